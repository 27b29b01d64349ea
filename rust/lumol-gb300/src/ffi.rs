//! Raw declarations of the C ABI of `include/lumol_gb300.h` (same names, same
//! layouts).  Everything here is `unsafe`; `engine.rs` wraps it.
#![allow(non_camel_case_types, dead_code)]
use std::os::raw::{c_char, c_void};

pub const LG_OK: i32 = 0;
pub const LG_ERR_ARGUMENT: i32 = 1;
pub const LG_ERR_CUDA: i32 = 2;
pub const LG_ERR_STATE: i32 = 3;
pub const LG_ERR_CAPACITY: i32 = 4;
pub const LG_ERR_NONFINITE: i32 = 5;
pub const LG_ERR_NO_DEVICE: i32 = 6;

pub const LG_PAIR_ABSENT: i32 = 0;
pub const LG_PAIR_NULL: i32 = 1;
pub const LG_PAIR_LJ: i32 = 2;
pub const LG_PAIR_BUCKINGHAM: i32 = 3;
pub const LG_PAIR_HARMONIC: i32 = 4;
pub const LG_PAIR_BMH: i32 = 5;
pub const LG_PAIR_MORSE: i32 = 6;
pub const LG_PAIR_GAUSSIAN: i32 = 7;
pub const LG_PAIR_MIE: i32 = 8;

pub const LG_RESTRICT_NONE: i32 = 0;
pub const LG_RESTRICT_INTRA: i32 = 1;
pub const LG_RESTRICT_INTER: i32 = 2;
pub const LG_RESTRICT_EXCLUDE12: i32 = 3;
pub const LG_RESTRICT_EXCLUDE13: i32 = 4;
pub const LG_RESTRICT_EXCLUDE14: i32 = 5;
pub const LG_RESTRICT_SCALE14: i32 = 6;

pub const LG_COULOMB_NONE: i32 = 0;
pub const LG_COULOMB_EWALD: i32 = 1;
pub const LG_COULOMB_WOLF: i32 = 2;

pub const LG_PRECISION_FP64: i32 = 0;
pub const LG_PRECISION_MIXED: i32 = 1;

pub const LG_TERM_PAIRS: u32 = 1;
pub const LG_TERM_TAIL: u32 = 2;
pub const LG_TERM_BONDS: u32 = 4;
pub const LG_TERM_ANGLES: u32 = 8;
pub const LG_TERM_COUL_REAL: u32 = 16;
pub const LG_TERM_COUL_SELF: u32 = 32;
pub const LG_TERM_COUL_KSPACE: u32 = 64;
pub const LG_TERM_DIHEDRALS: u32 = 128;
pub const LG_TERM_ALL: u32 = 255;

pub const LG_WANT_FORCES: u32 = 1;
pub const LG_WANT_ENERGY: u32 = 2;
pub const LG_WANT_VIRIAL: u32 = 4;

pub const LG_INTEGRATOR_VELOCITY_VERLET: i32 = 0;
pub const LG_INTEGRATOR_VERLET: i32 = 1;
pub const LG_INTEGRATOR_LEAP_FROG: i32 = 2;
pub const LG_THERMOSTAT_NONE: i32 = 0;
pub const LG_THERMOSTAT_BERENDSEN: i32 = 1;
pub const LG_THERMOSTAT_RESCALE: i32 = 2;
pub const LG_THERMOSTAT_CSVR: i32 = 3;
pub const LG_CONTROL_REMOVE_TRANSLATION: u32 = 1;
pub const LG_CONTROL_REWRAP: u32 = 2;
pub const LG_CONTROL_REMOVE_ROTATION: u32 = 4;
pub const LG_BAROSTAT_NONE: i32 = 0;
pub const LG_BAROSTAT_BERENDSEN: i32 = 1;

pub const LG_SYNC_DOWNLOAD: u32 = 1;
pub const LG_SYNC_TRUST_HOST: u32 = 2;
pub const LG_SYS_NONFINITE: u32 = 1;

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct lg_pair {
    pub kind: i32,
    pub shifted: i32,
    pub restriction: i32,
    pub tail: i32,
    pub p0: f64,
    pub p1: f64,
    pub p2: f64,
    pub cutoff: f64,
    pub scale14: f64,
    pub p3: f64,
    pub p4: f64,
    pub table_size: i32,
    pub table_pad: i32,
    pub table_max: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct lg_bonded {
    pub kind: i32,
    pub n: i32,
    pub k: f64,
    pub x0: f64,
    pub a: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct lg_coulomb {
    pub kind: i32,
    pub restriction: i32,
    pub kmax: i32,
    pub pad: i32,
    pub cutoff: f64,
    pub alpha: f64,
    pub scale14: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct lg_options {
    pub device: i32,
    pub precision: i32,
    pub skin: f64,
    pub threads_per_atom: i32,
    pub flags: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct lg_md_params {
    pub integrator: i32,
    pub thermostat: i32,
    pub timestep: f64,
    pub temperature: f64,
    pub tau: f64,
    pub tolerance: f64,
    pub seed: u64,
    pub controls: u32,
    pub reserved: u32,
}

#[repr(C)]
pub struct lg_engine {
    _private: [u8; 0],
}

extern "C" {
    pub fn lg_version() -> i32;
    pub fn lg_last_error(engine: *const lg_engine) -> *const c_char;
    pub fn lg_create(options: *const lg_options, n_systems: i32, engine: *mut *mut lg_engine) -> i32;
    pub fn lg_destroy(engine: *mut lg_engine);

    pub fn lg_set_cell(e: *mut lg_engine, s: i32, matrix: *const f64) -> i32;
    pub fn lg_set_particles(e: *mut lg_engine, s: i32, n: i64, kinds: *const i32, charges: *const f64,
                            masses: *const f64, molecules: *const i32) -> i32;
    pub fn lg_set_bonds(e: *mut lg_engine, s: i32, n: i64, bonds: *const i32, pots: *const lg_bonded) -> i32;
    pub fn lg_set_angles(e: *mut lg_engine, s: i32, n: i64, angles: *const i32, pots: *const lg_bonded) -> i32;
    pub fn lg_set_dihedrals(e: *mut lg_engine, s: i32, n: i64, dihedrals: *const i32, pots: *const lg_bonded)
                            -> i32;
    pub fn lg_set_pairs(e: *mut lg_engine, s: i32, n_kinds: i32, table: *const lg_pair) -> i32;
    pub fn lg_set_coulomb(e: *mut lg_engine, s: i32, coulomb: *const lg_coulomb) -> i32;

    pub fn lg_compute(e: *mut lg_engine, s: i32, positions: *const f64, terms: u32, want: u32, forces: *mut f64,
                      energy: *mut f64, virial: *mut f64) -> i32;
    pub fn lg_molecular_virial(e: *mut lg_engine, s: i32, positions: *const f64, terms: u32, virial: *mut f64)
                               -> i32;

    pub fn lg_md_setup_ex(e: *mut lg_engine, s: i32, params: *const lg_md_params) -> i32;
    pub fn lg_md_set_barostat(e: *mut lg_engine, s: i32, kind: i32, pressure: f64, tau: f64) -> i32;
    pub fn lg_get_cell(e: *mut lg_engine, s: i32, matrix: *mut f64) -> i32;
    pub fn lg_md_set_state(e: *mut lg_engine, s: i32, positions: *const f64, velocities: *const f64) -> i32;
    pub fn lg_md_get_state(e: *mut lg_engine, s: i32, positions: *mut f64, velocities: *mut f64) -> i32;
    pub fn lg_md_run(e: *mut lg_engine, nsteps: i64) -> i32;
    pub fn lg_md_integrate(e: *mut lg_engine, positions: *mut f64, velocities: *mut f64, nsteps: i64) -> i32;
    pub fn lg_md_propagate(e: *mut lg_engine, positions: *mut f64, velocities: *mut f64, nsteps: i64,
                           flags: u32) -> i32;
    pub fn lg_system_status(e: *mut lg_engine, flags: *mut u32, clear: i32) -> i32;

    pub fn lg_mc_init(e: *mut lg_engine, s: i32, positions: *const f64, energy: *mut f64) -> i32;
    pub fn lg_mc_move_molecule_cost(e: *mut lg_engine, s: i32, molecule: i64, new_positions: *const f64,
                                    cost: *mut f64) -> i32;
    pub fn lg_mc_move_all_molecules_cost(e: *mut lg_engine, s: i32, new_cell: *const f64,
                                         new_positions: *const f64, cost: *mut f64) -> i32;
    pub fn lg_mc_update(e: *mut lg_engine, s: i32, molecule_positions: *const f64, energy: *mut f64) -> i32;
    pub fn lg_mc_restore(e: *mut lg_engine, s: i32) -> i32;

    pub fn lg_ewald_kspace_noalloc(d_positions: *const f64, d_charges: *const f64, n: i64,
                                   cell_lengths: *const f64, alpha: f64, kmax: i32, d_forces: *mut f64,
                                   d_energy: *mut f64, d_virial: *mut f64, stream: *mut c_void) -> i32;
}
