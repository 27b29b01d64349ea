//! `GlobalPotential` + `GlobalCache` + `CoulombicPotential` objects backed by
//! the engine (lumol-core/src/energy/global/mod.rs:84-202).
//!
//! Two objects share one engine: `GpuPairs` carries every pair potential of
//! the system (shift and tails included) and is registered with
//! `System::add_global_potential`, while the System's own pair table stays
//! empty, so sys/compute.rs:37-55 counts nothing twice; `GpuCoulomb` is the
//! `CoulombicPotential` registered with `System::set_coulomb_potential`
//! (Ewald or Wolf parameters of ewald.rs:278-305 / wolf.rs:68-84).  The terms
//! masks of `lg_compute` split the work between them.  Bonds, angles and
//! dihedral angles stay with Lumol's own host loops (the engine also knows
//! them, to derive the bond paths of the pair restrictions).
use lumol_core::energy::{CoulombicPotential, GlobalCache, GlobalPotential, PairRestriction};
use lumol_core::{Configuration, Matrix3, Vector3D};

use crate::engine::{as_f64, compute, Shared};
use crate::ffi::*;

const PAIR_TERMS: u32 = LG_TERM_PAIRS | LG_TERM_TAIL;
const COULOMB_TERMS: u32 = LG_TERM_COUL_REAL | LG_TERM_COUL_SELF | LG_TERM_COUL_KSPACE;

/// The pair potentials of a system on the engine.
#[derive(Clone)]
pub struct GpuPairs {
    pub(crate) engine: Shared,
    pub(crate) max_cutoff: f64,
}

impl GpuPairs {
    pub fn new(engine: Shared, max_cutoff: f64) -> GpuPairs {
        GpuPairs { engine, max_cutoff }
    }
}

impl GlobalPotential for GpuPairs {
    fn cutoff(&self) -> Option<f64> {
        Some(self.max_cutoff)
    }

    fn energy(&self, configuration: &Configuration) -> f64 {
        let engine = self.engine.lock();
        compute(&engine, configuration.particles().position, PAIR_TERMS, LG_WANT_ENERGY, None).0
    }

    /// Accumulates into `forces`, as GlobalPotential::forces does (ewald.rs:499).
    fn forces(&self, configuration: &Configuration, forces: &mut [Vector3D]) {
        let engine = self.engine.lock();
        compute(&engine, configuration.particles().position, PAIR_TERMS, LG_WANT_FORCES, Some(forces));
    }

    fn atomic_virial(&self, configuration: &Configuration) -> Matrix3 {
        let engine = self.engine.lock();
        compute(&engine, configuration.particles().position, PAIR_TERMS, LG_WANT_VIRIAL, None).1
    }

    fn molecular_virial(&self, configuration: &Configuration) -> Matrix3 {
        let engine = self.engine.lock();
        let mut virial = [0.0; 9];
        engine.check(unsafe {
            lg_molecular_virial(engine.raw(), 0, as_f64(configuration.particles().position), PAIR_TERMS,
                                virial.as_mut_ptr())
        });
        crate::engine::matrix(&virial)
    }
}

/// EnergyCache's GlobalCache hooks (cache.rs:180-186, 211-217): the engine
/// keeps its own cache, so both potentials' costs go through one call, made
/// by the pairs object; the Coulomb object returns zero for the same move.
impl GlobalCache for GpuPairs {
    fn move_molecule_cost(&self, _: &Configuration, molecule_id: usize, new_positions: &[Vector3D]) -> f64 {
        let engine = self.engine.lock();
        let mut cost = 0.0;
        engine.check(unsafe {
            lg_mc_move_molecule_cost(engine.raw(), 0, molecule_id as i64, as_f64(new_positions), &mut cost)
        });
        cost
    }

    fn update(&self) {
        let engine = self.engine.lock();
        let mut energy = 0.0;
        // the new positions were recorded by the cost call; the engine reads them there
        engine.check(unsafe { lg_mc_update(engine.raw(), 0, std::ptr::null(), &mut energy) });
    }
}

/// Ewald or Wolf summation on the engine.
#[derive(Clone)]
pub struct GpuCoulomb {
    pub(crate) engine: Shared,
    pub(crate) parameters: lg_coulomb,
}

impl GpuCoulomb {
    /// Ewald::new(cutoff, kmax, alpha) (ewald.rs:278-305); alpha None selects
    /// the reference's default pi / cutoff.
    pub fn ewald(engine: Shared, cutoff: f64, kmax: usize, alpha: Option<f64>) -> GpuCoulomb {
        let parameters = lg_coulomb {
            kind: LG_COULOMB_EWALD,
            kmax: kmax as i32,
            cutoff,
            alpha: alpha.unwrap_or(0.0),
            scale14: 1.0,
            ..Default::default()
        };
        GpuCoulomb::install(engine, parameters)
    }

    /// Wolf::new(cutoff) (wolf.rs:68-84).
    pub fn wolf(engine: Shared, cutoff: f64) -> GpuCoulomb {
        let parameters = lg_coulomb { kind: LG_COULOMB_WOLF, cutoff, scale14: 1.0, ..Default::default() };
        GpuCoulomb::install(engine, parameters)
    }

    fn install(engine: Shared, parameters: lg_coulomb) -> GpuCoulomb {
        {
            let e = engine.lock();
            e.check(unsafe { lg_set_coulomb(e.raw(), 0, &parameters) });
        }
        GpuCoulomb { engine, parameters }
    }
}

impl GlobalPotential for GpuCoulomb {
    fn cutoff(&self) -> Option<f64> {
        Some(self.parameters.cutoff)
    }

    fn energy(&self, configuration: &Configuration) -> f64 {
        let engine = self.engine.lock();
        compute(&engine, configuration.particles().position, COULOMB_TERMS, LG_WANT_ENERGY, None).0
    }

    fn forces(&self, configuration: &Configuration, forces: &mut [Vector3D]) {
        let engine = self.engine.lock();
        compute(&engine, configuration.particles().position, COULOMB_TERMS, LG_WANT_FORCES, Some(forces));
    }

    fn atomic_virial(&self, configuration: &Configuration) -> Matrix3 {
        let engine = self.engine.lock();
        compute(&engine, configuration.particles().position, COULOMB_TERMS, LG_WANT_VIRIAL, None).1
    }

    fn molecular_virial(&self, configuration: &Configuration) -> Matrix3 {
        let engine = self.engine.lock();
        let mut virial = [0.0; 9];
        engine.check(unsafe {
            lg_molecular_virial(engine.raw(), 0, as_f64(configuration.particles().position), COULOMB_TERMS,
                                virial.as_mut_ptr())
        });
        crate::engine::matrix(&virial)
    }
}

impl GlobalCache for GpuCoulomb {
    /// Counted in GpuPairs::move_molecule_cost (one engine call per move).
    fn move_molecule_cost(&self, _: &Configuration, _: usize, _: &[Vector3D]) -> f64 {
        0.0
    }

    fn update(&self) {}
}

impl CoulombicPotential for GpuCoulomb {
    /// CoulombicPotential::set_restriction (global/mod.rs:197-202).
    fn set_restriction(&mut self, restriction: PairRestriction) {
        let (kind, scale14) = match restriction {
            PairRestriction::None => (LG_RESTRICT_NONE, 1.0),
            PairRestriction::IntraMolecular => (LG_RESTRICT_INTRA, 1.0),
            PairRestriction::InterMolecular => (LG_RESTRICT_INTER, 1.0),
            PairRestriction::Exclude12 => (LG_RESTRICT_EXCLUDE12, 1.0),
            PairRestriction::Exclude13 => (LG_RESTRICT_EXCLUDE13, 1.0),
            PairRestriction::Exclude14 => (LG_RESTRICT_EXCLUDE14, 1.0),
            PairRestriction::Scale14(s) => (LG_RESTRICT_SCALE14, s),
        };
        self.parameters.restriction = kind;
        self.parameters.scale14 = scale14;
        let engine = self.engine.lock();
        engine.check(unsafe { lg_set_coulomb(engine.raw(), 0, &self.parameters) });
    }
}
