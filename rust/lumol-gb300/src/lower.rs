//! A Lumol `System` lowered into the engine: particles, cell, bonds, and the
//! pair table of the same TOML input (lumol-input/src/interactions/pairs.rs:57-139),
//! because `PairPotential` is an opaque `Box<dyn>` that cannot be downcast
//! (lumol-core/src/energy/mod.rs:134-163).  `check_pairs` then evaluates every
//! lowered pair on the engine and compares it with Lumol's own trait object.
use std::collections::BTreeMap;

use lumol_core::energy::PairInteraction;
use lumol_core::{System, Vector3D};

use crate::engine::{compute, Engine, Shared};
use crate::ffi::*;

/// One pair of the input's `[pairs]` table, as the engine takes it (the
/// parameter order of the INTEGRATION table: LJ sigma, epsilon; Buckingham a,
/// c, rho; ...).
#[derive(Clone, Copy)]
pub struct PairSpec {
    pub pair: lg_pair,
}

/// Creates an engine for `system` with the given pair table (kind names to
/// PairSpec) and options; the Coulomb potential is installed by
/// `potential::GpuCoulomb`.
pub fn lower(system: &System, pairs: &BTreeMap<(String, String), PairSpec>, options: lg_options) -> Shared {
    let engine = Engine::new(options);
    let n = system.size();
    let mut kinds_of: BTreeMap<String, i32> = BTreeMap::new();
    let mut kinds = Vec::with_capacity(n);
    for name in system.particles().name {
        let next = kinds_of.len() as i32;
        kinds.push(*kinds_of.entry(name.clone()).or_insert(next));
    }
    let charges: Vec<f64> = system.particles().charge.to_vec();
    let masses: Vec<f64> = system.particles().mass.to_vec();
    let mut molecules = vec![0i32; n];
    let mut bonds = Vec::new();
    for (m, molecule) in system.molecules().enumerate() {
        for i in molecule.indexes() {
            molecules[i] = m as i32;
        }
        for bond in molecule.bonds() {
            bonds.push(bond.i() as i32);
            bonds.push(bond.j() as i32);
        }
    }
    let cell = system.cell.matrix();
    let matrix = [cell[0][0], cell[0][1], cell[0][2], cell[1][0], cell[1][1], cell[1][2], cell[2][0], cell[2][1],
                  cell[2][2]];
    let nk = kinds_of.len();
    let mut table = vec![lg_pair::default(); nk * nk];
    for (a, ka) in &kinds_of {
        for (b, kb) in &kinds_of {
            let key = if a <= b { (a.clone(), b.clone()) } else { (b.clone(), a.clone()) };
            if let Some(spec) = pairs.get(&key) {
                table[(*ka as usize) * nk + *kb as usize] = spec.pair;
            }
        }
    }
    // bonds carry no potential here: Lumol's own loops keep the bonded terms;
    // the engine only derives the bond paths of the pair restrictions
    let none = vec![lg_bonded { kind: LG_PAIR_ABSENT, ..Default::default() }; bonds.len() / 2];
    engine.check(unsafe { lg_set_cell(engine.raw(), 0, matrix.as_ptr()) });
    engine.check(unsafe {
        lg_set_particles(engine.raw(), 0, n as i64, kinds.as_ptr(), charges.as_ptr(), masses.as_ptr(),
                         molecules.as_ptr())
    });
    engine.check(unsafe { lg_set_bonds(engine.raw(), 0, (bonds.len() / 2) as i64, bonds.as_ptr(), none.as_ptr()) });
    engine.check(unsafe { lg_set_pairs(engine.raw(), 0, nk as i32, table.as_ptr()) });
    Shared::new(engine)
}

/// The probe of the lowered pair table: for every pair of kinds, two atoms of
/// those kinds in an engine of their own at 16 distances up to the cutoff;
/// the engine's energy must equal `interaction.energy(r)` (pairs.rs:185-243)
/// to 1e-12 relative, or this panics (no silent fallback).
pub fn check_pairs(pairs: &BTreeMap<(String, String), (PairSpec, PairInteraction)>, options: lg_options) {
    for ((a, b), (spec, interaction)) in pairs {
        let engine = Engine::new(options);
        let length = 4.0 * spec.pair.cutoff + 10.0;
        let matrix = [length, 0.0, 0.0, 0.0, length, 0.0, 0.0, 0.0, length];
        let kinds = [0i32, if a == b { 0 } else { 1 }];
        let nk = if a == b { 1 } else { 2 };
        let table = vec![spec.pair; nk * nk];
        engine.check(unsafe { lg_set_cell(engine.raw(), 0, matrix.as_ptr()) });
        engine.check(unsafe {
            lg_set_particles(engine.raw(), 0, 2, kinds.as_ptr(), [0.0, 0.0].as_ptr(), [1.0, 1.0].as_ptr(),
                             [0, 1].as_ptr())
        });
        engine.check(unsafe { lg_set_pairs(engine.raw(), 0, nk as i32, table.as_ptr()) });
        for k in 1..=16 {
            let r = spec.pair.cutoff * (k as f64) / 16.5;
            let positions = [Vector3D::new(0.0, 0.0, 0.0), Vector3D::new(r, 0.0, 0.0)];
            let (energy, _) = compute(&engine, &positions, LG_TERM_PAIRS, LG_WANT_ENERGY, None);
            let expected = interaction.energy(r);
            let scale = expected.abs().max(1e-300);
            assert!((energy - expected).abs() <= 1e-12 * scale,
                    "the lowered pair potential ({}, {}) gives {} at r = {}, Lumol's gives {}",
                    a, b, energy, r, expected);
        }
    }
}
