//! Monte Carlo on the engine (lumol-sim/src/mc/moves/mod.rs:44-84): moves whose
//! cost goes through `EnergyCache`, which reaches `GpuPairs` (the engine's
//! cache) through the GlobalCache hooks, and the NPT `Resize` move, whose cost
//! is the engine's `move_all_molecules_cost` (sys/cache.rs:238-292).
use rand::distributions::{Distribution, Uniform};
use rand::RngCore;

use lumol_core::{EnergyCache, Matrix3, System, Vector3D};
use lumol_sim::mc::{MCDegreeOfFreedom, MCMove};

use crate::engine::{as_f64, Shared};
use crate::ffi::*;

/// Resize::new(pressure, delta) (mc/moves/resize.rs:14-128) with the energy
/// change computed on the engine.  `prepare` changes the System as the
/// reference does (cell scaled by cbrt((V + delta) / V), molecules moved with
/// their centres of mass); `cost` installs that configuration on the engine;
/// `apply` keeps it (`lg_mc_update`), `restore` puts the previous one back on
/// both sides (`lg_mc_restore`).
pub struct GpuResize {
    engine: Shared,
    pressure: f64,
    delta: f64,
    range: Uniform<f64>,
    previous: Option<(lumol_core::UnitCell, Vec<Vector3D>)>,
    maximum_cutoff: Option<f64>,
}

impl GpuResize {
    pub fn new(engine: Shared, pressure: f64, delta: f64) -> GpuResize {
        assert!(delta > 0.0, "delta must be positive in Resize move");
        GpuResize { engine, pressure, delta, range: Uniform::new(-delta, delta), previous: None, maximum_cutoff: None }
    }
}

impl MCMove for GpuResize {
    fn describe(&self) -> &str {
        "resizing of the cell"
    }

    fn setup(&mut self, system: &System) {
        assert!(!system.cell.is_infinite(), "cannot use `Resize` move with infinite simulation cell");
        self.maximum_cutoff = system.maximum_cutoff();
    }

    fn degrees_of_freedom(&self) -> MCDegreeOfFreedom {
        MCDegreeOfFreedom::AllMolecules
    }

    fn prepare(&mut self, system: &mut System, rng: &mut dyn RngCore) -> bool {
        let delta = self.range.sample(rng);
        let old_cell = system.cell;
        self.previous = Some((old_cell, system.particles().position.to_vec()));
        let volume = system.volume();
        let scaling_factor = f64::cbrt((volume + delta) / volume);
        system.cell.scale_mut(Matrix3::one() * scaling_factor);
        let cell = system.cell;
        for mut molecule in system.molecules_mut() {
            let old_com = molecule.as_ref().center_of_mass();
            let delta_com = cell.cartesian(&old_cell.fractional(&old_com)) - old_com;
            for position in molecule.particles_mut().position.iter_mut() {
                *position += delta_com;
            }
        }
        true
    }

    fn cost(&self, system: &System, beta: f64, cache: &mut EnergyCache) -> f64 {
        // the engine keeps the cache: Lumol's EnergyCache is not used for this move
        cache.unused();
        let engine = self.engine.lock();
        let m = system.cell.matrix();
        let matrix = [m[0][0], m[0][1], m[0][2], m[1][0], m[1][1], m[1][2], m[2][0], m[2][1], m[2][2]];
        let mut delta_energy = 0.0;
        engine.check(unsafe {
            lg_mc_move_all_molecules_cost(engine.raw(), 0, matrix.as_ptr(), as_f64(system.particles().position),
                                          &mut delta_energy)
        });
        let old_volume = self.previous.as_ref().expect("prepare before cost").0.volume();
        let new_volume = system.volume();
        beta * (delta_energy + self.pressure * (new_volume - old_volume))
            - (system.molecules().count() as f64) * f64::ln(new_volume / old_volume)
    }

    fn apply(&mut self, _: &mut System) {
        let engine = self.engine.lock();
        let mut energy = 0.0;
        engine.check(unsafe { lg_mc_update(engine.raw(), 0, std::ptr::null(), &mut energy) });
    }

    fn restore(&mut self, system: &mut System) {
        let (cell, positions) = self.previous.take().expect("prepare before restore");
        system.cell = cell;
        for (position, old) in system.particles_mut().position.iter_mut().zip(positions) {
            *position = old;
        }
        let engine = self.engine.lock();
        engine.check(unsafe { lg_mc_restore(engine.raw(), 0) });
    }

    fn update_amplitude(&mut self, scaling_factor: Option<f64>) {
        if let Some(s) = scaling_factor {
            self.delta *= s;
            self.range = Uniform::new(-self.delta, self.delta);
        }
    }
}
