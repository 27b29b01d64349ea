//! Molecular dynamics on the engine: an `Integrator` for drop-in use inside
//! Lumol's own `MolecularDynamics`, and a `Propagator` that keeps the state
//! on the device between the steps the outputs read
//! (lumol-sim/src/md/integrators.rs:10-17, lumol-sim/src/propagator.rs:24-44).
use lumol_core::{DegreesOfFreedom, System, UnitCell};
use lumol_sim::md::Integrator;
use lumol_sim::propagator::{Propagator, TemperatureStrategy};

use crate::engine::{as_f64_mut, Shared};
use crate::ffi::*;

/// VelocityVerlet (integrators.rs:19-70) on the engine.  Every `integrate`
/// call is one step through `lg_md_integrate`: the host arrays are uploaded
/// only when a thermostat, control or user changed them on the host, and the
/// new state is copied back so that Lumol's host thermostats, controls and
/// outputs see it.
pub struct GpuVelocityVerlet {
    engine: Shared,
    timestep: f64,
}

impl GpuVelocityVerlet {
    pub fn new(engine: Shared, timestep: f64) -> GpuVelocityVerlet {
        GpuVelocityVerlet { engine, timestep }
    }
}

impl Integrator for GpuVelocityVerlet {
    /// VelocityVerlet::setup: accelerations := 0 (integrators.rs:40-42).
    fn setup(&mut self, _: &System) {
        let params = lg_md_params {
            integrator: LG_INTEGRATOR_VELOCITY_VERLET,
            timestep: self.timestep,
            ..Default::default()
        };
        let engine = self.engine.lock();
        engine.check(unsafe { lg_md_setup_ex(engine.raw(), 0, &params) });
    }

    fn integrate(&mut self, system: &mut System) {
        let engine = self.engine.lock();
        let particles = system.particles_mut();
        engine.check(unsafe {
            lg_md_integrate(engine.raw(), as_f64_mut(particles.position), as_f64_mut(particles.velocity), 1)
        });
    }
}

/// What the device propagator integrates with (md/integrators.rs,
/// md/thermostats.rs, md/controls.rs), lowered to lg_md_params once.
#[derive(Clone, Copy)]
pub struct DeviceDynamics {
    pub params: lg_md_params,
    /// BerendsenBarostat::new(timestep, pressure, tau): Some((pressure, tau))
    pub barostat: Option<(f64, f64)>,
}

/// MolecularDynamics (md/molecular_dynamics.rs:11-83) with its integrator,
/// thermostat and controls on the device, and lazy host synchronisation:
/// `Simulation::run` calls `propagate` once per step and lets the outputs
/// read `System` at the steps their frequency selects (simulations.rs:87-92);
/// this propagator copies the state back only at those steps (`sync_every`,
/// the outputs' smallest frequency); `sync` copies it on demand.
pub struct GpuMolecularDynamics {
    engine: Shared,
    dynamics: DeviceDynamics,
    sync_every: u64,
}

impl GpuMolecularDynamics {
    pub fn new(engine: Shared, dynamics: DeviceDynamics, sync_every: u64) -> GpuMolecularDynamics {
        GpuMolecularDynamics { engine, dynamics, sync_every: sync_every.max(1) }
    }
}

impl Propagator for GpuMolecularDynamics {
    fn temperature_strategy(&self) -> TemperatureStrategy {
        TemperatureStrategy::Velocities
    }

    fn degrees_of_freedom(&self, _: &System) -> DegreesOfFreedom {
        DegreesOfFreedom::Particles
    }

    fn setup(&mut self, _: &System) {
        let engine = self.engine.lock();
        engine.check(unsafe { lg_md_setup_ex(engine.raw(), 0, &self.dynamics.params) });
        if let Some((pressure, tau)) = self.dynamics.barostat {
            engine.check(unsafe { lg_md_set_barostat(engine.raw(), 0, LG_BAROSTAT_BERENDSEN, pressure, tau) });
        }
    }

    fn propagate(&mut self, system: &mut System) {
        // Simulation::run increments system.step after this call
        let next = system.step + 1;
        let flags = if next % self.sync_every == 0 { LG_SYNC_DOWNLOAD } else { 0 };
        let engine = self.engine.lock();
        {
            let particles = system.particles_mut();
            engine.check(unsafe {
                lg_md_propagate(engine.raw(), as_f64_mut(particles.position), as_f64_mut(particles.velocity), 1,
                                flags)
            });
        }
        if self.dynamics.barostat.is_some() && flags != 0 {
            let mut m = [0.0; 9];
            engine.check(unsafe { lg_get_cell(engine.raw(), 0, m.as_mut_ptr()) });
            system.cell = UnitCell::ortho(m[0], m[4], m[8]);
        }
    }

    // Propagator::finish takes `&System`, so the last state cannot be written
    // back here: a caller that reads the system after a run whose last step
    // is not an output step calls `sync`.
}

/// The device state copied into `system` (for callers of the propagator that
/// read the system between its output steps).
pub fn sync(engine: &Shared, system: &mut System) {
    let e = engine.lock();
    let particles = system.particles_mut();
    e.check(unsafe {
        lg_md_get_state(e.raw(), 0, as_f64_mut(particles.position), as_f64_mut(particles.velocity))
    });
}
