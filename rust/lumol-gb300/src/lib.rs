//! Lumol on a GB300: the engine of `include/lumol_gb300.h` behind Lumol's own
//! plugin traits, so that a `Simulation` built from the same input runs
//! unchanged.
//!
//! * `potential::GpuPairs` (GlobalPotential + GlobalCache) carries the pair
//!   potentials, `potential::GpuCoulomb` (CoulombicPotential) Ewald or Wolf;
//!   both share one engine (`engine::Shared`).
//! * `md::GpuVelocityVerlet` is an `Integrator` for Lumol's own
//!   `MolecularDynamics`; `md::GpuMolecularDynamics` is a `Propagator` that
//!   runs integrator, thermostat, controls and barostat on the device and
//!   copies the state back only at the steps outputs read.
//! * `mc::GpuResize` is the NPT `Resize` move on the engine's cache.
//! * `lower` builds the engine from a `System` and the pair table of the same
//!   TOML input, and checks every lowered pair potential against Lumol's own
//!   trait object before use.
//!
//! The kernels are built for sm_103a by `build.rs`; there is no CPU fallback.
pub mod engine;
pub mod ffi;
pub mod lower;
pub mod mc;
pub mod md;
pub mod potential;

pub use engine::{Engine, Shared};
pub use lower::{lower, PairSpec};
