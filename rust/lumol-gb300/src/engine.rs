//! A safe owner of one `lg_engine` handle, shared by the trait objects of
//! this crate through `Arc<Mutex<_>>` (a handle is not re-entrant; Lumol's
//! own SharedEwald serialises its cache the same way, ewald.rs:847-875).
use std::ffi::CStr;
use std::ptr;
use std::sync::{Arc, Mutex, MutexGuard};

use lumol_core::{Matrix3, Vector3D};

use crate::ffi::*;

/// The engine: a batch of one system (a Lumol `System`).
pub struct Engine {
    raw: *mut lg_engine,
}

// The handle is used under a Mutex only.
unsafe impl Send for Engine {}

impl Engine {
    /// `lg_create`: panics, as the reference does on invalid input, when no
    /// device is visible (the engine has no CPU fallback) or on a bad option.
    pub fn new(options: lg_options) -> Engine {
        let mut raw = ptr::null_mut();
        let status = unsafe { lg_create(&options, 1, &mut raw) };
        if status != LG_OK {
            panic!("{}", last_error(ptr::null()));
        }
        Engine { raw }
    }

    pub fn raw(&self) -> *mut lg_engine {
        self.raw
    }

    /// Turns a status into the reference's behaviour: a panic with the message.
    pub fn check(&self, status: i32) {
        if status != LG_OK {
            panic!("{}", last_error(self.raw));
        }
    }
}

impl Drop for Engine {
    fn drop(&mut self) {
        unsafe { lg_destroy(self.raw) };
    }
}

pub fn last_error(raw: *const lg_engine) -> String {
    unsafe {
        let msg = lg_last_error(raw);
        if msg.is_null() {
            String::from("lumol-gb300: unknown error")
        } else {
            CStr::from_ptr(msg).to_string_lossy().into_owned()
        }
    }
}

/// The engine shared between the potentials, the integrator and the moves.
#[derive(Clone)]
pub struct Shared(pub Arc<Mutex<Engine>>);

impl Shared {
    pub fn new(engine: Engine) -> Shared {
        Shared(Arc::new(Mutex::new(engine)))
    }

    pub fn lock(&self) -> MutexGuard<'_, Engine> {
        self.0.lock().expect("lumol-gb300 engine mutex poisoned")
    }
}

/// `&[Vector3D]` as the 3n doubles the C ABI reads (`Vector3D` is a single
/// `[f64; 3]` field, lumol-core/src/types/vectors.rs:59).
pub fn as_f64(v: &[Vector3D]) -> *const f64 {
    v.as_ptr() as *const f64
}

pub fn as_f64_mut(v: &mut [Vector3D]) -> *mut f64 {
    v.as_mut_ptr() as *mut f64
}

/// A row-major `Matrix3` (lumol-core/src/types/matrix.rs:73) from 9 doubles.
pub fn matrix(m: &[f64; 9]) -> Matrix3 {
    Matrix3::new([[m[0], m[1], m[2]], [m[3], m[4], m[5]], [m[6], m[7], m[8]]])
}

/// One `lg_compute` call of system 0: `(forces accumulated into `forces` when
/// given, energy, virial)`.
pub fn compute(engine: &Engine, positions: &[Vector3D], terms: u32, want: u32,
               forces: Option<&mut [Vector3D]>) -> (f64, Matrix3) {
    let mut energy = 0.0;
    let mut virial = [0.0; 9];
    let f = match forces {
        Some(f) => as_f64_mut(f),
        None => ptr::null_mut(),
    };
    engine.check(unsafe {
        lg_compute(engine.raw(), 0, as_f64(positions), terms, want, f, &mut energy, virial.as_mut_ptr())
    });
    (energy, matrix(&virial))
}
