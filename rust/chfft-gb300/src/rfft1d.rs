//! `RFft1D<T>` (reference: src/rfft1d.rs:32-313): N reals <-> N/2 + 1 bins.
use std::marker::PhantomData;
use std::os::raw::c_int;

use num_complex::Complex;

use crate::{ffi, GpuFloat, Handle};

pub struct RFft1D<T> {
    plan: Handle,
    len: usize,
    _t: PhantomData<T>,
}

impl<T: GpuFloat> RFft1D<T> {
    /// src/rfft1d.rs:73; panics "invalid length" for an odd `len`.
    pub fn new(len: usize) -> Self {
        let plan = Handle::create(|p| unsafe { ffi::chfft_rfft1d_create(T::DTYPE, len, p) });
        RFft1D { plan, len, _t: PhantomData }
    }

    /// src/rfft1d.rs:101
    pub fn setup(&mut self, len: usize) {
        ffi::check(unsafe { ffi::chfft_plan_setup(self.plan.0, len, std::ptr::null()) });
        self.len = len;
    }

    fn run_fwd(&mut self, method: c_int, source: &[T]) -> Vec<Complex<T>> {
        let mut out = vec![Complex::new(T::zero(), T::zero()); (self.len >> 1) + 1];
        // The library checks source.len() against the plan: "invalid length".
        ffi::check(unsafe {
            ffi::chfft_execute(self.plan.0, method, source.as_ptr().cast(), source.len(),
                               out.as_mut_ptr().cast(), out.len())
        });
        out
    }

    fn run_back(&mut self, method: c_int, source: &[Complex<T>]) -> Vec<T> {
        let mut out = vec![T::zero(); self.len];
        ffi::check(unsafe {
            ffi::chfft_execute(self.plan.0, method, source.as_ptr().cast(), source.len(),
                               out.as_mut_ptr().cast(), out.len())
        });
        out
    }

    pub fn forward(&mut self, source: &[T]) -> Vec<Complex<T>> {
        self.run_fwd(ffi::FORWARD, source)
    }
    pub fn forward0(&mut self, source: &[T]) -> Vec<Complex<T>> {
        self.run_fwd(ffi::FORWARD0, source)
    }
    pub fn forwardu(&mut self, source: &[T]) -> Vec<Complex<T>> {
        self.run_fwd(ffi::FORWARDU, source)
    }
    pub fn forwardn(&mut self, source: &[T]) -> Vec<Complex<T>> {
        self.run_fwd(ffi::FORWARDN, source)
    }
    pub fn backward(&mut self, source: &[Complex<T>]) -> Vec<T> {
        self.run_back(ffi::BACKWARD, source)
    }
    pub fn backward0(&mut self, source: &[Complex<T>]) -> Vec<T> {
        self.run_back(ffi::BACKWARD0, source)
    }
    pub fn backwardu(&mut self, source: &[Complex<T>]) -> Vec<T> {
        self.run_back(ffi::BACKWARDU, source)
    }
    pub fn backwardn(&mut self, source: &[Complex<T>]) -> Vec<T> {
        self.run_back(ffi::BACKWARDN, source)
    }
}
