//! `CFft1D<T>` (reference: src/cfft1d.rs:53-468).
use std::marker::PhantomData;
use std::os::raw::c_int;

use num_complex::Complex;

use crate::{ffi, GpuFloat, Handle};

pub struct CFft1D<T> {
    plan: Handle,
    #[allow(dead_code)]
    len: usize,
    _t: PhantomData<T>,
}

impl<T: GpuFloat> CFft1D<T> {
    /// A plan with no length yet (src/cfft1d.rs:68).
    pub fn new() -> Self {
        Self::with_len(0)
    }

    /// A plan for `len` points (src/cfft1d.rs:83).
    pub fn with_len(len: usize) -> Self {
        let plan = Handle::create(|p| unsafe { ffi::chfft_cfft1d_create(T::DTYPE, len, p) });
        CFft1D { plan, len, _t: PhantomData }
    }

    /// Re-plan for `len` points (src/cfft1d.rs:103).
    pub fn setup(&mut self, len: usize) {
        ffi::check(unsafe { ffi::chfft_plan_setup(self.plan.0, len, std::ptr::null()) });
        self.len = len;
    }

    fn run(&mut self, method: c_int, source: &[Complex<T>]) -> Vec<Complex<T>> {
        // num-complex's Complex<T> is #[repr(C)] {re, im}: the C ABI's layout.
        let mut out = vec![Complex::new(T::zero(), T::zero()); source.len()];
        ffi::check(unsafe {
            ffi::chfft_execute(self.plan.0, method, source.as_ptr().cast(), source.len(),
                               out.as_mut_ptr().cast(), out.len())
        });
        self.len = source.len(); // a new length re-plans (src/cfft1d.rs:216-218)
        out
    }

    fn run_inplace(&mut self, method: c_int, source: &mut [Complex<T>]) {
        ffi::check(unsafe {
            ffi::chfft_execute(self.plan.0, method, source.as_ptr().cast(), source.len(),
                               source.as_mut_ptr().cast(), source.len())
        });
        self.len = source.len();
    }

    pub fn forward(&mut self, source: &[Complex<T>]) -> Vec<Complex<T>> {
        self.run(ffi::FORWARD, source)
    }
    pub fn forward0(&mut self, source: &[Complex<T>]) -> Vec<Complex<T>> {
        self.run(ffi::FORWARD0, source)
    }
    pub fn forwardu(&mut self, source: &[Complex<T>]) -> Vec<Complex<T>> {
        self.run(ffi::FORWARDU, source)
    }
    pub fn forwardn(&mut self, source: &[Complex<T>]) -> Vec<Complex<T>> {
        self.run(ffi::FORWARDN, source)
    }
    pub fn backward(&mut self, source: &[Complex<T>]) -> Vec<Complex<T>> {
        self.run(ffi::BACKWARD, source)
    }
    pub fn backward0(&mut self, source: &[Complex<T>]) -> Vec<Complex<T>> {
        self.run(ffi::BACKWARD0, source)
    }
    pub fn backwardu(&mut self, source: &[Complex<T>]) -> Vec<Complex<T>> {
        self.run(ffi::BACKWARDU, source)
    }
    pub fn backwardn(&mut self, source: &[Complex<T>]) -> Vec<Complex<T>> {
        self.run(ffi::BACKWARDN, source)
    }
    pub fn forward0i(&mut self, source: &mut [Complex<T>]) {
        self.run_inplace(ffi::FORWARD0I, source)
    }
    pub fn backward0i(&mut self, source: &mut [Complex<T>]) {
        self.run_inplace(ffi::BACKWARD0I, source)
    }
    pub fn forwardui(&mut self, source: &mut [Complex<T>]) {
        self.run_inplace(ffi::FORWARDUI, source)
    }
    pub fn backwardui(&mut self, source: &mut [Complex<T>]) {
        self.run_inplace(ffi::BACKWARDUI, source)
    }
}

impl<T: GpuFloat> Default for CFft1D<T> {
    fn default() -> Self {
        Self::new()
    }
}
