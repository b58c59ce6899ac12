//! `CFft2D<T>` (reference: src/cfft2d.rs:58-376): M rows of N points,
//! flattened row-major for the GPU and split back into rows.
use std::marker::PhantomData;
use std::os::raw::c_int;

use num_complex::Complex;

use crate::{ffi, GpuFloat, Handle};

pub struct CFft2D<T> {
    plan: Handle,
    #[allow(dead_code)]
    shape: (usize, usize),
    _t: PhantomData<T>,
}

impl<T: GpuFloat> CFft2D<T> {
    /// src/cfft2d.rs:75
    pub fn new() -> Self {
        Self::with_len(0, 0)
    }

    /// src/cfft2d.rs:93
    pub fn with_len(len_m: usize, len_n: usize) -> Self {
        let plan = Handle::create(|p| unsafe { ffi::chfft_cfft2d_create(T::DTYPE, len_m, len_n, p) });
        CFft2D { plan, shape: (len_m, len_n), _t: PhantomData }
    }

    /// src/cfft2d.rs:114
    pub fn setup(&mut self, len_m: usize, len_n: usize) {
        ffi::check(unsafe { ffi::chfft_cfft2d_setup(self.plan.0, len_m, len_n) });
        self.shape = (len_m, len_n);
    }

    fn run(&mut self, method: c_int, source: &[Vec<Complex<T>>]) -> Vec<Vec<Complex<T>>> {
        let m = source.len();
        if m == 0 {
            return Vec::new(); // src/cfft2d.rs:333-335
        }
        let n = source[0].len();
        let mut flat = Vec::with_capacity(m * n);
        for row in source {
            assert_eq!(row.len(), n, "rows of a 2-D transform have one length");
            flat.extend_from_slice(row);
        }
        let mut out = vec![Complex::new(T::zero(), T::zero()); m * n];
        ffi::check(unsafe {
            ffi::chfft_execute_2d(self.plan.0, method, flat.as_ptr().cast(), m, n, out.as_mut_ptr().cast())
        });
        self.shape = (m, n); // a new shape re-plans (src/cfft2d.rs:336-338)
        out.chunks(n.max(1)).map(|r| r.to_vec()).collect()
    }

    pub fn forward(&mut self, source: &[Vec<Complex<T>>]) -> Vec<Vec<Complex<T>>> {
        self.run(ffi::FORWARD, source)
    }
    pub fn forward0(&mut self, source: &[Vec<Complex<T>>]) -> Vec<Vec<Complex<T>>> {
        self.run(ffi::FORWARD0, source)
    }
    pub fn forwardu(&mut self, source: &[Vec<Complex<T>>]) -> Vec<Vec<Complex<T>>> {
        self.run(ffi::FORWARDU, source)
    }
    pub fn forwardn(&mut self, source: &[Vec<Complex<T>>]) -> Vec<Vec<Complex<T>>> {
        self.run(ffi::FORWARDN, source)
    }
    pub fn backward(&mut self, source: &[Vec<Complex<T>>]) -> Vec<Vec<Complex<T>>> {
        self.run(ffi::BACKWARD, source)
    }
    pub fn backward0(&mut self, source: &[Vec<Complex<T>>]) -> Vec<Vec<Complex<T>>> {
        self.run(ffi::BACKWARD0, source)
    }
    pub fn backwardu(&mut self, source: &[Vec<Complex<T>>]) -> Vec<Vec<Complex<T>>> {
        self.run(ffi::BACKWARDU, source)
    }
}

impl<T: GpuFloat> Default for CFft2D<T> {
    fn default() -> Self {
        Self::new()
    }
}
