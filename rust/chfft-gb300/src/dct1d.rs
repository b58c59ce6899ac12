//! `Dct1D<T>` and `DctType` (reference: src/dct1d.rs:30-410).
use std::marker::PhantomData;
use std::os::raw::c_int;

use crate::{ffi, GpuFloat, Handle};

/// src/dct1d.rs:37-44
#[derive(Debug, Clone, Copy, PartialEq, Eq)]
pub enum DctType {
    /// DCT-II
    Two,
    /// DCT-III
    Three,
}

fn type_id(t: DctType) -> c_int {
    match t {
        DctType::Two => ffi::DCT_TWO,
        DctType::Three => ffi::DCT_THREE,
    }
}

pub struct Dct1D<T> {
    plan: Handle,
    len: usize,
    _t: PhantomData<T>,
}

impl<T: GpuFloat> Dct1D<T> {
    /// src/dct1d.rs:53; panics "invalid length" for an odd `len`.
    pub fn new(dct_type: DctType, len: usize, is_ortho: bool) -> Self {
        let plan = Handle::create(|p| unsafe {
            ffi::chfft_dct1d_create(T::DTYPE, type_id(dct_type), len, is_ortho as c_int, p)
        });
        Dct1D { plan, len, _t: PhantomData }
    }

    /// src/dct1d.rs:74
    pub fn setup(&mut self, dct_type: DctType, len: usize, is_ortho: bool) {
        ffi::check(unsafe { ffi::chfft_dct1d_setup(self.plan.0, type_id(dct_type), len, is_ortho as c_int) });
        self.len = len;
    }

    fn run(&mut self, method: c_int, source: &[T]) -> Vec<T> {
        let mut out = vec![T::zero(); self.len];
        ffi::check(unsafe {
            ffi::chfft_execute(self.plan.0, method, source.as_ptr().cast(), source.len(),
                               out.as_mut_ptr().cast(), out.len())
        });
        out
    }

    pub fn forward(&mut self, source: &[T]) -> Vec<T> {
        self.run(ffi::FORWARD, source)
    }
    pub fn forward0(&mut self, source: &[T]) -> Vec<T> {
        self.run(ffi::FORWARD0, source)
    }
    pub fn forwardu(&mut self, source: &[T]) -> Vec<T> {
        self.run(ffi::FORWARDU, source)
    }
    pub fn forwardn(&mut self, source: &[T]) -> Vec<T> {
        self.run(ffi::FORWARDN, source)
    }
}
