//! `Mdct1D<T, F>` (reference: src/mdct1d.rs:30-292). The window table is
//! evaluated on the host from `window_func(len, i)` exactly as the
//! reference's calc_window does (src/mdct1d.rs:91-93) and handed to the
//! library as a custom window.
use std::marker::PhantomData;
use std::os::raw::c_int;

use num_traits::cast;

use crate::{ffi, GpuFloat, Handle};

/// sin(pi (p + 1/2) / l), the reference's sine window (src/mdct1d.rs:42-44).
fn sine_window<T: GpuFloat>(l: usize, p: usize) -> T {
    (T::PI() * (cast::<_, T>(p).unwrap() + cast(0.5).unwrap()) / cast(l).unwrap()).sin()
}

/// sin(pi/2 sin^2(pi (p + 1/2) / l)), the Vorbis window (src/mdct1d.rs:46-53).
fn vorbis_window<T: GpuFloat>(l: usize, p: usize) -> T {
    let s = (T::PI() * (cast::<_, T>(p).unwrap() + cast(0.5).unwrap()) / cast(l).unwrap()).sin();
    (s.powi(2) * T::PI() * cast(0.5).unwrap()).sin()
}

pub struct Mdct1D<T, F: Fn(usize, usize) -> T> {
    plan: Handle,
    len: usize,
    window_func: F,
    _t: PhantomData<T>,
}

impl<T: GpuFloat> Mdct1D<T, fn(usize, usize) -> T> {
    /// src/mdct1d.rs:62
    pub fn with_sine(len: usize) -> Self {
        Self::new(sine_window::<T>, len)
    }

    /// src/mdct1d.rs:72
    pub fn with_vorbis(len: usize) -> Self {
        Self::new(vorbis_window::<T>, len)
    }
}

impl<T: GpuFloat, F: Fn(usize, usize) -> T> Mdct1D<T, F> {
    fn table(window_func: &F, len: usize) -> Vec<T> {
        (0..len).map(|i| window_func(len, i)).collect()
    }

    /// src/mdct1d.rs:101; panics "invalid length" unless 4 divides `len`.
    pub fn new(window_func: F, len: usize) -> Self {
        if len & 3 != 0 {
            panic!("invalid length")
        }
        let w = Self::table(&window_func, len);
        let plan = Handle::create(|p| unsafe {
            ffi::chfft_mdct1d_create(T::DTYPE, len, ffi::WINDOW_CUSTOM, w.as_ptr().cast(), p)
        });
        Mdct1D { plan, len, window_func, _t: PhantomData }
    }

    /// src/mdct1d.rs:126
    pub fn setup(&mut self, len: usize) {
        if len & 3 != 0 {
            panic!("invalid length")
        }
        let w = Self::table(&self.window_func, len);
        ffi::check(unsafe { ffi::chfft_plan_setup(self.plan.0, len, w.as_ptr().cast()) });
        self.len = len;
    }

    fn run(&mut self, method: c_int, source: &[T], out_len: usize) -> Vec<T> {
        let mut out = vec![T::zero(); out_len];
        ffi::check(unsafe {
            ffi::chfft_execute(self.plan.0, method, source.as_ptr().cast(), source.len(),
                               out.as_mut_ptr().cast(), out.len())
        });
        out
    }

    /// N windowed samples -> N/2 coefficients, unnormalised (src/mdct1d.rs:149).
    pub fn forward(&mut self, source: &[T]) -> Vec<T> {
        self.run(ffi::FORWARD, source, self.len >> 1)
    }
    /// N/2 coefficients -> N windowed samples (src/mdct1d.rs:164).
    pub fn backward(&mut self, source: &[T]) -> Vec<T> {
        self.run(ffi::BACKWARD, source, self.len)
    }
    pub fn forwardu(&mut self, source: &[T]) -> Vec<T> {
        self.run(ffi::FORWARDU, source, self.len >> 1)
    }
    pub fn backwardu(&mut self, source: &[T]) -> Vec<T> {
        self.run(ffi::BACKWARDU, source, self.len)
    }
}
