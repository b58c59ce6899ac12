//! chfft's public API (`CFft1D`, `CFft2D`, `RFft1D`, `Dct1D` + `DctType`,
//! `Mdct1D`; src/lib.rs:21-25 of chfft 0.3.4) as handles to GPU plans of
//! libchfft_gb300 (include/chfft_gpu.h). Names, constructors, `setup`,
//! method names, scaling, output types and panics are the reference's;
//! every transform runs on the GPU.
//!
//! ```no_run
//! use chfft::CFft1D;
//! use num_complex::Complex;
//! let input = [Complex::new(2.0, 0.0), Complex::new(1.0, 1.0),
//!              Complex::new(0.0, 3.0), Complex::new(2.0, 4.0)];
//! let mut fft = CFft1D::<f64>::with_len(input.len());
//! let output = fft.forward(&input);
//! ```
mod cfft1d;
mod cfft2d;
mod dct1d;
mod ffi;
mod mdct1d;
mod rfft1d;

pub use cfft1d::CFft1D;
pub use cfft2d::CFft2D;
pub use dct1d::{Dct1D, DctType};
pub use mdct1d::Mdct1D;
pub use rfft1d::RFft1D;

use std::os::raw::c_int;

/// The element types the GPU library has plans for (the reference's
/// `Float + FloatConst + NumAssign` bound, instantiated for f32 and f64).
pub trait GpuFloat: num_traits::Float + num_traits::FloatConst + num_traits::NumAssign + Copy + 'static {
    #[doc(hidden)]
    const DTYPE: c_int;
}

impl GpuFloat for f32 {
    const DTYPE: c_int = ffi::F32;
}

impl GpuFloat for f64 {
    const DTYPE: c_int = ffi::F64;
}

/// A plan handle: destroyed on drop. Plans are `Send` (the reference's are
/// plain data) and, like `&mut self` plans, not shared between threads.
struct Handle(ffi::Plan);

unsafe impl Send for Handle {}

impl Drop for Handle {
    fn drop(&mut self) {
        unsafe {
            ffi::chfft_plan_destroy(self.0);
        }
    }
}

impl Handle {
    fn create(f: impl FnOnce(*mut ffi::Plan) -> c_int) -> Self {
        let mut plan: ffi::Plan = std::ptr::null_mut();
        ffi::check(f(&mut plan));
        Handle(plan)
    }
}
