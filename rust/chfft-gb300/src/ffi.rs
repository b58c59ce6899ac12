//! Declarations of the C ABI in include/chfft_gpu.h that the plan types use.
use std::os::raw::{c_char, c_int, c_void};

#[repr(C)]
pub struct PlanS {
    _private: [u8; 0],
}
pub type Plan = *mut PlanS;

pub const F32: c_int = 0;
pub const F64: c_int = 1;

pub const OK: c_int = 0;
pub const EINVAL_LEN: c_int = 1;

pub const FORWARD: c_int = 0;
pub const FORWARD0: c_int = 1;
pub const FORWARDU: c_int = 2;
pub const FORWARDN: c_int = 3;
pub const BACKWARD: c_int = 4;
pub const BACKWARD0: c_int = 5;
pub const BACKWARDU: c_int = 6;
pub const BACKWARDN: c_int = 7;
pub const FORWARD0I: c_int = 8;
pub const BACKWARD0I: c_int = 9;
pub const FORWARDUI: c_int = 10;
pub const BACKWARDUI: c_int = 11;

pub const DCT_TWO: c_int = 2;
pub const DCT_THREE: c_int = 3;

pub const WINDOW_CUSTOM: c_int = 2;

extern "C" {
    pub fn chfft_cfft1d_create(dtype: c_int, len: usize, out: *mut Plan) -> c_int;
    pub fn chfft_cfft2d_create(dtype: c_int, len_m: usize, len_n: usize, out: *mut Plan) -> c_int;
    pub fn chfft_rfft1d_create(dtype: c_int, len: usize, out: *mut Plan) -> c_int;
    pub fn chfft_dct1d_create(dtype: c_int, dct_type: c_int, len: usize, is_ortho: c_int, out: *mut Plan) -> c_int;
    pub fn chfft_mdct1d_create(dtype: c_int, len: usize, window: c_int, table: *const c_void, out: *mut Plan)
        -> c_int;
    pub fn chfft_plan_destroy(plan: Plan) -> c_int;
    pub fn chfft_plan_setup(plan: Plan, len: usize, table: *const c_void) -> c_int;
    pub fn chfft_cfft2d_setup(plan: Plan, len_m: usize, len_n: usize) -> c_int;
    pub fn chfft_dct1d_setup(plan: Plan, dct_type: c_int, len: usize, is_ortho: c_int) -> c_int;
    pub fn chfft_execute(plan: Plan, method: c_int, src: *const c_void, src_len: usize, dst: *mut c_void,
                         dst_len: usize) -> c_int;
    pub fn chfft_execute_2d(plan: Plan, method: c_int, src: *const c_void, len_m: usize, len_n: usize,
                            dst: *mut c_void) -> c_int;
    pub fn chfft_last_error() -> *const c_char;
}

/// The reference's error behaviour: `panic!("invalid length")` for the
/// length errors (src/rfft1d.rs:75, src/dct1d.rs:55, src/mdct1d.rs:103),
/// a panic with the library's message for anything else (a CUDA error).
pub fn check(rc: c_int) {
    match rc {
        OK => {}
        EINVAL_LEN => panic!("invalid length"),
        _ => {
            let msg = unsafe { std::ffi::CStr::from_ptr(chfft_last_error()) };
            panic!("chfft_gb300: {}", msg.to_string_lossy())
        }
    }
}
