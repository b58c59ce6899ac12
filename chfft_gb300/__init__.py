"""chfft_gb300: chfft's transforms on GB300 (sm_103a) behind chfft's API.

Python mirror of chfft 0.3.4's public types (src/lib.rs:21-25):
``CFft1D``, ``CFft2D``, ``RFft1D``, ``Dct1D`` + ``DctType``, ``Mdct1D``, with
the same constructors, ``setup`` methods and method names (``forward``,
``forward0``, ``forwardu``, ``forwardn``, ``backward``... and the in-place
``forward0i``... of CFft1D). Each call goes through the C ABI of
libchfft_gb300.so (include/chfft_gpu.h) into hand-written CUDA kernels;
there is no CPU fallback, and importing fails loudly if the library is not
built. ``RuntimeError("invalid length")`` (as ``InvalidLength``) stands for
the reference's ``panic!("invalid length")``.

The element type follows the reference's generic parameter: ``dtype=np.float32``
is ``CFft1D::<f32>``, ``np.float64`` is ``CFft1D::<f64>``. Complex arrays are
numpy complex64/complex128 (interleaved re, im: num-complex's layout).

Beyond the reference's one-transform-per-call methods, every plan offers
``execute_batch`` (host arrays, many transforms) and ``execute_device``
(device pointers on a CUDA stream).
"""
from __future__ import annotations

import ctypes
import enum
import math
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libchfft_gb300.so")

# chfft_status
OK, EINVAL_LEN, EINVAL, EUNSUPPORTED, ECUDA, ENOMEM, ETIMEOUT = range(7)

METHODS = {
    "forward": 0, "forward0": 1, "forwardu": 2, "forwardn": 3,
    "backward": 4, "backward0": 5, "backwardu": 6, "backwardn": 7,
    "forward0i": 8, "backward0i": 9, "forwardui": 10, "backwardui": 11,
}
_BACKWARD = {"backward", "backward0", "backwardu", "backwardn", "backward0i", "backwardui"}

KIND_CFFT1D, KIND_CFFT2D, KIND_RFFT1D, KIND_DCT1D, KIND_MDCT1D, KIND_CFFT3D = range(6)


class ChfftError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class InvalidLength(ChfftError, ValueError):
    """The reference's ``panic!("invalid length")``."""


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int), ("dtype", ctypes.c_int),
        ("len", ctypes.c_size_t), ("len_m", ctypes.c_size_t), ("len_n", ctypes.c_size_t),
        ("fft_len", ctypes.c_size_t), ("algorithm", ctypes.c_int), ("padded_len", ctypes.c_size_t),
        ("npass", ctypes.c_int), ("radix", ctypes.c_int * 24),
        ("seq_per_cta", ctypes.c_int), ("threads_per_cta", ctypes.c_int), ("smem_per_cta", ctypes.c_size_t),
        ("in_elems", ctypes.c_size_t), ("out_elems", ctypes.c_size_t), ("device_bytes", ctypes.c_size_t),
        ("cluster_ctas", ctypes.c_int), ("cluster_n1", ctypes.c_size_t), ("cluster_n2", ctypes.c_size_t),
        ("cluster_max_batch", ctypes.c_size_t), ("len_l", ctypes.c_size_t),
    ]


_lib = None


def lib() -> ctypes.CDLL:
    """Load libchfft_gb300.so (built by chfft_gb300._build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m chfft_gb300._build`")
    L = ctypes.CDLL(LIB_PATH)
    sz, vp, i, pp = ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)
    sigs = {
        "chfft_cfft1d_create": [i, sz, pp],
        "chfft_cfft2d_create": [i, sz, sz, pp],
        "chfft_cfft3d_create": [i, sz, sz, sz, pp],
        "chfft_rfft1d_create": [i, sz, pp],
        "chfft_dct1d_create": [i, i, sz, i, pp],
        "chfft_mdct1d_create": [i, sz, i, vp, pp],
        "chfft_plan_destroy": [vp],
        "chfft_plan_setup": [vp, sz, vp],
        "chfft_cfft2d_setup": [vp, sz, sz],
        "chfft_dct1d_setup": [vp, i, sz, i],
        "chfft_execute": [vp, i, vp, sz, vp, sz],
        "chfft_execute_2d": [vp, i, vp, sz, sz, vp],
        "chfft_execute_3d": [vp, i, vp, sz, sz, sz, vp],
        "chfft_execute_device_split": [vp, i, vp, vp, vp, vp, sz, vp],
        "chfft_execute_device_strided": [vp, i, vp, sz, sz, vp, sz, sz, sz, vp],
        "chfft_execute_batch": [vp, i, vp, vp, sz],
        "chfft_execute_device": [vp, i, vp, vp, sz, vp],
        "chfft_plan_wait": [vp, vp],
        "chfft_plan_get_info": [vp, ctypes.POINTER(PlanInfo)],
        "chfft_factorize": [sz, sz, vp, vp, sz],
        "chfft_digit_reversal": [vp, vp, sz, vp, sz],
        "chfft_swap_list": [vp, sz, vp],
        "chfft_chirp_index_device": [sz, vp, vp],
    }
    for name, args in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    for name in ("chfft_last_error", "chfft_status_string", "chfft_version"):
        getattr(L, name).restype = ctypes.c_char_p
    L.chfft_status_string.argtypes = [ctypes.c_int]
    L.chfft_plan_compiler_available.restype = ctypes.c_int
    L.chfft_plan_compiler_cache_size.restype = ctypes.c_size_t
    _lib = L
    return L


def _check(rc: int):
    if rc == OK:
        return
    msg = lib().chfft_last_error().decode() or lib().chfft_status_string(rc).decode()
    if rc == EINVAL_LEN:
        raise InvalidLength(rc, msg if msg.startswith("invalid length") else "invalid length: " + msg)
    raise ChfftError(rc, msg)


def version() -> str:
    return lib().chfft_version().decode()


def plan_compiler_available() -> bool:
    """Whether plan-time specialised kernels (NVRTC) can be used (CHFFT_JIT selects when)."""
    return bool(lib().chfft_plan_compiler_available())


def plan_compiler_cache_size() -> int:
    """Specialised kernels compiled so far in this process."""
    return int(lib().chfft_plan_compiler_cache_size())


def _dtype_id(dtype) -> int:
    d = np.dtype(dtype)
    if d in (np.float32, np.complex64):
        return 0
    if d in (np.float64, np.complex128):
        return 1
    raise TypeError(f"unsupported dtype {d}")


def _real(did):
    return np.float32 if did == 0 else np.float64


def _cplx(did):
    return np.complex64 if did == 0 else np.complex128


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


class _Plan:
    kind = -1

    def __init__(self, dtype):
        self._did = _dtype_id(dtype)
        self._h = ctypes.c_void_p()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.chfft_plan_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def info(self) -> PlanInfo:
        out = PlanInfo()
        _check(lib().chfft_plan_get_info(self._h, ctypes.byref(out)))
        return out

    def _in_dtype(self, method):
        raise NotImplementedError

    def _out_dtype(self, method):
        raise NotImplementedError

    def _host(self, method: str, src, out_len: int):
        src = np.ascontiguousarray(src, self._in_dtype(method))
        out = np.empty(out_len, self._out_dtype(method))
        _check(lib().chfft_execute(self._h, METHODS[method], _ptr(src), src.shape[-1] if src.ndim else 0,
                                   _ptr(out), out_len))
        return out

    def execute_batch(self, method: str, src: np.ndarray) -> np.ndarray:
        """Many transforms on host memory: src has shape (batch, per-transform input)."""
        info = self.info()
        back = method in _BACKWARD
        src = np.ascontiguousarray(src, self._in_dtype(method))
        batch = src.shape[0]
        out_elems, in_elems = self._sizes(back)
        if src.size != batch * in_elems:
            raise InvalidLength(EINVAL_LEN, "invalid length")
        out = np.empty((batch, out_elems), self._out_dtype(method))
        _check(lib().chfft_execute_batch(self._h, METHODS[method], _ptr(src), _ptr(out), batch))
        del info
        return out

    def execute_device_split(self, method: str, d_re: int, d_im: int, d_out_re: int, d_out_im: int, batch: int,
                             stream: int = 0):
        """CFft1D on split-complex device arrays (real / imaginary parts apart)."""
        _check(lib().chfft_execute_device_split(self._h, METHODS[method], ctypes.c_void_p(d_re), ctypes.c_void_p(d_im),
                                                ctypes.c_void_p(d_out_re), ctypes.c_void_p(d_out_im), batch,
                                                ctypes.c_void_p(stream)))

    def execute_device_strided(self, method: str, d_src: int, istride: int, idist: int, d_dst: int, ostride: int,
                               odist: int, batch: int, stream: int = 0):
        """CFft1D on strided device layouts (element i of transform t at t * dist + i * stride)."""
        _check(lib().chfft_execute_device_strided(self._h, METHODS[method], ctypes.c_void_p(d_src), istride, idist,
                                                  ctypes.c_void_p(d_dst), ostride, odist, batch,
                                                  ctypes.c_void_p(stream)))

    def execute_device(self, method: str, d_src: int, d_dst: int, batch: int, stream: int = 0):
        """`batch` transforms on device pointers, enqueued on a CUDA stream handle."""
        _check(lib().chfft_execute_device(self._h, METHODS[method], ctypes.c_void_p(d_src), ctypes.c_void_p(d_dst),
                                          batch, ctypes.c_void_p(stream)))

    def wait(self, stream: int = 0):
        """Synchronise `stream`; raises (status ETIMEOUT) if a bounded device-side
        wait of this plan's launches gave up since the last check."""
        _check(lib().chfft_plan_wait(self._h, ctypes.c_void_p(stream)))

    def _sizes(self, back: bool):
        raise NotImplementedError


class CFft1D(_Plan):
    """CFft1D<T> (src/cfft1d.rs:53-468)."""

    kind = KIND_CFFT1D

    def __init__(self, len: int = 0, dtype=np.float64):
        super().__init__(dtype)
        self._len = len
        _check(lib().chfft_cfft1d_create(self._did, len, ctypes.byref(self._h)))

    @classmethod
    def new(cls, dtype=np.float64):
        return cls(0, dtype)

    @classmethod
    def with_len(cls, len: int, dtype=np.float64):
        return cls(len, dtype)

    def setup(self, len: int):
        _check(lib().chfft_plan_setup(self._h, len, None))
        self._len = len

    def _in_dtype(self, method):
        return _cplx(self._did)

    _out_dtype = _in_dtype

    def _sizes(self, back):
        return self._len, self._len

    def _run(self, method, source):
        source = np.ascontiguousarray(source, _cplx(self._did))
        n = source.shape[-1]
        out = np.empty(n, _cplx(self._did))
        _check(lib().chfft_execute(self._h, METHODS[method], _ptr(source), n, _ptr(out), n))
        self._len = n
        return out

    def _run_inplace(self, method, source: np.ndarray):
        if source.dtype != _cplx(self._did) or not source.flags.c_contiguous:
            raise TypeError("in-place methods need a contiguous array of the plan's complex dtype")
        n = source.shape[-1]
        _check(lib().chfft_execute(self._h, METHODS[method], _ptr(source), n, _ptr(source), n))
        self._len = n

    def forward(self, source): return self._run("forward", source)
    def forward0(self, source): return self._run("forward0", source)
    def forwardu(self, source): return self._run("forwardu", source)
    def forwardn(self, source): return self._run("forwardn", source)
    def backward(self, source): return self._run("backward", source)
    def backward0(self, source): return self._run("backward0", source)
    def backwardu(self, source): return self._run("backwardu", source)
    def backwardn(self, source): return self._run("backwardn", source)
    def forward0i(self, source): self._run_inplace("forward0i", source)
    def backward0i(self, source): self._run_inplace("backward0i", source)
    def forwardui(self, source): self._run_inplace("forwardui", source)
    def backwardui(self, source): self._run_inplace("backwardui", source)


class CFft2D(_Plan):
    """CFft2D<T> (src/cfft2d.rs:58-376); arrays are (len_m, len_n) row-major."""

    kind = KIND_CFFT2D

    def __init__(self, len_m: int = 0, len_n: int = 0, dtype=np.float64):
        super().__init__(dtype)
        self._shape = (len_m, len_n)
        _check(lib().chfft_cfft2d_create(self._did, len_m, len_n, ctypes.byref(self._h)))

    @classmethod
    def new(cls, dtype=np.float64):
        return cls(0, 0, dtype)

    @classmethod
    def with_len(cls, len_m: int, len_n: int, dtype=np.float64):
        return cls(len_m, len_n, dtype)

    def setup(self, len_m: int, len_n: int):
        _check(lib().chfft_cfft2d_setup(self._h, len_m, len_n))
        self._shape = (len_m, len_n)

    def _in_dtype(self, method):
        return _cplx(self._did)

    _out_dtype = _in_dtype

    def _sizes(self, back):
        return self._shape[0] * self._shape[1], self._shape[0] * self._shape[1]

    def _run(self, method, source):
        source = np.ascontiguousarray(source, _cplx(self._did))
        if source.size == 0:
            return np.empty((0, 0), _cplx(self._did))
        m, n = source.shape
        out = np.empty((m, n), _cplx(self._did))
        _check(lib().chfft_execute_2d(self._h, METHODS[method], _ptr(source), m, n, _ptr(out)))
        self._shape = (m, n)
        return out

    def forward(self, source): return self._run("forward", source)
    def forward0(self, source): return self._run("forward0", source)
    def forwardu(self, source): return self._run("forwardu", source)
    def forwardn(self, source): return self._run("forwardn", source)
    def backward(self, source): return self._run("backward", source)
    def backward0(self, source): return self._run("backward0", source)
    def backwardu(self, source): return self._run("backwardu", source)


class CFft3D(_Plan):
    """3-D complex transform of (len_l, len_m, len_n) row-major arrays: no
    reference counterpart (chfft stops at CFft2D); CFft2D's methods and
    scales extended by one axis."""

    kind = KIND_CFFT3D

    def __init__(self, len_l: int = 0, len_m: int = 0, len_n: int = 0, dtype=np.float64):
        super().__init__(dtype)
        self._shape = (len_l, len_m, len_n)
        _check(lib().chfft_cfft3d_create(self._did, len_l, len_m, len_n, ctypes.byref(self._h)))

    @classmethod
    def with_len(cls, len_l: int, len_m: int, len_n: int, dtype=np.float64):
        return cls(len_l, len_m, len_n, dtype)

    def _in_dtype(self, method):
        return _cplx(self._did)

    _out_dtype = _in_dtype

    def _sizes(self, back):
        n = self._shape[0] * self._shape[1] * self._shape[2]
        return n, n

    def _run(self, method, source):
        source = np.ascontiguousarray(source, _cplx(self._did))
        if source.size == 0:
            return np.empty(source.shape, _cplx(self._did))
        l, m, n = source.shape
        out = np.empty((l, m, n), _cplx(self._did))
        _check(lib().chfft_execute_3d(self._h, METHODS[method], _ptr(source), l, m, n, _ptr(out)))
        self._shape = (l, m, n)
        return out

    def forward(self, source): return self._run("forward", source)
    def forward0(self, source): return self._run("forward0", source)
    def forwardu(self, source): return self._run("forwardu", source)
    def forwardn(self, source): return self._run("forwardn", source)
    def backward(self, source): return self._run("backward", source)
    def backward0(self, source): return self._run("backward0", source)
    def backwardu(self, source): return self._run("backwardu", source)


class RFft1D(_Plan):
    """RFft1D<T> (src/rfft1d.rs:32-313): N reals <-> N/2+1 complex bins."""

    kind = KIND_RFFT1D

    def __init__(self, len: int, dtype=np.float64):
        super().__init__(dtype)
        self._len = len
        _check(lib().chfft_rfft1d_create(self._did, len, ctypes.byref(self._h)))

    @classmethod
    def new(cls, len: int, dtype=np.float64):
        return cls(len, dtype)

    def setup(self, len: int):
        _check(lib().chfft_plan_setup(self._h, len, None))
        self._len = len

    def _in_dtype(self, method):
        return _cplx(self._did) if method in _BACKWARD else _real(self._did)

    def _out_dtype(self, method):
        return _real(self._did) if method in _BACKWARD else _cplx(self._did)

    def _sizes(self, back):
        h = self._len // 2 + 1
        return (self._len, h) if back else (h, self._len)

    def forward(self, source): return self._host("forward", source, self._len // 2 + 1)
    def forward0(self, source): return self._host("forward0", source, self._len // 2 + 1)
    def forwardu(self, source): return self._host("forwardu", source, self._len // 2 + 1)
    def forwardn(self, source): return self._host("forwardn", source, self._len // 2 + 1)
    def backward(self, source): return self._host("backward", source, self._len)
    def backward0(self, source): return self._host("backward0", source, self._len)
    def backwardu(self, source): return self._host("backwardu", source, self._len)
    def backwardn(self, source): return self._host("backwardn", source, self._len)


class DctType(enum.IntEnum):
    """DctType (src/dct1d.rs:37-43)."""

    Two = 2
    Three = 3


class Dct1D(_Plan):
    """Dct1D<T> (src/dct1d.rs:30-410): DCT-II / DCT-III of even length."""

    kind = KIND_DCT1D

    def __init__(self, dct_type: DctType, len: int, is_ortho: bool, dtype=np.float64):
        super().__init__(dtype)
        self._len = len
        _check(lib().chfft_dct1d_create(self._did, int(dct_type), len, int(is_ortho), ctypes.byref(self._h)))

    @classmethod
    def new(cls, dct_type: DctType, len: int, is_ortho: bool, dtype=np.float64):
        return cls(dct_type, len, is_ortho, dtype)

    def setup(self, dct_type: DctType, len: int, is_ortho: bool):
        _check(lib().chfft_dct1d_setup(self._h, int(dct_type), len, int(is_ortho)))
        self._len = len

    def _in_dtype(self, method):
        return _real(self._did)

    _out_dtype = _in_dtype

    def _sizes(self, back):
        return self._len, self._len

    def forward(self, source): return self._host("forward", source, self._len)
    def forward0(self, source): return self._host("forward0", source, self._len)
    def forwardu(self, source): return self._host("forwardu", source, self._len)
    def forwardn(self, source): return self._host("forwardn", source, self._len)


def sine_window(l: int, p: int) -> float:
    """sine_window (src/mdct1d.rs:42-44)."""
    return math.sin(math.pi * (p + 0.5) / l)


def vorbis_window(l: int, p: int) -> float:
    """vorbis_window (src/mdct1d.rs:46-53)."""
    return math.sin(math.sin(math.pi * (p + 0.5) / l) ** 2 * math.pi * 0.5)


class Mdct1D(_Plan):
    """Mdct1D<T, F> (src/mdct1d.rs:30-292): MDCT N -> N/2, IMDCT N/2 -> N.

    ``Mdct1D(window_func, len)`` evaluates ``window_func(len, i)`` for i < len
    like the reference's calc_window (src/mdct1d.rs:91-93); ``with_sine`` and
    ``with_vorbis`` use the built-in windows generated on the GPU in FP64.
    """

    kind = KIND_MDCT1D

    def __init__(self, window_func, len: int, dtype=np.float64, _builtin: int | None = None):
        super().__init__(dtype)
        self._len = len
        self._wf = window_func
        self._builtin = _builtin
        if _builtin is not None:
            _check(lib().chfft_mdct1d_create(self._did, len, _builtin, None, ctypes.byref(self._h)))
        else:
            w = self._window(len)
            _check(lib().chfft_mdct1d_create(self._did, len, 2, _ptr(w) if w is not None else None,
                                             ctypes.byref(self._h)))

    def _window(self, len):
        if len % 4 or len == 0:
            raise InvalidLength(EINVAL_LEN, "invalid length")
        return np.array([self._wf(len, i) for i in range(len)], _real(self._did))

    @classmethod
    def new(cls, window_func, len: int, dtype=np.float64):
        return cls(window_func, len, dtype)

    @classmethod
    def with_sine(cls, len: int, dtype=np.float64):
        return cls(sine_window, len, dtype, _builtin=0)

    @classmethod
    def with_vorbis(cls, len: int, dtype=np.float64):
        return cls(vorbis_window, len, dtype, _builtin=1)

    def setup(self, len: int):
        w = None if self._builtin is not None else self._window(len)
        _check(lib().chfft_plan_setup(self._h, len, _ptr(w) if w is not None else None))
        self._len = len

    def _in_dtype(self, method):
        return _real(self._did)

    _out_dtype = _in_dtype

    def _sizes(self, back):
        return (self._len, self._len // 2) if back else (self._len // 2, self._len)

    def forward(self, source): return self._host("forward", source, self._len // 2)
    def forwardu(self, source): return self._host("forwardu", source, self._len // 2)
    def backward(self, source): return self._host("backward", source, self._len)
    def backwardu(self, source): return self._host("backwardu", source, self._len)


# ---- uneven batches ----------------------------------------------------------

class BatchJob(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("method", ctypes.c_int), ("len", ctypes.c_size_t),
                ("in_offset", ctypes.c_size_t), ("out_offset", ctypes.c_size_t), ("option", ctypes.c_int)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("jobs", ctypes.c_size_t), ("tasks", ctypes.c_size_t), ("ctas", ctypes.c_uint),
                ("smem_per_cta", ctypes.c_size_t), ("workspace_bytes", ctypes.c_size_t),
                ("four_step_lengths", ctypes.c_size_t), ("one_cta_lengths", ctypes.c_size_t),
                ("class_tile", ctypes.c_int * 12)]


KINDS = {"cfft1d": KIND_CFFT1D, "rfft1d": KIND_RFFT1D, "dct1d": KIND_DCT1D, "mdct1d": KIND_MDCT1D}


def job_bytes(kind: str, n: int):
    """(input bytes, output bytes) of one f32 forward job."""
    if kind == "cfft1d":
        return 8 * n, 8 * n
    if kind == "rfft1d":
        return 4 * n, 8 * (n // 2 + 1)
    if kind == "dct1d":
        return 4 * n, 4 * n
    return 4 * n, 2 * n  # mdct1d: n reals -> n/2 reals


def pack_jobs(specs, align: int = 16):
    """specs: [(kind, n, method, option)] -> (jobs array, input bytes, output bytes, offsets)."""
    jobs = (BatchJob * len(specs))()
    ib = ob = 0
    offs = []
    for i, (kind, n, method, option) in enumerate(specs):
        bi, bo = job_bytes(kind, n)
        jobs[i] = BatchJob(KINDS[kind], METHODS[method], n, ib, ob, option)
        offs.append((ib, ob))
        ib += (bi + align - 1) // align * align
        ob += (bo + align - 1) // align * align
    return jobs, ib, ob, offs


class Batch:
    """Uneven batch: many f32 forward transforms in one work-queue launch."""

    def __init__(self, specs, dtype=np.float32):
        L = lib()
        for name, args in {
            "chfft_batch_create": [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)],
            "chfft_batch_execute": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
            "chfft_batch_execute_graph": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
            "chfft_batch_wait": [ctypes.c_void_p, ctypes.c_void_p],
            "chfft_batch_get_info": [ctypes.c_void_p, ctypes.POINTER(BatchInfo)],
            "chfft_batch_autotune": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_float)],
            "chfft_batch_destroy": [ctypes.c_void_p],
        }.items():
            getattr(L, name).argtypes = args
            getattr(L, name).restype = ctypes.c_int
        self.specs = list(specs)
        self.jobs, self.in_bytes, self.out_bytes, self.offsets = pack_jobs(self.specs)
        self._h = ctypes.c_void_p()
        _check(L.chfft_batch_create(_dtype_id(dtype), ctypes.cast(self.jobs, ctypes.c_void_p), len(self.specs),
                                    ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.chfft_batch_destroy(h)
            self._h = None

    def info(self) -> BatchInfo:
        out = BatchInfo()
        _check(lib().chfft_batch_get_info(self._h, ctypes.byref(out)))
        return out

    def execute(self, d_in: int, d_out: int, stream: int = 0, graph: bool = False):
        fn = lib().chfft_batch_execute_graph if graph else lib().chfft_batch_execute
        _check(fn(self._h, ctypes.c_void_p(d_in), ctypes.c_void_p(d_out), ctypes.c_void_p(stream)))

    def wait(self, stream: int = 0):
        _check(lib().chfft_batch_wait(self._h, ctypes.c_void_p(stream)))

    def autotune(self, d_in: int, d_out: int, stream: int = 0, reps: int = 3) -> float:
        """Per-class tile widths timed on this batch (chfft_batch_autotune); the winner's ms."""
        best = ctypes.c_float(0)
        _check(lib().chfft_batch_autotune(self._h, ctypes.c_void_p(d_in), ctypes.c_void_p(d_out),
                                          ctypes.c_void_p(stream), reps, ctypes.byref(best)))
        return best.value


# ---- index arithmetic (bit-exact with the reference's plan code) -----------

def factorize(len: int, max_prime: int = 7):
    """prime_factorization(len, max) (src/prime_factorization.rs:66-113)."""
    v = np.zeros(64, np.uint64)
    c = np.zeros(64, np.uint64)
    k = lib().chfft_factorize(len, max_prime, _ptr(v), _ptr(c), 64)
    if k < 0:
        raise ChfftError(-k, lib().chfft_last_error().decode())
    return [(int(v[i]), int(c[i])) for i in range(k)]


def digit_reversal(factors):
    """calc_bitreverse (src/precompute_utils.rs:70-91) for a factor list."""
    total = 1
    for v, c in factors:
        total *= v ** c
    vals = np.array([f[0] for f in factors] or [0], np.uint64)
    cnts = np.array([f[1] for f in factors] or [0], np.uint64)
    out = np.zeros(total, np.uint64)
    _check(lib().chfft_digit_reversal(_ptr(vals), _ptr(cnts), len(factors), _ptr(out), total))
    return out


def swap_list(gather):
    """calc_bitreverse2inplace (src/precompute_utils.rs:93-104)."""
    g = np.ascontiguousarray(gather, np.uint64)
    out = np.zeros_like(g)
    _check(lib().chfft_swap_list(_ptr(g), g.size, _ptr(out)))
    return out


def chirp_index_device(len: int, d_out: int, stream: int = 0):
    """(i*i) % 2N for i < len, written by a GPU kernel to device memory."""
    _check(lib().chfft_chirp_index_device(len, ctypes.c_void_p(d_out), ctypes.c_void_p(stream)))


__all__ = [
    "CFft1D", "CFft2D", "CFft3D", "RFft1D", "Dct1D", "DctType", "Mdct1D", "sine_window", "vorbis_window",
    "ChfftError", "InvalidLength", "PlanInfo", "factorize", "digit_reversal", "swap_list", "chirp_index_device",
    "lib", "version",
]
