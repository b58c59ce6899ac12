/*
 * chfft_gpu.h — C ABI of the GB300 (sm_103a) transform engine.
 *
 * This is the drop-in boundary below chfft's public Rust API
 * (src/lib.rs:21-25 of chfft 0.3.4). Each plan handle stands for one of the
 * reference's plan structs and keeps its semantics: the plan owns its
 * tables, is not thread-safe (the Rust methods take &mut self) and CFft1D /
 * CFft2D plans re-plan when handed a different length, as
 * src/cfft1d.rs:216-218 and src/cfft2d.rs:336-338 do. Errors are status
 * codes; CHFFT_EINVAL_LEN is the reference's `panic!("invalid length")`
 * (src/rfft1d.rs:75, src/dct1d.rs:55, src/mdct1d.rs:103).
 *
 * Data layout: complex values are interleaved {re, im} pairs of the working
 * dtype (num-complex's #[repr(C)] Complex<T>); 2-D arrays are row-major
 * M x N (the Rust wrapper flattens &[Vec<Complex<T>>]).
 *
 * Host-pointer calls copy to the device, run, copy back and synchronise.
 * Device-pointer calls enqueue on the given stream and return at once.
 * There is no CPU fallback: every transform runs in this library's kernels.
 */
#ifndef CHFFT_GPU_H
#define CHFFT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CHFFT_API __attribute__((visibility("default")))

typedef enum chfft_status {
  CHFFT_OK = 0,
  CHFFT_EINVAL_LEN = 1,    /* the reference's panic!("invalid length") */
  CHFFT_EINVAL = 2,        /* null pointer, unknown enum value, method not offered by the type */
  CHFFT_EUNSUPPORTED = 3,  /* size this build does not handle */
  CHFFT_ECUDA = 4,         /* CUDA runtime error (message in chfft_last_error) */
  CHFFT_ENOMEM = 5,        /* device allocation failed */
  CHFFT_ETIMEOUT = 6       /* a bounded device-side wait gave up */
} chfft_status;

typedef enum chfft_dtype { CHFFT_F32 = 0, CHFFT_F64 = 1 } chfft_dtype;

typedef enum chfft_kind {
  CHFFT_KIND_CFFT1D = 0,
  CHFFT_KIND_CFFT2D = 1,
  CHFFT_KIND_RFFT1D = 2,
  CHFFT_KIND_DCT1D = 3,
  CHFFT_KIND_MDCT1D = 4,
  CHFFT_KIND_CFFT3D = 5 /* no counterpart in the reference: a native 3-D layout */
} chfft_kind;

/* The reference's method names (src/cfft1d.rs:270-455 and the same names
 * on the other types). Each type accepts the subset it defines:
 *   CFft1D: all 12;  CFft2D and CFft3D: FORWARD..BACKWARDU (no BACKWARDN, no in-place);
 *   RFft1D: FORWARD..BACKWARDN;  Dct1D: FORWARD..FORWARDN;
 *   Mdct1D: FORWARD, FORWARDU, BACKWARD, BACKWARDU. */
typedef enum chfft_method {
  CHFFT_FORWARD = 0,
  CHFFT_FORWARD0 = 1,
  CHFFT_FORWARDU = 2,
  CHFFT_FORWARDN = 3,
  CHFFT_BACKWARD = 4,
  CHFFT_BACKWARD0 = 5,
  CHFFT_BACKWARDU = 6,
  CHFFT_BACKWARDN = 7,
  CHFFT_FORWARD0I = 8,
  CHFFT_BACKWARD0I = 9,
  CHFFT_FORWARDUI = 10,
  CHFFT_BACKWARDUI = 11
} chfft_method;

/* DctType::{Two, Three} (src/dct1d.rs:37-43). */
typedef enum chfft_dct_type { CHFFT_DCT_TWO = 2, CHFFT_DCT_THREE = 3 } chfft_dct_type;

/* Mdct1D windows: with_sine / with_vorbis (src/mdct1d.rs:62-75) or a
 * caller-evaluated window table (Mdct1D::new(window_func, len),
 * src/mdct1d.rs:101-121, calc_window :91-93: the reference evaluates window_func(len, i) for
 * i < len at setup; the wrapper does the same and passes the values). */
typedef enum chfft_window { CHFFT_WINDOW_SINE = 0, CHFFT_WINDOW_VORBIS = 1, CHFFT_WINDOW_CUSTOM = 2 } chfft_window;

typedef struct chfft_plan_s* chfft_plan;

/* ---- plan construction (one per reference constructor) ------------------ */

/* CFft1D::with_len (src/cfft1d.rs:83-92); len 0 gives CFft1D::new (:68-75). */
CHFFT_API int chfft_cfft1d_create(int dtype, size_t len, chfft_plan* out);
/* CFft2D::with_len (src/cfft2d.rs:93-103); 0 x 0 gives CFft2D::new. */
CHFFT_API int chfft_cfft2d_create(int dtype, size_t len_m, size_t len_n, chfft_plan* out);
/* 3-D complex transform of a row-major len_l x len_m x len_n array. No
 * counterpart in the reference (chfft stops at CFft2D, src/cfft2d.rs); it
 * extends CFft2D's semantics by one axis: the same methods and scales
 * (1/(L M N) for BACKWARD), rows of len_n first, then the len_m axis, then
 * the len_l axis. Each axis length must fit one CTA's engine (mixed radix
 * or Bluestein), as for CFft2D. 0 x 0 x 0 gives an empty plan. */
CHFFT_API int chfft_cfft3d_create(int dtype, size_t len_l, size_t len_m, size_t len_n, chfft_plan* out);
/* RFft1D::new (src/rfft1d.rs:73-90): odd len -> CHFFT_EINVAL_LEN. */
CHFFT_API int chfft_rfft1d_create(int dtype, size_t len, chfft_plan* out);
/* Dct1D::new (src/dct1d.rs:53-62): odd len -> CHFFT_EINVAL_LEN. */
CHFFT_API int chfft_dct1d_create(int dtype, int dct_type, size_t len, int is_ortho, chfft_plan* out);
/* Mdct1D::new / with_sine / with_vorbis (src/mdct1d.rs:62-121):
 * len % 4 != 0 -> CHFFT_EINVAL_LEN. window_table (len values of the working
 * dtype, host memory) is read only for CHFFT_WINDOW_CUSTOM. */
CHFFT_API int chfft_mdct1d_create(int dtype, size_t len, int window, const void* window_table, chfft_plan* out);
CHFFT_API int chfft_plan_destroy(chfft_plan plan);

/* ---- re-plan (the reference's setup methods) ---------------------------- */

/* CFft1D::setup (src/cfft1d.rs:103), RFft1D::setup (src/rfft1d.rs:101),
 * Mdct1D::setup (src/mdct1d.rs:126; a custom window must be re-supplied
 * through window_table, NULL keeps sine/vorbis). */
CHFFT_API int chfft_plan_setup(chfft_plan plan, size_t len, const void* window_table);
/* CFft2D::setup (src/cfft2d.rs:114-124). */
CHFFT_API int chfft_cfft2d_setup(chfft_plan plan, size_t len_m, size_t len_n);
/* Dct1D::setup (src/dct1d.rs:74-86). */
CHFFT_API int chfft_dct1d_setup(chfft_plan plan, int dct_type, size_t len, int is_ortho);

/* ---- execution ---------------------------------------------------------- */

/* One transform on host memory: the reference call `plan.method(&src)`.
 * src_len / dst_len count elements of the method's input / output type
 * (complex for complex sides, reals for real sides). For CFft1D a src_len
 * different from the plan's length re-plans; for the in-place methods src
 * and dst may be the same buffer. RFft1D / Dct1D / Mdct1D reject a length
 * mismatch with CHFFT_EINVAL_LEN. dst_len must equal the output length. */
CHFFT_API int chfft_execute(chfft_plan plan, int method, const void* src, size_t src_len, void* dst,
                            size_t dst_len);
/* CFft2D::method(&rows) on a row-major len_m x len_n host array (re-plans
 * when the shape differs from the plan's). */
CHFFT_API int chfft_execute_2d(chfft_plan plan, int method, const void* src, size_t len_m, size_t len_n,
                               void* dst);
/* CFft3D on a row-major len_l x len_m x len_n host array (re-plans when the
 * shape differs from the plan's; an empty shape returns at once). */
CHFFT_API int chfft_execute_3d(chfft_plan plan, int method, const void* src, size_t len_l, size_t len_m, size_t len_n,
                               void* dst);
/* `batch` independent transforms on host memory, each laid out back to back
 * (input and output strides are the per-transform element counts). */
CHFFT_API int chfft_execute_batch(chfft_plan plan, int method, const void* src, void* dst, size_t batch);
/* `batch` transforms on device memory, enqueued on `stream` (a cudaStream_t,
 * NULL for the legacy default stream). d_src == d_dst is allowed for
 * complex-to-complex kinds. */
CHFFT_API int chfft_execute_device(chfft_plan plan, int method, const void* d_src, void* d_dst, size_t batch,
                                   void* stream);

/* CFft1D on split-complex device arrays: real and imaginary parts in
 * separate arrays of the working dtype, `batch` transforms back to back in
 * each (no counterpart in the reference, whose Complex<T> is interleaved,
 * src/cfft1d.rs:270). Any CFft1D method; source and destination arrays may
 * be the same. Plans whose length fits one CTA (algorithm 0 or 1 in
 * chfft_plan_info); others get CHFFT_EUNSUPPORTED. */
CHFFT_API int chfft_execute_device_split(chfft_plan plan, int method, const void* d_src_re, const void* d_src_im,
                                         void* d_dst_re, void* d_dst_im, size_t batch, void* stream);

/* CFft1D on strided device layouts: element i of transform t at
 * t * idist + i * istride of d_src (complex elements) and t * odist +
 * i * ostride of d_dst: matrix columns, padded rows, interleaved channels
 * (no counterpart in the reference, which takes contiguous slices). Any
 * CFft1D method; strides in [1, 2^31). d_src == d_dst only with the same
 * layout on both sides, and the layouts must not map two elements of the
 * batch to one address. One-CTA lengths; others get CHFFT_EUNSUPPORTED. */
CHFFT_API int chfft_execute_device_strided(chfft_plan plan, int method, const void* d_src, size_t istride,
                                           size_t idist, void* d_dst, size_t ostride, size_t odist, size_t batch,
                                           void* stream);

/* Waits for `stream`, then reports CHFFT_ETIMEOUT if a bounded device-side
 * wait in one of this plan's launches gave up since the last check (the
 * launch then returned without hanging and its output is incomplete; the
 * pipelined four-step launch of CFft1D plans waits on other CTAs' tiles).
 * The host-memory calls make this check themselves. No counterpart in the
 * reference: chfft's transforms are synchronous CPU calls. */
CHFFT_API int chfft_plan_wait(chfft_plan plan, void* stream);

/* Device execution that allocates nothing. No counterpart in the reference
 * (chfft allocates a new Vec for every result).
 *
 * For callers that cannot allocate device memory when they run a transform:
 * code running while a stream is captured into a CUDA graph, real-time loops
 * that must not wait on the allocator, hosts whose device memory belongs to a
 * pool they do not control. chfft_execute_device grows the plan's workspace
 * with cudaMalloc on a large batch; this variant runs CFft1D plans on the
 * four-step path (lengths beyond one CTA, see chfft_plan_info.algorithm 2/3)
 * with the workspace taken from a fixed array of CHFFT_NOALLOC_SCRATCH_BYTES
 * that the library defines per device and every GPU that loads the library
 * holds until the process exits. It calls no cudaMalloc/cudaFree and no
 * allocating library routine; it always uses the library's own kernels
 * (never the plan-time compiler). Inputs and outputs are the caller's device
 * buffers, as for chfft_execute_device.
 *
 * Limits and rules: one transform's workspace (8 or 16 bytes x the FFT
 * length, twice that for Bluestein lengths) must fit the array, else the call
 * returns CHFFT_EUNSUPPORTED with the sizes in chfft_last_error; larger
 * batches run in chunks that fit. The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture. All calls share the array
 * and it keeps the last call's contents (nothing in it needs to start at
 * zero), so calls whose work overlaps on the GPU (different streams, no
 * ordering) race on it. A device reset (cudaDeviceReset) discards the array's
 * contents with the context; the next call looks the address up again in the
 * new context. Other plans get CHFFT_EINVAL. */
#define CHFFT_NOALLOC_SCRATCH_BYTES (16u << 20)
CHFFT_API int chfft_execute_device_noalloc(chfft_plan plan, int method, const void* d_src, void* d_dst, size_t batch,
                                           void* stream);

/* ---- uneven batches ------------------------------------------------------ */

/* Many transforms of mixed kinds and lengths in one launch fed by a device
 * work queue (one CTA per task; each CTA takes its task by ticket when it
 * starts). No counterpart in the reference (one chfft call is one
 * transform); each job means the reference call `plan.method(&src)` of its
 * kind at its length. Jobs are f32 forward methods of CFft1D, RFft1D, Dct1D
 * (DCT-II) and Mdct1D; lengths from 2 up to 2^18 (C2C) and a 7-smooth half
 * length for real kinds beyond 8192. Lengths beyond one CTA run as four-step
 * task chains synchronised by device counters (bounded waits:
 * CHFFT_SPIN_LIMIT polls, about a second by default; chfft_batch_wait
 * reports a wait that gave up as CHFFT_ETIMEOUT). */
typedef struct chfft_batch_job {
  int kind;          /* CHFFT_KIND_CFFT1D, _RFFT1D, _DCT1D (type II), _MDCT1D */
  int method;        /* a forward method of the kind (CHFFT_FORWARD, ...) */
  size_t len;        /* the plan length (the reference's `len`) */
  size_t in_offset;  /* bytes from the input base to this job's input */
  size_t out_offset; /* bytes from the output base to this job's output */
  int option;        /* Dct1D: is_ortho; Mdct1D: CHFFT_WINDOW_SINE or _VORBIS */
} chfft_batch_job;

typedef struct chfft_batch_s* chfft_batch;

typedef struct chfft_batch_info {
  size_t jobs, tasks;
  unsigned ctas;              /* CTAs per launch */
  size_t smem_per_cta;
  size_t workspace_bytes;     /* four-step intermediates */
  size_t four_step_lengths, one_cta_lengths;
  /* Widest four-step tile (columns / rows) per class of four-step items,
   * 0 for a class the batch has: index group * 4 + size, group 0 C2C,
   * 1 C2C Bluestein, 2 real kinds; size 0..3 for a four-step length of at
   * most 2^14, 2^15, 2^16, or more. Default 64 (the widest that fits a
   * CTA); chfft_batch_autotune times the alternatives. */
  int class_tile[12];
} chfft_batch_info;

/* Builds every table and the task queue (device memory). */
CHFFT_API int chfft_batch_create(int dtype, const chfft_batch_job* jobs, size_t njobs, chfft_batch* out);
/* One launch on `stream`: d_in / d_out are the bases the job
 * offsets refer to. Asynchronous. */
CHFFT_API int chfft_batch_execute(chfft_batch batch, const void* d_in, void* d_out, void* stream);
/* The same launch captured once into a CUDA graph (re-captured when the base
 * pointers change) and replayed on `stream`. */
CHFFT_API int chfft_batch_execute_graph(chfft_batch batch, const void* d_in, void* d_out, void* stream);
/* Waits for `stream`; CHFFT_ETIMEOUT if a task gave up waiting for its
 * dependencies (the launch then returned without hanging). */
CHFFT_API int chfft_batch_wait(chfft_batch batch, void* stream);
CHFFT_API int chfft_batch_get_info(chfft_batch batch, chfft_batch_info* info);
/* Tile widths chosen by timing this batch (no counterpart in the reference,
 * whose factor order is fixed, src/prime_factorization.rs:66-113): for each
 * class of four-step items present, in turn, the widest tile is tried at 16,
 * 32 and 64 with the other classes held, each candidate timed as the median
 * of `reps` launches on d_in / d_out (CUDA events on `stream`), and the class
 * keeps the fastest. The batch then runs with the chosen widths; *best_ms
 * (may be null) gets the winner's time. CHFFT_ETIMEOUT if a launch's
 * dependency wait gave up. */
CHFFT_API int chfft_batch_autotune(chfft_batch batch, const void* d_in, void* d_out, void* stream, int reps,
                                   float* best_ms);
CHFFT_API int chfft_batch_destroy(chfft_batch batch);

/* ---- plan inspection ---------------------------------------------------- */

typedef struct chfft_plan_info {
  int kind, dtype;
  size_t len, len_m, len_n;  /* user lengths */
  size_t fft_len;            /* length of the complex core FFT */
  int algorithm;             /* 0 mixed radix in shared memory, 1 fused Bluestein, 2 four-step, 3 four-step Bluestein,
                                4 Rader (CFft1D of a prime length whose length - 1 is 7-smooth, rows fitting one
                                CTA, with CHFFT_RADER=1 at plan creation; Chirp-Z otherwise) */
  size_t padded_len;         /* Bluestein convolution length M (0 otherwise) */
  int npass;                 /* radix passes of the core FFT */
  int radix[24];
  int seq_per_cta, threads_per_cta;
  size_t smem_per_cta;
  size_t in_elems, out_elems; /* per transform, in the method's element type (forward direction) */
  size_t device_bytes;        /* tables + workspace held by the plan */
  /* Latency form: batches of at most cluster_max_batch transforms run the
   * complex core (CFft1D: N; RFft1D and Dct1D: N/2; Mdct1D: N/4) one
   * transform per thread-block cluster of cluster_ctas CTAs (the core split
   * cluster_n1 x cluster_n2 over the cluster, exchange through distributed
   * shared memory); the real kinds' pre- and post-processing run in
   * launches of their own around it. 0 when the plan has none. Cores of
   * 7-smooth lengths from 64 to 2^20 with such a split that fits a CTA's
   * shared memory (CHFFT_CLUSTER=0 at plan creation turns it off, 8 or 16
   * forces the cluster size). */
  int cluster_ctas;
  size_t cluster_n1, cluster_n2, cluster_max_batch;
  size_t len_l; /* CFft3D: the outer axis (len_m, len_n the others) */
} chfft_plan_info;

CHFFT_API int chfft_plan_get_info(chfft_plan plan, chfft_plan_info* info);

/* ---- tuning (no reference counterpart) -----------------------------------
 * chfft fixes one plan per length: the factor order of
 * src/prime_factorization.rs:66-113 and the Chirp-Z length of
 * src/cfft1d.rs:114-140. Here the launch structure of a plan has knobs, an
 * exhaustive autotuner times them, and a learned cost model (a 3-layer MLP
 * trained on the GPU) proposes them for lengths it has not timed. A knob at
 * -1 / 0 is left to the built-in heuristic. */
typedef struct chfft_plan_config {
  int k1;                  /* 1: one butterfly per thread and pass, 0: several, -1 auto */
  int seq_per_cta;         /* sequences per CTA of the row kernels, 0 auto */
  int max_radix;           /* f32 plan-time kernels: 16 or 32, 0 auto (32) */
  int jit;                 /* plan-time specialised kernels: 1 always, 0 never, -1 policy (CHFFT_JIT) */
  long long bluestein_len; /* Bluestein convolution length M (7-smooth, >= 2N-1), 0 auto */
  int fs_n1;               /* four-step column length n1 (n1 | N), 0 auto */
  int tile_cols;           /* four-step and 2-D column tile width, 0 auto */
  int l2_chunk_mb;         /* four-step chunk budget in MiB (the workspace), 0 auto (512) */
  int tc_precision;        /* f32 radix-16 passes on the tensor cores (power-of-two CFft1D
                              lengths >= 16, plan-time compiled): 0 off (FP32 cores),
                              1 FP16 hi+lo, 2 BF16 hi+lo, 3 BF16 hi+mid+lo; FP32 accumulation */
  int min_blocks_per_sm;   /* plan-time kernels: CTAs per SM their launch bounds target
                              (the register budget), 0 auto */
  int balanced;            /* plan-time kernels with mixed radices: 1 / -1 (auto) every thread
                              takes maxR / R butterflies of a radix-R pass, 0 one butterfly per
                              thread and pass (threads idle through the larger radices) */
  int l2_prefetch;         /* retired (next-wave L2 prefetch measured slower everywhere): ignored,
                              always reported 0; kept so the struct layout does not change */
  int l2_evict_hints;      /* retired (L2 eviction priorities on the two-launch four-step passes,
                              superseded by the pipelined launch's own hints): ignored, reported 0 */
  int col_elems_per_thread; /* column / four-step kernels of the several-butterflies variant:
                               complex elements a thread holds (16 or 32), 0 the dtype's
                               default (32 f32, 16 f64) */
} chfft_plan_config;

CHFFT_API void chfft_plan_config_default(chfft_plan_config* cfg);
/* Applies cfg (rebuilding the plan's tables when the Bluestein length or the
 * four-step split changes). Knobs a plan cannot use are ignored; invalid
 * values fall back to the heuristic. */
CHFFT_API int chfft_plan_set_config(chfft_plan plan, const chfft_plan_config* cfg);
CHFFT_API int chfft_plan_get_config(chfft_plan plan, chfft_plan_config* cfg);
/* The autotuner's search space for `batch` transforms: up to cap configs into
 * out, their number into *n. tune_jit != 0 adds the jit / max_radix knobs. */
CHFFT_API int chfft_plan_candidates(chfft_plan plan, size_t batch, int tune_jit, chfft_plan_config* out, int cap,
                                    int* n);
/* Cost-model features of (plan, batch, cfg): CHFFT_FEATURES floats. */
#define CHFFT_FEATURES 48
CHFFT_API int chfft_plan_features(chfft_plan plan, size_t batch, const chfft_plan_config* cfg, float* out);
/* Exhaustive autotune: times every candidate (the method on `batch`
 * transforms of device scratch data, median of `reps` launches after one
 * warm-up), leaves the plan on the fastest, and reports each candidate and
 * its milliseconds (up to cap) plus the index of the best. */
CHFFT_API int chfft_autotune(chfft_plan plan, int method, size_t batch, int reps, int tune_jit,
                             chfft_plan_config* cfgs, float* ms, int cap, int* n, int* best);

/* Learned cost model: an MLP CHFFT_FEATURES -> hidden -> hidden -> 1 (ReLU,
 * FP32) predicting log milliseconds, trained with Adam by this library's own
 * CUDA forward / backward kernels. Inputs are standardised with the training
 * set's moments, kept in the model. */
typedef struct chfft_mlp_s* chfft_mlp;
CHFFT_API int chfft_mlp_create(int hidden, unsigned seed, chfft_mlp* out);
CHFFT_API int chfft_mlp_destroy(chfft_mlp m);
CHFFT_API int chfft_mlp_num_params(chfft_mlp m);
/* Parameters, flat: W1 (hidden x F), b1, W2 (hidden x hidden), b2, W3 (hidden), b3. */
CHFFT_API int chfft_mlp_get_params(chfft_mlp m, float* out);
CHFFT_API int chfft_mlp_set_params(chfft_mlp m, const float* p);
/* Feature / target moments used to standardise (F means, F stds, target mean, target std). */
CHFFT_API int chfft_mlp_set_moments(chfft_mlp m, const float* mean, const float* std, float y_mean, float y_std);
CHFFT_API int chfft_mlp_get_moments(chfft_mlp m, float* mean, float* std, float* y_mean, float* y_std);
/* Loss 0.5 * mean((f(x) - y)^2) over standardised rows and its gradient
 * (num_params floats) from the GPU kernels: the quantity a gradient check
 * compares. X is n x CHFFT_FEATURES raw features, y raw log ms. */
CHFFT_API int chfft_mlp_loss_grad(chfft_mlp m, const float* X, const float* y, int n, float* loss, float* grad);
/* Computes the moments from (X, y), then runs `epochs` of mini-batch Adam. */
CHFFT_API int chfft_mlp_train(chfft_mlp m, const float* X, const float* y, int n, int epochs, int batch, float lr,
                              unsigned seed, float* final_loss);
CHFFT_API int chfft_mlp_predict(chfft_mlp m, const float* X, int n, float* y);
/* Picks the candidate with the lowest predicted time and applies it. */
CHFFT_API int chfft_plan_propose(chfft_plan plan, size_t batch, chfft_mlp m, int tune_jit, chfft_plan_config* chosen);

/* ---- index arithmetic (bit-exact with the reference's plan code) -------- */

/* prime_factorization(len, max) (src/prime_factorization.rs:66-113):
 * writes up to cap (value, count) pairs, returns the number of factors
 * (0 when a prime exceeds max_prime; the reference's Chirp-Z trigger). */
CHFFT_API int chfft_factorize(size_t len, size_t max_prime, size_t* values, size_t* counts, size_t cap);
/* calc_bitreverse (src/precompute_utils.rs:70-91) for an explicit factor list;
 * writes prod(value^count) entries. */
CHFFT_API int chfft_digit_reversal(const size_t* values, const size_t* counts, size_t nfactors, size_t* out,
                                   size_t out_cap);
/* calc_bitreverse2inplace (src/precompute_utils.rs:93-104), in O(n). */
CHFFT_API int chfft_swap_list(const size_t* gather, size_t n, size_t* out);
/* Chirp-Z table indices (i*i) % 2N for i < len (src/cfft1d.rs:123-128),
 * computed by a GPU kernel into device memory d_out (len uint64 values). */
CHFFT_API int chfft_chirp_index_device(size_t len, uint64_t* d_out, void* stream);

/* ---- plan-time kernel specialisation ------------------------------------ */

/* Plans can run kernels specialised to their exact radix sequence, lengths
 * and launch shape, compiled with NVRTC for sm_103a on first use and cached
 * for the life of the process. CHFFT_JIT selects when: "0"/"off" never,
 * "auto" (default) for launches of at least 2^18 elements, anything else
 * always. Returns 1 when NVRTC and the driver API can be opened, 0 otherwise
 * (reason in chfft_last_error; plans then use the library's kernels). */
CHFFT_API int chfft_plan_compiler_available(void);
/* Number of specialised kernels compiled so far in this process. */
CHFFT_API size_t chfft_plan_compiler_cache_size(void);

/* ---- diagnostics -------------------------------------------------------- */

/* Message of the last failure on the calling thread ("" if none). */
CHFFT_API const char* chfft_last_error(void);
CHFFT_API const char* chfft_status_string(int status);
/* Library version string. */
CHFFT_API const char* chfft_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CHFFT_GPU_H */
