// chfft_execute_device_noalloc: four-step CFft1D execution without device
// allocation.
//
// Some callers cannot allocate device memory at the point where they run a
// transform: code that runs while a CUDA stream is being captured into a
// graph, real-time audio/radar loops that must not block in the allocator,
// and hosts whose device memory is handed out by a pool they do not own.
// chfft_execute_device grows the plan's workspace with cudaMalloc on the
// first large batch; this entry point instead takes the workspace of the
// four-step path from the fixed array below, which every GPU that loads the
// library holds until the process exits.
#include <cuda_runtime.h>

#include <exception>
#include <mutex>
#include <new>
#include <string>

#include "../../include/chfft_gpu.h"
#include "plan.hpp"

namespace chfft {

int plan_four_step(chfft_plan plan, int method, const BigCore** big, bool* back, double* scale);
int record_error(int code, const std::string& msg);
void clear_error();

namespace {

// The shared scratch: CHFFT_NOALLOC_SCRATCH_BYTES per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[CHFFT_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// Per device: the scratch's device address and the context it was looked
// up in (a device reset makes a new context, and the address is looked up
// again there).
void* g_scratch_ptr[kMaxDevices] = {};
void* g_scratch_ctx[kMaxDevices] = {};

int fail(int code, const std::string& msg) { return record_error(code, msg); }

// The driver's cuCtxGetCurrent, or null when it cannot be had.
typedef int (*CtxGetCurrent)(void**);
CtxGetCurrent ctx_getter() {
  static std::once_flag once;
  static CtxGetCurrent fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrent>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// Device address of the scratch on the current device, looked up once per
// device and context (host code only sees a stand-in for the array's name).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(CHFFT_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(CHFFT_EUNSUPPORTED, "device ordinal out of range");
  void* ctx = nullptr;
  if (CtxGetCurrent get = ctx_getter()) get(&ctx);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(CHFFT_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
    g_scratch_ctx[dev] = ctx;
  }
  *out = g_scratch_ptr[dev];
  return CHFFT_OK;
}

}  // namespace
}  // namespace chfft

extern "C" int chfft_execute_device_noalloc(chfft_plan plan, int method, const void* d_src, void* d_dst,
                                            size_t batch, void* stream) {
  using namespace chfft;
  clear_error();
  const BigCore* big = nullptr;
  bool back = false;
  double scale = 1.0;
  int rc = plan_four_step(plan, method, &big, &back, &scale);
  if (rc != CHFFT_OK) return rc;
  if (batch == 0) return CHFFT_OK;
  if (!d_src || !d_dst) return fail(CHFFT_EINVAL, "null buffer");
  const size_t per = big->work_bytes_per_transform();
  if (per > (size_t)CHFFT_NOALLOC_SCRATCH_BYTES) {
    return fail(CHFFT_EUNSUPPORTED, "length " + std::to_string(big->n) + " needs " + std::to_string(per) +
                                        " bytes of scratch per transform; the no-allocation entry point has " +
                                        std::to_string((size_t)CHFFT_NOALLOC_SCRATCH_BYTES));
  }
  void* scratch = nullptr;
  rc = scratch_address(&scratch);
  if (rc != CHFFT_OK) return rc;
  try {
    // Every workspace element is written by the column pass before the row
    // pass reads it, so the scratch needs no clearing between calls.
    big->exec(d_src, d_dst, scratch, (long long)batch, back, scale, static_cast<cudaStream_t>(stream),
              (long long)((size_t)CHFFT_NOALLOC_SCRATCH_BYTES / per), /*library_only=*/true);
  } catch (const Fail& f) {
    return fail(f.code, f.msg);
  } catch (const std::bad_alloc&) {
    return fail(CHFFT_ENOMEM, "host allocation failed");
  } catch (const std::exception& x) {
    return fail(CHFFT_EINVAL, x.what());
  }
  return CHFFT_OK;
}
