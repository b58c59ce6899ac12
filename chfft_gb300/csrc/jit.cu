// Plan-time kernel specialisation.
//
// The plan compiler emits, for one plan, the kernel template of its kind
// instantiated with a StatCore: FFT length, Bluestein length, sequences per
// CTA, tile stride and the exact radix sequence become template constants,
// so the pass bodies compile to straight-line code with constant indices
// and strides. The instance is compiled with NVRTC for sm_103a at first use
// and cached per process (and per device). NVRTC and the CUDA driver API are
// opened with dlopen on first use, so the library itself loads on hosts
// without a GPU or without NVRTC; when either is missing the plan keeps the
// run-time-stage kernels compiled into the library.
#include <dlfcn.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "jit.hpp"
#include "jit_headers.inc"  // generated by _build.py: kernel headers as strings

namespace chfft {
namespace {

typedef int CUresult;
typedef struct CUmod_st* CUmodule;
typedef struct CUfunc_st* CUfunction;
typedef struct CUstream_st* CUstream;
typedef int nvrtcResult;
typedef struct _nvrtcProgram* nvrtcProgram;
constexpr int kAttrMaxDynSmem = 8;  // CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES

struct Api {
  bool tried = false, ok = false;
  std::string why;
  CUresult (*cuModuleLoadData)(CUmodule*, const void*) = nullptr;
  CUresult (*cuModuleGetFunction)(CUfunction*, CUmodule, const char*) = nullptr;
  CUresult (*cuLaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                             CUstream, void**, void**) = nullptr;
  CUresult (*cuFuncSetAttribute)(CUfunction, int, int) = nullptr;
  CUresult (*cuOccupancyMaxActiveBlocksPerMultiprocessor)(int*, CUfunction, int, size_t) = nullptr;
  nvrtcResult (*nvrtcCreateProgram)(nvrtcProgram*, const char*, const char*, int, const char* const*,
                                    const char* const*) = nullptr;
  nvrtcResult (*nvrtcAddNameExpression)(nvrtcProgram, const char*) = nullptr;
  nvrtcResult (*nvrtcCompileProgram)(nvrtcProgram, int, const char* const*) = nullptr;
  nvrtcResult (*nvrtcGetLoweredName)(nvrtcProgram, const char*, const char**) = nullptr;
  nvrtcResult (*nvrtcGetCUBINSize)(nvrtcProgram, size_t*) = nullptr;
  nvrtcResult (*nvrtcGetCUBIN)(nvrtcProgram, char*) = nullptr;
  nvrtcResult (*nvrtcGetProgramLogSize)(nvrtcProgram, size_t*) = nullptr;
  nvrtcResult (*nvrtcGetProgramLog)(nvrtcProgram, char*) = nullptr;
  nvrtcResult (*nvrtcDestroyProgram)(nvrtcProgram*) = nullptr;
};

Api g_api;
std::mutex g_mu;

struct Entry {
  CUfunction fn = nullptr;
  int smem_set = 0;
  bool failed = false;
};
std::unordered_map<std::string, Entry> g_cache;

template <class F>
bool sym(void* h, const char* name, F* out) {
  *out = reinterpret_cast<F>(dlsym(h, name));
  return *out != nullptr;
}

bool load_api() {
  if (g_api.tried) return g_api.ok;
  g_api.tried = true;
  void* cu = dlopen("libcuda.so.1", RTLD_NOW | RTLD_GLOBAL);
  if (!cu) {
    g_api.why = "libcuda.so.1 not found";
    return false;
  }
  void* rtc = nullptr;
  const char* cands[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                         "/usr/local/cuda/lib64/libnvrtc.so"};
  for (const char* c : cands)
    if ((rtc = dlopen(c, RTLD_NOW | RTLD_GLOBAL))) break;
  if (!rtc) {
    g_api.why = "libnvrtc not found";
    return false;
  }
  bool ok = sym(cu, "cuModuleLoadData", &g_api.cuModuleLoadData) &&
            sym(cu, "cuModuleGetFunction", &g_api.cuModuleGetFunction) &&
            sym(cu, "cuLaunchKernel", &g_api.cuLaunchKernel) &&
            sym(cu, "cuFuncSetAttribute", &g_api.cuFuncSetAttribute) &&
            sym(cu, "cuOccupancyMaxActiveBlocksPerMultiprocessor", &g_api.cuOccupancyMaxActiveBlocksPerMultiprocessor) &&
            sym(rtc, "nvrtcCreateProgram", &g_api.nvrtcCreateProgram) &&
            sym(rtc, "nvrtcAddNameExpression", &g_api.nvrtcAddNameExpression) &&
            sym(rtc, "nvrtcCompileProgram", &g_api.nvrtcCompileProgram) &&
            sym(rtc, "nvrtcGetLoweredName", &g_api.nvrtcGetLoweredName) &&
            sym(rtc, "nvrtcGetCUBINSize", &g_api.nvrtcGetCUBINSize) &&
            sym(rtc, "nvrtcGetCUBIN", &g_api.nvrtcGetCUBIN) &&
            sym(rtc, "nvrtcGetProgramLogSize", &g_api.nvrtcGetProgramLogSize) &&
            sym(rtc, "nvrtcGetProgramLog", &g_api.nvrtcGetProgramLog) &&
            sym(rtc, "nvrtcDestroyProgram", &g_api.nvrtcDestroyProgram);
  if (!ok) {
    g_api.why = "missing NVRTC / driver entry points";
    return false;
  }
  g_api.ok = true;
  return true;
}

const char* kernel_template(Kernel k) {
  switch (k) {
    case Kernel::C2C: return "chfft::kern::k_c2c";
    case Kernel::COLS: return "chfft::kern::k_cols";
    case Kernel::R2C: return "chfft::kern::k_r2c";
    case Kernel::C2R: return "chfft::kern::k_c2r";
    case Kernel::DCT2: return "chfft::kern::k_dct2";
    case Kernel::DCT3: return "chfft::kern::k_dct3";
    case Kernel::MDCT: return "chfft::kern::k_mdct";
    case Kernel::IMDCT: return "chfft::kern::k_imdct";
    case Kernel::COLS_TW: return "chfft::kern::k_cols_tw";
    case Kernel::ROWS_T: return "chfft::kern::k_rows_t";
    case Kernel::ROWS_BB: return "chfft::kern::k_rows_bb";
    case Kernel::C2C_RADER: return "chfft::kern::k_c2c_rader";
  }
  return "";
}

// Tile pad period of a specialised kernel: the first pass's radix when even
// (its stride-R stores then become conflict-free), no padding otherwise.
int pad_period(const std::vector<int>& order) { return (!order.empty() && order[0] % 2 == 0) ? order[0] : 0; }

bool column_mapped(Kernel k) {
  return k == Kernel::COLS || k == Kernel::COLS_TW || k == Kernel::ROWS_T || k == Kernel::ROWS_BB;
}
bool four_step(Kernel k) { return k == Kernel::COLS_TW || k == Kernel::ROWS_T || k == Kernel::ROWS_BB; }

// Tile stride of a specialised kernel. Column-mapped passes give the lanes
// of one shared-memory wavefront (16 f32 / 8 f64 complex elements) tpb
// adjacent sequences times q = lanes / tpb adjacent elements; a stride that
// is q times an odd number puts all of them in distinct banks.
int tile_ld(int n, const std::vector<int>& order, int tpb, int dtype, bool column) {
  const int p = pad_period(order);
  int ld = n + (p > 0 ? n / p : 0);
  const int lanes = dtype == 0 ? 16 : 8;
  const int q = column ? std::max(1, lanes / std::max(1, tpb)) : 1;
  while (ld % (2 * q) != q) ld++;
  return ld;
}

// "chfft::StatCore<...>" of a specialised kernel.
std::string core_expression(Kernel k, int dtype, const Core& c, int n, const std::vector<int>& order, const Geo& g) {
  std::string s = "chfft::StatCore<";
  s += c.blue ? "true," : "false,";
  s += column_mapped(k) ? "true," : "false,";
  s += g.k1 ? "true," : "false,";
  // Default register budget: that of 512-thread CTAs, 2 per SM for the
  // one-butterfly and balanced variants, 1 otherwise; 3 for f32
  // one-butterfly complex kernels of radices up to 10, which fit it without
  // spilling (N = 1000: 30 -> 27 us measured).
  int rmax = 0;
  for (int r : order) rmax = std::max(rmax, r);
  const bool small_radix = dtype == 0 && rmax <= 10 && !c.blue && (k == Kernel::C2C || k == Kernel::COLS);
  // Rader rows hold up to 64 elements per thread in their two passes and fit
  // two CTAs per SM by shared memory: the register budget of two 512-thread CTAs.
  const int per512 = k == Kernel::C2C_RADER ? 1 : g.k1 ? (small_radix ? 3 : 2) : (g.ept > 0 ? 2 : 1);
  const int minb = g.min_blocks > 0 ? g.min_blocks : std::max(1, per512 * (kMaxThreads / std::max(32, g.threads)));
  s += std::to_string(n) + "," + std::to_string(c.n) + "," + std::to_string(g.tpb) + "," + std::to_string(g.ld) +
       "," + std::to_string(pad_period(order)) + "," + std::to_string(g.threads) + "," + std::to_string(minb) + "," +
       std::to_string(g.k1 ? 0 : g.ept);
  for (int r : order) s += "," + std::to_string(r);
  s += ">";
  return s;
}

std::string name_expression(Kernel k, int dtype, const Core& c, int n, const std::vector<int>& order, const Geo& g,
                            int mode) {
  std::string s = "&";
  s += kernel_template(k);
  s += dtype == 0 ? "<float, " : "<double, ";
  s += core_expression(k, dtype, c, n, order, g);
  if (four_step(k)) s += ", " + std::to_string(mode);
  s += ">";
  return s;
}

bool compile(const std::string& expr, Entry* e, std::string* log) {
  nvrtcProgram prog = nullptr;
  const char* src = "#include \"k_complex.cuh\"\n#include \"k_real.cuh\"\n#include \"tc_core.cuh\"\n";
  if (g_api.nvrtcCreateProgram(&prog, src, "chfft_plan.cu", kJitHeaderCount, kJitHeaderSrc, kJitHeaderNames) != 0) {
    *log = "nvrtcCreateProgram failed";
    return false;
  }
  g_api.nvrtcAddNameExpression(prog, expr.c_str());
  const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-lineinfo", "-DCHFFT_PLAN_TIME=1"};
  nvrtcResult rc = g_api.nvrtcCompileProgram(prog, 4, opts);
  if (rc != 0) {
    size_t n = 0;
    g_api.nvrtcGetProgramLogSize(prog, &n);
    log->assign(n, '\0');
    if (n) g_api.nvrtcGetProgramLog(prog, &(*log)[0]);
    g_api.nvrtcDestroyProgram(&prog);
    return false;
  }
  const char* lowered = nullptr;
  g_api.nvrtcGetLoweredName(prog, expr.c_str(), &lowered);
  std::string lname = lowered ? lowered : "";
  size_t sz = 0;
  g_api.nvrtcGetCUBINSize(prog, &sz);
  std::vector<char> cubin(sz);
  g_api.nvrtcGetCUBIN(prog, cubin.data());
  g_api.nvrtcDestroyProgram(&prog);
  CUmodule mod = nullptr;
  if (g_api.cuModuleLoadData(&mod, cubin.data()) != 0 || g_api.cuModuleGetFunction(&e->fn, mod, lname.c_str()) != 0) {
    *log = "module load failed";
    e->fn = nullptr;
    return false;
  }
  return true;
}

}  // namespace

int num_sms() {
  static int n[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 1;
  if (!n[dev]) cudaDeviceGetAttribute(&n[dev], cudaDevAttrMultiProcessorCount, dev);
  return n[dev] > 0 ? n[dev] : 1;
}

JitMode jit_mode() {
  const char* v = std::getenv("CHFFT_JIT");
  if (!v || !*v || !std::strcmp(v, "auto")) return JitMode::AUTO;
  if (!std::strcmp(v, "0") || !std::strcmp(v, "off")) return JitMode::OFF;
  return JitMode::ALWAYS;
}

bool jit_available(std::string* why) {
  std::lock_guard<std::mutex> lk(g_mu);
  bool ok = load_api();
  if (!ok && why) *why = g_api.why;
  return ok;
}

namespace {

// Geometry, stage list and arguments of a specialised launch.
struct Spec {
  Geo g;
  const StageList* sl = nullptr;
  std::vector<int> order;  // the passes' radices, first pass first
  KArgs a;
};

// False when the core has no specialised form for this geometry.
bool resolve(Kernel k, int dtype, const Core& c, const Geo& g0, const KArgs& a0, int mode, const FourStep* fs,
             Spec* out) {
  if (!c.stw.p) return false;
  if (k == Kernel::C2C_RADER && !c.order2.empty() && c.stw2.p) {
    // The Rader core's two-pass order, one butterfly per thread, on the
    // host's sequences per CTA.
    Geo g = g0;
    int per_seq = 0;
    for (int r : c.order2) per_seq = std::max(per_seq, (int)(c.st.n / r));
    g.k1 = true;
    g.ept = 0;
    g.threads = std::max(32, (g.tpb * per_seq + 31) / 32 * 32);
    if (g.threads > kMaxThreads) return false;
    g.ld = tile_ld(c.st.n, c.order2, g.tpb, dtype, false);
    g.smem = ((size_t)g.tpb * g.ld * cplx_bytes(dtype) + 15) / 16 * 16 + (size_t)g.tpb * (a0.ncols + 1) * cplx_bytes(dtype);
    if (g.smem > kMaxSmem) return false;
    out->a = a0;
    out->a.ld = g.ld;
    out->a.core.stw = c.stw2.p;
    out->g = g;
    out->sl = &c.st;
    out->order = c.order2;
    return true;
  }
  // Stage list: the radix-32 one where every thread holds 32 elements.
  const bool wide = !g0.k1 && g0.ept == 0 && g0.max_radix >= 32 && c.wide.p;
  const StageList& sl = wide ? c.sw : c.st;
  // The specialised tile uses its own pad period, hence its own stride.
  Geo g = g0;
  // Balanced variant of a one-butterfly-per-thread geometry whose radices
  // differ: every thread takes maxR / R butterflies of a radix-R pass, so no
  // thread idles through the passes of the largest radix.
  if (g.k1 && g.balance != 0) {
    int rmin = 1 << 30, rmax = 0;
    for (int r : pass_order(sl)) {
      rmin = std::min(rmin, r);
      rmax = std::max(rmax, r);
    }
    bool divides = rmax > 0;
    for (int r : pass_order(sl)) divides = divides && rmax % r == 0;
    if (rmax > rmin && divides) {
      g.k1 = false;
      g.ept = rmax;
      int th = threads_needed(sl, rmax, g.tpb, false);
      g.threads = std::max(32, ((th + 31) / 32) * 32);
    }
  }
  g.ld = tile_ld(sl.n, pass_order(sl), g.tpb, dtype, column_mapped(k));
  g.smem = (size_t)g.tpb * g.ld * cplx_bytes(dtype);
  if (k == Kernel::COLS_TW && (mode & 8) && fs)  // pass A's twiddle tables after the tile
    g.smem = (g.smem + 15) / 16 * 16 + (size_t)smem_twiddle_entries(g.tpb, fs->n1) * cplx_bytes(dtype);
  if (k == Kernel::C2C_RADER)  // the staged rows (stride a0.ncols) and X_0 per sequence after the tile
    g.smem = (g.smem + 15) / 16 * 16 + (size_t)g.tpb * (a0.ncols + 1) * cplx_bytes(dtype);
  if (g.smem > kMaxSmem) return false;
  if (wide) {
    int th = threads_needed(sl, ept_of(dtype), g.tpb, false);
    th = std::max(32, ((th + 31) / 32) * 32);
    if (th > kMaxThreads) return false;
    g.threads = th;
  }
  out->a = a0;
  out->a.ld = g.ld;
  if (wide) {
    out->a.core.st = sl;
    out->a.core.stw = c.wide.p;
  }
  out->g = g;
  out->sl = &sl;
  out->order = pass_order(sl);
  return true;
}

// The compiled kernel for expr with at least smem bytes of dynamic shared
// memory allowed (caller holds g_mu). Returns 0, 1 (unavailable) or 2.
int kernel_for(const std::string& expr, size_t smem, CUfunction* fn) {
  int dev = 0;
  cudaGetDevice(&dev);
  Entry& e = g_cache[std::to_string(dev) + "|" + expr];
  if (e.failed) return 1;
  if (!e.fn) {
    std::string log;
    if (!compile(expr, &e, &log)) {
      e.failed = true;
      if (std::getenv("CHFFT_JIT_VERBOSE")) fprintf(stderr, "chfft plan-time compile failed for %s:\n%s\n", expr.c_str(), log.c_str());
      return 1;
    }
  }
  if ((int)smem > 48 * 1024 && e.smem_set < (int)smem) {
    if (g_api.cuFuncSetAttribute(e.fn, kAttrMaxDynSmem, (int)smem) != 0) return 2;
    e.smem_set = (int)smem;
  }
  *fn = e.fn;
  return 0;
}

}  // namespace

int jit_launch(Kernel k, int dtype, const Core& c, const Geo& g0, const KArgs& a0, unsigned blocks,
               cudaStream_t stream, int mode, const FourStep* fs) {
  if (four_step(k) && !fs) return 1;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!load_api()) return 1;
  Spec sp;
  if (!resolve(k, dtype, c, g0, a0, mode, fs, &sp)) return 1;
  const Geo& g = sp.g;
  KArgs& a = sp.a;
  CUfunction fn = nullptr;
  const std::string expr = name_expression(k, dtype, c, sp.sl->n, sp.order, g, mode);
  if (int r = kernel_for(expr, g.smem, &fn)) return r;
  void* args[] = {const_cast<KArgs*>(&a), const_cast<FourStep*>(fs)};
  if (g_api.cuLaunchKernel(fn, blocks, 1, 1, g.threads, 1, 1, (unsigned)g.smem, (CUstream)stream, args, nullptr) != 0)
    return 2;
  return 0;
}

size_t tc_geometry(const Core& c, Kernel k, int tpb, int prec, int* ld_out) {
  if (c.dtype != 0 || c.blue || c.tc_s16 < 1 || !c.tcw.p || prec < 1 || prec > 3 || tpb < 1) return 0;
  const long long n = c.st.n;
  const long long rows = (long long)tpb * (n / 16);
  if (rows % 128 || rows / 128 > 16) return 0;
  int ld = (int)(n + n / 16);
  const int q = column_mapped(k) ? std::max(1, 16 / tpb) : 1;
  while (ld % (2 * q) != q) ld++;
  const size_t tile = (size_t)tpb * ld * 8;
  const size_t a_off = (tile + 1023) / 1024 * 1024;
  const size_t np = prec == 3 ? 3 : 2;
  const size_t smem = a_off + (size_t)(rows / 128) * np * 8192 + np * 2048 + 16;
  if (smem > kMaxSmem) return 0;
  if (ld_out) *ld_out = ld;
  return smem;
}

int jit_launch_tc(Kernel k, const Core& c, int prec, int tpb, const KArgs& a0, unsigned blocks, cudaStream_t stream,
                  int mode, const FourStep* fs) {
  if (four_step(k) && !fs) return 1;
  if (k != Kernel::C2C && !four_step(k)) return 1;
  int ld = 0;
  const size_t smem = tc_geometry(c, k, tpb, prec, &ld);
  if (!smem) return 1;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!load_api()) return 1;
  std::string expr = "&";
  expr += kernel_template(k);
  expr += "<float, chfft::TcCore<";
  expr += column_mapped(k) ? "true," : "false,";
  expr += std::to_string(c.st.n) + "," + std::to_string(tpb) + "," + std::to_string(ld) + "," + std::to_string(prec) +
          "," + std::to_string(c.tc_r0) + "," + std::to_string(c.tc_s16) + ">";
  if (four_step(k)) expr += ", " + std::to_string(mode);
  expr += ">";
  KArgs a = a0;
  a.ld = ld;
  a.tpb = tpb;
  a.core.stw = c.tcw.p;
  a.core.err = a0.err;
  int dev = 0;
  cudaGetDevice(&dev);
  Entry& e = g_cache[std::to_string(dev) + "|" + expr];
  if (e.failed) return 1;
  if (!e.fn) {
    std::string log;
    if (!compile(expr, &e, &log)) {
      e.failed = true;
      if (std::getenv("CHFFT_JIT_VERBOSE")) fprintf(stderr, "chfft plan-time compile failed for %s:\n%s\n", expr.c_str(), log.c_str());
      return 1;
    }
  }
  if ((int)smem > 48 * 1024 && e.smem_set < (int)smem) {
    if (g_api.cuFuncSetAttribute(e.fn, kAttrMaxDynSmem, (int)smem) != 0) return 2;
    e.smem_set = (int)smem;
  }
  void* args[] = {const_cast<KArgs*>(&a), const_cast<FourStep*>(fs)};
  if (g_api.cuLaunchKernel(e.fn, blocks, 1, 1, kTcThreads, 1, 1, (unsigned)smem, (CUstream)stream, args, nullptr) != 0)
    return 2;
  return 0;
}

size_t jit_cache_size() {
  std::lock_guard<std::mutex> lk(g_mu);
  size_t n = 0;
  for (auto& kv : g_cache)
    if (kv.second.fn) n++;
  return n;
}

}  // namespace chfft
