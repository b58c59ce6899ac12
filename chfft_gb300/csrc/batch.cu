// Uneven batches: many transforms of mixed kinds and lengths in one launch
// fed by a device task queue (k_batch.cu), optionally replayed from a CUDA
// graph.
//
// The host side groups the jobs by (kind, length, option), builds each
// distinct length's tables once (FP64-generated, like every plan), decides
// per length between a one-CTA task and a four-step task chain (column
// tiles; row tiles, which for Bluestein also run the spectrum product and
// the inverse FFT's first pass; the inverse's last pass; real-kind post
// tasks), and writes the task queue: the chains' steps interleaved item by
// item with a lag of a few waves between an item's steps, one-CTA tasks
// (by decreasing cost) filling the gaps and following. The queue and every
// table live in device memory; a launch only passes the input / output
// base pointers, so it can be captured once and replayed.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/chfft_gpu.h"
#include "jit.hpp"
#include "k_batch.cuh"
#include "plan.hpp"

namespace chfft {

int record_error(int code, const std::string& msg);
cudaError_t launch_batch(const BatchArgs& a, unsigned blocks, size_t smem, cudaStream_t stream);

namespace {

constexpr size_t kBatchSmemCap = 100 * 1024;  // per CTA: two CTAs of 512 threads per SM
// Tile classes of four-step items: kind group (C2C, C2C Bluestein, real
// kinds) x four-step length (<= 2^14, <= 2^15, <= 2^16, larger).
constexpr int kBatchClasses = 12;
constexpr int kMaxSplit = 512;                // four-step factors in the batch kernel

bool batch_fits(const StageList& st, int tpb) {
  return threads_needed(st, kBatchEpt, tpb) <= kBatchThreads && (size_t)tpb * smem_ld(st.n) * 8 <= kBatchSmemCap;
}

// Four-step tile width of a core: the widest power of two from kBatchTile
// to kBatchTileMax whose tile fits one CTA. Wider tiles mean fewer tasks, so
// less per-task overhead (ticket, descriptor, waits, signal) per element.
int fs_width(const StageList& st, int cap = kBatchTileMax) {
  int w = kBatchTile;
  while (w * 2 <= cap && batch_fits(st, w * 2)) w *= 2;
  return w;
}

// Tables of one complex core as the batch kernel runs it.
struct HostCore {
  BatchCore d{};
  DevBuf tw, chirp, bhat;
};

bool batch_split(long long m, int* n1, int* n2) {
  double best = 1e300;
  bool ok = false;
  for (long long d = 2; d <= kMaxSplit; d++) {
    if (m % d || m / d > kMaxSplit) continue;
    StageList a, b;
    if (!make_stages(d, &a) || !make_stages(m / d, &b) || !batch_fits(a, kBatchTile) || !batch_fits(b, kBatchTile))
      continue;
    const double score = std::fabs(std::log((double)d) - 0.5 * std::log((double)m));
    if (score < best) {
      best = score;
      *n1 = (int)d;
      *n2 = (int)(m / d);
      ok = true;
    }
  }
  return ok;
}

void gen(Table t, long long n, long long count, long long m, void* out, cudaStream_t s) {
  CHFFT_CUDA(gen_table<float>(t, n, count, m, out, s));
}

// B^ = FFT_M(conj chirp) / M, FP64, rounded to f32.
void bluestein_spectrum(long long n, long long m, void* out, cudaStream_t s) {
  DevBuf b64, w64;
  b64.ensure(m * sizeof(double2));
  CHFFT_CUDA(gen_table<double>(Table::BLUE_B, n, m, m, b64.p, s));
  Core c64;
  if (c64.build(m, 1, s) && !c64.blue) {
    KArgs a{};
    a.core = c64.desc();
    Geo g = row_geo(c64, 1);
    a.tpb = g.tpb;
    a.ld = g.ld;
    a.count = 1;
    a.in = b64.p;
    a.out = b64.p;
    a.scale = 1.0;
    a.in_dist = a.out_dist = m;
    CHFFT_CUDA(launch_kernel<double>(Kernel::C2C, false, g.k1, a, 1, g.threads, g.smem, s));
  } else {
    BigCore big64;
    if (!big64.build(m, 1, s)) throw Fail{CHFFT_EUNSUPPORTED, "Bluestein length " + std::to_string(m)};
    w64.ensure(big64.work_elems(1) * sizeof(double2));
    big64.exec(b64.p, b64.p, w64.p, 1, false, 1.0, s, 0, true);
  }
  CHFFT_CUDA(convert_from_f64<float>(static_cast<const double2*>(b64.p), out, m, s));
  CHFFT_CUDA(cudaStreamSynchronize(s));
}

// One-CTA core for length n (mixed radix, or Bluestein with a one-CTA M).
bool build_small(HostCore& hc, long long n, cudaStream_t s) {
  StageList st;
  if (make_stages(n, &st) && batch_fits(st, 1)) {
    hc.tw.ensure(n * 8);
    gen(Table::OMEGA, n, n, 0, hc.tw.p, s);
    hc.d.st = st;
    hc.d.tw = hc.tw.p;
    hc.d.n = (int)n;
    hc.d.blue = 0;
    return true;
  }
  long long hi = 1;
  while (hi < 2 * n - 1) hi <<= 1;
  for (long long m = 2 * n - 1; m <= hi; m++) {
    if (!make_stages(m, &st) || !batch_fits(st, 1)) continue;
    hc.tw.ensure(m * 8);
    hc.chirp.ensure(n * 8);
    hc.bhat.ensure(m * 8);
    gen(Table::OMEGA, m, m, 0, hc.tw.p, s);
    gen(Table::CHIRP, n, n, 0, hc.chirp.p, s);
    bluestein_spectrum(n, m, hc.bhat.p, s);
    hc.d.st = st;
    hc.d.tw = hc.tw.p;
    hc.d.chirp = hc.chirp.p;
    hc.d.bhat = hc.bhat.p;
    hc.d.n = (int)n;
    hc.d.blue = 1;
    return true;
  }
  return false;
}

// Four-step tables for length n (Bluestein with a four-step M when n has a
// prime factor above 7 and blue_ok).
struct HostBig {
  HostCore ca, cb;
  DevBuf lo, hi, chirp, bhat;
  FourStep fs{};
  bool blue = false;
  long long m = 0;
};

bool build_big(HostBig& hb, long long n, bool blue_ok, cudaStream_t s) {
  int n1 = 0, n2 = 0;
  long long m = n;
  hb.blue = false;
  if (!factor_smooth(n).ok || !batch_split(n, &n1, &n2)) {
    if (!blue_ok) return false;
    long long lo_m = 2 * n - 1, hi_m = 1;
    while (hi_m < lo_m) hi_m <<= 1;
    m = -1;
    for (long long mm = lo_m; mm <= hi_m; mm++)
      if (factor_smooth(mm).ok && batch_split(mm, &n1, &n2)) {
        m = mm;
        break;
      }
    if (m < 0) return false;
    hb.blue = true;
  }
  hb.m = m;
  if (!build_small(hb.ca, n1, s) || !build_small(hb.cb, n2, s) || hb.ca.d.blue || hb.cb.d.blue) return false;
  const int sh = tw_shift_for(m), L = 1 << sh;
  const long long nhi = (m + L - 1) / L;
  hb.lo.ensure(L * 8);
  hb.hi.ensure(nhi * 8);
  gen(Table::OMEGA, m, L, 0, hb.lo.p, s);
  gen(Table::OMEGA_STRIDE, m, nhi, L, hb.hi.p, s);
  if (hb.blue) {
    hb.chirp.ensure(n * 8);
    hb.bhat.ensure(m * 8);
    gen(Table::CHIRP, n, n, 0, hb.chirp.p, s);
    bluestein_spectrum(n, m, hb.bhat.p, s);
  }
  hb.fs.n = m;
  hb.fs.n1 = n1;
  hb.fs.n2 = n2;
  hb.fs.tw_shift = sh;
  hb.fs.lo = hb.lo.p;
  hb.fs.hi = hb.hi.p;
  hb.fs.n_user = n;
  hb.fs.chirp = hb.chirp.p;
  hb.fs.bhat = hb.bhat.p;
  return true;
}

struct KindTables {
  DevBuf aux0, aux1;
};

}  // namespace

// A four-step item of the batch: its tables, its first counter and its
// tile class (for the per-class tile caps).
struct BigRef {
  int item, big, c0, cls;
};

struct BatchImpl {
  std::vector<std::unique_ptr<HostCore>> smalls;
  std::vector<std::unique_ptr<HostBig>> bigs;
  std::vector<std::unique_ptr<KindTables>> kinds;
  std::vector<BatchItem> items;                        // host copy (queue order of the jobs)
  std::vector<BigRef> big_items;
  std::vector<std::pair<double, BatchTask>> small_sorted;  // one-CTA tasks, longest first
  int caps[kBatchClasses] = {};                        // widest tile per class
  bool class_used[kBatchClasses] = {};
  DevBuf d_items, d_tasks, d_ctr, d_work;
  int ntasks = 0, nitems = 0, nctr = 0, nbig = 0;
  size_t smem = 0, work_bytes = 0;
  unsigned blocks = 0;  // CTAs per launch
  cudaStream_t stream = nullptr;
  // captured launch
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  const void* g_in = nullptr;
  void* g_out = nullptr;
  cudaStream_t g_stream = nullptr;

  ~BatchImpl() {
    drop_graph();
    if (stream) cudaStreamDestroy(stream);
  }

  void drop_graph() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (graph) cudaGraphDestroy(graph);
    graph_exec = nullptr;
    graph = nullptr;
  }

  // The task queue for the current tile caps, uploaded (see the queue-order
  // comment inside), and the shared memory per CTA it needs.
  void build_tasks(cudaStream_t s);

  void enqueue(const void* d_in, void* d_out, cudaStream_t s) {
    CHFFT_CUDA(cudaMemsetAsync(d_ctr.p, 0, (size_t)(nctr + 2) * sizeof(int), s));
    BatchArgs a{};
    a.tasks = static_cast<const BatchTask*>(d_tasks.p);
    a.ntasks = ntasks;
    a.items = static_cast<const BatchItem*>(d_items.p);
    a.ctr = static_cast<int*>(d_ctr.p);
    a.next = a.ctr + nctr;
    a.err = a.ctr + nctr + 1;
    a.in = static_cast<const char*>(d_in);
    a.out = static_cast<char*>(d_out);
    a.work = static_cast<char*>(d_work.p);
    // CHFFT_SPIN_LIMIT polls (default ~1 s); CHFFT_TEST_STALL=1 makes every
    // dependency unreachable (the waits run out, chfft_batch_wait reports it).
    a.spin_limit = (int)std::min<long long>(spin_limit(), 0x7fffffffLL);
    a.stall = stall_test();
    CHFFT_CUDA(launch_batch(a, blocks, smem, s));
  }
};

void BatchImpl::build_tasks(cudaStream_t s) {
  // Four-step tasks per item and step: A (columns), then B / BB (rows),
  // then C (Bluestein's last rows) or POST (real kinds' split).
  struct Group {
    int item, step;
    std::vector<BatchTask> t;
  };
  std::vector<std::vector<Group>> chains;
  for (const BigRef& r : big_items) {
    const int i = r.item, c0 = r.c0;
    const BatchItem& it = items[i];
    const HostBig& hb = *bigs[r.big];
    const int cap = caps[r.cls];
    const int wa = fs_width(hb.ca.d.st, cap), wb = fs_width(hb.cb.d.st, cap);
    const int na = (hb.fs.n2 + wa - 1) / wa, nb = (hb.fs.n1 + wb - 1) / wb;
    std::vector<Group> chain(hb.blue || it.kind != BK_C2C ? 3 : 2);
    for (int g = 0; g < (int)chain.size(); g++) chain[g] = Group{i, g, {}};
    for (int t = 0; t < na; t++) chain[0].t.push_back({BT_FS_A, i, wa, hb.blue ? 1 : 0, t, -1, 0, c0});
    if (hb.blue) {
      // Forward rows + spectrum + the inverse's rows (FS_BB), then the
      // inverse's n1-long rows with the chirp-out (FS_C).
      const int wc = fs_width(hb.ca.d.st, cap), nc = (hb.fs.n2 + wc - 1) / wc;
      for (int t = 0; t < nb; t++) chain[1].t.push_back({BT_FS_BB, i, wb, 0, t, c0, na, c0 + 1});
      for (int t = 0; t < nc; t++) chain[2].t.push_back({BT_FS_C, i, wc, 0, t, c0 + 1, nb, -1});
    } else {
      const int bmode = it.kind == BK_C2C ? 0 : 3;
      // A task whose counter nobody waits for (the last step of a C2C
      // item) skips the signal and its store fence.
      const int b_sig = it.kind != BK_C2C ? c0 + 1 : -1;
      for (int t = 0; t < nb; t++) chain[1].t.push_back({BT_FS_B, i, wb, bmode, t, c0, na, b_sig});
    }
    if (it.kind != BK_C2C) {
      const int pairs = (it.n + 3) / 4;
      for (int q = 0; q * kPostChunk < pairs; q++) chain[2].t.push_back({BT_POST, i, 1, 0, q, c0 + 1, nb, -1});
    }
    chains.push_back(std::move(chain));
  }
  // Queue order. Each four-step item's steps follow one another with a
  // lag of at least `lag` tickets (about two waves of resident CTAs), so a
  // step's inputs are normally complete when its CTAs start, and the items
  // in flight keep their intermediates in L2 (the level-by-level order
  // sent every intermediate through DRAM). A step is queued only after
  // every task it waits for, so a waited-for task is always held by a CTA
  // that is already running. One-CTA tasks (longest first) fill the gaps
  // where no step is due yet, and then follow.
  std::vector<BatchTask> tasks;
  {
    long long lag = 4LL * num_sms();
    if (const char* e = std::getenv("CHFFT_BATCH_LAG")) lag = std::max(0LL, std::atoll(e));
    const size_t nchain = chains.size();
    std::vector<int> next_step(nchain, 0);
    std::vector<size_t> step_end(nchain, 0);  // queue length after the item's last queued step
    size_t started = 0, small_next = 0, done_chains = 0;
    auto emit = [&](size_t c) {
      Group& g = chains[c][next_step[c]];
      tasks.insert(tasks.end(), g.t.begin(), g.t.end());
      step_end[c] = tasks.size();
      if (++next_step[c] == (int)chains[c].size()) done_chains++;
    };
    size_t oldest = 0;  // chains before it are done
    while (done_chains < nchain) {
      while (oldest < started && next_step[oldest] == (int)chains[oldest].size()) oldest++;
      // a due later step of a started item (oldest first)
      size_t due = nchain;
      for (size_t c = oldest; c < started; c++)
        if (next_step[c] < (int)chains[c].size() && tasks.size() >= step_end[c] + (size_t)lag) {
          due = c;
          break;
        }
      if (due < nchain) {
        emit(due);
      } else if (started < nchain) {
        emit(started++);
      } else if (small_next < small_sorted.size()) {
        tasks.push_back(small_sorted[small_next++].second);
      } else {
        for (size_t c = oldest; c < started; c++)
          if (next_step[c] < (int)chains[c].size()) {
            emit(c);
            break;
          }
      }
    }
    for (; small_next < small_sorted.size(); small_next++) tasks.push_back(small_sorted[small_next].second);
  }
  // ---- shared memory per CTA: the largest tile
  size_t smem_need = 16;
  for (const BatchTask& t : tasks) {
    const BatchItem& it = items[t.item];
    size_t need = 0;
    if (t.type == BT_SMALL) need = (size_t)t.count * smem_ld(it.core.st.n) * 8;
    else if (t.type == BT_FS_A || t.type == BT_FS_C) need = (size_t)t.count * smem_ld(it.ca.st.n) * 8;
    else if (t.type == BT_FS_B || t.type == BT_FS_BB) need = (size_t)t.count * smem_ld(it.cb.st.n) * 8;
    smem_need = std::max(smem_need, need);
  }
  // ---- upload
  ntasks = (int)tasks.size();
  smem = smem_need;
  d_tasks.ensure(std::max<size_t>(1, tasks.size()) * sizeof(BatchTask));
  if (!tasks.empty())
    CHFFT_CUDA(cudaMemcpyAsync(d_tasks.p, tasks.data(), tasks.size() * sizeof(BatchTask), cudaMemcpyHostToDevice, s));
  blocks = (unsigned)std::max(1, ntasks);
  CHFFT_CUDA(cudaStreamSynchronize(s));
  drop_graph();  // a captured launch holds the old task count
}

}  // namespace chfft

struct chfft_batch_s {
  chfft::BatchImpl impl;
};

using chfft::Fail;

extern "C" {

int chfft_batch_create(int dtype, const chfft_batch_job* jobs, size_t njobs, chfft_batch* out) {
  using namespace chfft;
  if (!out || (njobs && !jobs)) return record_error(CHFFT_EINVAL, "null argument");
  *out = nullptr;
  if (dtype != CHFFT_F32) return record_error(CHFFT_EUNSUPPORTED, "uneven batches run in f32");
  std::unique_ptr<chfft_batch_s> b(new chfft_batch_s());
  BatchImpl& B = b->impl;
  try {
    CHFFT_CUDA(cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking));
    cudaStream_t s = B.stream;
    // ---- validate and group
    struct Job {
      int kind, opt;
      long long n;
      double scale;
      size_t in, out, idx;
    };
    std::vector<Job> js;
    for (size_t i = 0; i < njobs; i++) {
      const chfft_batch_job& j = jobs[i];
      Job x{};
      x.n = (long long)j.len;
      x.in = j.in_offset;
      x.out = j.out_offset;
      x.idx = i;
      const double n = (double)j.len;
      switch (j.kind) {
        case CHFFT_KIND_CFFT1D:
          x.kind = BK_C2C;
          if (j.len < 2) return record_error(CHFFT_EINVAL_LEN, "invalid length");
          if (j.method == CHFFT_FORWARD || j.method == CHFFT_FORWARD0) x.scale = 1.0;
          else if (j.method == CHFFT_FORWARDU) x.scale = 1.0 / std::sqrt(n);
          else if (j.method == CHFFT_FORWARDN) x.scale = 1.0 / n;
          else return record_error(CHFFT_EINVAL, "uneven batches run forward methods");
          break;
        case CHFFT_KIND_RFFT1D:
          x.kind = BK_R2C;
          if ((j.len & 1) || j.len < 2) return record_error(CHFFT_EINVAL_LEN, "invalid length");
          if (j.method == CHFFT_FORWARD || j.method == CHFFT_FORWARD0) x.scale = 1.0;
          else if (j.method == CHFFT_FORWARDU) x.scale = 1.0 / std::sqrt(n);
          else if (j.method == CHFFT_FORWARDN) x.scale = 1.0 / n;
          else return record_error(CHFFT_EINVAL, "uneven batches run forward methods");
          break;
        case CHFFT_KIND_DCT1D:
          x.kind = BK_DCT2;
          x.opt = j.option != 0;
          if ((j.len & 1) || j.len < 2) return record_error(CHFFT_EINVAL_LEN, "invalid length");
          if (j.method == CHFFT_FORWARD || j.method == CHFFT_FORWARD0) x.scale = 1.0;
          else if (j.method == CHFFT_FORWARDU) x.scale = std::sqrt(2.0 / n);
          else if (j.method == CHFFT_FORWARDN) x.scale = 2.0 / n;
          else return record_error(CHFFT_EINVAL, "uneven batches run forward methods");
          break;
        case CHFFT_KIND_MDCT1D:
          x.kind = BK_MDCT;
          x.opt = j.option == CHFFT_WINDOW_VORBIS ? 1 : 0;
          if ((j.len & 3) || j.len < 4) return record_error(CHFFT_EINVAL_LEN, "invalid length");
          if (j.method == CHFFT_FORWARD) x.scale = std::sqrt(n / 2.0);
          else if (j.method == CHFFT_FORWARDU) x.scale = 1.0;
          else return record_error(CHFFT_EINVAL, "uneven batches run forward methods");
          break;
        default: return record_error(CHFFT_EINVAL, "unknown kind");
      }
      js.push_back(x);
    }
    std::stable_sort(js.begin(), js.end(), [](const Job& a, const Job& c) {
      return std::tie(a.kind, a.n, a.opt) < std::tie(c.kind, c.n, c.opt);
    });
    // ---- per-length tables
    std::map<long long, int> small_of, big_of;
    std::map<std::tuple<int, long long, int>, int> kind_of;
    auto core_len = [](int kind, long long n) { return kind == BK_C2C ? n : kind == BK_MDCT ? n / 4 : n / 2; };
    std::vector<BatchItem> items(js.size());
    long long work_elems = 0;

    std::vector<std::pair<double, BatchTask>>& small_sorted = B.small_sorted;
    int nctr = 0;
    for (size_t i = 0; i < js.size(); i++) {
      const Job& x = js[i];
      BatchItem& it = items[i];
      it.kind = x.kind;
      it.n = (int)x.n;
      it.ncore = (int)core_len(x.kind, x.n);
      it.scale = (float)x.scale;
      it.ortho = x.opt ? (float)std::sqrt(0.5) : 1.0f;
      it.in_off = (long long)x.in;
      it.out_off = (long long)x.out;
      const auto kkey = std::make_tuple(x.kind, x.n, x.opt);
      if (x.kind != BK_C2C && !kind_of.count(kkey)) {
        auto kt = std::make_unique<KindTables>();
        const long long h = x.n / 2, q = x.n / 4;
        if (x.kind == BK_R2C) {
          kt->aux0.ensure(h * 8);
          gen(Table::RCOEF, x.n, h, 0, kt->aux0.p, s);
        } else if (x.kind == BK_DCT2) {
          kt->aux0.ensure(h * 8);
          kt->aux1.ensure((h + 1) * 8);
          gen(Table::RCOEF, x.n, h, 0, kt->aux0.p, s);
          gen(Table::OMEGA4N_POS, x.n, h + 1, 0, kt->aux1.p, s);
        } else {
          kt->aux0.ensure(q * 8);
          kt->aux1.ensure(x.n * 4);
          gen(Table::MDCT_TW, x.n, q, 0, kt->aux0.p, s);
          gen(x.opt ? Table::VORBIS_WIN : Table::SINE_WIN, x.n, x.n, 0, kt->aux1.p, s);
        }
        kind_of[kkey] = (int)B.kinds.size();
        B.kinds.push_back(std::move(kt));
      }
      if (x.kind != BK_C2C) {
        const KindTables& kt = *B.kinds[kind_of[kkey]];
        it.aux0 = kt.aux0.p;
        it.aux1 = kt.aux1.p;
      }
      const long long nc = it.ncore;
      if (!small_of.count(nc) && !big_of.count(nc)) {
        auto hc = std::make_unique<HostCore>();
        if (build_small(*hc, nc, s)) {
          small_of[nc] = (int)B.smalls.size();
          B.smalls.push_back(std::move(hc));
        } else {
          auto hb = std::make_unique<HostBig>();
          if (!build_big(*hb, nc, true, s))
            return record_error(CHFFT_EUNSUPPORTED, "length " + std::to_string(x.n) + " is too long for a batch");
          big_of[nc] = (int)B.bigs.size();
          B.bigs.push_back(std::move(hb));
        }
      }
      if (small_of.count(nc)) {
        it.big = 0;
        it.core = B.smalls[small_of[nc]]->d;
      } else {
        const HostBig& hb = *B.bigs[big_of[nc]];
        if (hb.blue && x.kind != BK_C2C)
          return record_error(CHFFT_EUNSUPPORTED, "real kinds in a batch need a 7-smooth half length beyond 8192");
        it.big = hb.blue ? 2 : 1;
        it.ca = hb.ca.d;
        it.cb = hb.cb.d;
        it.fs = hb.fs;
        it.work_off = work_elems * 8;
        work_elems += hb.m;
        if (hb.blue || x.kind != BK_C2C) {
          it.work2_off = work_elems * 8;
          work_elems += hb.m;
        }
        // its tasks come from build_tasks (tile widths per class)
        const int grp = hb.blue ? 1 : (x.kind != BK_C2C ? 2 : 0);
        const int bucket = hb.m <= (1 << 14) ? 0 : hb.m <= (1 << 15) ? 1 : hb.m <= (1 << 16) ? 2 : 3;
        B.big_items.push_back(BigRef{(int)i, big_of[nc], nctr, grp * 4 + bucket});
        B.class_used[grp * 4 + bucket] = true;
        nctr += 4;
      }
    }
    // ---- one-CTA tasks: consecutive items of one (kind, length, option), up to tpb per task
    for (size_t i = 0; i < js.size();) {
      if (items[i].big) {
        i++;
        continue;
      }
      size_t j = i;
      while (j < js.size() && !items[j].big && js[j].kind == js[i].kind && js[j].n == js[i].n && js[j].opt == js[i].opt)
        j++;
      const StageList& st = items[i].core.st;
      int tpb = std::max(1, kBatchThreads / std::max(1, threads_needed(st, kBatchEpt, 1)));
      while (tpb > 1 && !batch_fits(st, tpb)) tpb--;
      for (size_t k = i; k < j; k += tpb) {
        const int cnt = (int)std::min<size_t>(tpb, j - k);
        const double cost = (double)cnt * st.n * std::log2((double)st.n + 1) * (items[i].core.blue ? 2 : 1);
        small_sorted.push_back({cost, BatchTask{BT_SMALL, (int)k, cnt, 0, 0, -1, 0, -1}});
      }
      i = j;
    }
    std::stable_sort(small_sorted.begin(), small_sorted.end(),
                     [](const std::pair<double, BatchTask>& a, const std::pair<double, BatchTask>& c) {
                       return a.first > c.first;
                     });
    // ---- upload
    B.nitems = (int)items.size();
    B.nctr = nctr;
    B.d_items.ensure(std::max<size_t>(1, items.size()) * sizeof(BatchItem));
    B.d_ctr.ensure((size_t)(nctr + 2) * sizeof(int));
    B.work_bytes = (size_t)work_elems * 8;
    B.d_work.ensure(std::max<size_t>(B.work_bytes, 256));
    if (!items.empty())
      CHFFT_CUDA(cudaMemcpyAsync(B.d_items.p, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice, s));
    B.items = std::move(items);
    for (int& c : B.caps) c = kBatchTileMax;
    B.build_tasks(s);
  } catch (const Fail& f) {
    return record_error(f.code, f.msg);
  }
  *out = b.release();
  return CHFFT_OK;
}

int chfft_batch_execute(chfft_batch batch, const void* d_in, void* d_out, void* stream) {
  if (!batch) return chfft::record_error(CHFFT_EINVAL, "null batch");
  try {
    batch->impl.enqueue(d_in, d_out, static_cast<cudaStream_t>(stream));
  } catch (const Fail& f) {
    return chfft::record_error(f.code, f.msg);
  }
  return CHFFT_OK;
}

int chfft_batch_execute_graph(chfft_batch batch, const void* d_in, void* d_out, void* stream) {
  if (!batch) return chfft::record_error(CHFFT_EINVAL, "null batch");
  chfft::BatchImpl& B = batch->impl;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  try {
    if (!B.graph_exec || B.g_in != d_in || B.g_out != d_out) {
      if (B.graph_exec) cudaGraphExecDestroy(B.graph_exec);
      if (B.graph) cudaGraphDestroy(B.graph);
      B.graph_exec = nullptr;
      B.graph = nullptr;
      cudaStream_t cap = B.stream;  // capture on the batch's own stream
      CHFFT_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
      B.enqueue(d_in, d_out, cap);
      CHFFT_CUDA(cudaStreamEndCapture(cap, &B.graph));
      CHFFT_CUDA(cudaGraphInstantiate(&B.graph_exec, B.graph, 0));
      B.g_in = d_in;
      B.g_out = d_out;
    }
    CHFFT_CUDA(cudaGraphLaunch(B.graph_exec, s));
  } catch (const Fail& f) {
    return chfft::record_error(f.code, f.msg);
  }
  return CHFFT_OK;
}

int chfft_batch_wait(chfft_batch batch, void* stream) {
  if (!batch) return chfft::record_error(CHFFT_EINVAL, "null batch");
  chfft::BatchImpl& B = batch->impl;
  int err = 0;
  cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  if (e == cudaSuccess)
    e = cudaMemcpy(&err, static_cast<int*>(B.d_ctr.p) + B.nctr + 1, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return chfft::record_error(CHFFT_ECUDA, cudaGetErrorString(e));
  if (err) return chfft::record_error(CHFFT_ETIMEOUT, "a batch task waited too long for its dependencies");
  return CHFFT_OK;
}

int chfft_batch_autotune(chfft_batch batch, const void* d_in, void* d_out, void* stream, int reps, float* best_ms) {
  using namespace chfft;
  if (!batch || reps < 1) return record_error(CHFFT_EINVAL, "null batch or reps < 1");
  BatchImpl& B = batch->impl;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  try {
    CHFFT_CUDA(cudaEventCreate(&e0));
    CHFFT_CUDA(cudaEventCreate(&e1));
    int err = 0;
    // Median of `reps` launches of the current task list (one launch first).
    auto time_it = [&]() -> float {
      B.build_tasks(B.stream);
      B.enqueue(d_in, d_out, s);
      std::vector<float> v;
      for (int r = 0; r < reps; r++) {
        CHFFT_CUDA(cudaEventRecord(e0, s));
        B.enqueue(d_in, d_out, s);
        CHFFT_CUDA(cudaEventRecord(e1, s));
        CHFFT_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        CHFFT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        v.push_back(ms);
      }
      CHFFT_CUDA(cudaMemcpy(&err, static_cast<int*>(B.d_ctr.p) + B.nctr + 1, sizeof(int), cudaMemcpyDeviceToHost));
      if (err) throw Fail{CHFFT_ETIMEOUT, "a batch task waited too long for its dependencies"};
      std::sort(v.begin(), v.end());
      return v[v.size() / 2];
    };
    float best = time_it();
    for (int c = 0; c < kBatchClasses; c++) {
      if (!B.class_used[c]) continue;
      int keep = B.caps[c];
      for (int cap : {16, 32, 64}) {
        if (cap == keep) continue;
        B.caps[c] = cap;
        const float t = time_it();
        if (t < best) {
          best = t;
          keep = cap;
        }
      }
      B.caps[c] = keep;
    }
    B.build_tasks(B.stream);
    if (best_ms) *best_ms = best;
  } catch (const Fail& f) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return record_error(f.code, f.msg);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return CHFFT_OK;
}

int chfft_batch_get_info(chfft_batch batch, chfft_batch_info* info) {
  if (!batch || !info) return chfft::record_error(CHFFT_EINVAL, "null argument");
  const chfft::BatchImpl& B = batch->impl;
  std::memset(info, 0, sizeof(*info));
  info->jobs = (size_t)B.nitems;
  info->tasks = (size_t)B.ntasks;
  info->ctas = B.blocks;
  info->smem_per_cta = B.smem;
  info->workspace_bytes = B.work_bytes;
  info->four_step_lengths = B.bigs.size();
  info->one_cta_lengths = B.smalls.size();
  for (int c = 0; c < chfft::kBatchClasses && c < 12; c++) info->class_tile[c] = B.class_used[c] ? B.caps[c] : 0;
  return CHFFT_OK;
}

int chfft_batch_destroy(chfft_batch batch) {
  delete batch;
  return CHFFT_OK;
}

}  // extern "C"
