// Persistent uneven-batch kernel (see k_batch.cuh). f32 only.
//
// Every task runs the same three steps: a kind-specific load phase into the
// shared-memory tile, the complex core on the tile (one call site for every
// task type, so the pass code is instantiated once), and a kind-specific
// store phase. Real-kind pre- and post-processing follow chfft's formulas
// (src/rfft1d.rs:128-148, src/dct1d.rs:248-289, src/mdct1d.rs:206-241).
#include "k_batch.cuh"

namespace chfft {
namespace {

using C = float2;

__device__ __forceinline__ C ldcg(const C* p) { return __ldcg(p); }

// DCT-II input reorder v = (x0, x2, ..., x_{N-2}, x_{N-1}, ..., x3, x1).
__device__ __forceinline__ float dct_v(const float* x, int n, int j) {
  return j < (n >> 1) ? x[2 * j] : x[2 * (n - 1 - j) + 1];
}

// z_i of a real kind's complex core input (i < ncore), scaled.
__device__ __forceinline__ C real_pre(const BatchItem& it, const char* in_base, long long i) {
  const float* x = reinterpret_cast<const float*>(in_base + it.in_off);
  if (it.kind == BK_R2C) return mk(x[2 * i] * it.scale, x[2 * i + 1] * it.scale);
  if (it.kind == BK_DCT2) {
    float re = dct_v(x, it.n, (int)(2 * i)), im = dct_v(x, it.n, (int)(2 * i + 1));
    if (i == 0) re *= it.ortho;
    return mk(re * it.scale, im * it.scale);
  }
  // MDCT: window, fold and pre-twiddle
  const float* w = static_cast<const float*>(it.aux1);
  const C* tw = static_cast<const C*>(it.aux0);
  const int lenh = it.n >> 1, lenq = lenh >> 1, leno = lenq - (lenq >> 1), len3q = lenh + lenq, len5q = lenh + len3q;
  const int k = (int)(i << 1);
  float re, im;
  if (i < leno) {
    re = x[len3q - 1 - k] * w[len3q - 1 - k] + x[len3q + k] * w[len3q + k];
    im = x[lenq + k] * w[lenq + k] - x[lenq - 1 - k] * w[lenq - 1 - k];
  } else {
    re = x[len3q - 1 - k] * w[len3q - 1 - k] - x[k - lenq] * w[k - lenq];
    im = x[lenq + k] * w[lenq + k] + x[len5q - 1 - k] * w[len5q - 1 - k];
  }
  return cmul(mk(re, im), __ldg(&tw[i]));
}

// R2C split (src/rfft1d.rs:136-148) / DCT-II post-twiddle (src/dct1d.rs:266-289)
// for pair index i of one transform; zk(k) returns core output Z_k.
template <class Z>
__device__ __forceinline__ void real_post(const BatchItem& it, char* out_base, int i, const Z& zk) {
  const int h = it.ncore, N = it.n;
  if (it.kind == BK_R2C) {
    C* o = reinterpret_cast<C*>(out_base + it.out_off);
    const int qlen = (N + 3) >> 2;
    if (i >= qlen) return;
    if (i == 0) {
      C z0 = zk(0);
      o[0] = mk(z0.x + z0.y, 0.f);
      o[h] = mk(z0.x - z0.y, 0.f);
      if ((N & 3) == 0) o[qlen] = cconj(zk(qlen));
    } else {
      C zi = zk(i), zh = zk(h - i);
      C x = cmul(__ldg(&static_cast<const C*>(it.aux0)[i]), csub(zi, cconj(zh)));
      o[i] = csub(zi, x);
      o[h - i] = cadd(zh, cconj(x));
    }
    return;
  }
  float* o = reinterpret_cast<float*>(out_base + it.out_off);
  const C* coef = static_cast<const C*>(it.aux0);
  const C* om = static_cast<const C*>(it.aux1);
  const int q2 = (N + 3) >> 2;
  if (i >= q2) return;
  if (i == 0) {
    C z0 = zk(0);
    o[0] = z0.x + z0.y;
    o[h] = (z0.x - z0.y) * __ldg(&om[h]).x;
    if ((N & 3) == 0) {
      C x = cmul(zk(q2), __ldg(&om[q2]));
      o[q2] = x.x;
      o[N - q2] = x.y;
    }
  } else {
    C zi = zk(i);
    C wconj = cconj(zk(h - i));
    C x = cmul(__ldg(&coef[i]), csub(zi, wconj));
    C j = cmul(cconj(csub(zi, x)), __ldg(&om[i]));
    o[i] = j.x;
    o[N - i] = j.y;
    C k = cmul(cadd(wconj, x), __ldg(&om[h - i]));
    o[h - i] = k.x;
    o[h + i] = k.y;
  }
}

// Bounded wait of thread 0 for a dependency counter. After a time-out (or
// once another task's wait timed out) the task goes on without its inputs;
// the host reads the error word and reports CHFFT_ETIMEOUT. A.stall (test
// hook) raises every target by one, so no dependency is ever met.
__device__ __forceinline__ void wait_for(const BatchArgs& A, int ctr, int target) {
  if (threadIdx.x == 0) {
    target += A.stall;
    int it = 0;
    while (ld_acquire(A.ctr + ctr) < target) {  // acquire: the producers' stores are visible after it
      if (++it > A.spin_limit || *(volatile int*)A.err) {
        atomicExch(A.err, 1);
        break;
      }
      __nanosleep(200);
    }
  }
  __syncthreads();
}

__device__ __forceinline__ void signal(const BatchArgs& A, int ctr) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(A.ctr + ctr, 1);
  }
}

// One task of the queue, ticket ti (s_item: the CTA's descriptor copy).
__device__ __forceinline__ void batch_task(const BatchArgs& A, int ti, unsigned char* smem_raw, BatchItem& s_item) {
  C* sbase = reinterpret_cast<C*>(smem_raw);
  const BatchTask tk = A.tasks[ti];
  {
    const int* src = reinterpret_cast<const int*>(A.items + tk.item);
    int* dst = reinterpret_cast<int*>(&s_item);
    for (int w = threadIdx.x; w < (int)(sizeof(BatchItem) / 4); w += blockDim.x) dst[w] = __ldg(src + w);
  }
  if (tk.wait_ctr >= 0) wait_for(A, tk.wait_ctr, tk.wait_target);  // ends with a barrier
  else __syncthreads();
  const BatchItem& it = s_item;
  const int tid = threadIdx.x, nth = blockDim.x;

  if (tk.type == BT_POST) {
    const C* z = reinterpret_cast<const C*>(A.work + it.work2_off);
    const int i = tk.tile * kPostChunk;
    for (int p = i + tid; p < i + kPostChunk; p += nth) real_post(it, A.out, p, [&](int k) { return ldcg(z + k); });
    if (tk.signal_ctr >= 0) signal(A, tk.signal_ctr);
    return;
  }

  // ---- the core and its tile
  const BatchCore& core = tk.type == BT_SMALL ? it.core : (tk.type == BT_FS_A || tk.type == BT_FS_C ? it.ca : it.cb);
  const int m = core.st.n;
  // SMALL: transforms in the task; FS_A / FS_B: tile width (a power of two).
  const int tpb = tk.count;
  const int lw = 31 - __clz(tpb);
  const SmemIO<C> sm{sbase, smem_ld(m)};
  const FourStep& fs = it.fs;

  // ---- load phase
  if (tk.type == BT_SMALL) {
    for (int b = tid; b < tpb * m; b += nth) {
      const int t = b / m, i = b - t * m;
      const BatchItem& x = A.items[tk.item + t];
      C v = czero<C>();
      if (i < core.n) {
        if (x.kind == BK_C2C)
          v = cscale(reinterpret_cast<const C*>(A.in + x.in_off)[i], x.scale);
        else
          v = real_pre(x, A.in, i);
        if (core.blue) v = cmul(v, __ldg(&static_cast<const C*>(core.chirp)[i]));
      }
      sm.store(t, i, v);
    }
  } else if (tk.type == BT_FS_A) {
    const int c0 = tk.tile * tpb;
    for (int b = tid; b < tpb * m; b += nth) {
      const int t = b & (tpb - 1), i = b >> lw;  // consecutive threads: adjacent columns
      const int col = c0 + t;
      C v = czero<C>();
      if (col < fs.n2) {
        const long long flat = (long long)i * fs.n2 + col;
        if (tk.mode == 2) {
          v = ldcg(reinterpret_cast<const C*>(A.work + it.work2_off) + flat);
        } else if (it.kind == BK_C2C) {
          if (tk.mode == 0 || flat < fs.n_user) {
            v = cscale(reinterpret_cast<const C*>(A.in + it.in_off)[flat], it.scale);
            if (tk.mode == 1) v = cmul(v, __ldg(&static_cast<const C*>(fs.chirp)[flat]));
          }
        } else {
          v = real_pre(it, A.in, flat);
        }
      }
      sm.store(t, i, v);
    }
  } else {  // BT_FS_B / BT_FS_BB: rows of n2 of the workspace; BT_FS_C: rows of n1 of the second workspace
    const int r0 = tk.tile * tpb;
    const bool c = tk.type == BT_FS_C;
    const C* w = reinterpret_cast<const C*>(A.work + (c ? it.work2_off : it.work_off));
    const int nrows = c ? fs.n2 : fs.n1;
    for (int b = tid; b < tpb * m; b += nth) {
      const int t = b / m, i = b - t * m;  // consecutive threads along a row
      const int row = r0 + t;
      sm.store(t, i, row < nrows ? ldcg(w + (long long)row * m + i) : czero<C>());
    }
  }
  __syncthreads();

  // ---- complex core
  // Between the two FFT rounds of a Bluestein core (one-CTA SMALL) or of an
  // FS_BB row tile: the spectrum product, conjugated for the inverse.
  auto between = [&]() {
    if (core.blue) {
      spectrum_phase<false>(sm, m, tpb, static_cast<const C*>(core.bhat));
      return;
    }
    // conj(X_k B^_k) at natural index k = k1 + n1 k2 (row k1, element k2)
    const int r0 = tk.tile * tpb;
    const C* bh = static_cast<const C*>(fs.bhat);
    for (int b = tid; b < tpb * m; b += nth) {
      const int t = b / m, k2 = b - t * m;
      const int k1 = min(r0 + t, fs.n1 - 1);  // rows past n1 are never stored
      sm.store(t, k2, cconj(cmul(sm.load(t, k2), __ldg(&bh[k1 + (long long)fs.n1 * k2]))));
    }
    __syncthreads();
  };
  const bool two_rounds = core.blue || tk.type == BT_FS_BB;
  // Two call sites rather than a loop over the rounds: a loop around the
  // passes makes the compiler spill.
  smem_passes<false, false, kBatchEpt>(core.st.all, m, 1, tpb, static_cast<const C*>(core.tw), sm);
  if (two_rounds) {
    between();
    smem_passes<false, false, kBatchEpt>(core.st.all, m, 1, tpb, static_cast<const C*>(core.tw), sm);
  }

  // ---- store phase
  if (tk.type == BT_SMALL) {
    const int L = core.n;
    if (core.blue) {  // Z_k = conj(Y_k) c_k, in place
      for (int b = tid; b < tpb * L; b += nth) {
        const int t = b / L, k = b - t * L;
        sm.store(t, k, cmul(cconj(sm.load(t, k)), __ldg(&static_cast<const C*>(core.chirp)[k])));
      }
      __syncthreads();
    }
    if (it.kind == BK_C2C || it.kind == BK_MDCT) {
      for (int b = tid; b < tpb * L; b += nth) {
        const int t = b / L, k = b - t * L;
        const BatchItem& x = A.items[tk.item + t];
        const C z = sm.load(t, k);
        if (x.kind == BK_C2C) {
          reinterpret_cast<C*>(A.out + x.out_off)[k] = z;
        } else {
          C r = cmul(z, cscale(__ldg(&static_cast<const C*>(x.aux0)[k]), x.scale));
          float* o = reinterpret_cast<float*>(A.out + x.out_off);
          o[2 * k] = -r.x;
          o[(x.n >> 1) - 1 - 2 * k] = r.y;
        }
      }
    } else {
      const int pairs = (it.n + 3) >> 2;
      for (int b = tid; b < tpb * pairs; b += nth) {
        const int t = b / pairs, i = b - t * pairs;
        real_post(A.items[tk.item + t], A.out, i, [&](int k) { return sm.load(t, k); });
      }
    }
  } else if (tk.type == BT_FS_A) {
    const int c0 = tk.tile * tpb;
    C* w = reinterpret_cast<C*>(A.work + it.work_off);
    const C* lo = static_cast<const C*>(fs.lo);
    const C* hi = static_cast<const C*>(fs.hi);
    for (int b = tid; b < tpb * m; b += nth) {
      const int t = b & (tpb - 1), k1 = b >> lw;
      const int col = c0 + t;
      if (col >= fs.n2) continue;
      const long long e = (long long)k1 * col;
      const C tw = cmul(__ldg(&hi[e >> fs.tw_shift]), __ldg(&lo[e & ((1LL << fs.tw_shift) - 1)]));
      w[(long long)k1 * fs.n2 + col] = cmul(sm.load(t, k1), tw);
    }
  } else if (tk.type == BT_FS_BB) {  // G[k1][m2] w_M^(k1 m2) -> second workspace [m2][k1]
    const int r0 = tk.tile * tpb;
    C* w2 = reinterpret_cast<C*>(A.work + it.work2_off);
    const C* lo = static_cast<const C*>(fs.lo);
    const C* hi = static_cast<const C*>(fs.hi);
    for (int b = tid; b < tpb * m; b += nth) {
      const int t = b & (tpb - 1), m2 = b >> lw;  // consecutive threads: adjacent k1
      const int k1 = r0 + t;
      if (k1 >= fs.n1) continue;
      const long long e = (long long)k1 * m2;
      const C tw = cmul(__ldg(&hi[e >> fs.tw_shift]), __ldg(&lo[e & ((1LL << fs.tw_shift) - 1)]));
      w2[k1 + (long long)fs.n1 * m2] = cmul(sm.load(t, m2), tw);
    }
  } else if (tk.type == BT_FS_C) {  // F[m2 + n2 m1]: conj(F) c_m, m < n_user
    const int r0 = tk.tile * tpb;
    C* o = reinterpret_cast<C*>(A.out + it.out_off);
    const C* ch = static_cast<const C*>(fs.chirp);
    for (int b = tid; b < tpb * m; b += nth) {
      const int t = b & (tpb - 1), m1 = b >> lw;  // consecutive threads: adjacent m2
      const int m2 = r0 + t;
      if (m2 >= fs.n2) continue;
      const long long k = m2 + (long long)fs.n2 * m1;
      if (k < fs.n_user) o[k] = cmul(cconj(sm.load(t, m1)), __ldg(&ch[k]));
    }
  } else {  // BT_FS_B: X[k1 + n1 k2]
    const int r0 = tk.tile * tpb;
    for (int b = tid; b < tpb * m; b += nth) {
      const int t = b & (tpb - 1), k2 = b >> lw;  // consecutive threads: adjacent k1
      const int row = r0 + t;
      if (row >= fs.n1) continue;
      const long long k = row + (long long)fs.n1 * k2;
      const C v = sm.load(t, k2);
      if (tk.mode == 0) {
        reinterpret_cast<C*>(A.out + it.out_off)[k] = v;
      } else if (tk.mode == 1) {
        reinterpret_cast<C*>(A.work + it.work2_off)[k] = cconj(cmul(v, __ldg(&static_cast<const C*>(fs.bhat)[k])));
      } else if (tk.mode == 2) {
        if (k < fs.n_user)
          reinterpret_cast<C*>(A.out + it.out_off)[k] =
              cmul(cconj(v), __ldg(&static_cast<const C*>(fs.chirp)[k]));
      } else {
        reinterpret_cast<C*>(A.work + it.work2_off)[k] = v;
      }
    }
  }
  if (tk.signal_ctr >= 0) signal(A, tk.signal_ctr);
}

// One CTA per task, each taking its ticket when it starts: a task then only
// waits on tickets taken earlier by CTAs that are running, so no order of
// residency can deadlock. (A loop of resident CTAs over the queue made the
// compiler spill 836 bytes per thread around the pass code.)
__global__ void __launch_bounds__(kBatchThreads, 2) k_batch(const BatchArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_task;
  // The task's item descriptor, copied once per task: its fields are read
  // all through the task, from shared memory instead of global memory.
  __shared__ __align__(16) BatchItem s_item;
  static_assert(sizeof(BatchItem) % 4 == 0, "item descriptor copied as 32-bit words");
  if (threadIdx.x == 0) s_task = atomicAdd(A.next, 1);
  __syncthreads();
  const int ti = s_task;
  if (ti < A.ntasks) batch_task(A, ti, smem_raw, s_item);
}

}  // namespace

cudaError_t launch_batch(const BatchArgs& a, unsigned blocks, size_t smem, cudaStream_t stream) {
  auto fn = k_batch;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  fn<<<blocks, kBatchThreads, smem, stream>>>(a);
  return cudaGetLastError();
}


}  // namespace chfft
