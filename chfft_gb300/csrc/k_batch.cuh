// Uneven-batch kernel: one launch runs a whole list of tasks of mixed kinds
// and lengths, taken in order from a device work queue (one task per CTA by
// ticket, or resident CTAs looping over the queue).
//
// Task types
//   SMALL  `count` consecutive transforms of one kind and length, whole in
//          one CTA (C2C, R2C, DCT-II, MDCT; mixed radix or Bluestein core)
//   FS_A   four-step column tile: 16-64 columns of length n1, pre-processing of
//          the kind fused into the load, w_m^(k1 n2) into the store
//   FS_B   four-step row tile: 16-64 rows of length n2, transposed store (plain,
//          Bluestein spectrum, Bluestein chirp-out, or the core output of a
//          real kind for its POST tasks)
//   POST   the R2C split / DCT-II post-twiddle of a four-step real kind
//   FS_BB  four-step Bluestein middle: a row tile's forward FFT (n2), the
//          spectrum product, the row FFT of the inverse transform (n2) and
//          its twiddle, stored transposed (the inverse's row-major n2 x n1)
//   FS_C   four-step Bluestein last: row FFTs of length n1 of that
//          intermediate, chirp-out store in natural order
// A four-step Bluestein item runs FS_A (chirp in), FS_BB, FS_C: the
// inverse FFT is split with the roles of n1 and n2 swapped, so its first
// pass works on the rows the forward FFT's last pass already holds.
// Dependencies are device counters: a task waits (bounded spin, thread 0)
// until its counter reaches the number of tiles of the step it consumes,
// and signals its own counter when done. A step is queued after every task
// it waits for (CTAs take tickets in order), so a waited-for task is always
// held by a CTA that is already running.
// Workspace written by other CTAs is read with L1-bypassing loads.
#pragma once

#include "kernels.cuh"

namespace chfft {

constexpr int kBatchThreads = 512;
constexpr int kBatchEpt = 16;   // complex elements per thread per pass (64 registers)
constexpr int kBatchTile = 16;     // narrowest four-step tile (columns / rows)
constexpr int kBatchTileMax = 64;  // widest four-step tile

enum BatchKind : int { BK_C2C = 0, BK_R2C = 1, BK_DCT2 = 2, BK_MDCT = 3 };
enum BatchTaskType : int { BT_SMALL = 0, BT_FS_A = 1, BT_FS_B = 2, BT_POST = 3, BT_FS_BB = 4, BT_FS_C = 5 };

struct BatchCore {
  StageList st;       // stages run (length M for Bluestein)
  const void* tw;     // omega_{st.n}
  const void* chirp;  // Bluestein
  const void* bhat;   // Bluestein
  int n;              // logical length
  int blue;
};

struct BatchItem {
  int kind;             // BatchKind
  int n;                // user length
  int ncore;            // complex core length (n, n/2, n/4)
  int big;              // 0 one CTA, 1 four-step, 2 four-step Bluestein
  float scale;
  float ortho;          // DCT-II first-input factor
  long long in_off;     // bytes from the input base
  long long out_off;    // bytes from the output base
  long long work_off;   // bytes from the workspace base (big items)
  long long work2_off;
  BatchCore core;       // one-CTA items
  BatchCore ca, cb;     // big items: column (n1) and row (n2) cores
  FourStep fs;          // big items
  const void* aux0;     // kind tables (coef, omega_4N, MDCT twiddle)
  const void* aux1;     // (omega_4N, window)
};

struct BatchTask {
  int type;         // BatchTaskType
  int item;         // first item
  int count;        // SMALL: consecutive items of the same kind / length; FS_A / FS_B: tile width
  int mode;         // FS_A: 0 plain, 1 chirp in; FS_B: 0 out, 1 spectrum, 2 chirp out, 3 core out (real kinds)
  int tile;         // FS_A / FS_B tile, POST chunk
  int wait_ctr, wait_target, signal_ctr;
};

struct BatchArgs {
  const BatchTask* tasks;
  int ntasks;
  const BatchItem* items;
  int* next;          // queue head
  int* ctr;           // dependency counters
  int* err;           // error word (1: a wait gave up)
  const char* in;
  char* out;
  char* work;
  int spin_limit;     // wait iterations (~0.2 us apart) before giving up
  int stall;          // test hook: 1 raises every dependency target by one (no wait is ever met)
};

constexpr int kPostChunk = 2048;  // pairs per POST task

}  // namespace chfft
