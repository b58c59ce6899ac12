// Host interface of the pipelined four-step launch (k_pipe.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace chfft {
namespace pipe {
struct PipeArgs;
}

// Whether N = n1 x n2 has a pipelined four-step kernel (n1, n2 in {256, 512, 1024}).
bool pipe_shape_ok(int n1, int n2);
// Dynamic shared memory of that kernel (0 if none).
size_t pipe_smem(int n1, int n2);
// Tiles per transform of pass A (columns) and pass B (rows); 0 if no kernel.
int pipe_tiles(int n1, int n2, int* ta, int* tb);
// Complex elements of the pass-A tiles' twiddle tables, and their
// generation (FP64, rounded once) into `out` on stream s.
size_t pipe_twiddle_elems(int n1, int n2);
cudaError_t pipe_twiddles(int n1, int n2, void* out, cudaStream_t s);
// One launch of `grid` CTAs over a.count transforms read from `in`.
// 0 ok, 1 unavailable (input not 16-byte aligned, no tensor-map encoder),
// 2 launch error.
int pipe_launch(int n1, int n2, const void* in, const pipe::PipeArgs& a, int grid, cudaStream_t s);

}  // namespace chfft
