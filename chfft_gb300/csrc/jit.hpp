// Plan-time kernel specialisation (jit.cu).
#pragma once

#include <string>

#include "plan.hpp"

namespace chfft {

enum class JitMode { OFF, AUTO, ALWAYS };

// CHFFT_JIT=0|off -> OFF, unset|auto -> AUTO (large batches), anything else -> ALWAYS.
JitMode jit_mode();
// Whether NVRTC and the driver API could be opened (reason in *why if not).
bool jit_available(std::string* why);
// Launch the plan-time specialised kernel for (kind, dtype, core, geometry),
// compiling it on first use. Returns 0 on success, 1 when unavailable (the
// caller launches the library kernel instead), 2 on a launch error.
int jit_launch(Kernel k, int dtype, const Core& c, const Geo& g, const KArgs& a, unsigned blocks, cudaStream_t stream,
               int mode = 0, const FourStep* fs = nullptr);
// Tensor-core variant: the kernel over a TcCore (radix-16 passes on the
// tensor cores at precision prec 1..3, tc.cuh / tc_core.cuh) for a core with
// a tensor-core pass order, tpb sequences per CTA. Same return codes; 1 also
// when the geometry does not qualify (see tc_geometry).
int jit_launch_tc(Kernel k, const Core& c, int prec, int tpb, const KArgs& a, unsigned blocks, cudaStream_t stream,
                  int mode = 0, const FourStep* fs = nullptr);
// Shared memory of a TcCore kernel for (core, tpb, prec), 0 if it does not
// qualify (row tiles of 128 radix-16 butterflies, at most 16 of them, and
// the shared-memory limit). ld receives the tile stride.
size_t tc_geometry(const Core& c, Kernel k, int tpb, int prec, int* ld);
// Streaming multiprocessors of the current device.
int num_sms();
// Number of specialised kernels compiled in this process.
size_t jit_cache_size();

}  // namespace chfft
