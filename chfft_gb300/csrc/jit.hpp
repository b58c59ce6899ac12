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
// Number of specialised kernels compiled in this process.
size_t jit_cache_size();

}  // namespace chfft
