// prof.h -- optional per-kernel-class CUDA-event timing on the library stream.
#pragma once

#include <cuda_runtime.h>

namespace xt {

enum ProfClass { PROF_KRON64 = 0, PROF_KRON32 = 1, PROF_ILU64 = 2, PROF_ILU32 = 3, PROF_DAMAGE = 4,
                 PROF_ORTH64 = 5, PROF_ORTH32 = 6, PROF_KRONDF = 7, PROF_NCLASS = 8 };

// Returns a token for prof_end, or -1 when profiling is off.
int prof_begin(int cls, cudaStream_t s);
void prof_end(int token, cudaStream_t s);
// Algorithmic bytes of the timed launch (summed per class; bench.py divides
// them by the summed time).  No-op for token -1.
void prof_bytes(int token, double bytes);
// Drops a record (a launch that turned out to have nothing to do: a step
// issued past the end of a device-driven GMRES cycle).  No-op for -1.
void prof_cancel(int token);

}  // namespace xt
