// Stand-in for the reference's precompiled header when its kernels -- the neighbour
// search (Simulation/DFSPH/ParticleSearch/ParticleSearchKernels.cu) and the step
// (Simulation/DFSPH/DFSPHKernels.cu) -- are compiled as plain C++ for the CPU. Test
// infrastructure only: it lets the oracle be checked against the reference's own kernel
// code, run here with one emulated CUDA thread at a time.
//
// Provides what those kernels use: the CUDA function qualifiers (as nothing), the
// built-in thread indices (set by the driver before each emulated thread), the three
// atomics the search calls (sequential, returning the old value), the standard headers
// the reference's precompiled header brings in, and the glm subset (glm_subset.h).
#ifndef VFD_REF_SEARCH_PCH_H
#define VFD_REF_SEARCH_PCH_H

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __forceinline__

struct RefDim3 {
    unsigned int x, y, z;
};
extern RefDim3 blockIdx, blockDim, threadIdx;

inline int atomicMin(int* a, int v) {
    const int o = *a;
    if (v < o) *a = v;
    return o;
}
inline int atomicMax(int* a, int v) {
    const int o = *a;
    if (v > o) *a = v;
    return o;
}
inline unsigned int atomicAdd(unsigned int* a, unsigned int v) {
    const unsigned int o = *a;
    *a = o + v;
    return o;
}

#include "glm_subset.h"

#endif
