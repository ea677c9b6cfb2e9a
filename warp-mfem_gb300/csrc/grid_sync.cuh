// Arrival and wait of the persistent kernels' grid barriers.  Each barrier is
// a 64-bit counter that is never reset: the k-th barrier of a launch over G
// CTAs releases when the counter reaches base + k * G, base being the counter
// at launch rounded down to G.  One thread per CTA arrives and waits, after a
// __syncthreads that orders the CTA's stores before its arrival.
//
// The arrival is a single add with release semantics and the wait spins on a
// load with acquire semantics: every store a CTA made before arriving is
// visible to every CTA once it sees the count complete.  On GB300 with 152
// CTAs this costs 1.94 us per barrier (partials round trip included), against
// 2.21 us for a full fence, a relaxed add, a relaxed spin and a second full
// fence.
#pragma once

namespace mfem {
namespace {

__device__ __forceinline__ void grid_arrive(unsigned long long *counter) {
    asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(counter) : "memory");
}

__device__ __forceinline__ unsigned long long grid_count(const unsigned long long *counter) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(counter) : "memory");
    return v;
}

}  // namespace
}  // namespace mfem
