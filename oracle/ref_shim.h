// ref_shim.h -- host emulation of the CUDA built-ins the reference kernels use,
// so their bodies compile with g++ and run as one sequential schedule.
//
// TEST INFRASTRUCTURE (oracle/_ref): a kernel "launch" visits every block and
// thread of the grid in order (blockIdx.y, blockIdx.x, threadIdx.y, threadIdx.x);
// atomics are plain read-modify-writes.  This is one legal schedule of the
// reference's kernels.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#define __global__
#define __device__
#define __host__

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct uint3s {
    unsigned x, y, z;
};
static uint3s blockIdx, threadIdx;
static dim3 blockDim, gridDim;

inline void __syncthreads() {}
inline int atomicAdd(int* a, int v) {
    int o = *a;
    *a += v;
    return o;
}
inline unsigned atomicInc(unsigned* a, unsigned lim) {
    unsigned o = *a;
    *a = (o >= lim) ? 0 : o + 1;
    return o;
}
inline unsigned long long atomicCAS(unsigned long long* a, unsigned long long cmp, unsigned long long v) {
    unsigned long long o = *a;
    if (o == cmp) *a = v;
    return o;
}
inline double __longlong_as_double(long long v) {
    double d;
    std::memcpy(&d, &v, 8);
    return d;
}
inline long long __double_as_longlong(double d) {
    long long v;
    std::memcpy(&v, &d, 8);
    return v;
}

template <typename K, typename... A>
void ref_launch(dim3 grid, dim3 block, K kernel, A... args) {
    gridDim = grid;
    blockDim = block;
    for (unsigned by = 0; by < grid.y; ++by)
        for (unsigned bx = 0; bx < grid.x; ++bx)
            for (unsigned ty = 0; ty < block.y; ++ty)
                for (unsigned tx = 0; tx < block.x; ++tx) {
                    blockIdx = {bx, by, 0};
                    threadIdx = {tx, ty, 0};
                    kernel(args...);
                }
}

// Stand-in for the two Data members init_and_sort_watershed_bound_labelsMFD uses.
struct Data {
    FILE* outlog;
    int sinkcount;
};
