// lem_wave.cuh -- helpers shared by the two dependency waves (accumulation and
// sediment routing): float-float arithmetic, warp lists, donor tests.
#pragma once

#include "lem_ctx.cuh"

namespace lem {

// Unevaluated sum hi + lo of two floats (Knuth two-sum), ~44 significant bits.
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
    const float s = __fadd_rn(a.x, b.x);
    const float bb = __fsub_rn(s, a.x);
    float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
    e = __fadd_rn(e, __fadd_rn(a.y, b.y));
    const float hi = __fadd_rn(s, e);
    return make_float2(hi, __fsub_rn(e, __fsub_rn(hi, s)));
}
__device__ __forceinline__ float2 ff_scale(float2 a, float p) {
    const float h = __fmul_rn(a.x, p);
    const float e = __fmaf_rn(a.x, p, -h);
    const float l = __fmaf_rn(a.y, p, e);
    const float hi = __fadd_rn(h, l);
    return make_float2(hi, __fsub_rn(l, __fsub_rn(hi, h)));
}
// order-preserving key of a canonical float-float value
__device__ __forceinline__ uint32_t fkey(float f) {
    uint32_t b = __float_as_uint(f);
    if (b == 0x80000000u) b = 0;
    return (b >> 31) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ unsigned long long ffkey(float2 v) {
    return ((unsigned long long)fkey(v.x) << 32) | fkey(v.y);
}

__device__ __forceinline__ int wsum(int v) { return __reduce_add_sync(0xffffffffu, v); }

__device__ __forceinline__ void wave_append(bool pred, int32_t value, int32_t* list, int32_t* count, int cap,
                                            uint32_t* err) {
    unsigned ballot = __ballot_sync(0xffffffffu, pred);
    if (!ballot) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(ballot) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(ballot));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pred) {
        const int pos = base + __popc(ballot & ((1u << lane) - 1));
        if (pos < cap)
            list[pos] = value;
        else
            atomicOr(err, ErrFlags::kCapacity);
    }
}

// The neighbour in direction d of cell (x, y) donates to it when its code has
// the bit of the opposite direction.
__device__ __forceinline__ bool donates(uint8_t code_n, int d) { return (code_n & dir_bit((d + 4) & 7)) != 0; }

constexpr int32_t kBlocked = 0x40000000;  // pending flag of a cell with a donor that never completes

}  // namespace lem
