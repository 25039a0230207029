// lem_wave.cuh -- helpers shared by the two dependency waves (accumulation and
// sediment routing): float-float arithmetic, warp lists, donor tests.
#pragma once

#include <cooperative_groups.h>

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
            raise_error(err, ErrFlags::kCapacity);
    }
}

// The neighbour in direction d of cell (x, y) donates to it when its code has
// the bit of the opposite direction.
__device__ __forceinline__ bool donates(uint8_t code_n, int d) { return (code_n & dir_bit((d + 4) & 7)) != 0; }

constexpr int32_t kBlocked = 0x40000000;  // pending flag of a cell with a donor that never completes

// Decrement with acquire-release semantics: the release publishes this
// thread's earlier stores (the finished cell) to whichever thread sees the
// count reach zero, and the acquire lets that thread read every donor.
__device__ __forceinline__ int32_t dec_acq_rel(int32_t* p) {
    int32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], -1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

constexpr int kWaveStack = 8;      // receivers a lane keeps for itself before spilling to the next round

// The dependency wave shared by flow accumulation and sediment routing, run by
// every thread of a cooperative launch.  A cell is ready once all its donors
// are finished (pending[c] counts them; kBlocked marks a donor that never
// finishes).  Lanes take ready cells from the round's list through one atomic
// head per warp request, so no lane idles while work is left.  A lane that
// finishes a cell decrements its receivers and carries on with the first one
// it made ready (it was that cell's last donor); further receivers made ready
// at the same time (MFD) go on the lane's own stack, and only when that is full
// to the next round's list.  Op::cell(c, x, y) computes and stores cell c,
// reading finished donors with ld.global.cg; Op::receivers(c, x, y, r) lists
// the nodes whose pending count c's completion decrements.  Returns the nodes
// this thread finished.
template <class Op>
__device__ int wave_walk(const Op& op, int32_t* pending, int32_t* list_a, int32_t* list_b, int W, int H,
                         DevScalars* sc) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    const size_t N = (size_t)W * H;
    const size_t gtid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    int32_t* cnt = sc->counters;  // [0..2] list sizes by round % 3, [3..5] take heads by round % 3
    if (gtid == 0) {
        cnt[1] = cnt[2] = 0;
        cnt[3] = cnt[4] = cnt[5] = 0;
    }
    grid.sync();
    int done = 0;
    for (int round = 0;; ++round) {
        const int32_t* in = (round & 1) ? list_b : list_a;
        int32_t* out = (round & 1) ? list_a : list_b;
        const int nin = *((volatile int32_t*)&cnt[round % 3]);
        if (nin == 0) break;
        if (round >= round_cap_of(sc)) {
            if (gtid == 0) raise_error(&sc->err, ErrFlags::kNoConverge);
            break;
        }
        if (gtid == 0) {
            cnt[(round + 2) % 3] = 0;      // size of the list after next (read before the last sync)
            cnt[3 + (round + 1) % 3] = 0;  // head of the next round
        }
        int32_t* head = &cnt[3 + round % 3];
        int32_t stack[kWaveStack];
        int sp = 0;
        int32_t cur = -1;
        bool more = true;  // warp-uniform: the round's list may still hold cells
        for (size_t guard = 0;; ++guard) {
            if (cur < 0 && sp > 0) cur = stack[--sp];
            const bool need = cur < 0;
            const unsigned m = __ballot_sync(0xffffffffu, need && more);
            if (m) {
                const int leader = __ffs(m) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(head, __popc(m));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (need) {
                    const int it = base + __popc(m & below);
                    if (it < nin) cur = __ldcg(in + it);
                }
                if (base + __popc(m) >= nin) more = false;
            }
            if (!__any_sync(0xffffffffu, cur >= 0)) break;
            if (guard > 2 * N + 64) {  // every cell is finished at most once
                if (lane == 0) raise_error(&sc->err, ErrFlags::kNoConverge);
                break;
            }
            int32_t spill[8];
            int nspill = 0;
            if (cur >= 0) {
                const int x = cur % W, y = cur / W;
                // the receivers first: they read static data only, so their
                // loads overlap the cell's own chain of loads
                int32_t rcv[8];
                const int nr = op.receivers(cur, x, y, rcv);
                for (int j = 0; j < nr; ++j) op.prefetch(rcv[j]);
                op.cell(cur, x, y);
                ++done;
                int32_t next = -1;
                for (int j = 0; j < nr; ++j) {
                    const int32_t r = rcv[j];
                    if (dec_acq_rel(pending + r) == 1) {
                        if (next < 0)
                            next = r;
                        else if (sp < kWaveStack)
                            stack[sp++] = r;
                        else
                            spill[nspill++] = r;
                    }
                }
                cur = next;
            }
            if (__any_sync(0xffffffffu, nspill > 0))
                for (int j = 0; j < 8; ++j)
                    wave_append(j < nspill, j < nspill ? spill[j] : 0, out, &cnt[(round + 1) % 3], (int)N, &sc->err);
        }
        grid.sync();
    }
    return done;
}

// ---------------------------------------------------------------------------
// 32x32 tiles of the two waves: cell classes of the halo, the kind of a cell's
// receiver, and the halo ring in a fixed order.
constexpr int kTH = kTile + 2;  // tile with its one-cell halo
constexpr uint8_t kKindIn = 0, kKindOutlet = 1, kKindEnd = 2;  // receiver: in the tile / in another tile / none
constexpr uint8_t kCellOff = 0;    // never a donor (outside the grid; for accumulation also nodata outside the catchment)
constexpr uint8_t kCellIn = 1;     // a cell the wave computes
constexpr uint8_t kCellBlock = 2;  // a donor that never completes

__device__ __forceinline__ bool in_tile(int lx, int ly) { return lx >= 0 && lx < kTile && ly >= 0 && ly < kTile; }
// index step of direction d inside a tile (row-major, kTile cells per row)
__device__ __forceinline__ int tile_step(int d) { return dir_dy(d) * kTile + dir_dx(d); }

// The outlets of a 32x32 tile (cells whose receiver lies in another tile) in
// cell order, with each outlet's slot: warp w ballots rows 4w..4w+3, and a
// prefix over the 8 warps' counts places them.  Called by all 256 threads;
// s_wcnt holds 8 ints; the caller synchronises before reading the lists.
__device__ __forceinline__ void list_outlets(const uint8_t* s_kind, int16_t* s_olist, int16_t* s_oslot, int* s_no,
                                             int* s_wcnt) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned m[4];
    int cnt = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        m[r] = __ballot_sync(0xffffffffu, s_kind[(4 * w + r) * kTile + lane] == kKindOutlet);
        cnt += __popc(m[r]);
    }
    if (lane == 0) s_wcnt[w] = cnt;
    __syncthreads();
    int base = 0;
    for (int i = 0; i < w; ++i) base += s_wcnt[i];
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int l = (4 * w + r) * kTile + lane;
        if ((m[r] >> lane) & 1u) {
            const int pos = base + __popc(m[r] & below);
            s_olist[pos] = (int16_t)l;
            s_oslot[l] = (int16_t)pos;
        }
        base += __popc(m[r]);
    }
    if (threadIdx.x == 255) *s_no = base;  // the last warp's end is the total
}

// The halo ring in a fixed order: top row, bottom row, left column, right column.
constexpr int kRing = 4 * kTH - 4;
constexpr int kRingChunks = (kRing + 31) / 32;
__device__ __forceinline__ int ring_halo(int i) {
    if (i < kTH) return i;
    if (i < 2 * kTH) return (kTH - 1) * kTH + (i - kTH);
    if (i < 2 * kTH + kTile) return (i - 2 * kTH + 1) * kTH;
    return (i - 2 * kTH - kTile + 1) * kTH + kTH - 1;
}

// The in-tile dependency wave of one block, in rounds: a round takes every
// queued cell (all its donors in the tile finished), computes it with
// op(c, round), which returns the in-tile receiver it releases (or -1), and
// queues that receiver when c was its last donor.  Cells are queued once, in
// an order where every donor comes before its receiver.  Rounds with at least
// kWaveBlockMin cells (the first ones: the sources) run on every thread of the
// block; the narrow rounds after them run on warp 0 alone, with a warp barrier
// between rounds and the queue appended by ballot, while the block's other
// warps wait at one block barrier (the SM runs other blocks meanwhile).
constexpr int kWaveBlockMin = 96;
template <class Op>
__device__ __forceinline__ void tile_wave(const Op& op, int32_t* s_pend, int16_t* s_q, int* s_qn, int* s_end,
                                          const bool (&src)[4], int lx, int ly0) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (src[q]) s_q[atomicAdd(s_qn, 1)] = (int16_t)((ly0 + 8 * q) * kTile + lx);
    int start = 0, end = 0, round = 0;
    for (;; ++round) {
        __syncthreads();
        if (threadIdx.x == 0) *s_end = *s_qn;
        __syncthreads();
        end = *s_end;
        if (end - start < kWaveBlockMin) break;  // block-uniform
        for (int i = start + threadIdx.x; i < end; i += blockDim.x) {
            const int c = s_q[i];
            const int r = op(c, round);
            if (r >= 0 && atomicSub(&s_pend[r], 1) == 1) s_q[atomicAdd(s_qn, 1)] = (int16_t)r;
        }
        start = end;
    }
    if (threadIdx.x < 32) {
        const unsigned below = (1u << (threadIdx.x & 31)) - 1u;
        int qn = end;  // every append of the block rounds is in: the barrier above came after them
        for (; start < end && round <= kTile * kTile; ++round) {
            for (int i0 = start; i0 < end; i0 += 32) {
                const int i = i0 + (int)threadIdx.x;
                int r = -1;
                if (i < end) {
                    r = op(s_q[i], round);
                    if (r >= 0 && atomicSub(&s_pend[r], 1) != 1) r = -1;
                }
                const unsigned b = __ballot_sync(0xffffffffu, r >= 0);
                if (r >= 0) s_q[qn + __popc(b & below)] = (int16_t)r;
                qn += __popc(b);
            }
            __syncwarp();  // the round's cells and queue entries, for the next round
            start = end;
            end = qn;
        }
        if (threadIdx.x == 0) *s_qn = qn;
    }
    __syncthreads();
}

// The wave of wave_walk with a whole warp per node: lane 0 takes a ready node,
// Op::cell_warp(c, x, y, lane) computes it with every lane, lane 0 releases its
// receivers and the warp carries on with the first it made ready.  For nodes
// whose own computation has parallel parts (the sediment programs).
template <class Op>
__device__ void wave_walk_warp(const Op& op, int32_t* pending, int32_t* list_a, int32_t* list_b, int W, int H,
                               DevScalars* sc) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    const size_t N = (size_t)W * H;
    const size_t gtid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int32_t* cnt = sc->counters;  // [0..2] list sizes by round % 3, [3..5] take heads by round % 3
    if (gtid == 0) {
        cnt[1] = cnt[2] = 0;
        cnt[3] = cnt[4] = cnt[5] = 0;
    }
    grid.sync();
    for (int round = 0;; ++round) {
        const int32_t* in = (round & 1) ? list_b : list_a;
        int32_t* out = (round & 1) ? list_a : list_b;
        const int nin = *((volatile int32_t*)&cnt[round % 3]);
        if (nin == 0) break;
        if (round >= round_cap_of(sc)) {
            if (gtid == 0) raise_error(&sc->err, ErrFlags::kNoConverge);
            break;
        }
        if (gtid == 0) {
            cnt[(round + 2) % 3] = 0;
            cnt[3 + (round + 1) % 3] = 0;
        }
        int32_t* head = &cnt[3 + round % 3];
        for (size_t guard = 0; guard <= N; ++guard) {
            int32_t cur = -1;
            if (lane == 0) {
                const int it = atomicAdd(head, 1);
                if (it < nin) cur = __ldcg(in + it);
            }
            cur = __shfl_sync(0xffffffffu, cur, 0);
            if (cur < 0) break;
            for (size_t chain = 0; cur >= 0 && chain <= N; ++chain) {
                const int x = cur % W, y = cur / W;
                // the receivers first (static data): their loads overlap the node's
                int32_t rcv[8];
                int nr = 0;
                if (lane == 0) {
                    nr = op.receivers(cur, x, y, rcv);
                    for (int j = 0; j < nr; ++j) op.prefetch(rcv[j]);
                }
                __syncwarp();
                op.cell_warp(cur, x, y, lane);
                __syncwarp();
                int32_t next = -1;
                if (lane == 0) {
                    for (int j = 0; j < nr; ++j) {
                        if (dec_acq_rel(pending + rcv[j]) == 1) {
                            if (next < 0) {
                                next = rcv[j];
                            } else {
                                const int p = atomicAdd(&cnt[(round + 1) % 3], 1);
                                if (p < (int)N) out[p] = rcv[j];
                            }
                        }
                    }
                }
                cur = __shfl_sync(0xffffffffu, next, 0);
            }
        }
        grid.sync();
    }
}

// Brings the line holding p into L2 (a hint: no value is read).
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Receivers of cell (x, y) by its direction code: in-grid, in-catchment cells.
__device__ __forceinline__ int code_receivers(const uint8_t* __restrict__ fd, const uint8_t* __restrict__ mask,
                                              int32_t cur, int x, int y, int W, int H, int32_t* r) {
    const uint8_t code = __ldg(fd + cur);
    int nr = 0;
    for (int d = 0; d < 8; ++d) {
        if (!(code & dir_bit(d))) continue;
        const int rx = x + dir_dx(d), ry = y + dir_dy(d);
        if (rx < 0 || rx >= W || ry < 0 || ry >= H) continue;
        const int32_t n = ry * W + rx;
        if (__ldg(mask + n)) r[nr++] = n;
    }
    return nr;
}

}  // namespace lem
