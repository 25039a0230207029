// lem_fd.cu -- flow-direction stage: FlowDirs, plateau routing, sink flooding.
//
// Restates cuFlowDirection (FD_kernels/routeflow.cu:686-975) and its kernels in
// FD_kernels/newflow.cu.  Elevations stay fp64 in HBM (the reference's state);
// comparisons use order-preserving integer keys and slope magnitudes an fp32
// approximation with a certified error bound, so the common path issues no FP64
// instruction.  A cell whose steepest-descent choice cannot be certified (near
// tie) recomputes the reference's fp64 quotients exactly.

#include <cooperative_groups.h>

#include "lem_ctx.cuh"
#include "lem_tma.cuh"

#include <cudaTypedefs.h>

namespace cg = cooperative_groups;

namespace lem {

namespace {

constexpr int FD_BX = 32;
constexpr int FD_BY = 8;
constexpr float kFar = 20000000.0f;  // shortest_paths_plateaus_initMFD (newflow.cu:252)

__device__ __forceinline__ unsigned long long key_nodata() { return dkey(-9999.0); }

__device__ __forceinline__ int warp_sum(int v) { return __reduce_add_sync(0xffffffffu, v); }
// The DEM of a warp's valid lanes (a warp of 32 aligned cells lies in one DEM), -1 without one.
__device__ __forceinline__ int warp_dem(const DemCtx& dc, size_t cell, bool valid) {
    return __reduce_max_sync(0xffffffffu, valid ? dem_at(dc, cell) : -1);
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u < v ? u : v;
    }
    return v;
}

// Exclusive prefix sum over a block of 256 threads; s_scan holds 9 ints;
// *total receives the block's sum.  Every thread of the block calls it.
__device__ __forceinline__ int block_exclusive_scan(int v, int* s_scan, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_scan[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int x = lane < 8 ? s_scan[lane] : 0;
        int ix = x;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, ix, o);
            if (lane >= o) ix += t;
        }
        if (lane < 8) s_scan[lane] = ix - x;
        if (lane == 7) s_scan[8] = ix;
    }
    __syncthreads();
    const int ex = s_scan[wid] + incl - v;
    *total = s_scan[8];
    __syncthreads();  // s_scan is free for the next call
    return ex;
}

// Warp-aggregated append of `pred` lanes to list[*count].
__device__ __forceinline__ void warp_append(bool pred, int32_t value, int32_t* list, int32_t* count, int cap,
                                            uint32_t* err) {
    unsigned ballot = __ballot_sync(0xffffffffu, pred);
    if (!ballot) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(ballot) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(ballot));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pred) {
        int pos = base + __popc(ballot & ((1u << lane) - 1));
        if (pos < cap)
            list[pos] = value;
        else
            raise_error(err, ErrFlags::kCapacity);
    }
}

// entry d (N, NE, ... NW) of a cell's 8 slopes held as two float4
__device__ __forceinline__ void set_slope(float4& a, float4& b, int d, float v) {
    switch (d) {
        case 0: a.x = v; break;
        case 1: a.y = v; break;
        case 2: a.z = v; break;
        case 3: a.w = v; break;
        case 4: b.x = v; break;
        case 5: b.y = v; break;
        case 6: b.z = v; break;
        default: b.w = v; break;
    }
}

// --------------------------------------------------------------------------
// FlowDirs (newflow.cu:49-174) of one cell from its 3x3 neighbourhood staged in
// shared memory: elevation keys (0 = outside the grid or NaN, never compared)
// and the fp32 head/tail split of each elevation, at pitch P.  sa/sb hold the
// cell's persistent slopes; the downslope entries are replaced (the others
// keep their stale values, newflow.cu:126-140) and *touched says whether any
// was.
struct FdCell {
    uint8_t cs = kMaskedCode, cm = kMaskedCode;  // SFD and MFD codes
    int is_sink = 0, is_flat = 0;
    bool is_cand = false, has_equal = false;
    uint8_t eqm = 0;                            // directions of the equal-height neighbours
    unsigned long long low = ~0ull;             // the cell's key when it is in the catchment
};

template <int P>
__device__ __forceinline__ FdCell fd_cell(const unsigned long long* __restrict__ skey, const float* __restrict__ shi,
                                         const float* __restrict__ slo, int li, bool mk, float4& sa, float4& sb,
                                         bool* touched, const ModelConsts& k) {
    FdCell o;
    *touched = false;
    if (mk) o.cs = o.cm = 0;  // a NaN elevation compares false with every neighbour: no direction
    if (mk && skey[li] != 0) {
        const unsigned long long ks = skey[li];
        const unsigned long long knd = key_nodata();
        const float hs = shi[li], ls = slo[li];
        // the fp32 estimate of the slope towards d (from the head/tail split of z)
        auto nb = [&](int d) { return li + dir_dy(d) * P + dir_dx(d); };
        auto est = [&](int d) { return ((hs - shi[nb(d)]) + (ls - slo[nb(d)])) * k.inv_len[d]; };
        o.low = ks;
        int up = 0, flat = 0;
        uint32_t aspect = 0, cand = 0;
        int bestd = -1;
        float best = -1.0f, second = -1.0f, smin = 3.0e38f;
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            const unsigned long long kn = skey[nb(d)];
            if (kn == 0) continue;
            if (ks < kn) up += 1;
            if (ks == kn) {
                flat += 1;
                o.eqm |= (uint8_t)(1u << d);
            }
            if (ks > kn && kn != knd) {
                const float s = est(d);
                set_slope(sa, sb, d, s);  // kept unless the fp64 arithmetic below replaces it
                cand |= 1u << d;
                aspect |= dir_bit(d);
                smin = fminf(smin, s);
                if (s > best) {
                    second = best;
                    best = s;
                    bestd = d;
                } else if (s > second) {
                    second = s;
                }
            }
        }
        o.has_equal = flat > 0;
        if (cand) {
            // certify the steepest direction against the exact fp64 quotients
            const float zs_mag = fabsf(hs);
            const float inv_b = (bestd & 1) ? k.inv_len[1] : k.inv_len[0];  // the length depends on d's parity
            const float err_b = best * 1.0e-6f + fmaxf(zs_mag, 1.0f) * 1.0e-12f * inv_b;
            // Quick test with the largest per-direction error (the axial one):
            // every drop far above the split error and the runner-up clearly
            // below the best certify every direction, since the per-direction
            // tests below are monotone in the estimate and in the error.
            const float abs_max = fmaxf(zs_mag, 1.0f) * 1.0e-12f * fmaxf(k.inv_len[0], k.inv_len[1]);
            bool certain = !(smin < 1.0e5f * abs_max) &&
                           (second < 0.0f || second + (second * 1.0e-6f + abs_max) < best - err_b);
            if (!certain) {  // the full test, direction by direction
                certain = true;
                const unsigned long long kb = skey[nb(bestd)];
#pragma unroll
                for (int d = 0; d < 8; ++d) {
                    if (!((cand >> d) & 1u)) continue;
                    const float sd = est(d);
                    const float abs_d = fmaxf(zs_mag, 1.0f) * 1.0e-12f * k.inv_len[d];
                    // a drop close to the split error of z: the estimate is not
                    // within 1e-7 of the reference's slope (and may even round to 0,
                    // while the reference stores a positive slope that aveslope counts)
                    if (sd < 1.0e5f * abs_d) certain = false;
                    if (d == bestd) continue;
                    const float err_d = sd * 1.0e-6f + abs_d;
                    if (sd + err_d < best - err_b) continue;
                    if (((d ^ bestd) & 1) == 0 && skey[nb(d)] == kb && d > bestd) continue;  // exact tie
                    certain = false;
                }
            }
            if (!certain) {
                // the reference's arithmetic (newflow.cu:117,130-135)
                const double zs = dkey_inv(ks);
                double smax = 0.0;
                bestd = -1;
#pragma unroll
                for (int d = 0; d < 8; ++d) {
                    if (!((cand >> d) & 1u)) continue;
                    const double st = (zs - dkey_inv(skey[nb(d)])) / k.len[d];
                    set_slope(sa, sb, d, (float)st);
                    if (st > smax) {
                        smax = st;
                        bestd = d;
                    }
                }
            }
            *touched = true;
        }
        uint32_t asfd = bestd >= 0 ? dir_bit(bestd) : 0u;
        if (up > 7) {
            o.is_sink = 1;
            aspect = asfd = 0;
        }
        if (flat + up > 7 && up <= 7) {
            o.is_flat = 1;
            aspect = asfd = 0;
        }
        o.cs = (uint8_t)asfd;
        o.cm = (uint8_t)aspect;
    }
    // the plateau candidates (newflow.cu:234-350): masked-in cells with no
    // downslope direction start at distance 2e7, every other cell at 0
    o.is_cand = mk && o.cs == 0 && o.cm == 0;
    return o;
}

// The staged form of one elevation: its order-preserving key and fp32 split
// (0 outside the grid, which is never compared).
__device__ __forceinline__ void fd_stage(double v, bool in_grid, unsigned long long& key, float& hi, float& lo) {
    key = 0;
    hi = lo = 0.f;
    if (in_grid) {
        key = dkey(v);
        dsplit(v, hi, lo);
    }
}

// The block's sink and flat counts and lowest cell into its DEM's counters
// (pass 1; a block's cells lie in one DEM), one atomic each.
__device__ __forceinline__ void fd_counters(int is_sink, int is_flat, unsigned long long low, int dem_of_warp,
                                            DemCtx dc, int* s_sinks, int* s_flats, unsigned long long* s_low,
                                            int* s_dem) {
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    if (tid == 0) {
        *s_sinks = *s_flats = 0;
        *s_low = ~0ull;
        *s_dem = -1;
    }
    __syncthreads();
    const int s1 = warp_sum(is_sink), f1 = warp_sum(is_flat);
    low = warp_min_u64(low);
    if ((tid & 31) == 0) {
        if (s1) atomicAdd(s_sinks, s1);
        if (f1) atomicAdd(s_flats, f1);
        if (low != ~0ull) atomicMin(s_low, low);
        if (dem_of_warp >= 0) atomicMax(s_dem, dem_of_warp);
    }
    __syncthreads();
    if (tid == 0 && *s_dem >= 0) {
        DemOut& o = dc.out[*s_dem];
        if (*s_sinks) atomicAdd(&o.sink_counter, *s_sinks);
        if (*s_flats) atomicAdd(&o.flat_counter, *s_flats);
        if (*s_low != ~0ull) atomicMin(&o.lowest_key, *s_low);
    }
}

// FlowDirs on a 32x8 tile with a one-cell halo staged by plain loads (grids
// whose rows TMA cannot address: width not a multiple of 16).  Pass 1 writes
// the downslope slopes into the persistent 8-per-cell array and the sink/flat
// counters and lowest elevation; pass 2 writes codes only.
__global__ void __launch_bounds__(FD_BX* FD_BY)
    k_flowdirs(const double* __restrict__ z, const uint8_t* __restrict__ mask, float* __restrict__ slopes,
               uint8_t* __restrict__ sfd, uint8_t* __restrict__ mfd, float* __restrict__ sp,
               uint8_t* __restrict__ eqm, int32_t* plateau, ModelConsts k, DevScalars* sc, DemCtx dc, TileSet ts,
               int pass) {
    if (pass == 2 && sc->sinkcount_pass1 == 0) return;
    constexpr int P = FD_BX + 2;
    __shared__ unsigned long long skey[(FD_BY + 2) * P];
    __shared__ float shi[(FD_BY + 2) * P];
    __shared__ float slo[(FD_BY + 2) * P];
    __shared__ int s_cnt[FD_BX * FD_BY / 32 + 1];
    __shared__ int s_sinks, s_flats, s_dem;
    __shared__ unsigned long long s_low;
    const int W = k.W, H = k.H;
    const int t = ts.tile(blockIdx.x);
    const int x0 = (t % ts.tw) * kTile, y0 = (t / ts.tw) * kTile + blockIdx.y * FD_BY;
    const int tid = threadIdx.y * FD_BX + threadIdx.x;
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    const bool inb = x < W && y < H;
    const size_t self = (size_t)y * W + x;
    const uint8_t mk = inb ? mask[self] : 0;
    // the cell's persistent slopes, read before the halo so that the two loads overlap
    float4* const sp4 = (slopes && mk) ? reinterpret_cast<float4*>(slopes + 8 * self) : nullptr;
    float4 sa = make_float4(0.f, 0.f, 0.f, 0.f), sb = sa;
    if (sp4) {
        sa = sp4[0];
        sb = sp4[1];
    }
    for (int e = tid; e < (FD_BX + 2) * (FD_BY + 2); e += FD_BX * FD_BY) {
        const int ly = e / P, lx = e % P;
        const int gx = x0 + lx - 1, gy = y0 + ly - 1;
        const bool g = gx >= 0 && gx < W && gy >= 0 && gy < H;
        fd_stage(g ? z[(size_t)gy * W + gx] : 0.0, g, skey[e], shi[e], slo[e]);
    }
    __syncthreads();
    FdCell c;
    if (inb) {
        bool touched = false;
        c = fd_cell<P>(skey, shi, slo, (threadIdx.y + 1) * P + threadIdx.x + 1, mk != 0, sa, sb, &touched, k);
        if (sp4 && touched) {
            sp4[0] = sa;
            sp4[1] = sb;
        }
        sfd[self] = c.cs;
        mfd[self] = c.cm;
        sp[self] = c.is_cand ? kFar : 0.f;
        if (c.is_cand) eqm[self] = c.eqm;  // read by the plateau routing for its candidates only
    }
    // Only a candidate with an equal-height neighbour can be routed: the others
    // (single-cell pits, NaN cells) keep 2e7 and no direction, and stay off
    // the list the relaxation and the final directions work through.
    block_append(c.is_cand && c.has_equal, (int32_t)self, plateau, &sc->n_cand, (int)((size_t)W * H), &sc->err,
                 s_cnt);
    if (pass == 1)
        fd_counters(c.is_sink, c.is_flat, c.low, warp_dem(dc, self, mk != 0), dc, &s_sinks, &s_flats, &s_low,
                    &s_dem);
}

// ---------------------------------------------------------------------------
// FlowDirs with the tile moved by the Tensor Memory Accelerator.  A persistent
// grid of 32x8-thread blocks takes strips of 32 x ROWS cells (ROWS = 8, 16 or
// 32: the autotuned tile shape); each thread owns ROWS / 8 cells of a column.
// Per strip three tensor copies land in shared memory and complete on one
// mbarrier: the elevations with a one-cell halo (a 36 x (ROWS + 2) box of
// doubles from x0 - 2, so the inner coordinate stays 16-byte aligned; cells
// outside the grid read as zero and are masked by their coordinates), the mask
// (32 x ROWS bytes) and, in pass 1, the persistent slopes (ROWS rows of 256
// floats).  Two stages: the next strip's copies are issued before the current
// strip is computed, so they overlap its arithmetic and stores.
template <int ROWS>
struct FdTma {
    static constexpr int kBoxW = kTile + 4;          // doubles per elevation box row
    static constexpr int kStageW = kTile + 2;        // staged keys per row (pitch)
    static constexpr int kZBytes = kBoxW * (ROWS + 2) * 8;
    static constexpr int kMBytes = kTile * ROWS;
    static constexpr int kSBytes = 8 * kTile * ROWS * 4;
    static constexpr int kZOff = 0;
    static constexpr int kMOff = (kZBytes + 127) / 128 * 128;
    static constexpr int kSOff = kMOff + (kMBytes + 127) / 128 * 128;
    static constexpr int kStage = kSOff + kSBytes;   // bytes per pipeline stage (a multiple of 128)
    static constexpr int kKeys = kStageW * (ROWS + 2);
    static constexpr int kSmem = 2 * kStage + kKeys * 16 + 256;  // + room to align the base to 128 bytes
    static_assert(kStage % 128 == 0, "stages stay 128-byte aligned");
};

constexpr uint32_t kTmaSpin = 1u << 20;  // mbarrier polls before a wait gives up

template <int ROWS>
__global__ void __launch_bounds__(FD_BX* FD_BY, 4)
    k_flowdirs_tma(const __grid_constant__ CUtensorMap tm_z, const __grid_constant__ CUtensorMap tm_mask,
                   const __grid_constant__ CUtensorMap tm_slopes, float* __restrict__ slopes,
                   uint8_t* __restrict__ sfd, uint8_t* __restrict__ mfd, float* __restrict__ sp,
                   uint8_t* __restrict__ eqm, int32_t* plateau, ModelConsts k, DevScalars* sc, DemCtx dc, TileSet ts,
                   int pass) {
    using L = FdTma<ROWS>;
    constexpr int SPT = kTile / ROWS;  // strips per tile
    constexpr int P = L::kStageW;
    if (pass == 2 && sc->sinkcount_pass1 == 0) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // the copies' destinations are 128-byte aligned (the size carries the slack)
    unsigned char* const smem = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ int s_cnt[FD_BX * FD_BY / 32 + 1];
    __shared__ int s_sinks, s_flats, s_dem;
    __shared__ unsigned long long s_low;
    unsigned long long* skey = reinterpret_cast<unsigned long long*>(smem + 2 * L::kStage);
    float* shi = reinterpret_cast<float*>(smem + 2 * L::kStage + L::kKeys * 8);
    float* slo = shi + L::kKeys;
    const int W = k.W, H = k.H;
    const int tid = threadIdx.y * FD_BX + threadIdx.x;
    const int n_items = ts.n * SPT;
    const bool with_slopes = pass == 1 && slopes != nullptr;
    const uint32_t tx_bytes = L::kZBytes + L::kMBytes + (with_slopes ? L::kSBytes : 0);
    auto origin = [&](int item, int& x0, int& y0) {
        const int t = ts.tile(item / SPT);
        x0 = (t % ts.tw) * kTile;
        y0 = (t / ts.tw) * kTile + (item % SPT) * ROWS;
    };
    // one thread issues a strip's copies into a stage
    auto issue = [&](int item, int st) {
        int x0, y0;
        origin(item, x0, y0);
        unsigned char* base = smem + st * L::kStage;
        mbar_arrive_expect_tx(&s_bar[st], tx_bytes);
        tma_load_2d(base + L::kZOff, &tm_z, x0 - 2, y0 - 1, &s_bar[st]);
        tma_load_2d(base + L::kMOff, &tm_mask, x0, y0, &s_bar[st]);
        if (with_slopes) tma_load_2d(base + L::kSOff, &tm_slopes, 8 * x0, y0, &s_bar[st]);
    };
    if (tid == 0) {
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
        fence_mbarrier_init();
        if (blockIdx.x < n_items) issue(blockIdx.x, 0);
    }
    __syncthreads();
    int it = 0;
    for (int item = blockIdx.x; item < n_items; item += gridDim.x, ++it) {
        const int st = it & 1;
        // the next strip's copies go into the other stage, free since the end of the previous strip
        if (tid == 0 && item + (int)gridDim.x < n_items) {
            fence_proxy_async_shared();
            issue(item + gridDim.x, st ^ 1);
        }
        // every thread observes the copies' completion on the barrier
        const bool arrived = mbar_wait(&s_bar[st], (it >> 1) & 1, kTmaSpin);
        if (__syncthreads_or(!arrived)) {
            // the copies never arrived: give up, and let those in flight land
            // before the block's shared memory is released
            if (tid == 0) {
                raise_error(&sc->err, ErrFlags::kNoConverge);
                mbar_wait(&s_bar[st], (it >> 1) & 1, kTmaSpin);
                if (item + (int)gridDim.x < n_items) mbar_wait(&s_bar[st ^ 1], ((it + 1) >> 1) & 1, kTmaSpin);
            }
            __syncthreads();
            break;
        }
        int x0, y0;
        origin(item, x0, y0);
        const unsigned char* base = smem + st * L::kStage;
        const double* zb = reinterpret_cast<const double*>(base + L::kZOff);
        const uint8_t* mb = base + L::kMOff;
        const float* sb_ = reinterpret_cast<const float*>(base + L::kSOff);
        for (int e = tid; e < L::kKeys; e += FD_BX * FD_BY) {
            const int ly = e / P, lx = e % P;
            const int gx = x0 + lx - 1, gy = y0 + ly - 1;
            fd_stage(zb[ly * L::kBoxW + lx + 1], gx >= 0 && gx < W && gy >= 0 && gy < H, skey[e], shi[e], slo[e]);
        }
        __syncthreads();
        int n_sink = 0, n_flat = 0, dem_w = -1;
        unsigned long long low = ~0ull;
#pragma unroll
        for (int r = 0; r < ROWS / FD_BY; ++r) {
            const int ly = threadIdx.y + FD_BY * r;
            const int x = x0 + threadIdx.x, y = y0 + ly;
            const bool inb = x < W && y < H;
            const size_t self = (size_t)y * W + x;
            const bool mk = inb && mb[ly * kTile + threadIdx.x] != 0;
            float4 sa = make_float4(0.f, 0.f, 0.f, 0.f), sbb = sa;
            if (with_slopes && mk) {
                const float4* s4 = reinterpret_cast<const float4*>(sb_ + (ly * kTile + threadIdx.x) * 8);
                sa = s4[0];
                sbb = s4[1];
            }
            FdCell c;
            if (inb) {
                bool touched = false;
                c = fd_cell<P>(skey, shi, slo, (ly + 1) * P + threadIdx.x + 1, mk, sa, sbb, &touched, k);
                if (with_slopes && mk && touched) {
                    float4* g4 = reinterpret_cast<float4*>(slopes + 8 * self);
                    g4[0] = sa;
                    g4[1] = sbb;
                }
                sfd[self] = c.cs;
                mfd[self] = c.cm;
                sp[self] = c.is_cand ? kFar : 0.f;
                if (c.is_cand) eqm[self] = c.eqm;  // read by the plateau routing for its candidates only
            }
            block_append(c.is_cand && c.has_equal, (int32_t)self, plateau, &sc->n_cand, (int)((size_t)W * H),
                         &sc->err, s_cnt);
            n_sink += c.is_sink;
            n_flat += c.is_flat;
            low = c.low < low ? c.low : low;
            const int d = warp_dem(dc, self, mk);
            dem_w = d > dem_w ? d : dem_w;
        }
        if (pass == 1) fd_counters(n_sink, n_flat, low, dem_w, dc, &s_sinks, &s_flats, &s_low, &s_dem);
        __syncthreads();  // every thread is done with this stage before it is refilled
    }
}

// --------------------------------------------------------------------------
// Plateau routing (newflow.cu:234-350); k_flowdirs lists the candidates.
constexpr int kPT = 32;            // plateau tile edge (cells)
constexpr int kPH = kPT + 2;       // tile with its one-cell halo
constexpr int kTileSweeps = 2048;  // sweeps of one tile visit before it is re-queued

// Least fixpoint of sp = min(sp, sp[n] + dc) over equal-height in-grid
// neighbours (the route_plateausMFD loop, routeflow.cu:854-872), dc = 1 along
// the axes and 1.41 on the diagonals.  The grid is cut into 32x32 tiles and
// the dirty tiles wait in a queue that the blocks pull from until it drains
// (no grid barrier between visits).  A visit relaxes the tile to its local
// fixpoint in shared memory (Gauss-Seidel sweeps over the tile's active cells,
// with the halo read at the start of the visit), lowers the improved cells in
// memory with atomicMin and queues each neighbouring tile that holds an
// equal-height neighbour of one of them.  At the start every tile that holds a
// candidate is queued.  A tile leaves the queue when a block takes it, before
// the block reads its halo, so an improvement that lands later queues it
// again.  The fixpoint is unique, so the visiting order does not change the
// result.  Only candidates (sp > 0) ever change: every other cell is a source
// at 0.  Every poll of the queue is bounded, and the visits are capped at
// lem_limits.max_rounds times the tiles queued at the start.
constexpr int kQueueSpin = 1 << 20;  // polls of an empty but busy queue, or of an unwritten slot

// The tile queue is a ring of `cap` slots with a sequence number each (a
// bounded multi-producer multi-consumer queue): ticket p of the pushes (of the
// takes) owns slot p % cap, free for it once the slot's number reads p (ready
// for it once the number reads p + 1).  Tickets come from one atomicAdd each.
struct TileQueue {
    int32_t* val;  // [cap] entries
    int32_t* seq;  // [cap] sequence numbers
    int32_t* qc;   // [0] push tickets, [1] take tickets, [2] pending (queued or in a visit), [3] visits, [4] stop
    int cap;
    __device__ void stop(DevScalars* sc) const {
        raise_error(&sc->err, ErrFlags::kNoConverge);
        atomicExch(&qc[4], 1);
    }
    __device__ void push(int32_t t, DevScalars* sc) const {
        atomicAdd(&qc[2], 1);
        const int p = atomicAdd(&qc[0], 1), slot = p % cap;
        int spin = 0;  // the slot's previous entry is taken; its taker may still be reading it
        while (*((volatile int32_t*)&seq[slot]) != p && ++spin < kQueueSpin) __nanosleep(32);
        if (spin >= kQueueSpin) return stop(sc);
        val[slot] = t;
        __threadfence();
        atomicExch(&seq[slot], p + 1);
    }
    // the next tile, or -1 once nothing is queued and no visit runs (or the queue stopped)
    __device__ int32_t take(DevScalars* sc) const {
        const int c = atomicAdd(&qc[1], 1), slot = c % cap;
        for (int spin = 0; spin < kQueueSpin; ++spin) {
            if (*((volatile int32_t*)&seq[slot]) == c + 1) {
                const int32_t v = *((volatile int32_t*)&val[slot]);
                atomicExch(&seq[slot], c + cap);  // free for push ticket c + cap
                return v;
            }
            if (*((volatile int32_t*)&qc[2]) == 0 || *((volatile int32_t*)&qc[4])) return -1;
            __nanosleep(64);
        }
        stop(sc);
        return -1;
    }
};

__global__ void __launch_bounds__(256) k_plateau_relax(const uint8_t* __restrict__ eqm, float* sp,
                                                       const int32_t* __restrict__ cand, int32_t* tq, int tq_cap,
                                                       int32_t* mark, ModelConsts k, DevScalars* sc, int pass) {
    if (pass == 2 && sc->sinkcount_pass1 == 0) return;
    cg::grid_group grid = cg::this_grid();
    __shared__ float s_v[kPH * kPH];
    __shared__ int16_t s_acell[kPT * kPT];  // active cells (halo index)
    __shared__ uint8_t s_aeq[kPT * kPT];    //   directions of their equal-height neighbours
    __shared__ float s_av0[kPT * kPT];      //   their values at the start of the visit
    __shared__ int s_act[9];
    __shared__ int s_na, s_tile;
    const int W = k.W, H = k.H;
    const int TW = (W + kPT - 1) / kPT, TH = (H + kPT - 1) / kPT;
    const int n = sc->n_cand;
    const size_t gstride = (size_t)gridDim.x * blockDim.x;
    const size_t gtid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const TileQueue tqu{tq, tq + tq_cap, sc->counters, tq_cap};
    int32_t* const qc = tqu.qc;
    const int32_t qid = sc->round_id + 1;  // mark of a queued tile
    if (gtid == 0) qc[0] = qc[1] = qc[2] = qc[3] = qc[4] = 0;
    for (size_t i = gtid; i < (size_t)tq_cap; i += gstride) tqu.seq[i] = (int32_t)i;
    grid.sync();
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < (size_t)n; base += gstride) {
        const size_t i = base + threadIdx.x;
        bool fresh = false;
        int32_t t = -1;
        if (i < (size_t)n) {
            const int32_t c = cand[i];
            t = (c / W / kPT) * TW + (c % W) / kPT;
        }
        // candidates come in cell order: the lanes of a warp mostly share a
        // tile, and one lane per tile tests and sets its mark
        const unsigned peers = __match_any_sync(0xffffffffu, t);
        if (t >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1)
            fresh = __ldcg(mark + t) != qid && atomicExch(mark + t, qid) != qid;
        // one ticket reservation per warp; the ring is empty and holds every
        // tile, so no slot waits
        const unsigned b = __ballot_sync(0xffffffffu, fresh);
        const int lane = threadIdx.x & 31, leader = b ? __ffs(b) - 1 : 0;
        int at = 0;
        if (b && lane == leader) {
            atomicAdd(&qc[2], __popc(b));
            at = atomicAdd(&qc[0], __popc(b));
        }
        at = __shfl_sync(0xffffffffu, at, leader) + __popc(b & ((1u << lane) - 1));
        if (fresh) {
            tqu.val[at % tq_cap] = t;
            __threadfence();
            atomicExch(&tqu.seq[at % tq_cap], at + 1);
        }
    }
    grid.sync();
    const long long visit_cap = (long long)round_cap_of(sc) * max(1, *((volatile int32_t*)&qc[0]));
    // a thread owns 4 consecutive rows of one column: 4 * wy + q
    const int lx = threadIdx.x & 31, wy = threadIdx.x >> 5;
    for (;;) {
        if (threadIdx.x == 0) {
            int32_t t = tqu.take(sc);
            if (t >= 0 && atomicAdd(&qc[3], 1) >= visit_cap) {
                tqu.stop(sc);
                t = -1;
            }
            if (t >= 0) {
                atomicExch(mark + t, qid - 1);  // taken: a later improvement queues it again
                __threadfence();                // before the halo is read
            }
            s_tile = t;
        }
        __syncthreads();
        const int32_t t = s_tile;
        if (t < 0) break;  // block-uniform
        {
            const int tx0 = (t % TW) * kPT, ty0 = (t / TW) * kPT;
            // the distances of the tile and its halo, in one batch of
            // independent loads per thread, with the equal-height masks of
            // the thread's own cells (k_flowdirs stores them for candidates)
            constexpr int kLoads = (kPH * kPH + 255) / 256;
            float vv[kLoads];
#pragma unroll
            for (int i = 0; i < kLoads; ++i) {
                const int j = threadIdx.x + 256 * i;
                const int gx = tx0 - 1 + j % kPH, gy = ty0 - 1 + j / kPH;
                vv[i] = 0.f;  // outside the grid: a source, and no cell's equal neighbour
                if (j < kPH * kPH && gx >= 0 && gx < W && gy >= 0 && gy < H) vv[i] = __ldcg(sp + (size_t)gy * W + gx);
            }
            uint32_t m4[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int gx = tx0 + lx, gy = ty0 + 4 * wy + q;
                m4[q] = gx < W && gy < H ? eqm[(size_t)gy * W + gx] : 0u;
            }
#pragma unroll
            for (int i = 0; i < kLoads; ++i) {
                const int j = threadIdx.x + 256 * i;
                if (j < kPH * kPH) s_v[j] = vv[i];
            }
            if (threadIdx.x < 9) s_act[threadIdx.x] = 0;
            if (threadIdx.x == 0) s_na = 0;
            __syncthreads();
            // The tile's active cells, listed: candidates (start value above 0)
            // with an equal-height neighbour (a NaN cell, key 0, has none),
            // with the directions of those neighbours and their start values.
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int sidx = (4 * wy + q + 1) * kPH + lx + 1;
                const float v0 = s_v[sidx];
                const uint32_t m = v0 > 0.f ? m4[q] : 0u;
                const int slot = warp_slot(m != 0, &s_na);
                if (slot >= 0) {
                    s_acell[slot] = (int16_t)sidx;
                    s_aeq[slot] = (uint8_t)m;
                    s_av0[slot] = v0;
                }
            }
            __syncthreads();
            const int na = s_na;
            // Gauss-Seidel sweeps over the list, forward and backward in turn
            int sweep = 0;
            for (; sweep < kTileSweeps; ++sweep) {
                bool ch = false;
                for (int i = threadIdx.x; i < na; i += blockDim.x) {
                    const int j = (sweep & 1) ? na - 1 - i : i;
                    const int sidx = s_acell[j];
                    const uint32_t m = s_aeq[j];
                    const float cv = s_v[sidx];
                    float best = cv;
#pragma unroll
                    for (int d = 0; d < 8; ++d) {
                        const float nv = (m >> d) & 1u ? s_v[sidx + dir_dy(d) * kPH + dir_dx(d)] + ((d & 1) ? 1.41f : 1.0f)
                                                       : cv;
                        best = nv < best ? nv : best;
                    }
                    if (best < cv) {
                        s_v[sidx] = best;
                        ch = true;
                    }
                }
                if (!__syncthreads_or(ch)) break;
            }
            if (sweep == kTileSweeps && threadIdx.x == 0) s_act[4] = 1;  // not settled: visit again
            for (int i = threadIdx.x; i < na; i += blockDim.x) {
                const int sidx = s_acell[i];
                const int ly = sidx / kPH - 1, lx2 = sidx % kPH - 1;
                const int gx = tx0 + lx2, gy = ty0 + ly;
                const float v = s_v[sidx];
                if (gx < W && gy < H && v < s_av0[i] &&
                    __int_as_float(atomicMin(reinterpret_cast<int*>(sp) + (size_t)gy * W + gx, __float_as_int(v))) > v) {
                    // (the values are non-negative: their bits order as ints)
                    // a neighbouring tile can improve only through an
                    // equal-height neighbour of this cell that lies in it
                    uint32_t out = 0;  // directions leaving the tile
                    if (lx2 == 0) out |= 0xE0u;        // SW, W, NW
                    if (lx2 == kPT - 1) out |= 0x0Eu;  // NE, E, SE
                    if (ly == 0) out |= 0x83u;         // NW, N, NE
                    if (ly == kPT - 1) out |= 0x38u;   // SE, S, SW
#pragma unroll 1
                    for (uint32_t m = s_aeq[i] & out; m; m &= m - 1) {
                        const int d = __ffs(m) - 1;
                        const int nx = lx2 + dir_dx(d), ny = ly + dir_dy(d);
                        s_act[3 * (ny < 0 ? 0 : (ny >= kPT ? 2 : 1)) + (nx < 0 ? 0 : (nx >= kPT ? 2 : 1))] = 1;
                    }
                }
            }
            __threadfence();  // the lowered cells, before a neighbour is queued
            __syncthreads();
            if (threadIdx.x < 9 && s_act[threadIdx.x]) {
                const int ntx = t % TW + (int)(threadIdx.x % 3) - 1, nty = t / TW + (int)(threadIdx.x / 3) - 1;
                if (ntx >= 0 && ntx < TW && nty >= 0 && nty < TH) {
                    const int32_t nt = nty * TW + ntx;
                    if (atomicExch(mark + nt, qid) != qid) tqu.push(nt, sc);
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) atomicSub(&qc[2], 1);  // this visit is over (its pushes came first)
        }
    }
    grid.sync();
    if (gtid == 0) {
        sc->plateau_sweeps += qc[3];
        sc->round_id = qid + 1;
    }
}

// Final direction of a routed plateau cell: the first direction whose
// equal-height neighbour attains the cell's distance; pass 1 also stores the
// 1e-4 slope on that direction (newflow.cu:339-346).
__global__ void k_plateau_final(const uint8_t* __restrict__ eqm, const float* __restrict__ sp,
                                const int32_t* __restrict__ cand, uint8_t* sfd, uint8_t* mfd, float* slopes,
                                ModelConsts k, DevScalars* sc, int pass) {
    if (pass == 2 && sc->sinkcount_pass1 == 0) return;
    const int W = k.W;
    const int n = sc->n_cand;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (size_t)n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int32_t c = cand[i];
        const float v = sp[c];
        if (!(v < kFar)) continue;
        const int x = c % W, y = c / W;
        // the equal-height neighbours (k_flowdirs' mask: in the grid, NaN equal
        // to none) and their distances in one batch of loads
        const uint32_t eq = eqm[c];
        float vn[8];
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            vn[d] = 0.f;
            if ((eq >> d) & 1u) vn[d] = sp[(size_t)(y + dir_dy(d)) * W + x + dir_dx(d)];
        }
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            if (!((eq >> d) & 1u) || vn[d] + ((d & 1) ? 1.41f : 1.0f) != v) continue;
            sfd[c] = (uint8_t)dir_bit(d);
            mfd[c] = (uint8_t)dir_bit(d);
            if (slopes) slopes[8 * (size_t)c + d] = 0.0001f;
            break;
        }
    }
}

// --------------------------------------------------------------------------
// Sink flooding (floodingDriver, routeflow.cu:202-676).
// init_watershedMFD (newflow.cu:352-420): sink cells get a unique id (cell+1),
// other cells point at their SFD receiver, masked and edge cells are basin 0.
// The in-tile part of the labelling is done here as well: every cell of a
// 32x32 tile follows its path inside the tile (pointer jumping in shared
// memory) and keeps a pointer to where the path ends or leaves the tile.  A
// path ending at a sink points at the sink, whose id the equal-height merge
// may still change; one ending at basin 0 takes 0.  The global pointer
// jumping then crosses tiles only.
__global__ void __launch_bounds__(256)
    k_flood_init(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ sfd, uint8_t* __restrict__ sfd1,
                 int32_t* ws, int32_t* sinks, unsigned long long* raise, int32_t* bid, ModelConsts k,
                 DevScalars* sc, DemCtx dc, TileSet ts) {
    __shared__ int16_t s_nxt[kTile * kTile];  // next in-tile cell of the path; the cell itself at the path's end
    __shared__ int32_t s_end[kTile * kTile];  // at a path's end: what the cells draining to it take
    __shared__ int s_cnt[9];
    __shared__ int s_nsink, s_dem;
    const int W = k.W, H = k.H;
    const size_t N = (size_t)W * H;
    const int t = ts.tile(blockIdx.x);
    const int tx0 = (t % ts.tw) * kTile, ty0 = (t / ts.tw) * kTile;
    const int lx = threadIdx.x & 31, ly0 = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        s_nsink = 0;
        s_dem = -1;
    }
    __syncthreads();
    int nsink = 0;
    int32_t own[4];
    bool term[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx;
        const int x = tx0 + lx, y = ty0 + ly;
        const bool in = x < W && y < H;
        const size_t c = (size_t)y * W + x;
        int16_t nxt = (int16_t)l;
        int32_t endv = 0, ownv = 0;
        bool sink = false, tm = true;
        if (in) {
            const uint8_t s = sfd[c];
            sfd1[c] = s;
            if (mask[c]) {
                sink = (s == 0);
                const bool edge = x == W - 1 || y == 0 || y == H - 1;
                if (sink) {
                    endv = -(int32_t)c - 1;  // the cells above point at the sink
                    if (!edge) {
                        ownv = (int32_t)c + 1;
                        raise[c + 1] = dkey(0.0);
                    }
                } else if (!edge) {
                    const int d = bit_dir(s);
                    const int nx = x + dir_dx(d < 0 ? 0 : d), ny = y + dir_dy(d < 0 ? 0 : d);
                    if (d >= 0 && nx >= 0 && nx < W && ny >= 0 && ny < H) {
                        const int rlx = nx - tx0, rly = ny - ty0;
                        if (rlx >= 0 && rlx < kTile && rly >= 0 && rly < kTile) {
                            nxt = (int16_t)(rly * kTile + rlx);
                            tm = false;
                        } else {
                            endv = ownv = -(int32_t)((size_t)ny * W + nx) - 1;
                        }
                    }
                }
            }
        }
        s_nxt[l] = nxt;
        s_end[l] = endv;
        own[q] = ownv;
        term[q] = tm;
        nsink += sink ? 1 : 0;
        if (sink) atomicMax(&s_dem, dem_at(dc, c));  // one DEM per tile
        block_append(sink, (int32_t)c, sinks, &sc->n_sinks, (int)N, &sc->err, s_cnt);
    }
    nsink = warp_sum(nsink);
    if (lx == 0 && nsink) atomicAdd(&s_nsink, nsink);
    __syncthreads();
    for (int it = 0; it < 10; ++it) {  // in-tile paths are shorter than 2^10 cells
        bool ch = false;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int l = (ly0 + 8 * q) * kTile + lx;
            const int16_t nx = s_nxt[s_nxt[l]];
            if (nx != s_nxt[l]) {
                s_nxt[l] = nx;
                ch = true;
            }
        }
        if (!__syncthreads_or(ch)) break;  // every pointer is at its path's end
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx;
        const int x = tx0 + lx, y = ty0 + ly;
        if (x < W && y < H) ws[(size_t)y * W + x] = term[q] ? own[q] : s_end[s_nxt[l]];
    }
    if (threadIdx.x == 0 && s_nsink) {  // s_nsink is complete after the jumping loop's barriers
        atomicAdd(&dc.out[s_dem].sinkcount_pass1, s_nsink);
        atomicAdd(&sc->sinkcount_pass1, s_nsink);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        raise[0] = dkey(0.0);
        bid[0] = -1;  // numbered by the compaction once basin 0 is on an edge
    }
}

// init_watershed_sinkMFD loop (newflow.cu:430-460): equal-height sink cells
// adopt the largest neighbouring id until nothing changes.
__global__ void k_flood_merge(const double* __restrict__ z, int32_t* ws, const int32_t* __restrict__ sinks,
                              int32_t* merging, ModelConsts k, DevScalars* sc) {
    if (sc->sinkcount_pass1 == 0) return;
    cg::grid_group grid = cg::this_grid();
    const int W = k.W, H = k.H;
    const int n = sc->n_sinks;
    const size_t gtid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t gstride = (size_t)gridDim.x * blockDim.x;
    int32_t* nmerge = &sc->counters[6];
    if (gtid == 0) {
        sc->flag[0] = sc->flag[1] = sc->flag[2] = 0;
        *nmerge = 0;
    }
    grid.sync();
    // one sink: adopt the largest id of its equal-height neighbours; false for
    // a sink with none (a strict pit), which no later round needs to visit
    auto relax = [&](int32_t c, int& changed) {
        const int x = c % W, y = c / W;
        const unsigned long long kc = dkey(z[c]);
        const int32_t mine = __ldcg(ws + c);
        int32_t best = mine;
        bool eq = false;
        for (int d = 0; kc != 0 && d < 8; ++d) {
            const int nx = x + dir_dx(d), ny = y + dir_dy(d);
            if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
            const size_t nb = (size_t)ny * W + nx;
            if (dkey(z[nb]) != kc) continue;
            eq = true;
            const int32_t o = __ldcg(ws + nb);
            if (o > best) best = o;
        }
        if (best > mine) {
            atomicMax(ws + c, best);
            changed = 1;
        }
        return eq;
    };
    int round = 0;
    for (;; ++round) {
        if (gtid == 0) sc->flag[(round + 1) % 3] = 0;  // next round's flag; this round's is read after the sync
        int changed = 0;
        if (round == 0) {
            // every sink once; the ones with an equal-height neighbour are listed
            for (size_t base = (size_t)blockIdx.x * blockDim.x; base < (size_t)n; base += gstride) {
                const size_t i = base + threadIdx.x;
                bool eq = false;
                int32_t c = 0;
                if (i < (size_t)n) {
                    c = sinks[i];
                    eq = relax(c, changed);
                }
                warp_append(eq, c, merging, nmerge, (int)((size_t)W * H), &sc->err);
            }
        } else {
            const int m = *((volatile int32_t*)nmerge);
            for (size_t i = gtid; i < (size_t)m; i += gstride) relax(__ldcg(merging + i), changed);
        }
        if (changed) sc->flag[round % 3] = 1;
        grid.sync();
        if (*((volatile int32_t*)&sc->flag[round % 3]) == 0) break;
        if (round >= round_cap_of(sc)) {
            if (gtid == 0) raise_error(&sc->err, ErrFlags::kNoConverge);
            break;
        }
    }
    if (gtid == 0) sc->flood_sweeps = round + 1;
}

// identify_watershedMFD loop (newflow.cu:469-487): pointer jumping until every
// cell holds the label of the sink (or basin 0) its SFD path ends in.
__global__ void k_flood_jump(int32_t* ws, int32_t* list_a, int32_t* list_b, ModelConsts k, DevScalars* sc,
                             TileSet ts) {
    if (sc->sinkcount_pass1 == 0) return;
    cg::grid_group grid = cg::this_grid();
    __shared__ int s_cnt[9];
    const size_t N = (size_t)k.W * k.H;
    const size_t gstride = (size_t)gridDim.x * blockDim.x;
    const size_t gtid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    int32_t* cnt = sc->counters + 3;
    if (gtid == 0) {
        cnt[0] = 0;
        cnt[1] = 0;
        cnt[2] = 0;
    }
    grid.sync();
    // round 0 over every visited cell
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < ts.span(); base += gstride) {
        int x, y;
        const bool in = ts.cell(base + threadIdx.x, k.W, k.H, x, y);
        const size_t c = (size_t)y * k.W + x;
        bool keep = false;
        if (in) {
            int32_t v = __ldcg(ws + c);
            if (v < 0) {
                v = __ldcg(ws + (-(size_t)v - 1));
                ws[c] = v;
                keep = v < 0;
            }
        }
        block_append(keep, (int32_t)c, list_a, &cnt[0], (int)N, &sc->err, s_cnt);
    }
    grid.sync();
    int round = 0;
    for (;; ++round) {
        const int32_t* in = (round & 1) ? list_b : list_a;
        int32_t* out = (round & 1) ? list_a : list_b;
        const int nin = *((volatile int32_t*)&cnt[round % 3]);
        if (nin == 0) break;
        if (round >= min(64, round_cap_of(sc))) {  // pointer jumping halves every path per round
            if (gtid == 0) raise_error(&sc->err, ErrFlags::kNoConverge);
            break;
        }
        if (gtid == 0) cnt[(round + 2) % 3] = 0;
        for (size_t base = (size_t)blockIdx.x * blockDim.x; base < (size_t)nin; base += gstride) {
            const size_t i = base + threadIdx.x;
            bool keep = false;
            int32_t c = 0;
            if (i < (size_t)nin) {
                c = in[i];
                int32_t v = __ldcg(ws + c);
                if (v < 0) {
                    v = __ldcg(ws + (-(size_t)v - 1));
                    ws[c] = v;
                    keep = v < 0;
                }
            }
            block_append(keep, c, out, &cnt[(round + 1) % 3], (int)N, &sc->err, s_cnt);
        }
        grid.sync();
    }
    if (gtid == 0) sc->label_rounds = round + 1;
}

__device__ __forceinline__ uint64_t edge_hash(unsigned long long key, int logcap) {
    return (key * 0x9E3779B97F4A7C15ull) >> (64 - logcap);
}

// Live capacity of the basin-pair table: 8 slots per label that can own a
// basin (the sink cells, plus basin 0), rounded up to a power of two, at
// least 1024, at most the allocated capacity.  A basin borders about three
// others on average (the basin graph is nearly planar), so the table is at
// most about half full and linear probing stays short, and the table of a
// grid with few sinks is small enough to stay in L2.
__device__ __forceinline__ int edge_logcap(const DevScalars* sc, int logmax) {
    const long long want = 8ll * ((long long)sc->n_sinks + 1);
    int l = 10;
    while (l < logmax && (1ll << l) < want) ++l;
    const int lim = sc->edge_log_cap;  // lem_set_limits: a smaller table (full tables raise kCapacity)
    return (lim > 0 && lim < l) ? lim : l;
}

__global__ void k_edge_clear(unsigned long long* ekey, unsigned long long* ewt, int logmax, DevScalars* sc) {
    if (sc->sinkcount_pass1 == 0) return;
    const size_t cap = 1ull << edge_logcap(sc, logmax);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (size_t)gridDim.x * blockDim.x) {
        ekey[i] = ~0ull;
        ewt[i] = ~0ull;
    }
}

__device__ __forceinline__ void edge_insert(unsigned long long* ekey, unsigned long long* ewt, int logcap,
                                            unsigned long long key, unsigned long long w, DevScalars* sc) {
    const uint64_t capm = (1ull << logcap) - 1;
    uint64_t h = edge_hash(key, logcap);
    for (int probes = 0;; ++probes) {
        unsigned long long cur = ekey[h];
        if (cur == ~0ull) cur = atomicCAS(ekey + h, ~0ull, key);
        if (cur == ~0ull || cur == key) {
            if (w < __ldcg(ewt + h)) atomicMin(ewt + h, w);
            return;
        }
        h = (h + 1) & capm;
        if (probes >= 4096) {
            raise_error(&sc->err, ErrFlags::kCapacity);
            return;
        }
    }
}

constexpr int FE_BX = 32, FE_BY = 8;
constexpr int kEdgeSlotsLog2 = 7;
constexpr int kEdgeSlots = 1 << kEdgeSlotsLog2;  // block-local pair table (a 32x8 tile borders few basin pairs)

// identify_watershed_boundary_write_backMFD (newflow.cu:787-877): the minimum
// boundary height per unordered basin pair, in an open-addressing table.  A
// cell pair with different labels is a boundary at the higher cell's height
// (the reference visits it from the cell with zs[this] >= zs[idx]).  Labels and
// height keys of a 32x8 tile and its halo sit in shared memory, so interior
// cells cost eight shared-memory compares; the tile's pairs are first reduced
// in a block-local table and then merged into the global one, one insert per
// distinct pair and tile.
__global__ void __launch_bounds__(FE_BX* FE_BY)
    k_flood_edges(const double* __restrict__ z, const uint8_t* __restrict__ mask, const int32_t* __restrict__ ws,
                  unsigned long long* ekey, unsigned long long* ewt, int logmax, ModelConsts k, DevScalars* sc,
                  TileSet ts) {
    if (sc->sinkcount_pass1 == 0) return;
    __shared__ int32_t sw[FE_BY + 2][FE_BX + 2];
    __shared__ unsigned long long sk[FE_BY + 2][FE_BX + 2];
    __shared__ unsigned long long tkey[kEdgeSlots], twt[kEdgeSlots];
    const int W = k.W, H = k.H;
    const int logcap = edge_logcap(sc, logmax);
    const int tl = ts.tile(blockIdx.x);
    const int x0 = (tl % ts.tw) * kTile, y0 = (tl / ts.tw) * kTile + blockIdx.y * FE_BY;
    const int tid = threadIdx.y * FE_BX + threadIdx.x;
    for (int t = tid; t < kEdgeSlots; t += FE_BX * FE_BY) {
        tkey[t] = ~0ull;
        twt[t] = ~0ull;
    }
    for (int t = tid; t < (FE_BX + 2) * (FE_BY + 2); t += FE_BX * FE_BY) {
        const int ly = t / (FE_BX + 2), lx = t % (FE_BX + 2);
        const int gx = x0 + lx - 1, gy = y0 + ly - 1;
        int32_t lab = -1;  // outside the grid: no neighbour
        unsigned long long key = 0;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            const size_t g = (size_t)gy * W + gx;
            lab = ws[g];
            key = dkey(z[g]);
        }
        sw[ly][lx] = lab;
        sk[ly][lx] = key;
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    const int lx = threadIdx.x + 1, ly = threadIdx.y + 1;
    if (x < W && y < H && mask[(size_t)y * W + x]) {
        const int32_t a = sw[ly][lx];
        const unsigned long long kz = sk[ly][lx];
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            const int32_t b = sw[ly + dir_dy(d)][lx + dir_dx(d)];
            // a negative label is a pointer the jumping left when it stopped
            // at its round cap (an error is raised): no basin to pair
            if (a < 0 || b < 0 || b == a) continue;
            const unsigned long long kn = sk[ly + dir_dy(d)][lx + dir_dx(d)];
            if (kz == 0 || kn == 0 || kz < kn) continue;  // zs[this] >= zs[idx] is false for NaN
            const unsigned long long key = ((unsigned long long)(uint32_t)min(a, b) << 32) | (uint32_t)max(a, b);
            uint32_t h = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - kEdgeSlotsLog2));
            bool done = false;
            for (int p = 0; p < kEdgeSlots; ++p) {
                const unsigned long long cur = atomicCAS(&tkey[h], ~0ull, key);
                if (cur == ~0ull || cur == key) {
                    atomicMin(&twt[h], kz);
                    done = true;
                    break;
                }
                h = (h + 1) & (kEdgeSlots - 1);
            }
            if (!done) edge_insert(ekey, ewt, logcap, key, kz, sc);
        }
    }
    __syncthreads();
    for (int t = tid; t < kEdgeSlots; t += FE_BX * FE_BY) {
        if (tkey[t] != ~0ull) edge_insert(ekey, ewt, logcap, tkey[t], twt[t], sc);
    }
}

// Compact the table into an edge list and count the labels on edges
// (data->sinkcount, newflow.cu:1044-1045).  Labels on edges start unreached.
__global__ void k_flood_compact(const unsigned long long* __restrict__ ekey, const unsigned long long* __restrict__ ewt,
                                int logmax, int32_t* ea, int32_t* eb, unsigned long long* ew,
                                unsigned long long* raise, int32_t* seen, int32_t* bid, int32_t* blab,
                                DevScalars* sc, DemCtx dc) {
    if (sc->sinkcount_pass1 == 0) return;
    __shared__ int s_cnt[9];
    const int32_t epoch = sc->epoch;
    const size_t cap = 1ull << edge_logcap(sc, logmax);
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < (size_t)cap; base += (size_t)gridDim.x * blockDim.x) {
        const size_t i = base + threadIdx.x;
        bool has = false;
        int32_t a = 0, b = 0;
        unsigned long long w = 0;
        int d = -1, nd = 0;
        bool fa_ = false, fb_ = false;
        if (i < (size_t)cap) {
            const unsigned long long key = ekey[i];
            if (key != ~0ull) {
                has = true;
                a = (int32_t)(key >> 32);
                b = (int32_t)(key & 0xffffffffu);
                w = ewt[i];
                // labels are cell + 1 of one DEM; basin 0 is counted once per DEM it borders
                d = dem_at(dc, (size_t)(a != 0 ? a : b) - 1);
                // most labels are on many edges (basin 0 on most): test before the atomic
                fa_ = __ldcg(seen + a) != epoch && atomicExch(seen + a, epoch) != epoch;
                fb_ = __ldcg(seen + b) != epoch && atomicExch(seen + b, epoch) != epoch;
                if (a != 0 && fa_) ++nd;
                if (b != 0 && fb_) ++nd;
                if ((a == 0 || b == 0) && *((volatile int32_t*)&dc.out[d].zero_seen) != epoch &&
                    atomicExch(&dc.out[d].zero_seen, epoch) != epoch)
                    ++nd;
                if (a != 0) raise[a] = ~0ull;
                if (b != 0) raise[b] = ~0ull;
            }
        }
        // number the basins first seen here: one atomic per block
        const int pa = block_reserve(fa_, &sc->n_basins, s_cnt);
        if (pa >= 0) {
            bid[a] = pa;
            blab[pa] = a;
        }
        const int pb = block_reserve(fb_, &sc->n_basins, s_cnt);
        if (pb >= 0) {
            bid[b] = pb;
            blab[pb] = b;
        }
        // one atomic per DEM and warp for the label counts
        const unsigned grp = __match_any_sync(0xffffffffu, nd ? d : -1);
        const int gsum = __reduce_add_sync(grp, nd);
        if (nd && (grp & ((1u << (threadIdx.x & 31)) - 1)) == 0) atomicAdd(&dc.out[d].sinkcount, gsum);
        // the edge list: one atomic per block
        const int pe = block_reserve(has, &sc->n_edges, s_cnt);
        if (pe >= 0) {
            ea[pe] = a;
            eb[pe] = b;
            ew[pe] = w;
        }
    }
}

// Spill heights.  The Kruskal pass of routeflow.cu:520-572 gives every basin
// that can drain to basin 0 the smallest height h at which it connects to
// basin 0 through boundaries no higher than h: its minimax distance to basin 0
// over the basin-pair edges.  It is computed here as the fixpoint raise(a) =
// min over edges (a, b, w) of max(w, raise(b)), basin 0 at 0, with basins
// numbered compactly.  The kernel first groups the edges by basin (the edges
// of basin 0 left out: nothing lowers it), then relaxes in rounds: the first
// sweeps the edge list for the edges of basin 0; every later round only the
// edges of the basins lowered since the round before.
__global__ void k_flood_spill(const int32_t* __restrict__ ea, const int32_t* __restrict__ eb,
                              const unsigned long long* __restrict__ ew, unsigned long long* raise, int32_t* comp,
                              unsigned long long* cdist, unsigned long long* cmaxw, const int32_t* __restrict__ bid,
                              const int32_t* __restrict__ blab, int32_t* stamp, unsigned long long* bdist,
                              int32_t* euv, int32_t* adj_e, int32_t* adj_v, int32_t* cursor, int list_cap,
                              DevScalars* sc) {
    if (sc->sinkcount_pass1 == 0) return;
    const int n = sc->n_edges;
    const int nb = sc->n_basins;
    if (nb > list_cap) {  // `cursor` holds list_cap entries
        if (blockIdx.x == 0 && threadIdx.x == 0) raise_error(&sc->err, ErrFlags::kCapacity);
        return;
    }
    cg::grid_group grid = cg::this_grid();
    __shared__ int s_scan[9];
    const size_t gtid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t gstride = (size_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int32_t z = nb > 0 ? bid[0] : -1;  // basin 0 is on an edge whenever it borders a basin
    // The edges grouped by basin: offsets in comp (nb + 1 entries), chunk sums
    // of their prefix sum in cmaxw; both are idle until the walled-in pass.
    int32_t* const off = comp;
    int32_t* const csum = reinterpret_cast<int32_t*>(cmaxw);
    for (size_t i = gtid; i < (size_t)nb; i += gstride) {
        bdist[i] = (int32_t)i == z ? 0ull : ~0ull;
        stamp[i] = -1;
        cursor[i] = 0;
    }
    if (gtid == 0) sc->flag[0] = sc->flag[1] = sc->flag[2] = 0;
    grid.sync();
    for (size_t i = gtid; i < (size_t)n; i += gstride) {  // degrees
        const int32_t a = bid[ea[i]], b = bid[eb[i]];
        euv[2 * i] = a;
        euv[2 * i + 1] = b;
        if (a != z && b != z) {
            atomicAdd(cursor + a, 1);
            atomicAdd(cursor + b, 1);
        }
    }
    grid.sync();
    // exclusive prefix sum of the degrees: per chunk of at least 256 basins,
    // then over the chunk sums (block 0), then within the chunks again
    const int chunk = max(256, (nb + (int)gridDim.x - 1) / (int)gridDim.x);
    const int nchunks = (nb + chunk - 1) / chunk;
    const int c0 = min(nb, (int)blockIdx.x * chunk), c1 = min(nb, c0 + chunk);
    if ((int)blockIdx.x < nchunks) {
        int part = 0;
        for (int i = c0 + (int)threadIdx.x; i < c1; i += blockDim.x) part += cursor[i];
        int total = 0;
        block_exclusive_scan(part, s_scan, &total);
        if (threadIdx.x == 0) csum[blockIdx.x] = total;
    }
    grid.sync();
    if (blockIdx.x == 0) {
        int carry = 0;
        for (int b0 = 0; b0 < nchunks; b0 += blockDim.x) {
            const int b = b0 + (int)threadIdx.x;
            const int v = b < nchunks ? csum[b] : 0;
            int total = 0;
            const int ex = block_exclusive_scan(v, s_scan, &total);
            if (b < nchunks) csum[b] = carry + ex;
            carry += total;
        }
        if (threadIdx.x == 0) off[nb] = carry;
    }
    grid.sync();
    if ((int)blockIdx.x < nchunks) {
        int carry = csum[blockIdx.x];
        for (int i0 = c0; i0 < c1; i0 += blockDim.x) {
            const int i = i0 + (int)threadIdx.x;
            const int v = i < c1 ? cursor[i] : 0;
            int total = 0;
            const int ex = block_exclusive_scan(v, s_scan, &total);
            if (i < c1) {
                off[i] = carry + ex;
                cursor[i] = carry + ex;  // where the basin's next edge goes
            }
            carry += total;
        }
    }
    grid.sync();
    for (size_t i = gtid; i < (size_t)n; i += gstride) {
        const int32_t a = euv[2 * i], b = euv[2 * i + 1];
        if (a == z || b == z) continue;
        const int pa = atomicAdd(cursor + a, 1), pb = atomicAdd(cursor + b, 1);
        adj_e[pa] = (int32_t)i;
        adj_v[pa] = b;
        adj_e[pb] = (int32_t)i;
        adj_v[pb] = a;
    }
    grid.sync();
    // Round r relaxes the edges of every basin lowered in round r - 1 or
    // earlier in round r (its stamp: the last round that lowered it), from
    // the distance the basin has when its warp reaches it; a round that
    // lowers nothing ends the loop.
    const size_t warp = gtid >> 5, nwarps = gstride >> 5;
    int round = 1;
    for (;; ++round) {
        if (gtid == 0) sc->flag[(round + 1) % 3] = 0;
        bool lowered = false;
        if (round == 1) {
            for (size_t i = gtid; i < (size_t)n; i += gstride) {
                const int2 uv = *reinterpret_cast<const int2*>(euv + 2 * i);
                if (uv.x != z && uv.y != z) continue;
                const int32_t v = uv.x == z ? uv.y : uv.x;
                const unsigned long long cv = ew[i];
                if (cv < __ldcg(bdist + v) && atomicMin(bdist + v, cv) > cv) {
                    stamp[v] = round;
                    lowered = true;
                }
            }
        } else {
            // the edge lists of a warp's 32 basins that are active,
            // concatenated and relaxed 32 edges at a time; a lane finds the
            // basin of its edge by a search over the lanes' prefix sums
            for (size_t u0 = warp * 32; u0 < (size_t)nb; u0 += nwarps * 32) {
                const size_t mine = u0 + lane;
                const bool act = mine < (size_t)nb && __ldcg(stamp + mine) >= round - 1;
                int j0 = 0, deg = 0;
                unsigned long long du = 0;
                if (act) {
                    j0 = off[mine];
                    deg = off[mine + 1] - j0;
                    du = __ldcg(bdist + mine);
                }
                int incl = deg;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                const int total = __shfl_sync(0xffffffffu, incl, 31);
                for (int t0 = 0; t0 < total; t0 += 32) {
                    const int t = t0 + lane;
                    int k = 0;  // the first lane whose inclusive sum exceeds t
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const int pk = __shfl_sync(0xffffffffu, incl, k + step - 1);
                        if (pk <= t) k += step;
                    }
                    const int kin = __shfl_sync(0xffffffffu, incl, k);
                    const int kdeg = __shfl_sync(0xffffffffu, deg, k);
                    const int kj0 = __shfl_sync(0xffffffffu, j0, k);
                    const unsigned long long kdu = __shfl_sync(0xffffffffu, du, k);
                    if (t < total) {
                        const int j = kj0 + t - (kin - kdeg);
                        const int32_t v = adj_v[j];
                        const unsigned long long w = ew[adj_e[j]];
                        const unsigned long long cv = w > kdu ? w : kdu;
                        if (cv < __ldcg(bdist + v) && atomicMin(bdist + v, cv) > cv) {
                            stamp[v] = round;
                            lowered = true;
                        }
                    }
                }
            }
        }
        if (__any_sync(0xffffffffu, lowered) && lane == 0 && __ldcg(&sc->flag[round % 3]) == 0)
            sc->flag[round % 3] = 1;
        grid.sync();
        if (*((volatile int32_t*)&sc->flag[round % 3]) == 0) break;
        if (round >= round_cap_of(sc)) {
            if (gtid == 0) raise_error(&sc->err, ErrFlags::kNoConverge);
            break;
        }
    }
    for (size_t i = gtid; i < (size_t)nb; i += gstride) {
        const int32_t L = blab[i];
        if (L != 0) raise[L] = __ldcg(bdist + i);
    }
    if (gtid == 0) raise[0] = 0ull;
    if (gtid == 0) {
        sc->spill_rounds = round + 1;
        sc->flag[3] = 0;
    }
    grid.sync();
    // Basins that never reach basin 0 (walled in by NaN elevations, or a grid
    // with no nodata and no open edge): the Kruskal pass leaves every basin of
    // such a component the weight of the component's last merge, i.e. its
    // largest spanning-tree edge (routeflow.cu:562-572).  It equals the largest
    // minimax distance from any one basin of the component to the others.
    for (size_t i = gtid; i < (size_t)n; i += gstride)
        if (raise[ea[i]] == ~0ull || raise[eb[i]] == ~0ull) sc->flag[3] = 1;
    grid.sync();
    if (*((volatile int32_t*)&sc->flag[3])) {
        // (a) component label = smallest basin label, by min-propagation over edges
        for (size_t i = gtid; i < (size_t)n; i += gstride) {
            if (raise[ea[i]] == ~0ull) comp[ea[i]] = ea[i];
            if (raise[eb[i]] == ~0ull) comp[eb[i]] = eb[i];
        }
        if (gtid == 0) sc->flag[0] = sc->flag[1] = sc->flag[2] = 0;
        grid.sync();
        for (int r = 0;; ++r) {
            if (gtid == 0) sc->flag[(r + 1) % 3] = 0;
            int ch = 0;
            for (size_t i = gtid; i < (size_t)n; i += gstride) {
                const int32_t a = ea[i], b = eb[i];
                if (raise[a] != ~0ull || raise[b] != ~0ull) continue;
                const int32_t ca = __ldcg(comp + a), cb = __ldcg(comp + b);
                if (ca < cb) { atomicMin(comp + b, ca); ch = 1; }
                if (cb < ca) { atomicMin(comp + a, cb); ch = 1; }
            }
            if (ch) sc->flag[r % 3] = 1;
            grid.sync();
            if (*((volatile int32_t*)&sc->flag[r % 3]) == 0) break;
            if (r >= round_cap_of(sc)) {
                if (gtid == 0) raise_error(&sc->err, ErrFlags::kNoConverge);
                break;
            }
        }
        // (b) minimax distance to the component's label basin, in cdist
        for (size_t i = gtid; i < (size_t)n; i += gstride) {
            const int32_t a = ea[i], b = eb[i];
            if (raise[a] == ~0ull) cdist[a] = (comp[a] == a) ? 0ull : ~0ull;
            if (raise[b] == ~0ull) cdist[b] = (comp[b] == b) ? 0ull : ~0ull;
        }
        if (gtid == 0) sc->flag[0] = sc->flag[1] = sc->flag[2] = 0;
        grid.sync();
        for (int r = 0;; ++r) {
            if (gtid == 0) sc->flag[(r + 1) % 3] = 0;
            int ch = 0;
            for (size_t i = gtid; i < (size_t)n; i += gstride) {
                const int32_t a = ea[i], b = eb[i];
                if (raise[a] != ~0ull || raise[b] != ~0ull) continue;
                const unsigned long long w = ew[i];
                const unsigned long long da = __ldcg(cdist + a), db = __ldcg(cdist + b);
                const unsigned long long ca = w > db ? w : db, cb = w > da ? w : da;
                if (ca < da) { atomicMin(cdist + a, ca); ch = 1; }
                if (cb < db) { atomicMin(cdist + b, cb); ch = 1; }
            }
            if (ch) sc->flag[r % 3] = 1;
            grid.sync();
            if (*((volatile int32_t*)&sc->flag[r % 3]) == 0) break;
            if (r >= round_cap_of(sc)) {
                if (gtid == 0) raise_error(&sc->err, ErrFlags::kNoConverge);
                break;
            }
        }
        // (c) the component's largest distance, gathered at its label basin
        for (size_t i = gtid; i < (size_t)n; i += gstride) {
            const int32_t a = ea[i], b = eb[i];
            if (raise[a] == ~0ull && comp[a] != a) atomicMax(cdist + comp[a], cdist[a]);
            if (raise[b] == ~0ull && comp[b] != b) atomicMax(cdist + comp[b], cdist[b]);
        }
        grid.sync();
        for (size_t i = gtid; i < (size_t)n; i += gstride) {
            const int32_t a = ea[i], b = eb[i];
            if (raise[a] == ~0ull) cmaxw[a] = cdist[comp[a]];
            if (raise[b] == ~0ull) cmaxw[b] = cdist[comp[b]];
        }
        grid.sync();
        for (size_t i = gtid; i < (size_t)n; i += gstride) {
            const int32_t a = ea[i], b = eb[i];
            if (raise[a] == ~0ull) raise[a] = cmaxw[a];
            if (raise[b] == ~0ull) raise[b] = cmaxw[b];
        }
    }
    grid.sync();
    if (gtid == 0) raise[0] = dkey(0.0);
}

// raise_watershedMFD (newflow.cu:879-894) into the scratch DEM of pass 2.
__global__ void k_flood_raise(const double* __restrict__ z, const uint8_t* __restrict__ mask,
                              const int32_t* __restrict__ ws, const unsigned long long* __restrict__ raise,
                              double* __restrict__ zf, ModelConsts k, DevScalars* sc, DemCtx dc, TileSet ts) {
    if (sc->sinkcount_pass1 == 0) return;
    for (size_t v0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v0 < ts.span();
         v0 += (size_t)gridDim.x * blockDim.x) {
        int x, y;
        if (!ts.cell(v0, k.W, k.H, x, y)) continue;
        const size_t c = (size_t)y * k.W + x;
        double v = z[c];
        const uint8_t mk = mask[c];
        const int dm = dem_at(dc, c);
        // the basin's raise is read alongside the DEM's sink count
        const int32_t lab = ws[c];  // negative only where the jumping stopped at its round cap
        const unsigned long long r = (mk && lab >= 0) ? raise[lab] : 0ull;
        // a DEM without sinks keeps its DEM: its second pass repeats the first
        if (mk && dc.out[dm].sinkcount_pass1 != 0) {
            const unsigned long long kv = dkey(v);
            if (kv != 0 && kv < r) v = dkey_inv(r);  // zs < raise is false for NaN
        }
        zf[c] = v;
    }
}

// Epilogue of cuFlowDirection (routeflow.cu:934-953) and the host outlet check
// of routeflow.cu:738-741, which the reference applies after its device copy.
__global__ void k_fd_epilogue(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ sfd,
                              const uint8_t* __restrict__ mfd, uint8_t* __restrict__ fd, ModelConsts k, TileSet ts) {
    for (size_t v0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v0 < ts.span();
         v0 += (size_t)gridDim.x * blockDim.x) {
        int x, y;
        if (!ts.cell(v0, k.W, k.H, x, y)) continue;
        const size_t c = (size_t)y * k.W + x;
        uint8_t v = sfd[c];
        if (k.flow_type != 0 && mask[c] && mfd[c] != 0) v = mfd[c];
        fd[c] = v;
    }
}

// Per DEM: the outlet flows west (routeflow.cu:953) and testoutletislowest
// (routeflow.cu:171-199,740-741) lowers it below the lowest cell of the DEM.
__global__ void k_fd_outlets(uint8_t* __restrict__ fd, double* z, DemCtx dc) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= dc.n || !dc.in[d].active) return;
    DemOut& o = dc.out[d];
    const int outlet = o.outlet;
    fd[outlet] = 16;
    if (o.sinkcount_pass1 == 0) o.sinkcount = 0;
    const double zo = z[outlet];
    o.outlet_z_clim = zo;  // SetClimateMatrices ran before testoutletislowest lowers it (lem.cpp:80-84)
    o.outlet_clim = outlet;
    unsigned long long low = o.lowest_key;
    const unsigned long long k1000 = dkey(1000.0);
    if (low > k1000) low = k1000;
    if (low < dkey(zo)) z[outlet] = dkey_inv(low) - 0.0001;
}

__global__ void k_fd_reset(DevScalars* sc, DemCtx dc) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d == 0) {
        sc->epoch += 1;
        sc->sinkcount_pass1 = 0;
        sc->flood_sweeps = sc->label_rounds = sc->spill_rounds = 0;
        sc->plateau_sweeps = 0;
        sc->n_cand = 0;
        sc->n_sinks = 0;
        sc->n_edges = 0;
        sc->n_basins = 0;
    }
    if (d < dc.n) {
        DemOut& o = dc.out[d];
        o.lowest_key = ~0ull;
        o.sink_counter = o.flat_counter = 0;
        o.sinkcount_pass1 = 0;
        o.sinkcount = 0;
    }
}

__global__ void k_cand_reset(DevScalars* sc) { sc->n_cand = 0; }

}  // namespace

int coop_blocks_for(const void* kernel, int threads, size_t smem) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
    if (per < 1) per = 1;
    return sms * per;
}

static lem_status coop(const char* name, const void* fn, int blocks, void** args, const Launch& L) {
    L.pre(name);
    LEM_CUDA_TRY(coop_launch(fn, blocks, args, L.st));
    L.post();
    return LEM_OK;
}

static int flat_blocks(size_t n, int threads, int cap_blocks) {
    size_t b = (n + threads - 1) / threads;
    if (b > (size_t)cap_blocks) b = cap_blocks;
    if (b < 1) b = 1;
    return (int)b;
}

template <int ROWS>
static lem_status launch_flowdirs_tma(const DevState& s, const ModelConsts& k, const Launch& L, const TileSet& ts,
                                      int pass, int shape) {
    const FdTmaMaps& m = *s.fd_tma;
    const int items = ts.n * (kTile / ROWS);
    const int blocks = items < m.blocks[shape] ? items : m.blocks[shape];
    if (blocks < 1) return LEM_OK;
    L.pre("k_flowdirs");
    k_flowdirs_tma<ROWS><<<blocks, dim3(FD_BX, FD_BY), FdTma<ROWS>::kSmem, L.st>>>(
        pass == 1 ? m.z[shape] : m.zf[shape], m.mask[shape], m.slopes[shape], pass == 1 ? s.slopes : nullptr, s.sfd,
        s.mfd, s.sp, s.eqm, s.list_a, k, s.sc, s.dems, ts, pass);
    L.post();
    LEM_CUDA_TRY(cudaGetLastError());
    return LEM_OK;
}

// One pass of FlowDirs + plateau routing.  Pass 1 reads the stage's DEM and
// updates the persistent slopes; pass 2 reads the raised DEM.
static lem_status direction_pass(const DevState& s, const ModelConsts& k, const Launch& L, int pass) {
    const int T = 256, big = 152 * 32;
    const TileSet ts = tiles_of(s, k.W);
    const size_t span = ts.span();
    const dim3 fdb(FD_BX, FD_BY), fdg(ts.n, kTile / FD_BY);
    const double* zz = pass == 1 ? s.z : s.zf;
    float* slopes = pass == 1 ? s.slopes : nullptr;
    if (pass == 2) LEM_LAUNCH(L, k_cand_reset, 1, 1, s.sc);
    if (s.fd_tma) {
        lem_status r = LEM_OK;
        switch (s.fd_rows) {
            case 1: r = launch_flowdirs_tma<16>(s, k, L, ts, pass, 1); break;
            case 2: r = launch_flowdirs_tma<32>(s, k, L, ts, pass, 2); break;
            default: r = launch_flowdirs_tma<8>(s, k, L, ts, pass, 0); break;
        }
        if (r != LEM_OK) return r;
    } else {
        LEM_LAUNCH(L, k_flowdirs, fdg, fdb, zz, s.mask, slopes, s.sfd, s.mfd, s.sp, s.eqm, s.list_a, k, s.sc, s.dems,
                   ts, pass);
    }
    {
        float* sp = s.sp;
        const uint8_t* eqm = s.eqm;
        const int32_t* cand = s.list_a;  // the candidates
        int32_t* tq = s.tq;
        int tq_cap = s.tq_cap;
        int32_t* mark = s.mark;
        ModelConsts kk = k;
        DevScalars* sc = s.sc;
        void* args[] = {(void*)&eqm,  (void*)&sp, (void*)&cand, (void*)&tq,  (void*)&tq_cap,
                        (void*)&mark, (void*)&kk, (void*)&sc,   (void*)&pass};
        lem_status r = coop("k_plateau_relax", (const void*)k_plateau_relax, s.coop_blocks[kCkPlateau], args, L);
        if (r != LEM_OK) return r;
    }
    LEM_LAUNCH(L, k_plateau_final, flat_blocks(span, T, big), T, s.eqm, s.sp, s.list_a, s.sfd, s.mfd, slopes, k, s.sc,
               pass);
    return LEM_OK;
}

lem_status launch_flow_direction(const DevState& s, const ModelConsts& k, const Launch& L) {
    const int T = 256, big = 152 * 32;
    const TileSet ts = tiles_of(s, k.W);
    const size_t span = ts.span();
    lem_status r;
    LEM_LAUNCH(L, k_fd_reset, (s.dems.n + 127) / 128, 128, s.sc, s.dems);
    if ((r = direction_pass(s, k, L, 1)) != LEM_OK) return r;
    // sink flooding on the pass-1 codes
    LEM_LAUNCH(L, k_flood_init, ts.n, 256, s.mask, s.sfd, s.sfd1, s.ws, s.list_b, s.raise, s.bid, k, s.sc, s.dems,
               ts);
    {
        const double* zz = s.z;
        int32_t* ws = s.ws;
        const int32_t* sinks = s.list_b;
        int32_t* merging = s.list_a;  // free until the pointer jumping
        ModelConsts kk = k;
        DevScalars* sc = s.sc;
        void* args[] = {(void*)&zz, (void*)&ws, (void*)&sinks, (void*)&merging, (void*)&kk, (void*)&sc};
        if ((r = coop("k_flood_merge", (const void*)k_flood_merge, s.coop_blocks[kCkMerge], args, L)) != LEM_OK) return r;
    }
    {
        int32_t* ws = s.ws;
        int32_t* la = s.list_a;
        int32_t* lb = s.pending;
        ModelConsts kk = k;
        DevScalars* sc = s.sc;
        TileSet tt = ts;
        void* args[] = {(void*)&ws, (void*)&la, (void*)&lb, (void*)&kk, (void*)&sc, (void*)&tt};
        if ((r = coop("k_flood_jump", (const void*)k_flood_jump, s.coop_blocks[kCkJump], args, L)) != LEM_OK) return r;
    }
    int logmax = 0;
    while ((1ll << logmax) < s.ecap) ++logmax;
    LEM_LAUNCH(L, k_edge_clear, flat_blocks((size_t)s.ecap, T, big), T, s.ekey, s.ewt, logmax, s.sc);
    {
        const dim3 eb(FE_BX, FE_BY), eg(ts.n, kTile / FE_BY);
        LEM_LAUNCH(L, k_flood_edges, eg, eb, s.z, s.mask, s.ws, s.ekey, s.ewt, logmax, k, s.sc, ts);
    }
    LEM_LAUNCH(L, k_flood_compact, flat_blocks((size_t)s.ecap, T, big), T, s.ekey, s.ewt, logmax, s.edge_a, s.edge_b,
               s.edge_w, s.raise, s.label_seen, s.bid, s.blab, s.sc, s.dems);
    {
        const int32_t* ea = s.edge_a;
        const int32_t* eb = s.edge_b;
        const unsigned long long* ew = s.edge_w;
        unsigned long long* raise = s.raise;
        int32_t* comp = s.comp;
        unsigned long long* cdist = s.cdist;
        unsigned long long* cmaxw = s.cmaxw;
        const int32_t* bidp = s.bid;
        const int32_t* blab = s.blab;
        int32_t* stamp = s.boff;
        unsigned long long* bdist = s.bdist;
        int32_t* euv = s.adj_v;
        // the basin-pair table is idle after compaction: 2 * ecap int32 each
        int32_t* adj_e = reinterpret_cast<int32_t*>(s.ekey);
        int32_t* adj_v = reinterpret_cast<int32_t*>(s.ewt);
        int32_t* cursor = s.pending;  // an int32 grid unused from the label jumping to the second direction pass
        int list_cap = (int)std::min<size_t>((size_t)k.W * k.H, (size_t)INT32_MAX);  // entries of `pending`
        DevScalars* sc = s.sc;
        void* args[] = {(void*)&ea,    (void*)&eb,    (void*)&ew,     (void*)&raise, (void*)&comp,
                        (void*)&cdist, (void*)&cmaxw, (void*)&bidp,   (void*)&blab,  (void*)&stamp,
                        (void*)&bdist, (void*)&euv,   (void*)&adj_e,  (void*)&adj_v, (void*)&cursor,
                        (void*)&list_cap, (void*)&sc};
        if ((r = coop("k_flood_spill", (const void*)k_flood_spill, s.coop_blocks[kCkSpill], args, L)) != LEM_OK) return r;
    }
    LEM_LAUNCH(L, k_flood_raise, flat_blocks(span, T, big), T, s.z, s.mask, s.ws, s.raise, s.zf, k, s.sc, s.dems,
               ts);
    if ((r = direction_pass(s, k, L, 2)) != LEM_OK) return r;
    LEM_LAUNCH(L, k_fd_epilogue, flat_blocks(span, T, big), T, s.mask, s.sfd, s.mfd, s.fd, k, ts);
    LEM_LAUNCH(L, k_fd_outlets, (s.dems.n + 127) / 128, 128, s.fd, s.z, s.dems);
    LEM_CUDA_TRY(cudaGetLastError());
    return LEM_OK;
}

namespace {
template <int ROWS>
lem_status fd_tma_shape(const DevState& s, const ModelConsts& k, FdTmaMaps* m, int shape,
                        PFN_cuTensorMapEncodeTiled_v12000 encode) {
    using L = FdTma<ROWS>;
    const cuuint64_t W = (cuuint64_t)k.W, H = (cuuint64_t)k.H;
    const cuuint32_t one[2] = {1, 1};
    auto enc = [&](CUtensorMap* map, CUtensorMapDataType type, void* base, cuuint64_t w, cuuint64_t stride,
                   cuuint32_t bw, cuuint32_t bh) {
        const cuuint64_t dims[2] = {w, H};
        const cuuint64_t strides[1] = {stride};
        const cuuint32_t box[2] = {bw, bh};
        return encode(map, type, 2, base, dims, strides, box, one, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    };
    if (enc(&m->z[shape], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, s.z, W, W * 8, L::kBoxW, ROWS + 2) != CUDA_SUCCESS ||
        enc(&m->zf[shape], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, s.zf, W, W * 8, L::kBoxW, ROWS + 2) != CUDA_SUCCESS ||
        enc(&m->mask[shape], CU_TENSOR_MAP_DATA_TYPE_UINT8, s.mask, W, W, kTile, ROWS) != CUDA_SUCCESS ||
        enc(&m->slopes[shape], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, s.slopes, 8 * W, W * 32, 8 * kTile, ROWS) !=
            CUDA_SUCCESS)
        return LEM_ERR_INVALID;
    LEM_CUDA_TRY(cudaFuncSetAttribute(k_flowdirs_tma<ROWS>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::kSmem));
    int per = 0, dev = 0, sms = 0;
    LEM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_flowdirs_tma<ROWS>, FD_BX * FD_BY, L::kSmem));
    LEM_CUDA_TRY(cudaGetDevice(&dev));
    LEM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    m->blocks[shape] = (per < 1 ? 1 : per) * sms;
    return LEM_OK;
}
}  // namespace

lem_status fd_tma_setup(const DevState& s, const ModelConsts& k, FdTmaMaps* maps) {
    if (k.W % 16 != 0) return LEM_ERR_INVALID;  // rows of the mask and elevations must be 16-byte multiples
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    LEM_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (!fn || q != cudaDriverEntryPointSuccess) return LEM_ERR_INVALID;
    const auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    lem_status r;
    if ((r = fd_tma_shape<8>(s, k, maps, 0, encode)) != LEM_OK) return r;
    if ((r = fd_tma_shape<16>(s, k, maps, 1, encode)) != LEM_OK) return r;
    return fd_tma_shape<32>(s, k, maps, 2, encode);
}

// cooperative kernels of this file, for the co-residency query at handle creation
const void* fd_coop_kernels[] = {(const void*)k_plateau_relax, (const void*)k_flood_merge,
                                 (const void*)k_flood_jump, (const void*)k_flood_spill};
extern const int fd_coop_kernel_count = 4;

}  // namespace lem
