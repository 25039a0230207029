// lem_fa.cu -- flow-accumulation stage.
//
// computeRunOffWeights (MOD_kernels/runoffweight.cu:21-113), calcpropsSFD /
// calcprops (:115-354) and correctmfdflow (FA_kernels/mfd_simple.cu:33-384).
// The reference rescans the whole grid once per dependency level with a host
// round trip per launch; here every cell is visited once.  A thread starts at a
// cell whose donors are all complete and walks downstream for as long as it is
// the last donor to finish at the receiver (an atomic in-degree decides), so a
// whole single-flow-direction tree finishes in one launch.  The sum of the
// donors is pulled in the reference's order E, SE, S, SW, W, NW, N, NE
// (mfd_simple.cu:95-165) as an fp32 pair (hi + lo) to keep ~44 bits.

#include <cooperative_groups.h>

#include <mutex>

#include "lem_wave.cuh"

namespace cg = cooperative_groups;

namespace lem {

namespace {

// k_fat_local's cell status: finished inside the tile, and waiting on an
// inflow from another tile somewhere upstream (its final value needs the
// coarse wave)
constexpr uint8_t kLaDone = 1, kLaWaits = 2;
constexpr int kLaOutlet = 1;  // final-pass entry: an outlet (stored by the coarse wave; counted only)

// calcrunoffweight (runoffweight.cu:21-58) plus the in-degrees of the wave.
// A donor outside the catchment is complete from the start when its DEM is
// nodata (correctmfdflow's okgrid, mfd_simple.cu:279-285) and never otherwise.
// Sum over a block of 256 threads (every thread calls it; the result is valid in thread 0).
__device__ __forceinline__ int block_sum_i(int v) {
    __shared__ int part[8];
    v = wsum(v);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < 8; ++w) t += part[w];
    return t;
}

__global__ void k_fa_prep(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd,
                          const float* __restrict__ stone, const float* __restrict__ totB, float* __restrict__ soilM,
                          float* __restrict__ w, float2* __restrict__ fa, const int32_t* __restrict__ chunk_start,
                          ModelConsts k, DemCtx dc, DevScalars* sc) {
    const int W = k.W;
    const Chunk ch = chunk_of(chunk_start, dc.n, dc.in);
    const DemIn& r = dc.in[ch.d];
    const float rain0 = (float)r.rain, rinc = (float)r.rain_inc;
    int nact = 0;
    bool untiled = false;
    // two cells per thread and iteration: both cells' inputs are loaded before
    // either is used, so each thread keeps two cells' loads in flight
    for (int64_t r0 = ch.first + threadIdx.x; r0 < ch.end; r0 += 2 * blockDim.x) {
        size_t i[2];
        int y[2];
        uint8_t mk[2] = {0, 0}, code[2] = {0, 0};
        float sto[2], tb[2], sm0[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int64_t ri = r0 + u * blockDim.x;
            int x;
            i[u] = ri < ch.end ? region_cell(r, ri, W, &x, &y[u]) : 0;
            if (ri < ch.end) {
                mk[u] = mask[i[u]];
                code[u] = fd[i[u]];
                sto[u] = stone[i[u]];
                tb[u] = totB[i[u]];
                sm0[u] = soilM[i[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (r0 + u * blockDim.x >= ch.end) continue;
            if (mk[u]) {
                ++nact;
                const float coeff =
                    (1.0f - 0.0085f * sto[u]) * expf(-0.0025f * tb[u] / 76.5f) * tanhf(0.6f + sm0[u] / 0.2f);
                const float myppt = (rain0 + (float)(y[u] - r.y0) * rinc) / 1000.0f;
                const float wi = myppt * coeff;
                float sm = sm0[u] + myppt * (1.0f - coeff);
                if (sm > 0.5f) sm = 0.5f;
                soilM[i[u]] = sm;
                w[i[u]] = wi;
                fa[i[u]] = make_float2(wi, 0.0f);
                untiled |= wi < 0.0f || (code[u] & (code[u] - 1));
            } else {
                w[i[u]] = -9999.0f;
                fa[i[u]] = make_float2(0.0f, 0.0f);
            }
        }
    }
    if (__syncthreads_or(untiled) && threadIdx.x == 0) sc->tiled_ok = 0;
    const int tot = __syncthreads_count(nact > 0) ? block_sum_i(nact) : 0;  // one atomic per block
    if (threadIdx.x == 0 && tot) atomicAdd(&dc.out[ch.d].n_active, tot);
}

// In-degrees and sources of the global accumulation wave, for the steps that
// take it (MFD, contributing area, or a step k_fa_prep sent off the tiled path).
__global__ void k_fa_pend(const double* __restrict__ z, const uint8_t* __restrict__ mask,
                          const uint8_t* __restrict__ fd, int32_t* __restrict__ pending, int32_t* __restrict__ contrib,
                          int32_t* ready, const int32_t* __restrict__ chunk_start, ModelConsts k, DemCtx dc,
                          DevScalars* sc, int gate) {
    if (gate && sc->tiled_ok) return;  // the tiled path accumulates this step
    const int W = k.W, H = k.H;
    const size_t N = (size_t)W * H;
    const Chunk ch = chunk_of(chunk_start, dc.n, dc.in);
    const DemIn& r = dc.in[ch.d];
    for (int64_t base = ch.first; base < ch.end; base += blockDim.x) {
        const int64_t ri = base + threadIdx.x;
        bool src = false;
        size_t i = 0;
        if (ri < ch.end) {
            int x, y;
            i = region_cell(r, ri, W, &x, &y);
            if (mask[i]) {
                if (contrib) contrib[i] = 1;
                int32_t pend = 0;
#pragma unroll
                for (int d = 0; d < 8; ++d) {
                    const int nx = x + dir_dx(d), ny = y + dir_dy(d);
                    if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
                    const size_t n = (size_t)ny * W + nx;
                    if (!donates(fd[n], d)) continue;
                    if (mask[n])
                        ++pend;
                    else if (z[n] != kNoData)
                        pend |= kBlocked;
                }
                pending[i] = pend;
                src = (pend == 0);
            } else {
                if (contrib) contrib[i] = 0;
                pending[i] = kBlocked;
            }
        }
        wave_append(src, (int32_t)i, ready, &sc->counters[0], (int)N, &sc->err);
    }
}

// calcprops (runoffweight.cu:141-354): slope-proportional partition, forcing a
// single-direction code back to one direction (and rewriting its slopes).
__global__ void k_calcprops(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd, float* slopes,
                            float* prop, size_t N) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        if (!mask[i]) continue;
        float s[8];
        float tot = 0.f;
        for (int j = 0; j < 8; ++j) {
            s[j] = slopes[8 * i + j];
            tot += s[j];
        }
        int cnt = 0;
        float p[8];
        for (int j = 0; j < 8; ++j) {
            p[j] = s[j] / tot;
            if (p[j] > 0) ++cnt;
        }
        const int d = bit_dir(fd[i]);
        if (d >= 0 && cnt > 1) {
            for (int j = 0; j < 8; ++j) {
                slopes[8 * i + j] = (j == d) ? 0.0001f : 0.0f;
                p[j] = (j == d) ? 1.0f : 0.0f;
            }
        }
        for (int j = 0; j < 8; ++j) prop[8 * i + j] = p[j];
    }
}

__device__ __forceinline__ float prop_of(const float* prop, const uint8_t* mask, size_t n, int slot) {
    return prop ? prop[8 * n + slot] : (mask[n] ? 1.0f : 0.0f);
}

// One cell of correctmfdflow's CalcMFD (mfd_simple.cu:31-171): the weight plus
// the donors' accumulation in the order E, SE, S, SW, W, NW, N, NE, a negative
// donor sum clamped to zero.
struct FaCell {
    const uint8_t* mask;
    const uint8_t* fd;
    const float* w;
    const float* prop;
    float2* fa;
    int32_t* contrib;
    DemCtx dc;
    int W, H;
    __device__ __forceinline__ void cell(int32_t cur, int x, int y) const {
        if (dc.of) atomicAdd(&dc.out[dc.of[cur]].fa_done, 1);  // a batch: count per DEM
        float2 acc = make_float2(0.f, 0.f);
        int32_t cacc = 1;
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            const int d = scan_dir(kk);
            const int nx = x + dir_dx(d), ny = y + dir_dy(d);
            if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
            const int32_t n = ny * W + nx;
            if (!donates(__ldg(fd + n), d)) continue;
            const float2 v = __ldcg(fa + n);
            const float p = prop_of(prop, mask, n, (d + 4) & 7);
            acc = ff_add(acc, p == 1.0f ? v : ff_scale(v, p));
            if (contrib && __ldg(mask + n)) cacc += __ldcg(contrib + n);
        }
        if (acc.x < 0.0f) acc = make_float2(0.f, 0.f);
        __stcg(fa + cur, ff_add(make_float2(__ldg(w + cur), 0.f), acc));
        if (contrib) __stcg(contrib + cur, cacc);
    }
    __device__ __forceinline__ int receivers(int32_t cur, int x, int y, int32_t* r) const {
        return code_receivers(fd, mask, cur, x, y, W, H, r);
    }
    __device__ __forceinline__ void prefetch(int32_t) const {}
};

// The accumulation wave: every source starts it; cells follow as their last
// donor finishes.  With gate set it runs only when the tiled path is off.
__global__ void k_fa_walk(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd,
                          const float* __restrict__ w, const float* __restrict__ prop, float2* fa, int32_t* pending,
                          int32_t* contrib, int32_t* list_a, int32_t* list_b, ModelConsts k, DevScalars* sc,
                          DemCtx dc, int gate) {
    if (gate && sc->tiled_ok) return;  // the tiled kernels did this step
    const FaCell op{mask, fd, w, prop, fa, contrib, dc, k.W, k.H};
    int done = wave_walk(op, pending, list_a, list_b, k.W, k.H, sc);
    done = wsum(done);
    if (!dc.of && (threadIdx.x & 31) == 0 && done) atomicAdd(&dc.out[0].fa_done, done);
}

// ---------------------------------------------------------------------------
// Tiled accumulation for single-receiver codes (SFD).  A chain walk through
// global memory pays an L2 round trip per cell on the longest flow path; here
// the grid is cut into 32x32 tiles and most of the path runs in shared memory.
//   local : per tile, the accumulation from inside the tile (la), the outlet
//           each entry cell drains to, and per outlet its entries and the
//           number of inflows from other tiles it waits for;
//   coarse: a wave over the outlets only: F(o) = la(o) + the final values of
//           the outlets of neighbouring tiles that flow into o's entries;
//   final : per tile, every other cell by the reference formula, with the
//           donors in other tiles taken at their final values.
// All sums are pulled in a fixed order, so results do not depend on timing.
// The decomposition is exact while no donor sum can be negative (CalcMFD
// clamps those to zero); k_fa_prep disables the path for a step with a
// negative weight or a multi-direction code, and the walk then runs instead.


__device__ __forceinline__ void tile_load(const double* __restrict__ z, const uint8_t* __restrict__ mask,
                                          const uint8_t* __restrict__ fd, int W, int H, int tx0, int ty0,
                                          uint8_t* s_code, uint8_t* s_cls) {
    for (int j = threadIdx.x; j < kTH * kTH; j += blockDim.x) {
        const int gx = tx0 - 1 + j % kTH, gy = ty0 - 1 + j / kTH;
        uint8_t c = 0, cl = kCellOff;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            const size_t g = (size_t)gy * W + gx;
            c = fd[g];
            if (mask[g])
                cl = kCellIn;
            else if (z[g] != kNoData)
                cl = kCellBlock;
        }
        s_code[j] = c;
        s_cls[j] = cl;
    }
}

__global__ void __launch_bounds__(256, 8)
    k_fat_local(const double* __restrict__ z, const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd,
                const float* __restrict__ w, float2* __restrict__ t_la, int32_t* __restrict__ t_dst,
                int32_t* __restrict__ t_pend, int32_t* __restrict__ t_orng, int32_t* __restrict__ t_ent,
                float2* __restrict__ fa, int32_t* __restrict__ n_meta, int32_t* __restrict__ n_ref,
                int4* __restrict__ f_idx, float2* __restrict__ f_la, int32_t* __restrict__ t_fcnt, int32_t* srcs,
                ModelConsts k, DevScalars* sc, DemCtx dc, TileSet ts) {
    if (!sc->tiled_ok) return;
    __shared__ uint8_t s_code[kTH * kTH];
    __shared__ uint8_t s_cls[kTH * kTH];
    __shared__ int32_t s_pend[kTile * kTile];
    __shared__ float2 s_la[kTile * kTile];
    __shared__ int16_t s_ptr[kTile * kTile];
    __shared__ uint8_t s_kind[kTile * kTile];
    __shared__ uint8_t s_ext[kTile * kTile];
    __shared__ uint8_t s_done[kTile * kTile];
    __shared__ int16_t s_oslot[kTile * kTile];
    __shared__ int16_t s_q[kTile * kTile];
    __shared__ int16_t s_olist[kTileEnt];
    __shared__ int32_t s_ocnt[kTileEnt];
    __shared__ int16_t s_ostart[kTileEnt];
    __shared__ int16_t s_ofill[kTileEnt];
    __shared__ int s_no, s_qn, s_qend, s_nn, s_fn, s_pool;
    __shared__ int s_wcnt[9];  // per-warp counts of the outlet list and the source append
    const int W = k.W, H = k.H, TW = (W + kTile - 1) / kTile;
    const int t = ts.tile(blockIdx.x);
    const int tx0 = (t % TW) * kTile, ty0 = (t / TW) * kTile;
    const int lx = threadIdx.x & 31, ly0 = threadIdx.x >> 5;
    float wq[4];  // the cells' weights, loaded alongside the halo
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int gx = tx0 + lx, gy = ty0 + ly0 + 8 * q;
        wq[q] = (gx < W && gy < H) ? w[(size_t)gy * W + gx] : 0.f;
    }
    tile_load(z, mask, fd, W, H, tx0, ty0, s_code, s_cls);
    if (threadIdx.x == 0) s_fn = s_pool = 0;
    __syncthreads();
    bool src[4];  // chain starts, fixed before any chain runs (a chain may enter them later)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx, hc = (ly + 1) * kTH + lx + 1;
        int32_t pend = kBlocked;
        uint8_t kind = kKindEnd, ext = 0;
        int16_t ptr = (int16_t)l;
        float wl = 0.f;
        int16_t dm = 0;  // the in-tile donors: bit k for direction scan_dir(k)
        if (s_cls[hc] == kCellIn) {
            pend = 0;
#pragma unroll
            for (int d = 0; d < 8; ++d) {
                const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
                if (!donates(s_code[nh], d)) continue;
                const uint8_t cl = s_cls[nh];
                if (cl == kCellBlock)
                    pend |= kBlocked;
                else if (cl == kCellIn) {
                    if (in_tile(lx + dir_dx(d), ly + dir_dy(d))) {
                        ++pend;
                        dm |= (int16_t)(1 << scan_index(d));
                    } else {
                        ++ext;
                    }
                }
            }
            const int d = bit_dir(s_code[hc]);
            if (d >= 0 && s_cls[hc + dir_dy(d) * kTH + dir_dx(d)] == kCellIn) {
                const int rlx = lx + dir_dx(d), rly = ly + dir_dy(d);
                if (in_tile(rlx, rly)) {
                    kind = kKindIn;
                    ptr = (int16_t)(rly * kTile + rlx);
                } else {
                    kind = kKindOutlet;
                }
            }
            wl = wq[q];
        }
        s_pend[l] = pend;
        src[q] = pend == 0;
        s_kind[l] = kind;
        s_ext[l] = ext;
        s_ptr[l] = ptr;
        s_la[l] = make_float2(wl, 0.f);
        s_done[l] = 0;
        s_oslot[l] = dm;  // the outlet slots are listed after the wave
    }
    if (threadIdx.x == 0) s_qn = 0;
    __syncthreads();
    // accumulation from inside the tile, in dependency order
    tile_wave(
        [&](int cur, int rnd) {
            // the in-tile donors, all loaded before the sum in scan order
            const uint32_t dm = (uint16_t)s_oslot[cur];
            float2 v[8];
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                v[kk] = (dm >> kk) & 1u ? s_la[cur + tile_step(scan_dir(kk))] : make_float2(0.f, 0.f);
            float2 acc = make_float2(0.f, 0.f);
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                if ((dm >> kk) & 1u) acc = ff_add(acc, v[kk]);
            if (acc.x < 0.0f) acc = make_float2(0.f, 0.f);
            s_la[cur] = ff_add(s_la[cur], acc);
            s_done[cur] = kLaDone;
            return s_kind[cur] == kKindIn ? (int)s_ptr[cur] : -1;
        },
        s_pend, s_q, &s_qn, &s_qend, src, lx, ly0);
    // The waiting cells: every finished cell downstream of an entry (a cell
    // with a donor in another tile), marked along each entry's in-tile path.
    // A walk stops where another walk has passed (it carries on from there).
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        int c = (ly0 + 8 * q) * kTile + lx;
        if (!s_ext[c]) continue;
        for (int guard = 0; guard < kTile * kTile; ++guard) {
            if (s_done[c] != kLaDone) break;  // not finished, or marked already
            s_done[c] = kLaDone | kLaWaits;
            if (s_kind[c] != kKindIn) break;
            c = s_ptr[c];
        }
    }
    __syncthreads();
    // the end of every in-tile path: pointer jumping (paths are shorter than 2^10 cells)
    for (int it = 0; it < 10; ++it) {  // in-tile paths are shorter than 2^10 cells
        bool ch = false;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int l = (ly0 + 8 * q) * kTile + lx;
            const int16_t nx = s_ptr[s_ptr[l]];
            if (nx != s_ptr[l]) {
                s_ptr[l] = nx;
                ch = true;
            }
        }
        if (!__syncthreads_or(ch)) break;  // every pointer is at its path's end
    }
    bool stray = false;  // a waiting cell whose in-tile path ends inside the tile
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx;
        if (s_ext[l]) {
            const int e = s_ptr[l];
            t_dst[(size_t)(ty0 + ly) * W + tx0 + lx] =
                s_kind[e] == kKindOutlet ? (int32_t)((ty0 + e / kTile) * W + tx0 + (e & (kTile - 1))) : -1;
        }
        stray |= s_done[l] == (kLaDone | kLaWaits) && s_kind[s_ptr[l]] != kKindOutlet;
    }
    // Such a tile keeps the second wave; every other tile writes its settled
    // cells here and leaves the final pass a program of nodes (see below).
    const bool second_wave = __syncthreads_or(stray);
    // outlets in cell order (they lie on the border: at most 124)
    list_outlets(s_kind, s_olist, s_oslot, &s_no, s_wcnt);
    if (threadIdx.x < kTileEnt) s_ocnt[threadIdx.x] = 0;
    __syncthreads();
    // inflows: ring cells of the halo that flow into the tile, grouped by the
    // outlet their entry drains to, in ring order
    int key[kRingChunks];
    int32_t donor[kRingChunks];
#pragma unroll
    for (int c = 0; c < kRingChunks; ++c) {
        const int i = c * 32 + lx;
        key[c] = -1;
        donor[c] = 0;
        if (threadIdx.x < 32 && i < kRing) {
            const int h = ring_halo(i);
            const int d = s_cls[h] == kCellIn ? bit_dir(s_code[h]) : -1;
            if (d >= 0) {
                const int hx = h % kTH + dir_dx(d), hy = h / kTH + dir_dy(d);
                if (hx >= 1 && hx <= kTile && hy >= 1 && hy <= kTile && s_cls[hy * kTH + hx] == kCellIn) {
                    const int e = (hy - 1) * kTile + hx - 1;
                    const int o = s_ptr[e];
                    if (s_kind[o] == kKindOutlet) {
                        key[c] = s_oslot[o];
                        donor[c] = (ty0 - 1 + h / kTH) * W + tx0 - 1 + h % kTH;
                        atomicAdd(&s_ocnt[key[c]], 1);
                    }
                }
            }
        }
    }
    __syncthreads();
    const int no = s_no;
    if (threadIdx.x == 0) {
        int a = 0;
        for (int i = 0; i < no; ++i) {
            s_ostart[i] = (int16_t)a;
            s_ofill[i] = (int16_t)a;
            a += s_ocnt[i];
        }
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const unsigned below = (1u << lx) - 1u;
#pragma unroll
        for (int c = 0; c < kRingChunks; ++c) {
            const unsigned peers = __match_any_sync(0xffffffffu, key[c]);
            const int base = key[c] >= 0 ? s_ofill[key[c]] : 0;
            __syncwarp();
            if (key[c] >= 0) {
                t_ent[(size_t)t * kTileEnt + base + __popc(peers & below)] = donor[c];
                if ((peers & below) == 0) s_ofill[key[c]] = (int16_t)(base + __popc(peers));
            }
            __syncwarp();
        }
    }
    const int j = threadIdx.x;
    bool ready = false;
    int32_t og = 0;
    if (j < no) {
        const int o = s_olist[j];
        const int32_t opend = ((s_done[o] & kLaDone) ? 0 : kBlocked) + s_ocnt[j];
        og = (ty0 + o / kTile) * W + tx0 + (o & (kTile - 1));
        t_orng[og] = ((int)s_ostart[j] << 16) | s_ocnt[j];
        t_pend[og] = opend;
        t_la[og] = s_la[o];
        ready = (opend == 0);
    }
    block_append(ready, og, srcs, &sc->tile_src, W * H, &sc->err, s_wcnt);
    if (threadIdx.x == 0) t_fcnt[t] = -1;
    if (second_wave) return;  // block-uniform

    // The final pass's program.  A waiting cell's accumulation is its local
    // one plus the inflows of every entry upstream of it.  That sum is the same
    // along a run of single-input cells, so it is kept per node (an entry, a
    // join of two waiting branches, or the outlet): the inflows the node takes
    // from other tiles plus the sums of the nodes at the top of its waiting
    // inputs.  s_nd: node index + 1 in the low half (0: not a node), the cell
    // above in the high half (a cell between nodes: its waiting donor, then
    // the node at the top of its run).
    int32_t* s_nd = s_pend;  // the in-degrees are spent
    int done = 0, dem = -1;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx, hc = (ly + 1) * kTH + lx + 1;
        const size_t g = (size_t)(ty0 + ly) * W + tx0 + lx;
        int32_t nd = 0;
        if (dem < 0 && s_cls[hc] == kCellIn) dem = dem_at(dc, g);
        if (s_done[l] == kLaDone) {
            if (s_kind[l] != kKindOutlet) {  // the coarse wave stores the outlets
                fa[g] = s_la[l];
                ++done;
            }
        } else if (s_done[l] == (kLaDone | kLaWaits)) {
            int ntd = 0, up = l;
#pragma unroll
            for (int d = 0; d < 8; ++d) {
                const int nlx = lx + dir_dx(d), nly = ly + dir_dy(d);
                const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
                if (in_tile(nlx, nly) && donates(s_code[nh], d) && s_cls[nh] == kCellIn &&
                    (s_done[nly * kTile + nlx] & kLaWaits)) {
                    ++ntd;
                    up = nly * kTile + nlx;
                }
            }
            nd = (s_ext[l] != 0 || ntd >= 2 || s_kind[l] == kKindOutlet) ? 1 : (up << 16);
        }
        s_nd[l] = nd;
    }
    done = wsum(done);
    dem = __reduce_max_sync(0xffffffffu, dem);  // one DEM per tile
    if ((threadIdx.x & 31) == 0 && done && dem >= 0) atomicAdd(&dc.out[dem].fa_done, done);
    __syncthreads();
    // pointer jumping: every cell between nodes finds the node at the top of its run
    for (int it = 0; it < 10; ++it) {  // in-tile runs are shorter than 2^10 cells
        int32_t nu[4];
        bool ch = false;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int l = (ly0 + 8 * q) * kTile + lx;
            nu[q] = -1;
            const int32_t v = s_nd[l];
            if (s_done[l] != (kLaDone | kLaWaits) || (v & 0xffff)) continue;
            const int32_t vp = s_nd[v >> 16];
            if (vp & 0xffff) continue;  // at the top
            nu[q] = vp & ~0xffff;
            ch = true;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (nu[q] >= 0) s_nd[(ly0 + 8 * q) * kTile + lx] = nu[q];
        if (!__syncthreads_or(ch)) break;
    }
    // node indices in the order the wave reached the cells (inputs first):
    // warp w numbers the nodes among queue entries 128 w .. 128 w + 127
    {
        const int qn = s_qn, wq = threadIdx.x >> 5;
        const unsigned below = (1u << lx) - 1u;
        unsigned b[4];
        int cnt = 0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int i = wq * 128 + r * 32 + lx;
            bool isn = false;
            if (i < qn) {
                const int c = s_q[i];
                isn = s_done[c] == (kLaDone | kLaWaits) && (s_nd[c] & 0xffff);
            }
            b[r] = __ballot_sync(0xffffffffu, isn);
            cnt += __popc(b[r]);
        }
        if (lx == 0) s_wcnt[wq] = cnt;
        __syncthreads();
        int base = 0;
        for (int i = 0; i < wq; ++i) base += s_wcnt[i];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if ((b[r] >> lx) & 1u) s_nd[s_q[wq * 128 + r * 32 + lx]] = base + __popc(b[r] & below) + 1;
            base += __popc(b[r]);
        }
        if (threadIdx.x == 255) s_nn = base;  // the last warp's end is the total
    }
    __syncthreads();
    const size_t tb = (size_t)t * kTile * kTile, pool = (size_t)t * kTilePool;
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx, hc = (ly + 1) * kTH + lx + 1;
        const size_t g = (size_t)(ty0 + ly) * W + tx0 + lx;
        const int32_t v = s_nd[l];
        const bool waits = s_done[l] == (kLaDone | kLaWaits), outlet = s_kind[l] == kKindOutlet;
        const int e = warp_slot(waits || outlet, &s_fn);
        if (outlet) {  // counted once the coarse wave stored it
            f_idx[tb + e] = make_int4((int)g, 0, kLaOutlet, 0);
        } else if (waits) {
            const int node = (v & 0xffff) ? (v & 0xffff) - 1 : (s_nd[v >> 16] & 0xffff) - 1;
            f_idx[tb + e] = make_int4((int)g, node, 0, 0);
            f_la[tb + e] = s_la[l];
        }
        if (!waits || !(v & 0xffff)) continue;
        // the node's inputs, in the donors' scan order: cells of other tiles, then node indices (negated)
        int nin = 0;
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            const int nlx = lx + dir_dx(d), nly = ly + dir_dy(d);
            const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
            if (!donates(s_code[nh], d) || s_cls[nh] != kCellIn) continue;
            if (!in_tile(nlx, nly) || (s_done[nly * kTile + nlx] & kLaWaits)) ++nin;
        }
        const int start = atomicAdd(&s_pool, nin);
        if (start + nin > kTilePool) {
            raise_error(&sc->err, ErrFlags::kCapacity);
            continue;
        }
        int m = 0;
#pragma unroll 1
        for (int kk = 0; kk < 8; ++kk) {
            const int d = scan_dir(kk);
            const int nlx = lx + dir_dx(d), nly = ly + dir_dy(d);
            const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
            if (!donates(s_code[nh], d) || s_cls[nh] != kCellIn) continue;
            int32_t ref;
            if (!in_tile(nlx, nly)) {
                ref = (ty0 + nly) * W + tx0 + nlx;
            } else {
                const int u = nly * kTile + nlx;
                if (!(s_done[u] & kLaWaits)) continue;
                const int32_t vu = s_nd[u];
                ref = -((vu & 0xffff) ? (vu & 0xffff) : (s_nd[vu >> 16] & 0xffff));
            }
            n_ref[pool + start + m] = ref;
            ++m;
        }
        n_meta[tb + (v & 0xffff) - 1] = start | (m << 11);
    }
    __syncthreads();
    if (threadIdx.x == 0) t_fcnt[t] = (s_nn << 16) | s_fn;
}

// One outlet of the coarse wave.
struct CoarseCell {
    const uint8_t* mask;
    const uint8_t* fd;
    const float2* t_la;
    const int32_t* t_orng;
    const int32_t* t_ent;
    const int32_t* t_dst;
    float2* fa;
    int W, H, TW;
    __device__ __forceinline__ void cell(int32_t o, int x, int y) const {
        const int t = (y / kTile) * TW + x / kTile;
        const int rng = __ldg(t_orng + o);
        const int start = rng >> 16, cnt = rng & 0xffff;
        const int32_t* list = t_ent + (size_t)t * kTileEnt + start;
        float2 acc = __ldg(t_la + o);
        for (int i = 0; i < cnt; i += 8) {
            float2 v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = (i + j < cnt) ? __ldcg(fa + __ldg(list + i + j)) : make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (i + j < cnt) acc = ff_add(acc, v[j]);
        }
        __stcg(fa + o, acc);
    }
    __device__ __forceinline__ int receivers(int32_t o, int x, int y, int32_t* r) const {
        const int d = bit_dir(__ldg(fd + o));
        const int32_t rc = (y + dir_dy(d)) * W + x + dir_dx(d);
        const int32_t dst = __ldg(t_dst + rc);
        r[0] = dst;
        return dst >= 0 ? 1 : 0;
    }
    // the receiving outlet's record, read first when this lane carries on with it
    __device__ __forceinline__ void prefetch(int32_t o) const {
        if (o >= 0) prefetch_l2(t_orng + o);
    }
};

__global__ void k_fat_coarse(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd,
                             const float2* __restrict__ t_la, const int32_t* __restrict__ t_orng,
                             const int32_t* __restrict__ t_ent, const int32_t* __restrict__ t_dst, float2* fa,
                             int32_t* t_pend, int32_t* list_a, int32_t* list_b, ModelConsts k, DevScalars* sc) {
    if (!sc->tiled_ok) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->counters[0] = sc->tile_src;
    const CoarseCell op{mask, fd, t_la, t_orng, t_ent, t_dst, fa, k.W, k.H, (k.W + kTile - 1) / kTile};
    wave_walk(op, t_pend, list_a, list_b, k.W, k.H, sc);
}

__global__ void __launch_bounds__(256)
    k_fat_final(const double* __restrict__ z, const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd,
                const float* __restrict__ w, const int32_t* __restrict__ t_pend, float2* fa,
                const int32_t* __restrict__ n_meta, const int32_t* __restrict__ n_ref, const int4* __restrict__ f_idx,
                const float2* __restrict__ f_la, const int32_t* __restrict__ t_fcnt, ModelConsts k, DevScalars* sc,
                DemCtx dc, TileSet ts) {
    if (!sc->tiled_ok) return;
    __shared__ uint8_t s_code[kTH * kTH];
    __shared__ uint8_t s_cls[kTH * kTH];
    __shared__ uint8_t s_hok[kTH * kTH];
    __shared__ float2 s_hval[kTH * kTH];
    __shared__ int32_t s_pend[kTile * kTile];
    __shared__ float2 s_val[kTile * kTile];
    __shared__ int16_t s_q[kTile * kTile];
    __shared__ int s_done, s_dem, s_qn, s_qend;
    const int W = k.W, H = k.H, TW = (W + kTile - 1) / kTile;
    const int t = ts.tile(blockIdx.x);
    const int fc = t_fcnt[t];
    if (fc >= 0) {
        // The tile's program: each node's sum of inflows, then every waiting
        // cell's local accumulation plus the sum of its node.  A node is valid
        // when every inflow upstream completed.
        const int ne = fc & 0xffff, nn = fc >> 16;
        const size_t tb = (size_t)t * kTile * kTile, pool = (size_t)t * kTilePool;
        float2* s_X = s_val;      // node sums
        int32_t* s_ok = s_pend;  // node valid
        // (the second wave's arrays are free here) per node: its largest input
        // node + 1 and its number of input nodes, and up to four input nodes
        int16_t* s_nin = s_q;                                     // (largest + 1) | count << 11
        int16_t* s_in4 = reinterpret_cast<int16_t*>(s_hval);      // [4 * node]
        for (int n = threadIdx.x; n < nn; n += blockDim.x) {
            const int meta = n_meta[tb + n];
            const int start = meta & 2047, nin = meta >> 11;
            float2 acc = make_float2(0.f, 0.f);
            int ok = 1, top = 0, cnt = 0;
            for (int j = 0; j < nin; ++j) {
                const int32_t ref = n_ref[pool + start + j];
                if (ref < 0) {  // an input node: added in the pass below
                    const int u = -ref - 1;
                    if (cnt < 4) s_in4[4 * n + cnt] = (int16_t)u;
                    ++cnt;
                    top = u + 1 > top ? u + 1 : top;
                    continue;
                }
                acc = ff_add(acc, __ldcg(fa + ref));
                ok &= t_pend[ref] == 0;
            }
            s_X[n] = acc;
            s_ok[n] = ok;
            s_nin[n] = (int16_t)(top | (cnt << 11));
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            // in index order (a node's inputs have smaller indices), a run of
            // nodes with no input inside the run at a time
            const int lane = threadIdx.x;
            for (int i = 0; i < nn;) {
                const int n = i + lane;
                int info = 0;
                if (n < nn) info = s_nin[n];
                const bool dep = n < nn && (info & 2047) - 1 >= i;
                const unsigned b = __ballot_sync(0xffffffffu, dep);
                const int run = b ? __ffs(b) - 1 : 32;  // lane 0's inputs all lie before i
                if (lane < run && n < nn) {
                    float2 acc = s_X[n];
                    int ok = s_ok[n];
                    const int cnt = info >> 11;
                    if (cnt <= 4) {
                        for (int j = 0; j < cnt; ++j) {
                            const int u = s_in4[4 * n + j];
                            acc = ff_add(acc, s_X[u]);
                            ok &= s_ok[u];
                        }
                    } else {  // more input nodes than kept: from memory, in the same order
                        const int meta = n_meta[tb + n];
                        for (int j = 0; j < (meta >> 11); ++j) {
                            const int32_t ref = n_ref[pool + (meta & 2047) + j];
                            if (ref >= 0) continue;
                            acc = ff_add(acc, s_X[-ref - 1]);
                            ok &= s_ok[-ref - 1];
                        }
                    }
                    s_X[n] = acc;
                    s_ok[n] = ok;
                }
                __syncwarp();
                i += run;
            }
        }
        __syncthreads();
        int done = 0, dem = -1;
        for (int e = threadIdx.x; e < ne; e += blockDim.x) {
            const int4 id = f_idx[tb + e];
            dem = dem_at(dc, (size_t)id.x);
            if (id.z & kLaOutlet) {
                done += t_pend[id.x] == 0;
                continue;
            }
            if (!s_ok[id.y]) continue;
            fa[id.x] = ff_add(f_la[tb + e], s_X[id.y]);
            ++done;
        }
        done = wsum(done);
        dem = __reduce_max_sync(0xffffffffu, dem);
        if ((threadIdx.x & 31) == 0 && done && dem >= 0) atomicAdd(&dc.out[dem].fa_done, done);
        return;
    }
    const int tx0 = (t % TW) * kTile, ty0 = (t / TW) * kTile;
    tile_load(z, mask, fd, W, H, tx0, ty0, s_code, s_cls);
    // donors in other tiles: outlets of their tiles, final after the coarse wave
    for (int j = threadIdx.x; j < kTH * kTH; j += blockDim.x) {
        const int hx = j % kTH, hy = j / kTH;
        if (hx != 0 && hx != kTH - 1 && hy != 0 && hy != kTH - 1) continue;
        const int gx = tx0 - 1 + hx, gy = ty0 - 1 + hy;
        uint8_t ok = 0;
        float2 v = make_float2(0.f, 0.f);
        if (gx >= 0 && gx < W && gy >= 0 && gy < H && mask[(size_t)gy * W + gx]) {
            const size_t g = (size_t)gy * W + gx;
            ok = t_pend[g] == 0;
            v = fa[g];
        }
        s_hok[j] = ok;
        s_hval[j] = v;
    }
    if (threadIdx.x == 0) s_done = 0, s_dem = -1;
    __syncthreads();
    const int lx = threadIdx.x & 31, ly0 = threadIdx.x >> 5;
    int done = 0, dem = -1;  // one DEM per tile
    bool outlet[4], src[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx, hc = (ly + 1) * kTH + lx + 1;
        int32_t pend = kBlocked;
        float wl = 0.f;
        outlet[q] = false;
        if (s_cls[hc] == kCellIn) {
            pend = 0;
#pragma unroll
            for (int d = 0; d < 8; ++d) {
                const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
                if (!donates(s_code[nh], d)) continue;
                const uint8_t cl = s_cls[nh];
                if (cl == kCellBlock)
                    pend |= kBlocked;
                else if (cl == kCellIn) {
                    if (in_tile(lx + dir_dx(d), ly + dir_dy(d)))
                        ++pend;
                    else if (!s_hok[nh])
                        pend |= kBlocked;
                }
            }
            const int d = bit_dir(s_code[hc]);
            if (d >= 0 && s_cls[hc + dir_dy(d) * kTH + dir_dx(d)] == kCellIn &&
                !in_tile(lx + dir_dx(d), ly + dir_dy(d))) {
                outlet[q] = true;
                if (t_pend[(size_t)(ty0 + ly) * W + tx0 + lx] == 0) ++done;
            }
            wl = w[(size_t)(ty0 + ly) * W + tx0 + lx];
            if (dem < 0) dem = dem_at(dc, (size_t)(ty0 + ly) * W + tx0 + lx);
        }
        s_pend[l] = pend;
        src[q] = pend == 0 && !outlet[q];
        s_val[l] = make_float2(wl, 0.f);
    }
    dem = __reduce_max_sync(0xffffffffu, dem);
    if ((threadIdx.x & 31) == 0 && dem >= 0) atomicMax(&s_dem, dem);
    if (threadIdx.x == 0) s_qn = 0;
    __syncthreads();
    tile_wave(
        [&](int cur, int rnd) {
            const int cx = cur & (kTile - 1), cy = cur / kTile, hc = (cy + 1) * kTH + cx + 1;
            float2 acc = make_float2(0.f, 0.f);
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                const int d = scan_dir(kk);
                const int nlx = cx + dir_dx(d), nly = cy + dir_dy(d);
                const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
                if (!donates(s_code[nh], d) || s_cls[nh] != kCellIn) continue;
                acc = ff_add(acc, in_tile(nlx, nly) ? s_val[nly * kTile + nlx] : s_hval[nh]);
            }
            if (acc.x < 0.0f) acc = make_float2(0.f, 0.f);
            const float2 v = ff_add(s_val[cur], acc);
            s_val[cur] = v;
            fa[(size_t)(ty0 + cy) * W + tx0 + cx] = v;
            ++done;
            const int d = bit_dir(s_code[hc]);
            if (d < 0) return -1;
            const int rlx = cx + dir_dx(d), rly = cy + dir_dy(d);
            const int rh = hc + dir_dy(d) * kTH + dir_dx(d);
            if (!in_tile(rlx, rly) || s_cls[rh] != kCellIn) return -1;
            // an outlet keeps the coarse wave's value
            const int dr = bit_dir(s_code[rh]);
            if (dr >= 0 && s_cls[rh + dir_dy(dr) * kTH + dir_dx(dr)] == kCellIn &&
                !in_tile(rlx + dir_dx(dr), rly + dir_dy(dr)))
                return -1;
            return rly * kTile + rlx;
        },
        s_pend, s_q, &s_qn, &s_qend, src, lx, ly0);
    done = wsum(done);
    if ((threadIdx.x & 31) == 0 && done) atomicAdd(&s_done, done);
    __syncthreads();
    if (threadIdx.x == 0 && s_done && s_dem >= 0) atomicAdd(&dc.out[s_dem].fa_done, s_done);
}

// correctmfdflow's first-iteration branch (mfd_simple.cu:336-349): the outlet
// becomes the first cell holding the largest accumulation.
__global__ void k_fa_argmax(const float2* __restrict__ fa, const int32_t* __restrict__ chunk_start, int W,
                            DemCtx dc, int phase) {
    const Chunk ch = chunk_of(chunk_start, dc.n, dc.in);
    const DemIn& r = dc.in[ch.d];
    DemOut& o = dc.out[ch.d];
    if (!r.outlet_from_fa) return;
    for (int64_t ri = ch.first + threadIdx.x; ri < ch.end; ri += blockDim.x) {
        int x, y;
        const size_t i = region_cell(r, ri, W, &x, &y);
        const float2 v = fa[i];
        if (v.x != v.x) continue;  // NaN never wins the host scan (mfd_simple.cu:341)
        const unsigned long long kk = ffkey(v);
        if (phase == 0)
            atomicMax(&o.fa_max_key, kk);
        else if (kk == o.fa_max_key)
            atomicMin(&o.argmax, (int32_t)i);
    }
}

// The DEM's outlet becomes the first cell of the largest accumulation; with
// none above zero the reference's scan leaves index 0, the region's first cell.
__global__ void k_fa_argmax_set(int W, DemCtx dc) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= dc.n || !dc.in[d].active || !dc.in[d].outlet_from_fa) return;
    const unsigned long long zero = ffkey(make_float2(0.f, 0.f));
    DemOut& o = dc.out[d];
    o.outlet = (o.fa_max_key > zero) ? o.argmax : dc.in[d].y0 * W + dc.in[d].x0;
}

__global__ void k_fa_reset(DevScalars* sc, DemCtx dc, int tiled) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d == 0) {
        sc->counters[0] = 0;
        sc->tiled_ok = tiled;
        sc->tile_src = 0;
    }
    if (d < dc.n) {
        DemOut& o = dc.out[d];
        o.fa_done = 0;
        o.n_active = 0;
        o.fa_max_key = 0ull;
        o.argmax = 0x7fffffff;
    }
}

}  // namespace

lem_status launch_flow_accumulation(const DevState& s, const ModelConsts& k, uint32_t flags, const Launch& L) {
    const size_t N = (size_t)k.W * k.H;
    const int T = 256;
    size_t nb = (N + T - 1) / T;
    const int blocks = (int)(nb > 152 * 32 ? 152 * 32 : nb);
    const int dem_blocks = (s.dems.n + 127) / 128;
    int32_t* contrib = (flags & LEM_STEP_CONTRIB) ? s.contrib : nullptr;
    const int tiled = (k.flow_type == 0 && !contrib) ? 1 : 0;
    LEM_LAUNCH(L, k_fa_reset, dem_blocks, 128, s.sc, s.dems, tiled);
    const float* prop = nullptr;
    if (k.flow_type != 0 && k.mfd_props) {
        LEM_LAUNCH(L, k_calcprops, blocks, T, s.mask, s.fd, s.slopes, s.prop, N);
        prop = s.prop;
    }
    LEM_LAUNCH(L, k_fa_prep, s.n_chunks, T, s.mask, s.fd, s.stone, s.totB, s.soilM, s.w, s.fa, s.chunk_start, k,
               s.dems, s.sc);
    LEM_LAUNCH(L, k_fa_pend, s.n_chunks, T, s.z, s.mask, s.fd, s.pending, contrib, s.list_a, s.chunk_start, k, s.dems,
               s.sc, tiled);
    if (tiled) {
        const TileSet ts = tiles_of(s, k.W);
        const int tiles = ts.n;
        LEM_LAUNCH(L, k_fat_local, tiles, 256, s.z, s.mask, s.fd, s.w, s.t_la, s.t_dst, s.t_pend, s.t_orng, s.t_ent,
                   s.fa, s.n_meta, s.p_ref, s.f_idx, s.f_ds, s.t_fcnt, s.list_b, k, s.sc, s.dems, ts);
        const uint8_t* mask = s.mask;
        const uint8_t* fd = s.fd;
        const float2* tla = s.t_la;
        const int32_t* torng = s.t_orng;
        const int32_t* tent = s.t_ent;
        const int32_t* tdst = s.t_dst;
        float2* fa = s.fa;
        int32_t* tpend = s.t_pend;
        int32_t* la = s.list_b;  // the outlets k_fat_local found ready
        int32_t* lb = s.list_a;
        ModelConsts kk = k;
        DevScalars* sc = s.sc;
        void* args[] = {(void*)&mask, (void*)&fd, (void*)&tla, (void*)&torng, (void*)&tent, (void*)&tdst,
                        (void*)&fa, (void*)&tpend, (void*)&la, (void*)&lb, (void*)&kk, (void*)&sc};
        L.pre("k_fat_coarse");
        LEM_CUDA_TRY(coop_launch((const void*)k_fat_coarse, s.coop_blocks[kCkFatCoarse], args, L.st));
        L.post();
        LEM_LAUNCH(L, k_fat_final, tiles, 256, s.z, s.mask, s.fd, s.w, s.t_pend, s.fa, s.n_meta, s.p_ref, s.f_idx,
                   s.f_ds, s.t_fcnt, k, s.sc, s.dems, ts);
    }
    {
        const uint8_t* mask = s.mask;
        const uint8_t* fd = s.fd;
        const float* w = s.w;
        float2* fa = s.fa;
        int32_t* pending = s.pending;
        int32_t* la = s.list_a;
        int32_t* lb = s.list_b;
        ModelConsts kk = k;
        DevScalars* sc = s.sc;
        DemCtx dc = s.dems;
        int gate = tiled;
        void* args[] = {(void*)&mask,    (void*)&fd, (void*)&w,  (void*)&prop, (void*)&fa,  (void*)&pending,
                        (void*)&contrib, (void*)&la, (void*)&lb, (void*)&kk,   (void*)&sc,  (void*)&dc,
                        (void*)&gate};
        L.pre("k_fa_walk");
        LEM_CUDA_TRY(coop_launch((const void*)k_fa_walk, s.coop_blocks[kCkFaWalk], args, L.st));
        L.post();
    }
    if (flags & LEM_STEP_SET_OUTLET_FROM_FA) {  // some DEM moves its outlet this step
        LEM_LAUNCH(L, k_fa_argmax, s.n_chunks, T, s.fa, s.chunk_start, k.W, s.dems, 0);
        LEM_LAUNCH(L, k_fa_argmax, s.n_chunks, T, s.fa, s.chunk_start, k.W, s.dems, 1);
        LEM_LAUNCH(L, k_fa_argmax_set, dem_blocks, 128, k.W, s.dems);
    }
    LEM_CUDA_TRY(cudaGetLastError());
    return LEM_OK;
}

// ---------------------------------------------------------------------------
// lem_accumulate_flow_noalloc: the accumulation wave on caller-owned buffers,
// with its intermediate data in one file-scope device array.
namespace {

constexpr size_t kNaCells = LEM_NOALLOC_MAX_CELLS;
constexpr size_t kNaHead = 1024;  // DevScalars and one DemOut, rounded up
constexpr size_t kNaOffDem = 512;
static_assert(sizeof(DevScalars) <= kNaOffDem && kNaOffDem + sizeof(DemOut) <= kNaHead, "scalar block");
constexpr size_t kNaOffCode = kNaHead;
constexpr size_t kNaOffMask = kNaOffCode + kNaCells;
constexpr size_t kNaOffPend = kNaOffMask + kNaCells;          // int32
constexpr size_t kNaOffListA = kNaOffPend + 4 * kNaCells;     // int32
constexpr size_t kNaOffListB = kNaOffListA + 4 * kNaCells;    // int32
constexpr size_t kNaOffW = kNaOffListB + 4 * kNaCells;        // float
constexpr size_t kNaOffFa = kNaOffW + 4 * kNaCells;           // float2
constexpr size_t kNaBytes = kNaOffFa + 8 * kNaCells;

// Scratch of the no-allocation entry point (every call shares it).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

struct NaDevice {
    unsigned char* base = nullptr;  // device address of g_noalloc_scratch
    int blocks = 0;                 // co-resident blocks of k_fa_walk
};
std::mutex g_na_mutex;
NaDevice g_na[64];

__global__ void k_na_reset(DevScalars* sc, DemOut* dem) {
    dem->fa_done = 0;
    dem->n_active = 0;
    sc->counters[0] = sc->counters[1] = sc->counters[2] = 0;
    sc->err = 0;
    sc->err_first = 0;
}

// Codes, mask, weights, initial accumulation and in-degrees from the caller's
// int32 codes and DEM (cells at -9999 are outside and complete with zero flow).
__global__ void k_na_prep(const int32_t* __restrict__ fd_in, const double* __restrict__ w_in,
                          const double* __restrict__ dem, uint8_t* __restrict__ code, uint8_t* __restrict__ mask,
                          float* __restrict__ w, float2* __restrict__ fa, int32_t* __restrict__ pending,
                          int32_t* ready, int W, int H, DevScalars* sc, DemOut* dem_out) {
    const size_t N = (size_t)W * H;
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < N; base += (size_t)gridDim.x * blockDim.x) {
        const size_t i = base + threadIdx.x;
        bool src = false, act = false;
        if (i < N) {
            const int x = (int)(i % W), y = (int)(i / W);
            const bool in = dem[i] != kNoData;
            code[i] = (uint8_t)(fd_in[i] & 0xff);
            mask[i] = in ? 1 : 0;
            const float wi = (float)w_in[i];
            w[i] = wi;
            fa[i] = make_float2(in ? wi : 0.0f, 0.0f);
            int32_t pend = in ? 0 : kBlocked;
            for (int d = 0; in && d < 8; ++d) {
                const int nx = x + dir_dx(d), ny = y + dir_dy(d);
                if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
                const size_t n = (size_t)ny * W + nx;
                if (donates((uint8_t)(fd_in[n] & 0xff), d) && dem[n] != kNoData) ++pend;
            }
            pending[i] = pend;
            src = in && pend == 0;
            act = in;
        }
        const unsigned nact = __ballot_sync(0xffffffffu, act);  // in-catchment cells, one atomic per warp
        if ((threadIdx.x & 31) == 0 && nact) atomicAdd(&dem_out->n_active, __popc(nact));
        wave_append(src, (int32_t)i, ready, &sc->counters[0], (int)N, &sc->err);
    }
}

__global__ void k_na_out(const float2* __restrict__ fa, double* __restrict__ out, size_t N) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (double)fa[i].x + (double)fa[i].y;
}

}  // namespace

extern "C" lem_status lem_accumulate_flow_noalloc(const int32_t* d_fd, const double* d_weight,
                                                  const double* d_dem, double* d_fa, int32_t width,
                                                  int32_t height, void* stream) {
    if (!d_fd || !d_weight || !d_dem || !d_fa || width < 1 || height < 1) return LEM_ERR_INVALID;
    const size_t N = (size_t)width * height;
    if (N > kNaCells) return LEM_ERR_CAPACITY;  // the static scratch holds LEM_NOALLOC_MAX_CELLS cells
    int dev = 0;
    LEM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return LEM_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    LEM_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
    NaDevice nd;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (cap == cudaStreamCaptureStatusNone || !g_na[dev].base) {
            // With that device current: the device address of the array.  It is
            // looked up again on every call outside a stream capture, so a
            // context torn down and created again (cudaDeviceReset) gets the
            // array's new address; inside a capture the address of the last
            // call on this device is used.
            void* ptr = nullptr;
            LEM_CUDA_TRY(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
            if (!g_na[dev].blocks) {
                int per = 0, sms = 0;
                LEM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fa_walk, 256, 0));
                LEM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
                g_na[dev].blocks = (per < 1 ? 1 : per) * sms;
            }
            g_na[dev].base = static_cast<unsigned char*>(ptr);
        }
        nd = g_na[dev];
    }
    DevScalars* sc = reinterpret_cast<DevScalars*>(nd.base);
    DemOut* dem = reinterpret_cast<DemOut*>(nd.base + kNaOffDem);
    uint8_t* code = nd.base + kNaOffCode;
    uint8_t* mask = nd.base + kNaOffMask;
    int32_t* pending = reinterpret_cast<int32_t*>(nd.base + kNaOffPend);
    int32_t* la = reinterpret_cast<int32_t*>(nd.base + kNaOffListA);
    int32_t* lb = reinterpret_cast<int32_t*>(nd.base + kNaOffListB);
    float* w = reinterpret_cast<float*>(nd.base + kNaOffW);
    float2* fa = reinterpret_cast<float2*>(nd.base + kNaOffFa);
    const int T = 256;
    const int blocks = (int)std::min<size_t>((N + T - 1) / T, 152 * 32);
    k_na_reset<<<1, 1, 0, st>>>(sc, dem);  // the array keeps the previous call's contents
    k_na_prep<<<blocks, T, 0, st>>>(d_fd, d_weight, d_dem, code, mask, w, fa, pending, la, width, height, sc, dem);
    LEM_CUDA_TRY(cudaGetLastError());
    {
        const uint8_t* m = mask;
        const uint8_t* c = code;
        const float* ww = w;
        const float* prop = nullptr;
        int32_t* contrib = nullptr;
        ModelConsts k{};
        k.W = width;
        k.H = height;
        int gate = 0;
        DemCtx dc{nullptr, nullptr, dem, 1};
        void* args[] = {(void*)&m, (void*)&c, (void*)&ww, (void*)&prop, (void*)&fa, (void*)&pending,
                        (void*)&contrib, (void*)&la, (void*)&lb, (void*)&k, (void*)&sc, (void*)&dc, (void*)&gate};
        LEM_CUDA_TRY(coop_launch((const void*)k_fa_walk, nd.blocks, args, st));
    }
    k_na_out<<<blocks, T, 0, st>>>(fa, d_fa, N);
    LEM_CUDA_TRY(cudaGetLastError());
    uint32_t err[2] = {0, 0};  // err and err_first
    DemOut counts{};
    LEM_CUDA_TRY(cudaMemcpyAsync(err, &sc->err, sizeof err, cudaMemcpyDeviceToHost, st));
    LEM_CUDA_TRY(cudaMemcpyAsync(&counts, dem, sizeof counts, cudaMemcpyDeviceToHost, st));
    LEM_CUDA_TRY(cudaStreamSynchronize(st));
    if (err[1] == ErrFlags::kCapacity || (err[0] & ErrFlags::kCapacity && err[1] != ErrFlags::kNoConverge))
        return LEM_ERR_CAPACITY;
    if (err[0]) return LEM_ERR_NOCONVERGE;
    // in-catchment cells the wave never reached (a cycle in the codes, or a
    // donor chain through one): they hold their own weight, as correctmfdflow
    // leaves them (mfd_simple.cu:72), and the call says so
    if (counts.fa_done < counts.n_active) return LEM_ERR_NOCONVERGE;
    return LEM_OK;
}

const void* fa_coop_kernels[] = {(const void*)k_fa_walk, (const void*)k_fat_coarse};
extern const int fa_coop_kernel_count = 2;

}  // namespace lem
