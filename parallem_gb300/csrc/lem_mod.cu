// lem_mod.cu -- process stage: erosion, sediment routing, surface update.
//
// erosionGPU (MOD_kernels/erosion.cu:69-186) runs ten kernels and ~20 host
// copies per step.  Here it is three passes over the grid:
//   k_erosion  aveslope + diff_erosion + conc_erosion + gelifluction
//              (eroincidep.cu:8-198), budget sums and FA_max in the epilogue;
//   k_sed_*    sedmfdaccum / MFDsedbud (mfd_accum.cu:32-483) as a dependency
//              wave like the accumulation (lem_fa.cu);
//   k_final    surface_change + weathering + Update_Surface +
//              update_nutrient_content + grow_vegetation (eroincidep.cu:200-327,
//              updates.cu:23-139) fused, with their budget sums.
// The climate grids of SetClimateMatrices (Data.cpp:211-303) are generated on
// the fly from the row index and the DEM.

#include <cooperative_groups.h>

#include "lem_wave.cuh"

namespace cg = cooperative_groups;

namespace lem {

namespace {

constexpr double kMinHeight = 467.228;  // Data.cpp:252

// Temperature of cell i (tempmat): T - (z - 467.228) * 0.0065 with z the DEM the
// grids were built from (the initial DEM during run-in, the DEM at the start of
// the step otherwise; the outlet uses its value before the stage-1 adjustment).
__device__ __forceinline__ float clim_temp(const DemIn& c, const double* z, const double* z_init, size_t i,
                                           int outlet_clim, double outlet_z) {
    double zc = c.from_current_dem ? (((int)i == outlet_clim) ? outlet_z : z[i]) : z_init[i];
    float hi, lo;
    dsplit(zc, hi, lo);
    return (float)c.temp - ((hi - (float)kMinHeight) + lo) * 0.0065f;
}

__device__ __forceinline__ double block_sum_d(float v, double* red) {
    // fp32 warp partials, fp64 across warps
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    const int wid = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[wid] = (double)v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
    return t;
}

__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v, unsigned long long* red) {
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u > v ? u : v;
    }
    const int wid = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[wid] = v;
    __syncthreads();
    unsigned long long m = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) m = red[i] > m ? red[i] : m;
    return m;
}

// five blocks per SM: a few spilled registers, measured faster than four or six
__global__ void __launch_bounds__(256, 5)
    k_erosion(const double* __restrict__ z, const double* __restrict__ z_init, const uint8_t* __restrict__ mask,
              const float* __restrict__ slopes, const float2* __restrict__ fa, const float* __restrict__ fines,
              const float* __restrict__ nut, const float* __restrict__ soilT, const float* __restrict__ stone,
              const float* __restrict__ totB, float* __restrict__ slopeptr, float* __restrict__ ero,
              float* __restrict__ inci, float* __restrict__ geli, float* __restrict__ depo,
              const uint8_t* __restrict__ fd, const int32_t* __restrict__ chunk_start, ModelConsts k, DemCtx dc,
              DevScalars* sc) {
    __shared__ double red[8];
    __shared__ unsigned long long redk[8];
    const Chunk ch = chunk_of(chunk_start, dc.n, dc.in);
    const DemIn& c = dc.in[ch.d];
    DemOut& o = dc.out[ch.d];
    const int W = k.W;
    const int outlet = o.outlet;
    const int outlet_clim = o.outlet_clim;  // the cell whose climate elevation is outlet_z_clim
    const double outlet_z = o.outlet_z_clim;
    if (ch.first == 0 && threadIdx.x == 0) o.base_level = z[outlet] - 0.00012;  // updates.cu:151
    float se = 0.f, si = 0.f, sg = 0.f;
    unsigned long long famax = 0;
    bool multi = false;
    for (int64_t ri = ch.first + threadIdx.x; ri < ch.end; ri += blockDim.x) {
        int x, y;
        const size_t i = region_cell(c, ri, W, &x, &y);
        // every input of the cell in one batch of loads, ahead of the mask test
        // and the arithmetic (the region's cells outside the catchment are few)
        const float2 f2 = fa[i];
        const uint8_t mk = mask[i], code = fd[i];
        const float4 a = reinterpret_cast<const float4*>(slopes)[2 * i];
        const float4 b = reinterpret_cast<const float4*>(slopes)[2 * i + 1];
        const float st = soilT[i], tb = totB[i], fi = fines[i], nu = nut[i], sto = stone[i];
        float T = clim_temp(c, z, z_init, i, outlet_clim, outlet_z);
        const unsigned long long fk = ffkey(f2);
        if (f2.x == f2.x) famax = fk > famax ? fk : famax;  // the reduction skips NaN (thrust::maximum order)
        if (!mk) {
            ero[i] = inci[i] = geli[i] = 0.0f;
            slopeptr[i] = 0.0f;
            continue;
        }
        // sedmfdaccum set-up (mfd_accum.cu:389-396): depo = 1e-5 in the catchment.
        // A multi-direction code among the routed cells (not row 0 / column 0,
        // mfd_accum.cu:42) sends the step's sediment routing to the walk.
        depo[i] = 0.00001f;
        if (x != 0 && y != 0) multi |= (code & (code - 1)) != 0;
        // aveslope (eroincidep.cu:8-37): mean of the positive entries
        const float sv[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        float total = 0.f;
        int nonzero = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            total += sv[j];
            nonzero += sv[j] > 0.f;
        }
        const float sp = (total > 0.f && nonzero > 0) ? total / (float)nonzero : 0.f;
        slopeptr[i] = sp;
        const float fav = f2.x + f2.y;
        const float veg = expf(-0.07f * tb / 76.5f);
        // diff_erosion (eroincidep.cu:39-87)
        float erod = (2.77e-6f * powf(fi, 1.14f) * (12.0f - nu)) + k.erod_const;
        if (erod < 0.f) erod = 0.f;
        float OF = (fav * 1000.0f) / 25.0f;
        if (OF > k.q_threshold) OF = k.q_threshold;
        float slope = sp;
        if (slope == 0.f) slope = 0.0001f;
        if (slope > 5.0f) slope = 5.0f;
        float e = ((erod * OF * OF * powf(slope, 1.67f) * (powf(110.0f - sto, 0.877f) / 61.7023f))) * veg;
        if (e > st) e = st;
        // conc_erosion (eroincidep.cu:89-152)
        float cslope = sp;
        if (cslope > 0.5f) cslope = 0.5f;
        // fa * cs^2/1e4 - Qthreshold cancels near the threshold: evaluate it on the
        // (hi, lo) accumulation and the split constants
        float f_temp = fmaf(f2.x, k.rescale_conc, -k.q_threshold) +
                       (fmaf(f2.x, k.rescale_conc_lo, f2.y * k.rescale_conc) - k.q_threshold_lo);
        float in;
        if (f_temp < 0.0f) {
            f_temp = 0.0f;
            in = 0.0f;
        } else {
            in = k.flow_a * powf(f_temp, k.flow_b) * (cslope == 0.0f ? 0.01f : cslope) * veg;
        }
        if (in > k.max_incision) in = k.max_incision;
        if (in > st) {
            const float bed = (1.0f - (st / in)) * 0.0001f * powf(f_temp, k.flow_b) * cslope * veg;
            in = st + bed;
            if (in > k.max_incision) in = k.max_incision;
        }
        // gelifluction (eroincidep.cu:154-198).  The quartic kappa(T) cancels near
        // its roots (T ~ -16.8 and 8.6 C) and the range test has edges at -20 and 8.87 C:
        // there the temperature and kappa take the reference's fp64 arithmetic.
        float kappa = k.kappa;
        if (T >= -20.f && T <= 8.87f)
            kappa = 0.15711f - 0.011835f * T - 0.001195f * T * T + 0.000038f * T * T * T + 0.000002f * T * T * T * T;
        if (fabsf(T - 8.87f) < 1e-3f || fabsf(T + 20.0f) < 1e-3f || fabsf(kappa) < 4e-3f) {
            const double zc = c.from_current_dem ? (((int)i == outlet_clim) ? outlet_z : z[i]) : z_init[i];
            const double Td = c.temp - ((zc - kMinHeight) * 0.0065);
            double kd = (double)k.kappa;
            if (Td >= -20. && Td <= 8.87)
                kd = 0.15711 - 0.011835 * Td - 0.001195 * Td * Td + 0.000038 * Td * Td * Td +
                     0.000002 * Td * Td * Td * Td;
            kappa = (float)kd;
            T = (float)Td;
        }
        // 1 - fa/Gflowlim cancels where fa approaches Gflowlim
        const float gap = ((k.g_flowlim - f2.x) + k.g_flowlim_lo) - f2.y;
        float scaler = gap / (k.g_flowlim + k.g_flowlim_lo);
        if (gap < 0.0f) scaler = 0.0f;
        float sthr = sp;
        if (sthr > k.g_slope) sthr = k.g_slope;
        float g = kappa * sthr * scaler;
        if ((e + g) > st) g = st - e;
        if (g < 0.f) g = 0.f;
        ero[i] = e;
        inci[i] = in;
        geli[i] = g;
        se += e;
        si += in;
        sg += g;
    }
    const double te = block_sum_d(se, red);
    const double ti = block_sum_d(si, red);
    const double tg = block_sum_d(sg, red);
    const unsigned long long fm = block_max_u64(famax, redk);
    const bool any_multi = __syncthreads_or(multi) != 0;
    if (threadIdx.x == 0) {
        atomicAdd(&o.tot_e, te);
        atomicAdd(&o.tot_i, ti);
        atomicAdd(&o.tot_g, tg);
        atomicMax(&o.fa_max_key, fm);
        if (any_multi) sc->sed_tiled_ok = 0;
    }
}

// In-degrees and sources of the global sediment wave, for the steps that take
// it (MFD, or a multi-direction code found by k_erosion): cells in row 0 or
// column 0 are never processed (mfd_accum.cu:42) and masked cells never
// complete, so a donor of either kind blocks its receiver for good.
__global__ void k_sed_prep(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd,
                           float* __restrict__ depo, int32_t* __restrict__ pending, int32_t* ready, ModelConsts k,
                           DevScalars* sc, TileSet ts) {
    if (sc->sed_tiled_ok) return;  // the tiled path routes this step
    const int W = k.W, H = k.H;
    const size_t N = (size_t)W * H;
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < ts.span(); base += (size_t)gridDim.x * blockDim.x) {
        int x, y;
        const bool in = ts.cell(base + threadIdx.x, W, H, x, y);
        const size_t i = (size_t)y * W + x;
        bool src = false;
        if (in) {
            int32_t pend = kBlocked;
            if (mask[i]) {
                if (x != 0 && y != 0) {
                    pend = 0;
#pragma unroll
                    for (int d = 0; d < 8; ++d) {
                        const int nx = x + dir_dx(d), ny = y + dir_dy(d);
                        if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
                        const size_t n = (size_t)ny * W + nx;
                        if (!donates(fd[n], d)) continue;
                        if (mask[n] && nx != 0 && ny != 0)
                            ++pend;
                        else
                            pend |= kBlocked;
                    }
                    src = (pend == 0);
                }
            }
            pending[i] = pend;
        }
        wave_append(src, (int32_t)i, ready, &sc->counters[0], (int)N, &sc->err);
    }
}

// The per-cell arithmetic of MFDsedbud (mfd_accum.cu:222-249), rounded the same
// way wherever it is evaluated (no contraction): deposition, the stone mix
// coefficients (stone = A + B * from, clamped, when the sediment column is not
// empty; stone kept otherwise) and the new soil thickness.
struct SedLocal {
    float dep, A, B, stn;
    bool nz;
};
__device__ __forceinline__ SedLocal sed_local(float ad, float ac, float ag, float e, float ic, float g, float st0,
                                              float stone0, float ddk, float dck, float dgk) {
    SedLocal r;
    r.dep = __fadd_rn(__fadd_rn(__fmul_rn(__fadd_rn(ad, e), ddk), __fmul_rn(__fadd_rn(ac, ic), dck)),
                      __fmul_rn(__fadd_rn(ag, g), dgk));
    const float sedthick = __fadd_rn(st0, r.dep);
    r.nz = sedthick != 0.0f;
    const float old = r.nz ? __fdiv_rn(st0, sedthick) : 0.0f;
    r.B = __fsub_rn(1.0f, old);
    r.A = r.nz ? __fmul_rn(old, stone0) : stone0;
    const float toterosion = __fadd_rn(__fadd_rn(e, ic), g);
    float stn = st0;
    if (toterosion >= sedthick) stn = 0.0f;
    if (sedthick > toterosion) stn = __fsub_rn(sedthick, toterosion);
    r.stn = stn;
    return r;
}
__device__ __forceinline__ float sed_mix(float A, float B, float from) {
    float sn = __fadd_rn(A, __fmul_rn(B, from));
    if (sn < 0.01f)
        sn = 0.01f;
    else if (sn > 99.9f)
        sn = 99.9f;
    return sn;
}
__device__ __forceinline__ void sed_store(size_t g, const SedLocal& L, float sn, float* depo, float* stone,
                                          float* fines, float* soilT) {
    depo[g] = L.dep;
    if (L.nz) {
        __stcg(stone + g, sn);
        fines[g] = __fsub_rn(100.0f, sn);
    }
    soilT[g] = L.stn;
}

// One cell of MFDsedbud (mfd_accum.cu:32-254): deposition from the donors'
// erosion, stone mixing with the donors' updated stone, new soil thickness.
struct SedCell {
    const uint8_t* mask;
    const uint8_t* fd;
    const float* prop;
    const float* ero;
    const float* inci;
    const float* geli;
    float* depo;
    float* stone;
    float* fines;
    float* soilT;
    DemCtx dc;
    int W, H;
    float ddk, dck, dgk;
    __device__ __forceinline__ void cell(int32_t cur, int x, int y) const {
        if (dc.of) atomicAdd(&dc.out[dc.of[cur]].sed_done, 1);  // a batch: count per DEM
        const float omd = 1.0f - ddk, omc = 1.0f - dck, omg = 1.0f - dgk;
        float ad = 0.f, ac = 0.f, ag = 0.f, from = 0.f;
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            const int d = scan_dir(kk);
            const int nx = x + dir_dx(d), ny = y + dir_dy(d);
            if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
            const int32_t n = ny * W + nx;
            if (!donates(__ldg(fd + n), d)) continue;
            const float p = prop ? __ldg(prop + 8 * (size_t)n + ((d + 4) & 7)) : 1.0f;
            ad = __fadd_rn(ad, __fmul_rn(p, __fmul_rn(__ldg(ero + n), omd)));
            ac = __fadd_rn(ac, __fmul_rn(p, __fmul_rn(__ldg(inci + n), omc)));
            ag = __fadd_rn(ag, __fmul_rn(p, __fmul_rn(__ldg(geli + n), omg)));
            from = __fadd_rn(from, __fmul_rn(p, __ldcg(stone + n)));
        }
        const SedLocal L = sed_local(ad, ac, ag, __ldg(ero + cur), __ldg(inci + cur), __ldg(geli + cur), soilT[cur],
                                     __ldcg(stone + cur), ddk, dck, dgk);
        sed_store(cur, L, L.nz ? sed_mix(L.A, L.B, from) : 0.0f, depo, stone, fines, soilT);
    }
    __device__ __forceinline__ int receivers(int32_t cur, int x, int y, int32_t* r) const {
        return code_receivers(fd, mask, cur, x, y, W, H, r);
    }
    __device__ __forceinline__ void prefetch(int32_t) const {}
};

// The sediment wave: every source starts it; cells follow as their last donor
// finishes.  With gate set it runs only when the tiled path is off.
__global__ void k_sed_walk(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd,
                           const float* __restrict__ prop, const float* __restrict__ ero,
                           const float* __restrict__ inci, const float* __restrict__ geli, float* depo, float* stone,
                           float* fines, float* soilT, int32_t* pending, int32_t* list_a, int32_t* list_b,
                           ModelConsts k, DevScalars* sc, DemCtx dc, int gate) {
    if (gate && sc->sed_tiled_ok) return;
    const SedCell op{mask, fd, prop, ero, inci, geli, depo, stone, fines, soilT, dc, k.W, k.H, k.ddk, k.dck, k.dgk};
    int done = wave_walk(op, pending, list_a, list_b, k.W, k.H, sc);
    done = wsum(done);
    if (!dc.of && (threadIdx.x & 31) == 0 && done) atomicAdd(&dc.out[0].sed_done, done);
}

// ---------------------------------------------------------------------------
// Tiled sediment routing for single-receiver codes, on the tiles of the tiled
// accumulation.  Deposition and soil thickness are local; only the stone mix
// carries the donors' new values downstream, through a clamp, so the coarse
// level cannot add partial sums.  Instead:
//   local : per tile, cells with no donor outside the tile upstream are
//           settled and stored; the others ("waiting" cells) are written as a
//           program per outlet, in dependency order: A, B, the sum C of the
//           settled donors and references to the waiting donors (earlier
//           slots of the same program, or cells of other tiles);
//   coarse: a wave over the outlets: an outlet whose inflows are all final
//           runs its program and stores its own new values;
//   final : per tile, the remaining waiting cells by the per-cell formula.
// Cell classes follow MFDsedbud: in-catchment cells off row 0 and column 0 are
// computed; every other in-grid donor blocks its receiver.

constexpr int kProgLocal = 256;  // program nodes the coarse evaluator keeps in local memory
constexpr int kFinNz = 1;      // final-pass slot: the cell's sediment column is not empty
constexpr int kFinOutlet = 2;  // final-pass slot: an outlet (the coarse wave stored it; counted only)
constexpr int kPool = kTilePool;
constexpr uint8_t kFDone = 1, kFTaint = 2;

// Maps of a value through a run of single-input cells: v -> clamp(a*v + b, lo, hi)
// as float4(a, b, lo, hi); lo > hi encodes the constant b (a cell whose
// sediment column is empty keeps its stone whatever its donors carry).
__device__ __forceinline__ float4 map_identity() { return make_float4(1.0f, 0.0f, -INFINITY, INFINITY); }
__device__ __forceinline__ float4 map_const(float c) { return make_float4(0.0f, c, INFINITY, -INFINITY); }
__device__ __forceinline__ float map_apply(const float4 m, float v) {
    if (m.z > m.w) return m.y;
    const float y = __fadd_rn(__fmul_rn(m.x, v), m.y);
    return y < m.z ? m.z : (y > m.w ? m.w : y);
}
// a single-input cell: from = C + v, stone = clamp(A + B * from) (or its old stone S)
__device__ __forceinline__ float4 map_cell(float A, float B, float C, bool nz, float S) {
    if (!nz) return map_const(S);
    return make_float4(B, __fadd_rn(A, __fmul_rn(B, C)), 0.01f, 99.9f);
}
// outer after inner
__device__ __forceinline__ float4 map_compose(const float4 outer, const float4 inner) {
    if (outer.z > outer.w) return outer;
    if (inner.z > inner.w) return map_const(map_apply(outer, inner.y));
    const float a1 = outer.x, b1 = outer.y;
    if (a1 == 0.0f) return map_const(map_apply(outer, 0.0f));
    const float L = __fadd_rn(__fmul_rn(a1, a1 > 0.0f ? inner.z : inner.w), b1);
    const float U = __fadd_rn(__fmul_rn(a1, a1 > 0.0f ? inner.w : inner.z), b1);
    const float lo = fmaxf(L, outer.z), hi = fminf(U, outer.w);
    if (lo > hi) return map_const(U < outer.z ? outer.z : outer.w);
    return make_float4(__fmul_rn(a1, inner.x), __fadd_rn(__fmul_rn(a1, inner.y), b1), lo, hi);
}

__device__ __forceinline__ void sed_tile_load(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd, int W,
                                              int H, int tx0, int ty0, uint8_t* s_code, uint8_t* s_cls) {
    for (int j = threadIdx.x; j < kTH * kTH; j += blockDim.x) {
        const int gx = tx0 - 1 + j % kTH, gy = ty0 - 1 + j / kTH;
        uint8_t c = 0, cl = kCellOff;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            const size_t g = (size_t)gy * W + gx;
            c = fd[g];
            cl = (mask[g] && gx != 0 && gy != 0) ? kCellIn : kCellBlock;
        }
        s_code[j] = c;
        s_cls[j] = cl;
    }
}

// Static part of a cell: deposition from all donors (in scan order), the mix
// coefficients and the new soil thickness; pend counts donors inside the tile,
// ext those outside, kBlocked marks a blocked donor.
struct SedInit {
    SedLocal L;
    int32_t pend;
    int ext;
    uint32_t dmask;  // the in-tile donors (sed_init_staged): bit k for direction scan_dir(k)
};
__device__ __forceinline__ SedInit sed_init(const uint8_t* s_code, const uint8_t* s_cls, int lx, int ly, int tx0,
                                            int ty0, int W, const float* __restrict__ ero,
                                            const float* __restrict__ inci, const float* __restrict__ geli,
                                            const float* __restrict__ soilT, const float* stone, const ModelConsts& k) {
    const float omd = 1.0f - k.ddk, omc = 1.0f - k.dck, omg = 1.0f - k.dgk;
    const int hc = (ly + 1) * kTH + lx + 1;
    SedInit r;
    r.pend = 0;
    r.ext = 0;
    r.dmask = 0;  // the wave of k_sedt_final derives its donors itself
    float ad = 0.f, ac = 0.f, ag = 0.f;
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
        const int d = scan_dir(kk);
        const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
        if (!donates(s_code[nh], d)) continue;
        const uint8_t cl = s_cls[nh];
        if (cl == kCellBlock) {
            r.pend |= kBlocked;
            continue;
        }
        if (cl != kCellIn) continue;
        const size_t n = (size_t)(ty0 + ly + dir_dy(d)) * W + tx0 + lx + dir_dx(d);
        ad = __fadd_rn(ad, __fmul_rn(1.0f, __fmul_rn(__ldg(ero + n), omd)));
        ac = __fadd_rn(ac, __fmul_rn(1.0f, __fmul_rn(__ldg(inci + n), omc)));
        ag = __fadd_rn(ag, __fmul_rn(1.0f, __fmul_rn(__ldg(geli + n), omg)));
        if (in_tile(lx + dir_dx(d), ly + dir_dy(d)))
            ++r.pend;
        else
            ++r.ext;
    }
    const size_t g = (size_t)(ty0 + ly) * W + tx0 + lx;
    r.L = sed_local(ad, ac, ag, __ldg(ero + g), __ldg(inci + g), __ldg(geli + g), soilT[g], __ldcg(stone + g), k.ddk,
                    k.dck, k.dgk);
    return r;
}

// sed_init on the tile's erosion terms staged in shared memory (kTH x kTH
// halo layout): the same sums in the same order.
__device__ __forceinline__ SedInit sed_init_staged(const uint8_t* s_code, const uint8_t* s_cls, const float* s_e,
                                                   const float* s_i, const float* s_g, int lx, int ly, float st0,
                                                   float stone0, const ModelConsts& k) {
    const float omd = 1.0f - k.ddk, omc = 1.0f - k.dck, omg = 1.0f - k.dgk;
    const int hc = (ly + 1) * kTH + lx + 1;
    SedInit r;
    r.pend = 0;
    r.ext = 0;
    r.dmask = 0;
    float ad = 0.f, ac = 0.f, ag = 0.f;
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
        const int d = scan_dir(kk);
        const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
        if (!donates(s_code[nh], d)) continue;
        const uint8_t cl = s_cls[nh];
        if (cl == kCellBlock) {
            r.pend |= kBlocked;
            continue;
        }
        if (cl != kCellIn) continue;
        ad = __fadd_rn(ad, __fmul_rn(1.0f, __fmul_rn(s_e[nh], omd)));
        ac = __fadd_rn(ac, __fmul_rn(1.0f, __fmul_rn(s_i[nh], omc)));
        ag = __fadd_rn(ag, __fmul_rn(1.0f, __fmul_rn(s_g[nh], omg)));
        if (in_tile(lx + dir_dx(d), ly + dir_dy(d))) {
            ++r.pend;
            r.dmask |= 1u << kk;
        } else {
            ++r.ext;
        }
    }
    r.L = sed_local(ad, ac, ag, s_e[hc], s_i[hc], s_g[hc], st0, stone0, k.ddk, k.dck, k.dgk);
    return r;
}

__global__ void __launch_bounds__(256, 5)
    k_sedt_local(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd, const float* __restrict__ ero,
                 const float* __restrict__ inci, const float* __restrict__ geli, float* depo, float* stone,
                 float* fines, float* soilT, int32_t* __restrict__ t_dst, int32_t* __restrict__ t_pend,
                 int32_t* __restrict__ t_orng, float2* __restrict__ t_out, float4* __restrict__ p_abc,
                 int32_t* __restrict__ p_ref, float4* __restrict__ p_map, uint8_t* __restrict__ t_stat,
                 int4* __restrict__ f_idx, float4* __restrict__ f_map, float2* __restrict__ f_ds,
                 int32_t* __restrict__ t_fcnt, int32_t* srcs, ModelConsts k, DevScalars* sc, DemCtx dc, TileSet ts) {
    if (!sc->sed_tiled_ok) return;
    __shared__ uint8_t s_code[kTH * kTH];
    __shared__ uint8_t s_cls[kTH * kTH];
    __shared__ int32_t s_pend[kTile * kTile];
    __shared__ float s_new[kTile * kTile];  // settled stone (the old stone until then)
    // A, B, deposition and soil thickness per cell; before them, the halo's
    // erosion terms (3 kTH x kTH floats) for the set-up
    __shared__ float s_coef[4 * kTile * kTile];
    float* const s_A = s_coef;
    float* const s_B = s_coef + kTile * kTile;
    float* const s_dep = s_coef + 2 * kTile * kTile;
    float* const s_stn = s_coef + 3 * kTile * kTile;
    float* const s_ero = s_coef;
    float* const s_inc = s_coef + kTH * kTH;
    float* const s_gel = s_coef + 2 * kTH * kTH;
    __shared__ int16_t s_ptr[kTile * kTile];
    __shared__ int16_t s_topo[kTile * kTile];
    __shared__ int16_t s_pos[kTile * kTile];
    __shared__ int16_t s_oslot[kTile * kTile];
    __shared__ uint8_t s_kind[kTile * kTile];
    __shared__ uint8_t s_ext[kTile * kTile];
    __shared__ uint8_t s_flag[kTile * kTile];
    __shared__ uint8_t s_nz[kTile * kTile];
    __shared__ int16_t s_olist[kTileEnt];
    __shared__ int32_t s_ocnt[kTileEnt];
    __shared__ int32_t s_pcnt[kTileEnt];
    __shared__ int16_t s_pstart[kTileEnt];
    __shared__ int16_t s_pfill[kTileEnt];
    __shared__ int16_t s_q[kTile * kTile];
    __shared__ int16_t s_rnd[kTile * kTile];
    __shared__ int s_no, s_nt, s_done, s_pool, s_dem, s_qn, s_qend, s_fn;
    __shared__ int s_wcnt[9];  // per-warp counts of the outlet list and the source append
    const int W = k.W, H = k.H, TW = (W + kTile - 1) / kTile;
    const int t = ts.tile(blockIdx.x);
    const int tx0 = (t % TW) * kTile, ty0 = (t / TW) * kTile;
    sed_tile_load(mask, fd, W, H, tx0, ty0, s_code, s_cls);
    for (int j = threadIdx.x; j < kTH * kTH; j += blockDim.x) {
        const int gx = tx0 - 1 + j % kTH, gy = ty0 - 1 + j / kTH;
        float e = 0.f, i = 0.f, g = 0.f;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            const size_t c = (size_t)gy * W + gx;
            e = __ldg(ero + c);
            i = __ldg(inci + c);
            g = __ldg(geli + c);
        }
        s_ero[j] = e;
        s_inc[j] = i;
        s_gel[j] = g;
    }
    if (threadIdx.x < kTileEnt) {
        s_ocnt[threadIdx.x] = 0;
        s_pcnt[threadIdx.x] = 0;
    }
    if (threadIdx.x == 0) s_nt = s_done = s_fn = 0, s_dem = -1;
    __syncthreads();
    const int lx = threadIdx.x & 31, ly0 = threadIdx.x >> 5;
    bool src[4];
    float cA[4], cB[4], cD[4], cS[4];  // the cells' coefficients until the staged terms are spent
    int dem = -1;  // one DEM per tile
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx, hc = (ly + 1) * kTH + lx + 1;
        int32_t pend = kBlocked;
        uint8_t kind = kKindEnd, ext = 0, nz = 0;
        int16_t ptr = (int16_t)l, dm = 0;
        float snew = 0.f;
        cA[q] = cB[q] = cD[q] = cS[q] = 0.f;
        if (s_cls[hc] == kCellIn) {
            const size_t g = (size_t)(ty0 + ly) * W + tx0 + lx;
            snew = __ldcg(stone + g);
            const SedInit in = sed_init_staged(s_code, s_cls, s_ero, s_inc, s_gel, lx, ly, soilT[g], snew, k);
            pend = in.pend;
            ext = (uint8_t)in.ext;
            dm = (int16_t)in.dmask;
            cA[q] = in.L.A;
            cB[q] = in.L.B;
            cD[q] = in.L.dep;
            cS[q] = in.L.stn;
            nz = in.L.nz;
            if (dem < 0) dem = dem_at(dc, (size_t)(ty0 + ly) * W + tx0 + lx);
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
        }
        s_pend[l] = pend;
        src[q] = pend == 0;
        s_kind[l] = kind;
        s_ext[l] = ext;
        s_ptr[l] = ptr;
        s_new[l] = snew;
        s_nz[l] = nz;
        s_flag[l] = 0;
        s_pos[l] = -1;
        s_oslot[l] = dm;  // the outlet slots are listed after the wave
    }
    dem = __reduce_max_sync(0xffffffffu, dem);
    if ((threadIdx.x & 31) == 0 && dem >= 0) atomicMax(&s_dem, dem);
    __syncthreads();  // the staged erosion terms are spent
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int l = (ly0 + 8 * q) * kTile + lx;
        s_A[l] = cA[q];
        s_B[l] = cB[q];
        s_dep[l] = cD[q];
        s_stn[l] = cS[q];
    }
    __syncthreads();
    // The waiting cells: every cell downstream of an entry (a cell with a donor
    // in another tile), marked along each entry's in-tile path before the wave.
    // A walk stops where another walk has passed (it carries on from there).
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        int c = (ly0 + 8 * q) * kTile + lx;
        if (!s_ext[c]) continue;
        for (int guard = 0; guard < kTile * kTile; ++guard) {
            if (s_flag[c] & kFTaint) break;
            s_flag[c] = kFTaint;
            if (s_kind[c] != kKindIn) break;
            c = s_ptr[c];
        }
    }
    // settle what depends on this tile only; order the waiting cells
    int done = 0;
    if (threadIdx.x == 0) s_qn = 0;
    __syncthreads();
    tile_wave(
        [&](int cur, int rnd) {
            const bool taint = (s_flag[cur] & kFTaint) != 0;
            if (!taint) {
                // every donor is inside the tile and settled; all of them are
                // loaded before the sum in scan order
                const uint32_t dm = (uint16_t)s_oslot[cur];
                float v[8];
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) v[kk] = (dm >> kk) & 1u ? s_new[cur + tile_step(scan_dir(kk))] : 0.f;
                float from = 0.f;
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                    if ((dm >> kk) & 1u) from = __fadd_rn(from, __fmul_rn(1.0f, v[kk]));
                // the cell's outputs are stored after the wave, coalesced
                if (s_nz[cur]) s_new[cur] = sed_mix(s_A[cur], s_B[cur], from);
                s_flag[cur] = kFDone;
                ++done;
            } else {
                s_flag[cur] = kFDone | kFTaint;
                s_rnd[cur] = (int16_t)rnd;  // a level for the coarse evaluation: inputs come from earlier rounds
                s_topo[atomicAdd(&s_nt, 1)] = (int16_t)cur;
            }
            return s_kind[cur] == kKindIn ? (int)s_ptr[cur] : -1;
        },
        s_pend, s_q, &s_qn, &s_qend, src, lx, ly0);
    // the settled cells' outputs (sed_store), one coalesced pass
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx;
        if (s_flag[l] != kFDone) continue;
        const size_t g = (size_t)(ty0 + ly) * W + tx0 + lx;
        depo[g] = s_dep[l];
        if (s_nz[l]) {
            const float sn = s_new[l];
            __stcg(stone + g, sn);
            fines[g] = __fsub_rn(100.0f, sn);
        }
        soilT[g] = s_stn[l];
    }
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
    bool stray = false;  // a waiting cell whose in-tile path ends inside the tile (at the DEM's outlet, say)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx;
        const size_t g = (size_t)(ty0 + ly) * W + tx0 + lx;
        if (s_ext[l]) {
            const int e = s_ptr[l];
            t_dst[g] = s_kind[e] == kKindOutlet ? (int32_t)((ty0 + e / kTile) * W + tx0 + (e & (kTile - 1))) : -1;
        }
        stray |= s_flag[l] == (kFDone | kFTaint) && s_kind[s_ptr[l]] != kKindOutlet;
        if (tx0 + lx < W && ty0 + ly < H) t_stat[g] = (s_flag[l] & kFDone) ? ((s_flag[l] & kFTaint) ? 2 : 1) : 0;
    }
    // Such a tile keeps the second wave for its waiting cells; in every other
    // tile each waiting cell's stone is a map of one program node's value,
    // stored by the final pass.
    const bool second_wave = __syncthreads_or(stray);
    list_outlets(s_kind, s_olist, s_oslot, &s_no, s_wcnt);
    __syncthreads();
    // inflows per outlet (ring cells flowing into the tile)
    if (threadIdx.x < kRing) {
        const int h = ring_halo(threadIdx.x);
        const int d = s_cls[h] == kCellIn ? bit_dir(s_code[h]) : -1;
        if (d >= 0) {
            const int hx = h % kTH + dir_dx(d), hy = h / kTH + dir_dy(d);
            if (hx >= 1 && hx <= kTile && hy >= 1 && hy <= kTile && s_cls[hy * kTH + hx] == kCellIn) {
                const int o = s_ptr[(hy - 1) * kTile + hx - 1];
                if (s_kind[o] == kKindOutlet) atomicAdd(&s_ocnt[s_oslot[o]], 1);
            }
        }
    }
    // program nodes: waiting cells draining to an outlet that take an inflow
    // from another tile, join two waiting branches, or are the outlet.  The
    // waiting cells between nodes pass one value on; they become the maps of
    // the nodes' inputs.
    int32_t* s_node = s_pend;  // the in-degrees are spent
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx, hc = (ly + 1) * kTH + lx + 1;
        bool node = false;
        if (s_flag[l] == (kFDone | kFTaint) && s_kind[s_ptr[l]] == kKindOutlet) {
            int ntd = 0;
#pragma unroll
            for (int d = 0; d < 8; ++d) {
                const int nlx = lx + dir_dx(d), nly = ly + dir_dy(d);
                const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
                if (in_tile(nlx, nly) && donates(s_code[nh], d) && s_cls[nh] == kCellIn &&
                    (s_flag[nly * kTile + nlx] & kFTaint))
                    ++ntd;
            }
            node = s_ext[l] != 0 || ntd >= 2 || s_kind[l] == kKindOutlet;
        }
        s_node[l] = node;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int l = (ly0 + 8 * q) * kTile + lx;
        if (s_node[l]) atomicAdd(&s_pcnt[s_oslot[s_ptr[l]]], 1);
    }
    // Every waiting cell between nodes: its map v -> stone from its one waiting
    // in-tile donor (in place of its own coefficients, which only nodes need
    // from here on).  Every waiting cell of a tile without a second wave also
    // takes a final-pass slot, with its deposition and soil thickness.
    int16_t* s_up = s_q;  // the node at the top of a cell's run (s_q is spent since the wave)
    const size_t fbase = (size_t)t * kTile * kTile;
    int fslot[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx, hc = (ly + 1) * kTH + lx + 1;
        const bool waits = s_flag[l] == (kFDone | kFTaint) && s_kind[s_ptr[l]] == kKindOutlet;
        fslot[q] = warp_slot(waits && !second_wave, &s_fn);
        if (!waits) continue;
        if (fslot[q] >= 0) f_ds[fbase + fslot[q]] = make_float2(s_dep[l], s_stn[l]);
        if (s_node[l]) continue;
        float Cc = 0.f;
#pragma unroll
        for (int k2 = 0; k2 < 8; ++k2) {
            const int d2 = scan_dir(k2);
            const int ulx = lx + dir_dx(d2), uly = ly + dir_dy(d2);
            const int uh = hc + dir_dy(d2) * kTH + dir_dx(d2);
            if (!in_tile(ulx, uly) || !donates(s_code[uh], d2) || s_cls[uh] != kCellIn) continue;
            const int u = uly * kTile + ulx;
            if (!(s_flag[u] & kFTaint)) Cc = __fadd_rn(Cc, __fmul_rn(1.0f, s_new[u]));
        }
        const float4 M = map_cell(s_A[l], s_B[l], Cc, s_nz[l] != 0, s_new[l]);
        s_A[l] = M.x;
        s_B[l] = M.y;
        s_dep[l] = M.z;
        s_stn[l] = M.w;
    }
    __syncthreads();
    // The maps of the cells between nodes, composed down each run from the node
    // at its top: afterwards s_up of such a cell is that node and its map takes
    // the node's value to its own stone.  One walk per node; no two walks
    // share a cell (a cell between nodes has one waiting donor).
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        const int l = (ly0 + 8 * q) * kTile + lx;
        if (!s_node[l] || s_kind[l] != kKindIn) continue;
        float4 F = map_identity();
        int c = l;
        for (int guard = 0; guard < kTile * kTile; ++guard) {
            const int d = bit_dir(s_code[(c / kTile + 1) * kTH + (c & (kTile - 1)) + 1]);
            c += dir_dy(d) * kTile + dir_dx(d);  // in the tile: c is not an outlet
            if (s_flag[c] != (kFDone | kFTaint) || s_node[c]) break;
            F = map_compose(make_float4(s_A[c], s_B[c], s_dep[c], s_stn[c]), F);
            s_A[c] = F.x;
            s_B[c] = F.y;
            s_dep[c] = F.z;
            s_stn[c] = F.w;
            s_up[c] = (int16_t)l;
            if (s_kind[c] != kKindIn) break;
        }
    }
    __syncthreads();
    const int no = s_no, nt = s_nt;
    if (threadIdx.x == 0) {
        int a = 0;
        for (int i = 0; i < no; ++i) {
            s_pstart[i] = (int16_t)a;
            s_pfill[i] = (int16_t)a;
            a += s_pcnt[i];
        }
        s_pool = 0;
    }
    __syncthreads();
    // node slots: grouped by outlet, in the order the cells were reached
    if (threadIdx.x < 32) {
        const unsigned below = (1u << lx) - 1u;
        for (int base = 0; base < nt; base += 32) {
            const int i = base + lx;
            int key = -1, c = 0;
            if (i < nt) {
                c = s_topo[i];
                if (s_node[c]) key = s_oslot[s_ptr[c]];
            }
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            const int fill = key >= 0 ? s_pfill[key] : 0;
            __syncwarp();
            if (key >= 0) {
                s_pos[c] = (int16_t)(fill + __popc(peers & below));
                if ((peers & below) == 0) s_pfill[key] = (int16_t)(fill + __popc(peers));
            }
            __syncwarp();
        }
    }
    __syncthreads();
    const size_t nbase = (size_t)t * kTile * kTile;
    const size_t pool = (size_t)t * kPool;
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx, hc = (ly + 1) * kTH + lx + 1;
        if (!s_node[l]) continue;
        const int pos = s_pos[l];
        const int first = s_pstart[s_oslot[s_ptr[l]]];
        int nin = 0;
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            const int nlx = lx + dir_dx(d), nly = ly + dir_dy(d);
            const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
            if (!donates(s_code[nh], d) || s_cls[nh] != kCellIn) continue;
            if (!in_tile(nlx, nly) || (s_flag[nly * kTile + nlx] & kFTaint)) ++nin;
        }
        const int start = atomicAdd(&s_pool, nin);
        if (start + nin > kPool) {
            raise_error(&sc->err, ErrFlags::kCapacity);
            continue;
        }
        float C = 0.f;
        int m = 0;
#pragma unroll 1
        for (int kk = 0; kk < 8; ++kk) {
            const int d = scan_dir(kk);
            const int nlx = lx + dir_dx(d), nly = ly + dir_dy(d);
            const int nh = hc + dir_dy(d) * kTH + dir_dx(d);
            if (!donates(s_code[nh], d) || s_cls[nh] != kCellIn) continue;
            if (!in_tile(nlx, nly)) {
                p_ref[pool + start + m] = (ty0 + nly) * W + tx0 + nlx;
                p_map[pool + start + m] = map_identity();
                ++m;
                continue;
            }
            int cur = nly * kTile + nlx;
            if (!(s_flag[cur] & kFTaint)) {
                C = __fadd_rn(C, __fmul_rn(1.0f, s_new[cur]));
                continue;
            }
            // the node that feeds this input, through the single-input cells in between
            float4 H = map_identity();
            if (!s_node[cur]) {
                H = make_float4(s_A[cur], s_B[cur], s_dep[cur], s_stn[cur]);
                cur = s_up[cur];
            }
            p_ref[pool + start + m] = -(s_pos[cur] - first + 1);
            p_map[pool + start + m] = H;
            ++m;
        }
        p_abc[nbase + pos] =
            make_float4(s_A[l], s_B[l], C, __int_as_float(start | (m << 11) | (s_nz[l] << 15) | ((int)s_rnd[l] << 16)));
    }
    // the final pass's slots: a node reads its own value, a cell between nodes
    // maps the value of the node at the top of its chain
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (fslot[q] < 0) continue;
        const int ly = ly0 + 8 * q, l = ly * kTile + lx;
        const bool node = s_node[l] != 0;
        const int src_node = node ? l : s_up[l];
        const int e = s_ptr[l];
        // (a chain always ends at a node; -1 only guards the final pass's read)
        const int vref = s_node[src_node] && s_pos[src_node] >= 0 ? (int)(fbase + s_pos[src_node]) : -1;
        f_idx[fbase + fslot[q]] = make_int4((ty0 + ly) * W + tx0 + lx, vref,
                                            (ty0 + e / kTile) * W + tx0 + (e & (kTile - 1)),
                                            (s_nz[l] ? kFinNz : 0) | (s_kind[l] == kKindOutlet ? kFinOutlet : 0));
        f_map[fbase + fslot[q]] = node ? map_identity() : make_float4(s_A[l], s_B[l], s_dep[l], s_stn[l]);
    }
    if (threadIdx.x == 0) t_fcnt[t] = second_wave ? -1 : s_fn;
    const int j = threadIdx.x;
    bool ready = false;
    int32_t og = 0;
    if (j < no) {
        const int o = s_olist[j];
        const int32_t opend = ((s_flag[o] & kFDone) ? 0 : kBlocked) + s_ocnt[j];
        og = (ty0 + o / kTile) * W + tx0 + (o & (kTile - 1));
        t_orng[og] = ((int)s_pstart[j] << 16) | s_pcnt[j];
        t_pend[og] = opend;
        t_out[og] = make_float2(s_dep[o], s_stn[o]);
        ready = (opend == 0);
    }
    block_append(ready, og, srcs, &sc->tile_src, W * H, &sc->err, s_wcnt);
    done = wsum(done);
    if ((threadIdx.x & 31) == 0 && done) atomicAdd(&s_done, done);
    __syncthreads();
    if (threadIdx.x == 0 && s_done && s_dem >= 0) atomicAdd(&dc.out[s_dem].sed_done, s_done);
}

// One outlet of the coarse sediment wave, a warp per outlet: its program
// level by level (nodes of one tile-wave round depend only on earlier rounds,
// and the program lists them by round), then its own stores by lane 0.
// Gathered program of one outlet, per warp: the nodes' coefficients, the
// first slot of each node's inputs, and per input either its mapped value
// (an input from another tile, final when the outlet is ready) or its map and
// the feeding node.  Programs larger than this take the inputs from memory.
constexpr int kGatherNodes = 64;
constexpr int kGatherInputs = 96;

struct SedCoarse {
    const uint8_t* fd;
    const int32_t* t_orng;
    const int32_t* t_dst;
    const float2* t_out;
    const float4* p_abc;
    const int32_t* p_ref;
    const float4* p_map;
    float* p_val;
    float* depo;
    float* stone;
    float* fines;
    float* soilT;
    float* s_vals;    // kProgLocal values per warp of the block
    float4* s_abc;    // kGatherNodes per warp
    int16_t* s_ib;    // kGatherNodes per warp: first input slot of the node
    float4* s_imap;   // kGatherInputs per warp: mapped value (.x) or map
    int32_t* s_iref;  // kGatherInputs per warp: 0 (mapped value) or the feeding node (negative)
    int W, TW;
    __device__ __forceinline__ void cell_warp(int32_t o, int x, int y, int lane) const {
        const int rng = __ldg(t_orng + o);
        const int cnt = rng & 0xffff;
        if (cnt == 0) return;  // settled inside its tile
        const int t = (y / kTile) * TW + x / kTile;
        const size_t nbase = (size_t)t * kTile * kTile + (rng >> 16);
        const size_t pool = (size_t)t * kPool;
        const int wq = threadIdx.x >> 5;
        float* vals = s_vals + wq * kProgLocal;
        float4* abc = s_abc + wq * kGatherNodes;
        int16_t* ib = s_ib + wq * kGatherNodes;
        float4* imap = s_imap + wq * kGatherInputs;
        int32_t* iref = s_iref + wq * kGatherInputs;
        // Gather: every node's coefficients and inputs in one batch of loads,
        // instead of a chain of loads per level of the program.
        bool gathered = cnt <= kGatherNodes;
        for (int c0 = 0, in0 = 0; gathered && c0 < cnt; c0 += 32) {
            const int j = c0 + lane;
            int nin = 0, start = 0;
            float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
            if (j < cnt) {
                r = __ldg(p_abc + nbase + j);
                const int meta = __float_as_int(r.w);
                start = meta & 2047;
                nin = (meta >> 11) & 15;
            }
            int incl = nin;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += v;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            if (in0 + total > kGatherInputs) {
                gathered = false;  // warp-uniform
                break;
            }
            const int b0 = in0 + incl - nin;
            if (j < cnt) {
                abc[j] = r;
                ib[j] = (int16_t)b0;
            }
            for (int jr = 0; jr < nin; ++jr) {
                const int32_t ref = __ldg(p_ref + pool + start + jr);
                const float4 mp = __ldg(p_map + pool + start + jr);
                if (ref >= 0) {
                    imap[b0 + jr] = make_float4(map_apply(mp, __ldcg(stone + ref)), 0.f, 0.f, 0.f);
                    iref[b0 + jr] = 0;
                } else {
                    imap[b0 + jr] = mp;
                    iref[b0 + jr] = ref;
                }
            }
            in0 += total;
        }
        __syncwarp();
        for (int i = 0; i < cnt;) {
            const int j = i + lane;
            float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
            int meta = -1;
            if (j < cnt) {
                r = gathered ? abc[j] : __ldg(p_abc + nbase + j);
                meta = __float_as_int(r.w);
            }
            const int lvl0 = __shfl_sync(0xffffffffu, meta >> 16, 0);
            // the run: the nodes from i on that share i's level (independent of one another)
            const unsigned same = __ballot_sync(0xffffffffu, j < cnt && (meta >> 16) == lvl0);
            const int run = same == 0xffffffffu ? 32 : __ffs(~same) - 1;
            const bool act = lane < run;
            if (act) {
                const int start = meta & 2047, nin = (meta >> 11) & 15;
                const bool nz = (meta >> 15) & 1;
                float from = r.z;
                if (gathered) {
                    const int b0 = ib[j];
                    for (int jr = 0; jr < nin; ++jr) {
                        const int32_t ref = iref[b0 + jr];
                        const float4 mp = imap[b0 + jr];
                        const float v = ref == 0 ? mp.x : map_apply(mp, vals[-ref - 1]);
                        from = __fadd_rn(from, __fmul_rn(1.0f, v));
                    }
                } else {
                    for (int jr = 0; jr < nin; ++jr) {
                        const int32_t ref = __ldg(p_ref + pool + start + jr);
                        const float4 mp = __ldg(p_map + pool + start + jr);
                        float v;
                        if (ref >= 0)
                            v = __ldcg(stone + ref);
                        else if (-ref - 1 < kProgLocal)
                            v = vals[-ref - 1];
                        else
                            v = __ldcg(p_val + nbase - ref - 1);
                        from = __fadd_rn(from, __fmul_rn(1.0f, map_apply(mp, v)));
                    }
                }
                const float sn = nz ? sed_mix(r.x, r.y, from) : r.x;
                if (j < kProgLocal) vals[j] = sn;
                __stcg(p_val + nbase + j, sn);  // the final pass maps every node's value onto its chain
            }
            __syncwarp();
            i += run;
        }
        if (lane == 0) {
            // the outlet is the last node of its program
            const int j = cnt - 1;
            const float sn = j < kProgLocal ? vals[j] : __ldcg(p_val + nbase + j);
            const int meta = __float_as_int(__ldg(p_abc + nbase + j).w);
            const float2 out = __ldg(t_out + o);
            depo[o] = out.x;
            if ((meta >> 15) & 1) {
                __stcg(stone + o, sn);
                fines[o] = __fsub_rn(100.0f, sn);
            }
            soilT[o] = out.y;
        }
        __syncwarp();  // the gather buffers are reused by the warp's next node
    }
    __device__ __forceinline__ int receivers(int32_t o, int x, int y, int32_t* r) const {
        const int d = bit_dir(__ldg(fd + o));
        const int32_t rc = (y + dir_dy(d)) * W + x + dir_dx(d);
        const int32_t dst = __ldg(t_dst + rc);
        r[0] = dst;
        return dst >= 0 ? 1 : 0;
    }
    // the receiving outlet's record, read first when this warp carries on with it
    __device__ __forceinline__ void prefetch(int32_t o) const {
        if (o >= 0) prefetch_l2(t_orng + o);
    }
};

__global__ void __launch_bounds__(256)
    k_sedt_coarse(const uint8_t* __restrict__ fd, const int32_t* __restrict__ t_orng,
                  const int32_t* __restrict__ t_dst, const float2* __restrict__ t_out,
                  const float4* __restrict__ p_abc, const int32_t* __restrict__ p_ref,
                  const float4* __restrict__ p_map, float* p_val, float* depo, float* stone, float* fines,
                  float* soilT, int32_t* t_pend, int32_t* list_a, int32_t* list_b, ModelConsts k, DevScalars* sc) {
    if (!sc->sed_tiled_ok) return;
    __shared__ float s_vals[8 * kProgLocal];
    __shared__ float4 s_abc[8 * kGatherNodes];
    __shared__ int16_t s_ib[8 * kGatherNodes];
    __shared__ float4 s_imap[8 * kGatherInputs];
    __shared__ int32_t s_iref[8 * kGatherInputs];
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->counters[0] = sc->tile_src;
    const SedCoarse op{fd,    t_orng, t_dst, t_out,  p_abc, p_ref,  p_map,  p_val,  depo,          stone,
                       fines, soilT,  s_vals, s_abc, s_ib,  s_imap, s_iref, k.W,    (k.W + kTile - 1) / kTile};
    wave_walk_warp(op, t_pend, list_a, list_b, k.W, k.H, sc);
}

constexpr uint8_t kStatNz = 4;  // k_sedt_final: flag in a waiting cell's status

__global__ void __launch_bounds__(256, 6)
    k_sedt_final(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd, const float* __restrict__ ero,
                 const float* __restrict__ inci, const float* __restrict__ geli, float* depo, float* stone,
                 float* fines, float* soilT, const int32_t* __restrict__ t_pend, const uint8_t* __restrict__ t_stat,
                 const int4* __restrict__ f_idx, const float4* __restrict__ f_map, const float2* __restrict__ f_ds,
                 const int32_t* __restrict__ t_fcnt, const float* __restrict__ p_val, ModelConsts k, DevScalars* sc,
                 DemCtx dc, TileSet ts) {
    if (!sc->sed_tiled_ok) return;
    const int t = ts.tile(blockIdx.x);
    const int nf = t_fcnt[t];
    const size_t fbase = (size_t)t * kTile * kTile;
    bool stalled = false;  // an outlet whose program never ran (a donor upstream never completes)
    // a thread's slots (a tile has at most kTile * kTile), kept for both passes
    int4 ev[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = (int)threadIdx.x + 256 * q;
        ev[q] = make_int4(0, 0, 0, kFinOutlet);
        if (nf >= 0 && i < nf) {
            ev[q] = f_idx[fbase + i];
            stalled |= t_pend[ev[q].z] != 0 || ev[q].y < 0;
        }
    }
    if (nf >= 0 && !__syncthreads_or(stalled)) {
        // every waiting cell is a program node or lies on a chain below one:
        // its stone is the map of that node's value
        int done = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = (int)threadIdx.x + 256 * q;
            if (i >= nf) continue;
            const int4 e = ev[q];
            ++done;
            if (e.w & kFinOutlet) continue;
            const float2 ds = f_ds[fbase + i];
            const bool nz = (e.w & kFinNz) != 0;
            const float4 mp = nz ? f_map[fbase + i] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float pv = nz ? __ldcg(p_val + e.y) : 0.f;
            depo[e.x] = ds.x;
            soilT[e.x] = ds.y;
            if (nz) {
                const float sn = map_apply(mp, pv);
                __stcg(stone + e.x, sn);
                fines[e.x] = __fsub_rn(100.0f, sn);
            }
        }
        if (nf > 0) {
            done = wsum(done);
            const int dem = dem_at(dc, (size_t)f_idx[fbase].x);
            if ((threadIdx.x & 31) == 0 && done && dem >= 0) atomicAdd(&dc.out[dem].sed_done, done);
        }
        return;
    }
    __shared__ uint8_t s_code[kTH * kTH];
    __shared__ uint8_t s_cls[kTH * kTH];
    __shared__ uint8_t s_hok[kTH * kTH];
    __shared__ float s_hval[kTH * kTH];
    __shared__ int32_t s_pend[kTile * kTile];
    __shared__ float s_new[kTile * kTile];
    __shared__ uint8_t s_stat[kTile * kTile];  // 1 settled, 2 waiting; kStatNz: the sediment column is not empty
    __shared__ float s_A[kTile * kTile];       // a waiting cell's deposition and stone-mix coefficients,
    __shared__ float s_B[kTile * kTile];       //   computed before the wave so that its rounds read no
    __shared__ float s_dep[kTile * kTile];     //   global memory
    __shared__ float s_stn[kTile * kTile];
    __shared__ int16_t s_q[kTile * kTile];
    __shared__ int s_done, s_dem, s_qn, s_qend;
    const int W = k.W, H = k.H, TW = (W + kTile - 1) / kTile;
    const int tx0 = (t % TW) * kTile, ty0 = (t / TW) * kTile;
    sed_tile_load(mask, fd, W, H, tx0, ty0, s_code, s_cls);
    if (threadIdx.x < kRing) {
        const int h = ring_halo(threadIdx.x);
        const int gx = tx0 - 1 + h % kTH, gy = ty0 - 1 + h / kTH;
        uint8_t ok = 0;
        float v = 0.f;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            const size_t g = (size_t)gy * W + gx;
            ok = t_pend[g] == 0;
            v = __ldcg(stone + g);
        }
        s_hok[h] = ok;
        s_hval[h] = v;
    }
    if (threadIdx.x == 0) s_done = 0, s_dem = -1;
    __syncthreads();
    const int lx = threadIdx.x & 31, ly0 = threadIdx.x >> 5;
    int done = 0, dem = -1;  // one DEM per tile
    bool src[4], outlet[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ly = ly0 + 8 * q, l = ly * kTile + lx, hc = (ly + 1) * kTH + lx + 1;
        int32_t pend = kBlocked;
        uint8_t st = 0;
        float v = 0.f;
        outlet[q] = false;
        if (s_cls[hc] == kCellIn) {
            const size_t g = (size_t)(ty0 + ly) * W + tx0 + lx;
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
                if (t_stat[g] == 2 && t_pend[g] == 0) ++done;
            }
            st = t_stat[g];
            v = __ldcg(stone + g);
            if (dem < 0) dem = dem_at(dc, g);
            if (st == 2 && !outlet[q]) {
                const SedInit in = sed_init(s_code, s_cls, lx, ly, tx0, ty0, W, ero, inci, geli, soilT, stone, k);
                s_A[l] = in.L.A;
                s_B[l] = in.L.B;
                s_dep[l] = in.L.dep;
                s_stn[l] = in.L.stn;
                if (in.L.nz) st |= kStatNz;
            }
        }
        s_pend[l] = pend;
        s_stat[l] = st;
        s_new[l] = v;
        src[q] = pend == 0;
    }
    dem = __reduce_max_sync(0xffffffffu, dem);
    if ((threadIdx.x & 31) == 0 && dem >= 0) atomicMax(&s_dem, dem);
    if (threadIdx.x == 0) s_qn = 0;
    __syncthreads();
    tile_wave(
        [&](int cur, int rnd) {
            const int cx = cur & (kTile - 1), cy = cur / kTile, hc = (cy + 1) * kTH + cx + 1;
            const int d = bit_dir(s_code[hc]);
            const int rlx = cx + (d >= 0 ? dir_dx(d) : 0), rly = cy + (d >= 0 ? dir_dy(d) : 0);
            const bool rin = d >= 0 && s_cls[hc + dir_dy(d) * kTH + dir_dx(d)] == kCellIn;
            if (rin && !in_tile(rlx, rly)) return -1;  // an outlet: the coarse wave stored it
            const uint8_t stc = s_stat[cur];
            if ((stc & 3) == 2) {
                float from = 0.f;
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) {
                    const int dd = scan_dir(kk);
                    const int nlx = cx + dir_dx(dd), nly = cy + dir_dy(dd);
                    const int nh = hc + dir_dy(dd) * kTH + dir_dx(dd);
                    if (!donates(s_code[nh], dd) || s_cls[nh] != kCellIn) continue;
                    from = __fadd_rn(from, __fmul_rn(1.0f, in_tile(nlx, nly) ? s_new[nly * kTile + nlx] : s_hval[nh]));
                }
                SedLocal L;
                L.A = s_A[cur];
                L.B = s_B[cur];
                L.dep = s_dep[cur];
                L.stn = s_stn[cur];
                L.nz = (stc & kStatNz) != 0;
                const float sn = L.nz ? sed_mix(L.A, L.B, from) : s_new[cur];
                s_new[cur] = sn;
                sed_store((size_t)(ty0 + cy) * W + tx0 + cx, L, sn, depo, stone, fines, soilT);
                ++done;
            }
            return rin ? rly * kTile + rlx : -1;
        },
        s_pend, s_q, &s_qn, &s_qend, src, lx, ly0);
    done = wsum(done);
    if ((threadIdx.x & 31) == 0 && done) atomicAdd(&s_done, done);
    __syncthreads();
    if (threadIdx.x == 0 && s_done && s_dem >= 0) atomicAdd(&dc.out[s_dem].sed_done, s_done);
}

__device__ __forceinline__ float dreybrodt(const float* tab, float T) {
    float u = (T - kTabT0) / kTabStep;
    u = fminf(fmaxf(u, 0.0f), (float)(kTabN - 2));
    const int j = (int)u;
    const float f = u - (float)j;
    return tab[j] + f * (tab[j + 1] - tab[j]);
}

// six blocks per SM: a few spilled registers, measured faster than four
__global__ void __launch_bounds__(256, 6)
    k_final(double* __restrict__ z, const double* __restrict__ z_init, const uint8_t* __restrict__ mask,
            const float2* __restrict__ fa, const float* __restrict__ ero, const float* __restrict__ inci,
            const float* __restrict__ geli, const float* __restrict__ depo, float* __restrict__ soilT,
            float* __restrict__ stone, float* __restrict__ fines, float* __restrict__ soilM,
            float* __restrict__ soilB, float* __restrict__ nut, float* __restrict__ totB, float* __restrict__ dz_out,
            float* __restrict__ wc_out, float* __restrict__ wp_out, const float* __restrict__ tab,
            const int32_t* __restrict__ chunk_start, ModelConsts k, DemCtx dc) {
    __shared__ double red[8];
    const int W = k.W;
    const Chunk ch = chunk_of(chunk_start, dc.n, dc.in);
    const DemIn& c = dc.in[ch.d];
    DemOut& o = dc.out[ch.d];
    const int outlet = o.outlet;
    const int outlet_clim = o.outlet_clim;  // the cell whose climate elevation is outlet_z_clim
    const double outlet_z = o.outlet_z_clim;
    const double base = o.base_level;
    const float rain0 = (float)c.rain, rinc = (float)c.rain_inc;
    const float dtemp_scalar = (float)(c.temp - c.temp0);
    float swc = 0.f, swp = 0.f, sbio = 0.f, sd = 0.f;
    for (int64_t ri = ch.first + threadIdx.x; ri < ch.end; ri += blockDim.x) {
        int x, y;
        const size_t i = region_cell(c, ri, W, &x, &y);
        // every input of the cell in one batch of loads, ahead of the mask test
        // and the arithmetic (the region's cells outside the catchment are few)
        const uint8_t mk = mask[i];
        const float dp = depo[i];
        const float e = ero[i], ic = inci[i], gl = geli[i];
        const double zold = z[i], z0 = z_init[i];
        const float2 f2 = fa[i];
        const float st0 = soilT[i], sn0 = stone[i], sm0 = soilM[i], tb = totB[i], sb0 = soilB[i];
        sd += dp;
        if (!mk) {
            totB[i] = 0.0f;  // grow_vegetation (updates.cu:102-105)
            if (dz_out) {
                dz_out[i] = 0.f;
                wc_out[i] = 0.f;
                wp_out[i] = 0.f;
            }
            continue;
        }
        const float dz = dp - e - ic - gl;  // surface_change (eroincidep.cu:404)
        const double zc = c.from_current_dem ? (((int)i == outlet_clim) ? outlet_z : zold) : z0;
        float zch, zcl;
        dsplit(zc, zch, zcl);
        const float T = (float)c.temp - ((zch - (float)kMinHeight) + zcl) * 0.0065f;
        const float rain = rain0 + (float)(y - c.y0) * rinc;
        const float fav = f2.x + f2.y;
        // weathering type 1 (eroincidep.cu:220-327)
        const float PE = 1.44f * (T + 6.0f) * (T + 6.0f);
        const float surface_flow = fav * 1000.0f;
        const float evap_trans = (rain + surface_flow <= PE) ? rain + surface_flow : rain + surface_flow - PE;
        float st = st0;
        const float lpco2 = (st > 0.1f ? -2.5f : -3.5f) + ((T - 15.0f) / 10.0f);
        const float Ca2eq = exp10f((lpco2 + dreybrodt(tab, T)) * (1.0f / 3.0f));
        float wC = 0.0148148148f * Ca2eq * (surface_flow / k.rescale_weather);
        if (wC <= 0.0f) wC = 0.0f;
        if (wC > 0.001f) wC = 0.001f;
        const float wP = 7.7e-5f * expf(-2.3f * st);
        st = st + wC * 0.02f + wP;
        float sn = sn0, sm = sm0;
        if (st <= 0.0f) {
            st = 0.0f;
            sn = 0.0f;
            fines[i] = 0.0f;
            sm = 0.02f;
        } else {
            if (wP > 0.f)
                sn += sn * (tanhf(e / st) * -tanhf(wC / wP));
            else
                sn += sn * tanhf(e / st);
            if (sn < 0.01f)
                sn = 0.01f;
            else if (sn > 99.9f)
                sn = 99.9f;
            fines[i] = 100.0f - sn;
            sm -= (1.e-3f * evap_trans / st);
            if (sm < 0.02f)
                sm = 0.02f;
            else if (sm > 0.5f)
                sm = 0.5f;
        }
        soilT[i] = st;
        stone[i] = sn;
        soilM[i] = sm;
        // Update_Surface (updates.cu:23-46); the outlet takes base - 1.2e-4 (:165,174)
        double zn = zold;
        if ((int)i == outlet) {
            zn = base - 0.00012;
        } else {
            zn = ((zn + (double)dz) - (double)wC) - (double)wP;
            if (zn <= base) zn = base + 0.01;
        }
        z[i] = zn;
        // update_nutrient_content (updates.cu:48-76)
        float nu;
        const float leaf_fall = tb / (72.8f * logf(tb + 1.4f));
        const float decomposition = sb0 * expf(0.12f * T - 5.75f);
        const float sb = sb0 + leaf_fall - decomposition;
        soilB[i] = sb;
        if (st == 0.0f && sb > 0.0f)
            nu = 100.0f;
        else if (st == 0.0f)
            nu = 0.0f;
        else
            nu = (sb / (1300.0f * st)) * 100.0f;
        if (nu > 100.f) nu = 100.f;
        nut[i] = nu;
        // grow_vegetation (updates.cu:78-139): delta_temp against the initial
        // climate grids (copytolastclimate is disabled, lem.cpp:102).  During the
        // run-in both grids come from the same DEM and scalars, so it is 0.
        float dT = 0.0f;
        if (c.from_current_dem) {
            float h1, l1, h0, l0;
            dsplit(zc, h1, l1);
            dsplit(z0, h0, l0);
            dT = dtemp_scalar - ((h1 - h0) + (l1 - l0)) * 0.0065f;
            if (fabsf(dT) < 1.0e-3f) {  // decide the branch with the reference's fp64 arithmetic
                const double t1 = c.temp - ((zc - kMinHeight) * 0.0065);
                const double t0 = c.temp0 - ((z0 - kMinHeight) * 0.0065);
                const double dd = t1 - t0;
                dT = dd > 0.0 ? fmaxf((float)dd, 1.17549435e-38f) : (dd < 0.0 ? -fmaxf((float)(-dd), 1.17549435e-38f) : 0.0f);
            }
        }
        const float tempeffect = 100.0f + (100.0f / (T + 15.0f));
        const float total_cc = (3000.0f + (5.0f * (rain - tempeffect))) / k.rescale_veg;
        float nb = tb;
        if (dT > 0.f) {
            const float r_plus = dT * (1.0f + tanhf((T - k.temp_inflex) / k.temp_sens));
            nb += ((r_plus * nb) * (1.0f - (nb / total_cc)));
        }
        if (dT < 0.f) {
            const float r_minus = dT * (1.0f - tanhf((T - k.temp_inflex) / k.temp_sens));
            nb += ((r_minus * nb) * (nb / total_cc));
        }
        if (dT == 0.f) nb = total_cc;
        if (nb < 1.f) nb = 1.0f;
        totB[i] = nb;
        if (dz_out) {
            dz_out[i] = dz;
            wc_out[i] = wC;
            wp_out[i] = wP;
        }
        swc += wC;
        swp += wP;
        sbio += nb;
    }
    const double t1 = block_sum_d(swc, red);
    const double t2 = block_sum_d(swp, red);
    const double t3 = block_sum_d(sbio, red);
    const double t4 = block_sum_d(sd, red);
    if (threadIdx.x == 0) {
        atomicAdd(&o.tot_wc, t1);
        atomicAdd(&o.tot_wp, t2);
        atomicAdd(&o.tot_bio, t3);
        atomicAdd(&o.tot_d, t4);
    }
}

__global__ void k_mod_reset(DevScalars* sc, DemCtx dc, int tiled) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d == 0) {
        sc->counters[0] = 0;
        sc->sed_tiled_ok = tiled;
        sc->tile_src = 0;
    }
    if (d < dc.n) {
        DemOut& o = dc.out[d];
        o.sed_done = 0;
        o.tot_e = o.tot_i = o.tot_g = o.tot_d = o.tot_wc = o.tot_wp = o.tot_bio = 0.0;
        o.fa_max_key = 0ull;
    }
}

}  // namespace

lem_status launch_erosion(const DevState& s, const ModelConsts& k, uint32_t flags, const Launch& L) {
    const int T = 256;
    const float* prop = (k.flow_type != 0 && k.mfd_props) ? s.prop : nullptr;
    const int tiled = (k.flow_type == 0 && !prop) ? 1 : 0;
    LEM_LAUNCH(L, k_mod_reset, (s.dems.n + 127) / 128, 128, s.sc, s.dems, tiled);
    LEM_LAUNCH(L, k_erosion, s.n_chunks, T, s.z, s.z_init, s.mask, s.slopes, s.fa, s.fines, s.nut, s.soilT, s.stone,
               s.totB, s.slopeptr, s.ero, s.inci, s.geli, s.depo, s.fd, s.chunk_start, k, s.dems, s.sc);
    const TileSet ts = tiles_of(s, k.W);
    {
        const size_t vb = (ts.span() + T - 1) / T;
        LEM_LAUNCH(L, k_sed_prep, (int)(vb > 152 * 32 ? 152 * 32 : vb), T, s.mask, s.fd, s.depo, s.pending, s.list_a,
                   k, s.sc, ts);
    }
    if (tiled) {
        const int tiles = ts.n;
        LEM_LAUNCH(L, k_sedt_local, tiles, 256, s.mask, s.fd, s.ero, s.inci, s.geli, s.depo, s.stone, s.fines,
                   s.soilT, s.t_dst, s.t_pend, s.t_orng, s.t_la, s.p_abc, s.p_ref, s.p_map, s.t_stat, s.f_idx,
                   s.f_map, s.f_ds, s.t_fcnt, s.list_b, k, s.sc, s.dems, ts);
        const uint8_t* fd = s.fd;
        const int32_t* torng = s.t_orng;
        const int32_t* tdst = s.t_dst;
        const float2* tout = s.t_la;
        const float4* pabc = s.p_abc;
        const int32_t* pref = s.p_ref;
        const float4* pmap = s.p_map;
        float* pval = s.p_val;
        float* depo = s.depo;
        float* stone = s.stone;
        float* fines = s.fines;
        float* soilT = s.soilT;
        int32_t* tpend = s.t_pend;
        int32_t* la = s.list_b;  // the outlets k_sedt_local found ready
        int32_t* lb = s.list_a;
        ModelConsts kk = k;
        DevScalars* sc = s.sc;
        void* args[] = {(void*)&fd,    (void*)&torng, (void*)&tdst,  (void*)&tout, (void*)&pabc, (void*)&pref,
                        (void*)&pmap,  (void*)&pval,  (void*)&depo,  (void*)&stone, (void*)&fines, (void*)&soilT, (void*)&tpend,
                        (void*)&la,    (void*)&lb,    (void*)&kk,    (void*)&sc};
        L.pre("k_sedt_coarse");
        LEM_CUDA_TRY(coop_launch((const void*)k_sedt_coarse, s.coop_blocks[kCkSedCoarse], args, L.st));
        L.post();
        LEM_LAUNCH(L, k_sedt_final, tiles, 256, s.mask, s.fd, s.ero, s.inci, s.geli, s.depo, s.stone, s.fines,
                   s.soilT, s.t_pend, s.t_stat, s.f_idx, s.f_map, s.f_ds, s.t_fcnt, s.p_val, k, s.sc, s.dems,
                   ts);
    }
    {
        const uint8_t* mask = s.mask;
        const uint8_t* fd = s.fd;
        const float* ero = s.ero;
        const float* inci = s.inci;
        const float* geli = s.geli;
        float* depo = s.depo;
        float* stone = s.stone;
        float* fines = s.fines;
        float* soilT = s.soilT;
        int32_t* pending = s.pending;
        int32_t* la = s.list_a;
        int32_t* lb = s.list_b;
        ModelConsts kk = k;
        DevScalars* sc = s.sc;
        DemCtx dc = s.dems;
        int gate = tiled;
        void* args[] = {(void*)&mask, (void*)&fd,    (void*)&prop,  (void*)&ero,     (void*)&inci,
                        (void*)&geli, (void*)&depo,  (void*)&stone, (void*)&fines,   (void*)&soilT,
                        (void*)&pending, (void*)&la, (void*)&lb,    (void*)&kk,      (void*)&sc, (void*)&dc,
                        (void*)&gate};
        L.pre("k_sed_walk");
        LEM_CUDA_TRY(coop_launch((const void*)k_sed_walk, s.coop_blocks[kCkSedWalk], args, L.st));
        L.post();
    }
    const bool diag = (flags & LEM_STEP_KEEP_DIAGNOSTICS) != 0;
    LEM_LAUNCH(L, k_final, s.n_chunks, T, s.z, s.z_init, s.mask, s.fa, s.ero, s.inci, s.geli, s.depo, s.soilT,
               s.stone, s.fines, s.soilM, s.soilB, s.nut, s.totB, diag ? s.dz : nullptr, diag ? s.wc : nullptr,
               diag ? s.wp : nullptr, s.temp_tab, s.chunk_start, k, s.dems);
    LEM_CUDA_TRY(cudaGetLastError());
    return LEM_OK;
}

const void* mod_coop_kernels[] = {(const void*)k_sed_walk, (const void*)k_sedt_coarse};
extern const int mod_coop_kernel_count = 2;

}  // namespace lem
