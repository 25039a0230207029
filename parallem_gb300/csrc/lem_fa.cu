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

#include "lem_wave.cuh"

namespace cg = cooperative_groups;

namespace lem {

namespace {

// calcrunoffweight (runoffweight.cu:21-58) plus the in-degrees of the wave.
// A donor outside the catchment is complete from the start when its DEM is
// nodata (correctmfdflow's okgrid, mfd_simple.cu:279-285) and never otherwise.
__global__ void k_fa_prep(const double* __restrict__ z, const uint8_t* __restrict__ mask,
                          const uint8_t* __restrict__ fd, const float* __restrict__ stone,
                          const float* __restrict__ totB, float* __restrict__ soilM, float* __restrict__ w,
                          float2* __restrict__ fa, int32_t* __restrict__ pending, int32_t* __restrict__ contrib,
                          int32_t* ready, ModelConsts k, ClimateNow c, DevScalars* sc) {
    const int W = k.W, H = k.H;
    const size_t N = (size_t)W * H;
    const float rain0 = (float)c.rain, rinc = (float)c.rain_inc;
    int nact = 0;
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < N; base += (size_t)gridDim.x * blockDim.x) {
        const size_t i = base + threadIdx.x;
        bool src = false;
        if (i < N) {
            const int x = (int)(i % W), y = (int)(i / W);
            if (mask[i]) {
                ++nact;
                const float coeff = (1.0f - 0.0085f * stone[i]) * expf(-0.0025f * totB[i] / 76.5f) *
                                    tanhf(0.6f + soilM[i] / 0.2f);
                const float myppt = (rain0 + (float)y * rinc) / 1000.0f;
                const float wi = myppt * coeff;
                float sm = soilM[i] + myppt * (1.0f - coeff);
                if (sm > 0.5f) sm = 0.5f;
                soilM[i] = sm;
                w[i] = wi;
                fa[i] = make_float2(wi, 0.0f);
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
                w[i] = -9999.0f;
                fa[i] = make_float2(0.0f, 0.0f);
                if (contrib) contrib[i] = 0;
                pending[i] = kBlocked;
            }
        }
        wave_append(src, (int32_t)i, ready, &sc->counters[0], (int)N, &sc->err);
    }
    nact = wsum(nact);
    if ((threadIdx.x & 31) == 0 && nact) atomicAdd(&sc->n_active, nact);
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

// The accumulation wave.  Round 0 starts at every source; MFD cells that
// release more than one receiver queue the extra ones for the next round.
__global__ void k_fa_walk(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd,
                          const float* __restrict__ w, const float* __restrict__ prop, float2* fa, int32_t* pending,
                          int32_t* contrib, int32_t* list_a, int32_t* list_b, ModelConsts k, DevScalars* sc) {
    cg::grid_group grid = cg::this_grid();
    const int W = k.W, H = k.H;
    const size_t N = (size_t)W * H;
    const size_t gstride = (size_t)gridDim.x * blockDim.x;
    const size_t gtid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    int32_t* cnt = sc->counters;  // cnt[0] holds the sources written by k_fa_prep
    if (gtid == 0) cnt[1] = cnt[2] = 0;
    grid.sync();
    int done = 0;
    int round = 0;
    for (;; ++round) {
        const int32_t* in = (round & 1) ? list_b : list_a;
        int32_t* out = (round & 1) ? list_a : list_b;
        const int nin = *((volatile int32_t*)&cnt[round % 3]);
        if (nin == 0) break;
        if (round > (1 << 24)) {
            if (gtid == 0) atomicOr(&sc->err, ErrFlags::kNoConverge);
            break;
        }
        if (gtid == 0) cnt[(round + 2) % 3] = 0;
        for (size_t base = (size_t)blockIdx.x * blockDim.x; base < (size_t)nin; base += gstride) {
            const size_t it = base + threadIdx.x;
            int32_t cur = it < (size_t)nin ? in[it] : -1;
            int32_t extra[8];
            int nextra = 0;
            for (size_t steps = 0; cur >= 0 && steps < N; ++steps) {
                const int x = cur % W, y = cur / W;
                float2 acc = make_float2(0.f, 0.f);
                int32_t cacc = 1;
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) {
                    const int d = scan_dir(kk);
                    const int nx = x + dir_dx(d), ny = y + dir_dy(d);
                    if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
                    const size_t n = (size_t)ny * W + nx;
                    if (!donates(fd[n], d)) continue;
                    const float2 v = __ldcg(fa + n);
                    const float p = prop_of(prop, mask, n, (d + 4) & 7);
                    acc = ff_add(acc, p == 1.0f ? v : ff_scale(v, p));
                    if (contrib && mask[n]) cacc += __ldcg(contrib + n);
                }
                if (acc.x < 0.0f) acc = make_float2(0.f, 0.f);
                __stcg(fa + cur, ff_add(make_float2(w[cur], 0.f), acc));
                if (contrib) __stcg(contrib + cur, cacc);
                ++done;
                __threadfence();
                // release the receivers
                const uint8_t code = fd[cur];
                int32_t next = -1;
                for (int d = 0; d < 8; ++d) {
                    if (!(code & dir_bit(d))) continue;
                    const int rx = x + dir_dx(d), ry = y + dir_dy(d);
                    if (rx < 0 || rx >= W || ry < 0 || ry >= H) continue;
                    const size_t r = (size_t)ry * W + rx;
                    if (!mask[r]) continue;
                    if (atomicSub(pending + r, 1) == 1) {
                        if (next < 0)
                            next = (int32_t)r;
                        else if (nextra < 8)
                            extra[nextra++] = (int32_t)r;
                    }
                }
                __threadfence();
                cur = next;
            }
            for (int j = 0; j < 8; ++j)
                wave_append(j < nextra, j < nextra ? extra[j] : 0, out, &cnt[(round + 1) % 3], (int)N, &sc->err);
        }
        grid.sync();
    }
    done = wsum(done);
    if ((threadIdx.x & 31) == 0 && done) atomicAdd(&sc->fa_done, done);
}

// correctmfdflow's first-iteration branch (mfd_simple.cu:336-349): the outlet
// becomes the first cell holding the largest accumulation.
__global__ void k_fa_argmax(const float2* __restrict__ fa, size_t N, DevScalars* sc, int phase) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = fa[i];
        if (v.x != v.x) continue;  // NaN never wins the host scan (mfd_simple.cu:341)
        const unsigned long long kk = ffkey(v);
        if (phase == 0)
            atomicMax(&sc->fa_max_key, kk);
        else if (kk == sc->fa_max_key)
            atomicMin(&sc->counters[7], (int32_t)i);
    }
}

__global__ void k_fa_argmax_set(DevScalars* sc) {
    const unsigned long long zero = ffkey(make_float2(0.f, 0.f));
    sc->outlet = (sc->fa_max_key > zero) ? sc->counters[7] : 0;
}

__global__ void k_fa_reset(DevScalars* sc) {
    sc->counters[0] = 0;
    sc->fa_done = 0;
    sc->n_active = 0;
    sc->fa_max_key = 0ull;
    sc->counters[7] = 0x7fffffff;
}

}  // namespace

lem_status launch_flow_accumulation(const DevState& s, const ModelConsts& k, const ClimateNow& c, uint32_t flags,
                                    const Launch& L) {
    const size_t N = (size_t)k.W * k.H;
    const int T = 256;
    size_t nb = (N + T - 1) / T;
    const int blocks = (int)(nb > 152 * 32 ? 152 * 32 : nb);
    LEM_LAUNCH(L, k_fa_reset, 1, 1, s.sc);
    const float* prop = nullptr;
    if (k.flow_type != 0 && k.mfd_props) {
        LEM_LAUNCH(L, k_calcprops, blocks, T, s.mask, s.fd, s.slopes, s.prop, N);
        prop = s.prop;
    }
    int32_t* contrib = (flags & LEM_STEP_CONTRIB) ? s.contrib : nullptr;
    LEM_LAUNCH(L, k_fa_prep, blocks, T, s.z, s.mask, s.fd, s.stone, s.totB, s.soilM, s.w, s.fa, s.pending, contrib,
               s.list_a, k, c, s.sc);
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
        void* args[] = {(void*)&mask, (void*)&fd, (void*)&w, (void*)&prop, (void*)&fa, (void*)&pending,
                        (void*)&contrib, (void*)&la, (void*)&lb, (void*)&kk, (void*)&sc};
        L.pre("k_fa_walk");
        LEM_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_fa_walk, dim3(s.max_coop_blocks), dim3(256), args,
                                                 0, L.st));
        L.post();
    }
    if (flags & LEM_STEP_SET_OUTLET_FROM_FA) {
        LEM_LAUNCH(L, k_fa_argmax, blocks, T, s.fa, N, s.sc, 0);
        LEM_LAUNCH(L, k_fa_argmax, blocks, T, s.fa, N, s.sc, 1);
        LEM_LAUNCH(L, k_fa_argmax_set, 1, 1, s.sc);
    }
    LEM_CUDA_TRY(cudaGetLastError());
    return LEM_OK;
}

const void* fa_coop_kernels[] = {(const void*)k_fa_walk};
extern const int fa_coop_kernel_count = 1;

}  // namespace lem
