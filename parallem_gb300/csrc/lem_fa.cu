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
    int W, H;
    __device__ __forceinline__ void cell(int32_t cur, int x, int y) const {
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
};

// The accumulation wave: every source starts it; cells follow as their last
// donor finishes.
__global__ void k_fa_walk(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fd,
                          const float* __restrict__ w, const float* __restrict__ prop, float2* fa, int32_t* pending,
                          int32_t* contrib, int32_t* list_a, int32_t* list_b, ModelConsts k, DevScalars* sc) {
    const FaCell op{mask, fd, w, prop, fa, contrib, k.W, k.H};
    int done = wave_walk(op, fd, mask, pending, list_a, list_b, k.W, k.H, sc);
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

// ---------------------------------------------------------------------------
// lem_accumulate_flow_noalloc: the accumulation wave on caller-owned buffers,
// with its intermediate data in one file-scope device array.
namespace {

constexpr size_t kNaCells = LEM_NOALLOC_MAX_CELLS;
constexpr size_t kNaHead = 1024;  // DevScalars, rounded up
static_assert(sizeof(DevScalars) <= kNaHead, "scalar block");
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

__global__ void k_na_reset(DevScalars* sc) {
    sc->counters[0] = sc->counters[1] = sc->counters[2] = 0;
    sc->fa_done = 0;
    sc->err = 0;
}

// Codes, mask, weights, initial accumulation and in-degrees from the caller's
// int32 codes and DEM (cells at -9999 are outside and complete with zero flow).
__global__ void k_na_prep(const int32_t* __restrict__ fd_in, const double* __restrict__ w_in,
                          const double* __restrict__ dem, uint8_t* __restrict__ code, uint8_t* __restrict__ mask,
                          float* __restrict__ w, float2* __restrict__ fa, int32_t* __restrict__ pending,
                          int32_t* ready, int W, int H, DevScalars* sc) {
    const size_t N = (size_t)W * H;
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < N; base += (size_t)gridDim.x * blockDim.x) {
        const size_t i = base + threadIdx.x;
        bool src = false;
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
        }
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
    NaDevice nd;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na[dev].base) {
            // once per device, with that device current: the device address of the array
            void* ptr = nullptr;
            LEM_CUDA_TRY(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
            int per = 0, sms = 0;
            LEM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fa_walk, 256, 0));
            LEM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            g_na[dev].base = static_cast<unsigned char*>(ptr);
            g_na[dev].blocks = (per < 1 ? 1 : per) * sms;
        }
        nd = g_na[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevScalars* sc = reinterpret_cast<DevScalars*>(nd.base);
    uint8_t* code = nd.base + kNaOffCode;
    uint8_t* mask = nd.base + kNaOffMask;
    int32_t* pending = reinterpret_cast<int32_t*>(nd.base + kNaOffPend);
    int32_t* la = reinterpret_cast<int32_t*>(nd.base + kNaOffListA);
    int32_t* lb = reinterpret_cast<int32_t*>(nd.base + kNaOffListB);
    float* w = reinterpret_cast<float*>(nd.base + kNaOffW);
    float2* fa = reinterpret_cast<float2*>(nd.base + kNaOffFa);
    const int T = 256;
    const int blocks = (int)std::min<size_t>((N + T - 1) / T, 152 * 32);
    k_na_reset<<<1, 1, 0, st>>>(sc);  // the array keeps the previous call's contents
    k_na_prep<<<blocks, T, 0, st>>>(d_fd, d_weight, d_dem, code, mask, w, fa, pending, la, width, height, sc);
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
        void* args[] = {(void*)&m, (void*)&c, (void*)&ww, (void*)&prop, (void*)&fa, (void*)&pending,
                        (void*)&contrib, (void*)&la, (void*)&lb, (void*)&k, (void*)&sc};
        LEM_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_fa_walk, dim3(nd.blocks), dim3(256), args, 0, st));
    }
    k_na_out<<<blocks, T, 0, st>>>(fa, d_fa, N);
    LEM_CUDA_TRY(cudaGetLastError());
    uint32_t err = 0;
    LEM_CUDA_TRY(cudaMemcpyAsync(&err, &sc->err, sizeof err, cudaMemcpyDeviceToHost, st));
    LEM_CUDA_TRY(cudaStreamSynchronize(st));
    if (err & ErrFlags::kCapacity) return LEM_ERR_CAPACITY;
    if (err) return LEM_ERR_NOCONVERGE;
    return LEM_OK;
}

const void* fa_coop_kernels[] = {(const void*)k_fa_walk};
extern const int fa_coop_kernel_count = 1;

}  // namespace lem
