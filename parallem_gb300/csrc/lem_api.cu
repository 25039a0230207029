// lem_api.cu -- the C ABI of include/lem_gb300.h: handle life cycle, field
// transfers, climate state and stage orchestration.

#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "lem_ctx.cuh"

namespace lem {

extern const void* fd_coop_kernels[];
extern const int fd_coop_kernel_count;
extern const void* fa_coop_kernels[];
extern const int fa_coop_kernel_count;
extern const void* mod_coop_kernels[];
extern const int mod_coop_kernel_count;

static thread_local std::string g_last_error;

struct Profiler {
    struct Rec {
        const char* name;
        int a, b;
    };
    std::vector<cudaEvent_t> pool;
    std::vector<Rec> recs;
    size_t used = 0;
    int open_a = -1;
    const char* open_name = nullptr;
    int take() {
        if (used == pool.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return -1;
            pool.push_back(e);
        }
        return (int)used++;
    }
};

void profiler_begin(Profiler* p, const char* name, cudaStream_t st) {
    const int a = p->take();
    if (a < 0) return;
    cudaEventRecord(p->pool[a], st);
    p->open_a = a;
    p->open_name = name;
}

void profiler_end(Profiler* p, cudaStream_t st) {
    if (p->open_a < 0) return;
    const int b = p->take();
    if (b < 0) return;
    cudaEventRecord(p->pool[b], st);
    p->recs.push_back({p->open_name, p->open_a, b});
    p->open_a = -1;
}

lem_status cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    g_last_error = buf;
    return LEM_ERR_CUDA;
}

}  // namespace lem

using namespace lem;

// The autotuner: over its next steps a handle runs every cooperative kernel
// with 1, 2 and 4 blocks per SM and with all its co-resident blocks in turn
// (step s of the tuning runs candidate s % 4, so the drift of the model state
// between steps falls on all candidates alike; the first step, under the
// default schedule, is not measured), times each with events, and keeps for
// each kernel the block count with the lowest mean time when it beats the
// default by more than the step-to-step noise.  The default is the block
// count every cooperative kernel can hold at once (4 per SM here), candidate
// kTuneDefault.  Results do not depend on the block count: every loop runs to
// a unique fixpoint and sums are pulled in a fixed order.
constexpr int kTuneCands = 4;
constexpr int kTuneBlocksPerSm[kTuneCands] = {1, 2, 4, 0};  // 0: every co-resident block
constexpr int kTuneDefault = 2;
constexpr double kTuneMargin = 0.97;  // a candidate replaces the default only below 97 % of its time
// The flow-direction kernel's tile shape tried in each candidate step (an
// index into kFdRows); the default shape is candidate kTuneDefault's.
constexpr int kTuneFdShape[kTuneCands] = {0, 2, 1, 0};  // the default candidate takes 32 x 16 tiles
const char* const kCoopNames[kCoopKernels] = {"k_plateau_relax", "k_flood_merge", "k_flood_jump", "k_flood_spill",
                                              "k_fat_coarse",    "k_fa_walk",     "k_sedt_coarse", "k_sed_walk"};
struct Tuner {
    int state = 0;  // 0 default schedule, 1 tuning, 2 tuned
    int step = -1;  // tuning step (-1: the unmeasured first one)
    int steps = 0;  // measured steps in all
    double coop_ms[kCoopKernels][kTuneCands] = {};  // device ms, summed over the steps of each candidate
    double fd_ms[kTuneCands] = {};                  // the flow-direction kernel, by candidate tile shape
    int coop_n[kTuneCands] = {};
    double default_ms = 0, tuned_ms = 0;
};

// A DEM of the handle as the host tracks it: its region and its climate state.
struct HostDem {
    bool active = false;
    int32_t x0 = 0, y0 = 0, w = 0, h = 0;
    double rain = 0, temp = 0, rain0 = 0, temp0 = 0;
    bool from_current = false;     // a recompute = 1 climate has been set
    bool outlet_set = false;
    uint32_t next_flags = 0;       // one-shot step flags of this DEM
};

struct lem_handle {
    DevState s{};
    ModelConsts k{};
    lem_params p{};
    cudaStream_t st = nullptr;
    int device = 0;
    bool batch = false;            // several DEMs packed into the grid
    bool dem_set = false;          // a single grid: its DEM was uploaded
    size_t N = 0;
    uint64_t launches = 0;
    std::vector<void*> allocs;
    std::vector<HostDem> dems;
    DemIn* dem_in = nullptr;       // device copies
    DemOut* dem_out = nullptr;
    uint16_t* dem_of = nullptr;
    int32_t* chunks = nullptr;
    int32_t* live = nullptr;       // device list of the tiles holding a DEM region (batch grids)
    bool live_dirty = true;        // a DEM joined or left since the list was uploaded
    DemOut* host_out = nullptr;    // pinned mirror of dem_out
    void* staging = nullptr;       // pinned host buffer for field conversions, grown on demand
    size_t staging_bytes = 0;
    DevScalars* host_sc = nullptr; // pinned mirror of the device scalars
    Profiler prof;
    bool profiling = false;
    bool graphs = false;           // steps replay a captured CUDA graph (lem_set_graphs)
    cudaGraphExec_t gexec = nullptr;
    int32_t gkey[3] = {-1, -1, -1};  // chunks, visited tiles and step flags the graph was captured for
    uint64_t glaunches = 0;        // kernel launches in one replay
    int sms = 0;                   // SMs of the handle's device
    Tuner tune;
    cudaEvent_t events[16] = {};
    FdTmaMaps fd_maps{};           // tensor maps of the TMA flow-direction kernel (when s.fd_tma is set)
    size_t device_bytes = 0;       // bytes of the handle's resident allocations
    cudaStream_t side = nullptr;   // exports' device-to-host copies (created on first use)
    std::vector<std::pair<void*, size_t>> pinned_free;  // exports' pinned host buffers for reuse
    int exports = 0;               // exports started and not yet waited for
    Launch launch() { return Launch{st, &launches, profiling ? &prof : nullptr}; }
};

struct lem_export {
    lem_handle* h = nullptr;
    int32_t x0 = 0, y0 = 0, w = 0, hgt = 0;  // the DEM's region when the export started
    std::vector<lem_field> fields;
    std::vector<size_t> off;               // byte offset of each field's raw copy in the staging
    size_t mask_off = 0, out_off = 0;      // the region's mask and DemOut (for the direction codes)
    size_t bytes = 0;
    void* host = nullptr;                  // pinned staging
    size_t host_cap = 0;
    cudaEvent_t done = nullptr;            // the device-to-host copy has finished
};

namespace {

template <class T>
lem_status dalloc(lem_handle* h, T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__) == LEM_ERR_CUDA ? LEM_ERR_NOMEM : LEM_ERR_NOMEM;
    h->allocs.push_back(q);
    h->device_bytes += sizeof(T) * (count ? count : 1);
    e = cudaMemsetAsync(q, 0, sizeof(T) * (count ? count : 1), h->st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync", __FILE__, __LINE__);
    *p = static_cast<T*>(q);
    return LEM_OK;
}

// log10(K1*KC*KH / (4*K2*gammaCa*gammaHCO3^2)) of weathering (eroincidep.cu:435-447,
// :470) in the reference's double arithmetic, tabulated over temperature.
void dreybrodt_table(std::vector<float>& tab) {
    tab.resize(kTabN);
    for (int j = 0; j < kTabN; ++j) {
        const double T = (double)kTabT0 + j * (double)kTabStep;
        const double t_abs = T + 273.16;
        const double t2 = t_abs * t_abs;
        const double ltemp = log10(t_abs);
        const double DHA = -0.4883 + 8.074e-4 * T;
        const double DHB = -0.3241 + 1.600e-4 * T;
        const double sqI = sqrt(0.1);
        const double denom1 = (-4. * DHA * sqI) / (1. + 5.e-8 * DHB * sqI);
        const double gammCa = pow(10., denom1);
        const double gammHCO3 = pow(10., (-DHA * sqI) / (1. + 5.4e-8 * DHB * sqI));
        const double K1 = pow(10., -356.3094 - 0.06091964 * t_abs + 21834.37 / t_abs + 126.8339 * ltemp - 1684915 / t2);
        const double K2 = pow(10., -107.8871 - 0.03252849 * t_abs + 5151.79 / t_abs + 38.92561 * ltemp - 563713.9 / t2);
        const double KC = pow(10., -171.9065 - 0.077993 * t_abs + 2839.319 / t_abs + 71.595 * ltemp);
        const double KH = pow(10., 108.3865 + 0.01985076 * t_abs - 6919.53 / t_abs - 40.45154 * ltemp + 669365.0 / t2);
        tab[j] = (float)log10((K1 * KC * KH) / (4. * K2 * gammCa * gammHCO3 * gammHCO3));
    }
}

bool field_is_int(lem_field f) {
    return f == LEM_F_MASK || f == LEM_F_FD || f == LEM_F_SFD || f == LEM_F_CONTRIB || f == LEM_F_WATERSHED ||
           f == LEM_F_DEM_ROUTED || f == LEM_F_SFD_PASS1;
}

float* float_field(lem_handle* h, lem_field f) {
    DevState& s = h->s;
    switch (f) {
        case LEM_F_RUNOFF: return s.w;
        case LEM_F_SLOPEPTR: return s.slopeptr;
        case LEM_F_STONE: return s.stone;
        case LEM_F_FINES: return s.fines;
        case LEM_F_SOILT: return s.soilT;
        case LEM_F_SOILM: return s.soilM;
        case LEM_F_SOILB: return s.soilB;
        case LEM_F_NUT: return s.nut;
        case LEM_F_TOTB: return s.totB;
        case LEM_F_ERO: return s.ero;
        case LEM_F_INCI: return s.inci;
        case LEM_F_GELI: return s.geli;
        case LEM_F_DEPO: return s.depo;
        case LEM_F_DZ: return s.dz;
        case LEM_F_WEATHER_C: return s.wc;
        case LEM_F_WEATHER_P: return s.wp;
        default: return nullptr;
    }
}

lem_status sync_scalars(lem_handle* h) {
    LEM_CUDA_TRY(cudaMemcpyAsync(h->host_sc, h->s.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->st));
    LEM_CUDA_TRY(cudaMemcpyAsync(h->host_out, h->dem_out, sizeof(DemOut) * h->dems.size(), cudaMemcpyDeviceToHost,
                                 h->st));
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    return LEM_OK;
}

lem_status ensure_staging(lem_handle* h, size_t bytes) {
    if (bytes <= h->staging_bytes) return LEM_OK;
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    if (h->staging) cudaFreeHost(h->staging);
    h->staging = nullptr;
    h->staging_bytes = 0;
    if (cudaMallocHost(&h->staging, bytes) != cudaSuccess) return LEM_ERR_NOMEM;
    h->staging_bytes = bytes;
    return LEM_OK;
}

__global__ void k_fill_f64(double* p, size_t n, double v) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}
__global__ void k_fill_u16(uint16_t* p, size_t n, uint16_t v) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

// A DEM joins (id >= 0) or leaves (id < 0) its region of the grid.  Joining:
// the DEM was uploaded into z; the mask follows it (createmask,
// MEM_kernels/memory.cu:229-238), the initial climate grids take it as their
// DEM, and every other field of the region starts at zero as in a new handle.
// Leaving: the region returns to nodata outside every DEM.
__global__ void k_region(DevState s, uint16_t* of, int W, int x0, int y0, int w, int h, int id) {
    const size_t n = (size_t)w * h;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t g = (size_t)(y0 + i / w) * W + x0 + i % w;
        if (id < 0) s.z[g] = kNoData;
        if (of) of[g] = id < 0 ? kNoDem : (uint16_t)id;
        const double zv = s.z[g];
        s.z_init[g] = zv;
        s.zf[g] = zv;
        s.mask[g] = (id >= 0 && zv != kNoData) ? 1 : 0;
        s.sfd[g] = s.mfd[g] = s.fd[g] = s.sfd1[g] = kMaskedCode;
        for (int j = 0; j < 8; ++j) s.slopes[8 * g + j] = 0.f;
        s.fa[g] = make_float2(0.f, 0.f);
        s.w[g] = s.slopeptr[g] = 0.f;
        s.stone[g] = s.fines[g] = s.soilT[g] = s.soilM[g] = s.soilB[g] = s.nut[g] = s.totB[g] = 0.f;
        s.ero[g] = s.inci[g] = s.geli[g] = s.depo[g] = s.dz[g] = s.wc[g] = s.wp[g] = 0.f;
        s.contrib[g] = 0;
        s.ws[g] = 0;
        s.sp[g] = 0.f;
    }
}

lem_status region_op(lem_handle* h, const HostDem& r, int id) {
    const size_t n = (size_t)r.w * r.h;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 32);
    k_region<<<blocks, 256, 0, h->st>>>(h->s, h->dem_of, h->k.W, r.x0, r.y0, r.w, r.h, id);
    LEM_CUDA_TRY(cudaGetLastError());
    return LEM_OK;
}

// Per-DEM inputs of the next stage (region, climate, flags) and the chunks of
// the streaming passes.
lem_status prepare(lem_handle* h) {
    const int n = (int)h->dems.size();
    std::vector<DemIn> in(n);
    std::vector<int32_t> chunk(n + 1, 0);
    bool any = false;
    for (int d = 0; d < n; ++d) {
        const HostDem& r = h->dems[d];
        DemIn& o = in[d];
        std::memset(&o, 0, sizeof o);
        chunk[d + 1] = chunk[d];
        if (!r.active) continue;
        if (h->batch && !r.outlet_set) return LEM_ERR_STATE;
        any = true;
        o.x0 = r.x0;
        o.y0 = r.y0;
        o.w = r.w;
        o.h = r.h;
        o.active = 1;
        o.from_current_dem = r.from_current ? 1 : 0;
        o.outlet_from_fa = (r.next_flags & LEM_STEP_SET_OUTLET_FROM_FA) ? 1 : 0;
        o.rain = r.rain;
        o.temp = r.temp;
        o.rain_inc = (r.rain * 2 - r.rain) / r.h;  // Data.cpp:246-249, rows of the DEM
        o.rain0 = r.rain0;
        o.temp0 = r.temp0;
        o.rain0_inc = (r.rain0 * 2 - r.rain0) / r.h;
        chunk[d + 1] += (int32_t)(((int64_t)r.w * r.h + kChunk - 1) / kChunk);
    }
    if (!any) return LEM_ERR_STATE;
    // pageable sources: the copies take the data before returning
    LEM_CUDA_TRY(cudaMemcpyAsync(h->dem_in, in.data(), sizeof(DemIn) * n, cudaMemcpyHostToDevice, h->st));
    LEM_CUDA_TRY(cudaMemcpyAsync(h->chunks, chunk.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, h->st));
    h->s.n_chunks = chunk[n];
    if (h->batch && h->live_dirty) {
        // the tiles covered by some DEM region, in ascending order
        const int tw = (h->k.W + kTile - 1) / kTile, th = (h->k.H + kTile - 1) / kTile;
        std::vector<uint8_t> on((size_t)tw * th, 0);
        for (const HostDem& r : h->dems) {
            if (!r.active) continue;
            for (int ty = r.y0 / kTile; ty < (r.y0 + r.h + kTile - 1) / kTile; ++ty)
                for (int tx = r.x0 / kTile; tx < (r.x0 + r.w + kTile - 1) / kTile; ++tx) on[(size_t)ty * tw + tx] = 1;
        }
        std::vector<int32_t> live;
        for (size_t t = 0; t < on.size(); ++t)
            if (on[t]) live.push_back((int32_t)t);
        LEM_CUDA_TRY(cudaMemcpyAsync(h->live, live.data(), sizeof(int32_t) * live.size(), cudaMemcpyHostToDevice,
                                     h->st));
        h->s.live = h->live;
        h->s.n_live = (int32_t)live.size();
        h->live_dirty = false;
    }
    return LEM_OK;
}

bool any_flag(const lem_handle* h, uint32_t f) {
    for (const HostDem& r : h->dems)
        if (r.active && (r.next_flags & f)) return true;
    return false;
}

// ---- field transfers of one DEM region (the whole grid for a single DEM)

lem_status set_region_field(lem_handle* h, const HostDem& r, lem_field f, const void* host) {
    const size_t n = (size_t)r.w * r.h;
    const size_t W = (size_t)h->k.W;
    const size_t off = (size_t)r.y0 * W + r.x0;
    DevState& s = h->s;
    lem_status st;
    if ((st = ensure_staging(h, n * 8 * sizeof(float))) != LEM_OK) return st;
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    if (f == LEM_F_DEM) {
        LEM_CUDA_TRY(cudaMemcpy2DAsync(s.z + off, W * 8, host, r.w * 8, r.w * 8, r.h, cudaMemcpyHostToDevice, h->st));
    } else if (f == LEM_F_SLOPES) {
        const double* src = static_cast<const double*>(host);
        float* t = static_cast<float*>(h->staging);
        for (size_t i = 0; i < 8 * n; ++i) t[i] = (float)src[i];
        LEM_CUDA_TRY(cudaMemcpy2DAsync(s.slopes + 8 * off, W * 32, t, r.w * 32, r.w * 32, r.h, cudaMemcpyHostToDevice,
                                       h->st));
    } else if (f == LEM_F_FA) {
        const double* src = static_cast<const double*>(host);
        float2* t = static_cast<float2*>(h->staging);
        for (size_t i = 0; i < n; ++i) {
            const float hi = (float)src[i];
            t[i] = make_float2(hi, (float)(src[i] - (double)hi));
        }
        LEM_CUDA_TRY(cudaMemcpy2DAsync(s.fa + off, W * 8, t, r.w * 8, r.w * 8, r.h, cudaMemcpyHostToDevice, h->st));
    } else if (f == LEM_F_FD || f == LEM_F_SFD) {
        // int32 codes; -9999 (outside the catchment) keeps its low byte 0xF1
        const int32_t* src = static_cast<const int32_t*>(host);
        uint8_t* t = static_cast<uint8_t*>(h->staging);
        for (size_t i = 0; i < n; ++i) t[i] = (uint8_t)(src[i] & 0xff);
        LEM_CUDA_TRY(cudaMemcpy2DAsync((f == LEM_F_FD ? s.fd : s.sfd) + off, W, t, r.w, r.w, r.h,
                                       cudaMemcpyHostToDevice, h->st));
    } else {
        if (field_is_int(f)) return LEM_ERR_INVALID;  // the mask, counts and labels are computed, not set
        float* dst = float_field(h, f);
        if (!dst) return LEM_ERR_INVALID;
        const double* src = static_cast<const double*>(host);
        float* t = static_cast<float*>(h->staging);
        for (size_t i = 0; i < n; ++i) t[i] = (float)src[i];
        LEM_CUDA_TRY(cudaMemcpy2DAsync(dst + off, W * 4, t, r.w * 4, r.w * 4, r.h, cudaMemcpyHostToDevice, h->st));
    }
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    return LEM_OK;
}

lem_status get_region_field(lem_handle* h, const HostDem& r, int id, lem_field f, void* host) {
    const size_t n = (size_t)r.w * r.h;
    const size_t W = (size_t)h->k.W;
    const size_t off = (size_t)r.y0 * W + r.x0;
    DevState& s = h->s;
    lem_status st;
    if ((st = ensure_staging(h, n * 8 * sizeof(float))) != LEM_OK) return st;
    if ((st = sync_scalars(h)) != LEM_OK) return st;
    const DemOut& o = h->host_out[id];
    auto get2d = [&](void* dst, const void* src, size_t elem) {
        return cudaMemcpy2D(dst, r.w * elem, src, W * elem, r.w * elem, r.h, cudaMemcpyDeviceToHost);
    };
    switch (f) {
        case LEM_F_DEM:
            LEM_CUDA_TRY(get2d(host, s.z + off, 8));
            return LEM_OK;
        case LEM_F_DEM_ROUTED:
            // without sinks the second pass does not run and the stage's DEM is the routed one
            LEM_CUDA_TRY(get2d(host, (o.sinkcount_pass1 ? s.zf : s.z) + off, 8));
            return LEM_OK;
        case LEM_F_MASK: {
            uint8_t* m = static_cast<uint8_t*>(h->staging);
            LEM_CUDA_TRY(get2d(m, s.mask + off, 1));
            int32_t* out = static_cast<int32_t*>(host);
            for (size_t i = 0; i < n; ++i) out[i] = m[i];
            return LEM_OK;
        }
        case LEM_F_FD:
        case LEM_F_SFD:
        case LEM_F_SFD_PASS1: {
            uint8_t* buf = static_cast<uint8_t*>(h->staging);
            const uint8_t* src = f == LEM_F_FD ? s.fd : (f == LEM_F_SFD ? s.sfd : s.sfd1);
            LEM_CUDA_TRY(get2d(buf, src + off, 1));
            LEM_CUDA_TRY(get2d(buf + n, s.mask + off, 1));
            const int64_t outlet = (int64_t)o.outlet;
            const int64_t ol = (outlet / (int64_t)W - r.y0) * r.w + (outlet % (int64_t)W - r.x0);
            int32_t* out = static_cast<int32_t*>(host);
            for (size_t i = 0; i < n; ++i) {
                int32_t v = buf[n + i] ? (int32_t)buf[i] : -9999;  // masked cells hold -9999 (newflow.cu:74)
                if (f == LEM_F_FD && (int64_t)i == ol) v = 16;       // routeflow.cu:953
                out[i] = v;
            }
            return LEM_OK;
        }
        case LEM_F_CONTRIB:
            LEM_CUDA_TRY(get2d(host, s.contrib + off, 4));
            return LEM_OK;
        case LEM_F_WATERSHED:
            LEM_CUDA_TRY(get2d(host, s.ws + off, 4));
            return LEM_OK;
        case LEM_F_SLOPES: {
            float* t = static_cast<float*>(h->staging);
            LEM_CUDA_TRY(get2d(t, s.slopes + 8 * off, 32));
            double* out = static_cast<double*>(host);
            for (size_t i = 0; i < 8 * n; ++i) out[i] = t[i];
            return LEM_OK;
        }
        case LEM_F_FA: {
            float2* t = static_cast<float2*>(h->staging);
            LEM_CUDA_TRY(get2d(t, s.fa + off, 8));
            double* out = static_cast<double*>(host);
            for (size_t i = 0; i < n; ++i) out[i] = (double)t[i].x + (double)t[i].y;
            return LEM_OK;
        }
        default: {
            float* src = float_field(h, f);
            if (!src) return LEM_ERR_INVALID;
            float* t = static_cast<float*>(h->staging);
            LEM_CUDA_TRY(get2d(t, src + off, 4));
            double* out = static_cast<double*>(host);
            for (size_t i = 0; i < n; ++i) out[i] = t[i];
            return LEM_OK;
        }
    }
}

lem_status totals_from_host(lem_handle* h, int id, lem_totals* o);
lem_status totals_of(lem_handle* h, int id, lem_totals* o) {
    lem_status r = sync_scalars(h);
    if (r != LEM_OK) return r;
    return totals_from_host(h, id, o);
}
// the budget row of DEM id from the host copy of the device scalars
lem_status totals_from_host(lem_handle* h, int id, lem_totals* o) {
    const DevScalars& g = *h->host_sc;
    const DemOut& d = h->host_out[id];
    std::memset(o, 0, sizeof *o);
    o->tot_e = d.tot_e;
    o->tot_i = d.tot_i;
    o->tot_g = d.tot_g;
    o->tot_d = d.tot_d;
    o->tot_weather_c = d.tot_wc;
    o->tot_weather_p = d.tot_wp;
    o->tot_bio = d.tot_bio;
    {
        // FA_max from its ordered key (the hi and lo words are ordered fp32 keys)
        auto unkey = [](uint32_t k) {
            uint32_t b = (k >> 31) ? (k & 0x7fffffffu) : ~k;
            float f;
            std::memcpy(&f, &b, 4);
            return f;
        };
        const unsigned long long fk = d.fa_max_key;
        double v = fk ? (double)unkey((uint32_t)(fk >> 32)) + (double)unkey((uint32_t)fk) : 0.0;
        o->fa_max = v > 0.0 ? v : 0.0;
    }
    const HostDem& hd = h->dems[id];
    o->rain = hd.rain;
    o->temp = hd.temp;
    o->sinkcount = d.sinkcount;
    // the outlet as an index of the DEM's own grid
    o->outlet = (int32_t)(((int64_t)d.outlet / h->k.W - hd.y0) * hd.w + ((int64_t)d.outlet % h->k.W - hd.x0));
    o->initial_sinks = d.sink_counter;
    o->initial_flats = d.flat_counter;
    o->plateau_sweeps = g.plateau_sweeps;
    o->flood_edges = g.n_edges;
    o->fa_uncomputed = d.n_active - d.fa_done;
    o->sed_uncomputed = d.n_active - d.sed_done;
    o->merge_rounds = g.flood_sweeps;
    o->label_rounds = g.label_rounds;
    o->spill_rounds = g.spill_rounds;
    return LEM_OK;
}

lem_status set_climate(HostDem& r, const lem_climate* c) {
    if (c->recompute) {
        r.rain = c->rain;
        r.temp = c->temp;
        r.from_current = true;
    } else if (r.from_current) {
        return LEM_ERR_STATE;
    }
    return LEM_OK;
}

}  // namespace

extern "C" {

const char* lem_status_string(lem_status s) {
    switch (s) {
        case LEM_OK: return "ok";
        case LEM_ERR_INVALID: return "invalid argument";
        case LEM_ERR_CAPACITY: return "capacity exceeded";
        case LEM_ERR_NOCONVERGE: return "iteration cap reached";
        case LEM_ERR_CUDA: return g_last_error.empty() ? "CUDA error" : g_last_error.c_str();
        case LEM_ERR_NOMEM: return "out of memory";
        case LEM_ERR_STATE: return "call out of order";
    }
    return "unknown status";
}

}  // extern "C"

namespace {

lem_status create_common(const lem_grid_desc* grid, const lem_params* params, int max_dems, bool batch,
                         lem_handle** out) {
    if (!grid || !params || !out) return LEM_ERR_INVALID;
    *out = nullptr;
    if (grid->width < 1 || grid->height < 1 || !(grid->cellsize > 0)) return LEM_ERR_INVALID;
    const size_t N = (size_t)grid->width * grid->height;
    if (N >= (size_t)0x7ffffff0) return LEM_ERR_INVALID;  // int32 cell indices
    if ((int)grid->cellsize < 1) return LEM_ERR_INVALID;
    if (max_dems < 1 || max_dems >= (int)kNoDem) return LEM_ERR_INVALID;
    lem_handle* h = new lem_handle();
    h->N = N;
    h->p = *params;
    h->batch = batch;
    h->dems.resize(max_dems);
    // mfd_accum.cu:406-407 clamps the travel distances before the first use
    if (h->p.ddk > 0.95) h->p.ddk = 0.95;
    if (h->p.dck > 0.9) h->p.dck = 0.9;
    cudaGetDevice(&h->device);
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete h;
        return cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__);
    }
    ModelConsts& k = h->k;
    k.W = grid->width;
    k.H = grid->height;
    k.csize = (int)grid->cellsize;
    k.flow_type = params->flow_direction_type;
    k.mfd_props = params->mfd_proportions;
    k.soil_struct = params->soil_struct;
    k.profile_permeability = params->profile_permeability;
    for (int d = 0; d < 8; ++d) {
        const float L = (float)k.csize * ((d % 2 == 0) ? 1.0f : 1.41f);  // newflow.cu:108-117
        k.len[d] = (double)L;
        k.inv_len[d] = (float)(1.0 / (double)L);
    }
    const double cs = grid->cellsize;
    k.q_threshold = (float)h->p.q_threshold;
    k.g_slope = (float)h->p.g_slope;
    k.kappa = (float)h->p.kappa;
    k.g_flowlim = (float)h->p.g_flowlim;
    k.flow_a = (float)h->p.flow_a;
    k.flow_b = (float)h->p.flow_b;
    k.max_incision = (float)h->p.max_incision;
    k.ddk = (float)h->p.ddk;
    k.dck = (float)h->p.dck;
    k.dgk = (float)h->p.dgk;
    k.temp_inflex = (float)h->p.temp_inflex;
    k.temp_sens = (float)h->p.temp_sens;
    k.rescale_conc = (float)(1 / (10000 / (cs * cs)));
    k.rescale_conc_lo = (float)((1 / (10000 / (cs * cs))) - (double)k.rescale_conc);
    k.q_threshold_lo = (float)(h->p.q_threshold - (double)k.q_threshold);
    k.g_flowlim_lo = (float)(h->p.g_flowlim - (double)k.g_flowlim);
    k.rescale_weather = (float)(10000 * (10000 / (cs * cs)));
    k.rescale_veg = (float)(10000 / (cs * cs));
    k.erod_const = (float)((0.043 * (params->soil_struct - 2.)) + (0.033 * (params->profile_permeability - 3.)));

    DevState& s = h->s;
    lem_status r = LEM_OK;
#define ALLOC(ptr, n)                             \
    if ((r = dalloc(h, &(ptr), (n))) != LEM_OK) { \
        lem_destroy(h);                           \
        return r;                                 \
    }
    ALLOC(s.z, N);
    ALLOC(s.zf, N);
    ALLOC(s.z_init, N);
    ALLOC(s.mask, N);
    ALLOC(s.slopes, 8 * N);
    ALLOC(s.sfd, N);
    ALLOC(s.mfd, N);
    ALLOC(s.fd, N);
    ALLOC(s.sfd1, N);
    ALLOC(s.sp, N);
    ALLOC(s.ws, N);
    ALLOC(s.pending, N);
    ALLOC(s.list_a, N);
    ALLOC(s.list_b, N);
    ALLOC(s.mark, N);
    ALLOC(s.eqm, N);
    {
        const int64_t ptiles = (int64_t)((k.W + 31) / 32) * ((k.H + 31) / 32);  // plateau tiles (32x32)
        s.tq_cap = (int32_t)(2 * ptiles + 32);
        ALLOC(s.tq, 2 * (size_t)s.tq_cap);
    }
    ALLOC(s.fa, N);
    ALLOC(s.w, N);
    ALLOC(s.slopeptr, N);
    ALLOC(s.stone, N);
    ALLOC(s.fines, N);
    ALLOC(s.soilT, N);
    ALLOC(s.soilM, N);
    ALLOC(s.soilB, N);
    ALLOC(s.nut, N);
    ALLOC(s.totB, N);
    ALLOC(s.ero, N);
    ALLOC(s.inci, N);
    ALLOC(s.geli, N);
    ALLOC(s.depo, N);
    ALLOC(s.dz, N);
    ALLOC(s.wc, N);
    ALLOC(s.wp, N);
    ALLOC(s.contrib, N);
    ALLOC(s.t_dst, N);
    ALLOC(s.t_pend, N);
    ALLOC(s.t_orng, N);
    ALLOC(s.t_la, N);
    {
        const size_t tiles = (size_t)((grid->width + kTile - 1) / kTile) * ((grid->height + kTile - 1) / kTile);
        ALLOC(s.t_ent, tiles * kTileEnt);
        ALLOC(s.p_abc, tiles * kTile * kTile);
        ALLOC(s.p_ref, tiles * kTilePool);
        ALLOC(s.p_map, tiles * kTilePool);
        ALLOC(s.p_val, tiles * kTile * kTile);
        ALLOC(s.f_idx, tiles * kTile * kTile);
        ALLOC(s.f_map, tiles * kTile * kTile);
        ALLOC(s.f_ds, tiles * kTile * kTile);
        ALLOC(s.t_fcnt, tiles);
        ALLOC(s.n_meta, tiles * kTile * kTile);
    }
    ALLOC(s.t_stat, N);
    if (params->flow_direction_type != 0 && params->mfd_proportions) {
        ALLOC(s.prop, 8 * N);
    }
    int64_t cap = 1024;
    while (cap < (int64_t)(N / 2)) cap <<= 1;
    s.ecap = cap;
    ALLOC(s.ekey, (size_t)cap);
    ALLOC(s.ewt, (size_t)cap);
    ALLOC(s.edge_a, (size_t)cap);
    ALLOC(s.edge_b, (size_t)cap);
    ALLOC(s.edge_w, (size_t)cap);
    ALLOC(s.raise, N + 1);
    ALLOC(s.label_seen, N + 1);
    ALLOC(s.comp, N + 1);
    ALLOC(s.cdist, N + 1);
    ALLOC(s.cmaxw, N + 1);
    ALLOC(s.bid, N + 1);
    ALLOC(s.blab, N + 1);
    ALLOC(s.boff, N + 2);
    ALLOC(s.bdist, N + 1);
    ALLOC(s.adj_v, 2 * (size_t)cap);
    ALLOC(s.sc, 1);
    ALLOC(s.temp_tab, (size_t)kTabN);
    ALLOC(h->dem_in, (size_t)max_dems);
    ALLOC(h->dem_out, (size_t)max_dems);
    ALLOC(h->chunks, (size_t)max_dems + 1);
    if (batch) {
        ALLOC(h->dem_of, N);
        ALLOC(h->live, (size_t)((grid->width + kTile - 1) / kTile) * ((grid->height + kTile - 1) / kTile));
    }
#undef ALLOC
    s.chunk_start = h->chunks;
    s.dems = DemCtx{h->dem_of, h->dem_in, h->dem_out, max_dems};
    s.live = nullptr;  // a single grid visits every tile; a batch lists its DEMs' tiles before each stage
    s.n_live = (int32_t)(((grid->width + kTile - 1) / kTile) * ((grid->height + kTile - 1) / kTile));
    std::vector<float> tab;
    dreybrodt_table(tab);
    e = cudaMemcpyAsync(s.temp_tab, tab.data(), sizeof(float) * kTabN, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = cudaMallocHost(&h->host_sc, sizeof(DevScalars));
    if (e == cudaSuccess) e = cudaMallocHost(&h->host_out, sizeof(DemOut) * max_dems);
    if (e != cudaSuccess) {
        lem_destroy(h);
        return LEM_ERR_NOMEM;
    }
    std::memset(h->host_sc, 0, sizeof(DevScalars));
    h->host_sc->round_id = 1;
    std::memset(h->host_out, 0, sizeof(DemOut) * max_dems);
    e = cudaMemcpyAsync(s.sc, h->host_sc, sizeof(DevScalars), cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess && batch) {
        // a batch grid starts as nodata outside every DEM
        const int blocks = (int)std::min<size_t>((N + 255) / 256, 152 * 32);
        k_fill_f64<<<blocks, 256, 0, h->st>>>(s.z, N, kNoData);
        k_fill_f64<<<blocks, 256, 0, h->st>>>(s.z_init, N, kNoData);
        k_fill_f64<<<blocks, 256, 0, h->st>>>(s.zf, N, kNoData);
        k_fill_u16<<<blocks, 256, 0, h->st>>>(h->dem_of, N, kNoDem);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemsetAsync(s.sfd, kMaskedCode, N, h->st);
        if (e == cudaSuccess) e = cudaMemsetAsync(s.mfd, kMaskedCode, N, h->st);
        if (e == cudaSuccess) e = cudaMemsetAsync(s.fd, kMaskedCode, N, h->st);
        if (e == cudaSuccess) e = cudaMemsetAsync(s.sfd1, kMaskedCode, N, h->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) {
        lem_destroy(h);
        return cuda_fail(e, "initial upload", __FILE__, __LINE__);
    }
    int blocks = 1 << 30;
    for (int i = 0; i < fd_coop_kernel_count; ++i) blocks = std::min(blocks, coop_blocks_for(fd_coop_kernels[i], 256, 0));
    for (int i = 0; i < fa_coop_kernel_count; ++i) blocks = std::min(blocks, coop_blocks_for(fa_coop_kernels[i], 256, 0));
    for (int i = 0; i < mod_coop_kernel_count; ++i) blocks = std::min(blocks, coop_blocks_for(mod_coop_kernels[i], 256, 0));
    s.max_coop_blocks = blocks;
    // each cooperative kernel's own co-residency bounds its launches (the
    // kernel arrays of the three files, in CoopKernel order)
    const void* const coop_fn[kCoopKernels] = {fd_coop_kernels[0], fd_coop_kernels[1], fd_coop_kernels[2],
                                               fd_coop_kernels[3], fa_coop_kernels[1], fa_coop_kernels[0],
                                               mod_coop_kernels[1], mod_coop_kernels[0]};
    for (int i = 0; i < kCoopKernels; ++i) {
        s.coop_cap[i] = coop_blocks_for(coop_fn[i], 256, 0);
        s.coop_blocks[i] = std::min(s.coop_cap[i], blocks);  // untuned: the blocks every one of them can hold
    }
    cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device);
    // the flow-direction tiles move by TMA where the grid's rows allow it
    s.fd_tma = nullptr;
    s.fd_rows = kTuneFdShape[kTuneDefault];
    if (fd_tma_setup(s, k, &h->fd_maps) == LEM_OK) s.fd_tma = &h->fd_maps;
    cudaGetLastError();  // a grid the maps cannot describe keeps the plain-load kernel
    *out = h;
    return LEM_OK;
}

// Per-kernel launches and device ms recorded since the last collection.
lem_status profile_collect(lem_handle* h, std::vector<lem_kernel_stat>& agg) {
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    agg.clear();
    for (const Profiler::Rec& r : h->prof.recs) {
        float ms = 0.f;
        LEM_CUDA_TRY(cudaEventElapsedTime(&ms, h->prof.pool[r.a], h->prof.pool[r.b]));
        size_t j = 0;
        while (j < agg.size() && std::strncmp(agg[j].name, r.name, sizeof(agg[j].name)) != 0) ++j;
        if (j == agg.size()) {
            lem_kernel_stat z{};
            std::strncpy(z.name, r.name, sizeof(z.name) - 1);
            agg.push_back(z);
        }
        agg[j].launches += 1;
        agg[j].total_ms += ms;
    }
    h->prof.recs.clear();
    h->prof.used = 0;
    return LEM_OK;
}

int coop_blocks_of(const lem_handle* h, int kernel, int cand) {
    const int cap = h->s.coop_cap[kernel];
    if (cand == kTuneDefault) return std::min(cap, h->s.max_coop_blocks);
    return kTuneBlocksPerSm[cand] == 0 ? cap : std::max(1, std::min(cap, kTuneBlocksPerSm[cand] * h->sms));
}

// The schedule of the tuner's current step.
void tune_apply(lem_handle* h) {
    const Tuner& t = h->tune;
    const int c = t.step < 0 ? kTuneDefault : t.step % kTuneCands;
    for (int i = 0; i < kCoopKernels; ++i) h->s.coop_blocks[i] = coop_blocks_of(h, i, c);
    h->s.fd_rows = kTuneFdShape[c];
}

// Books the kernel times of a tuning step; after the last one, keeps for every
// cooperative kernel its fastest block count (the default unless another is
// clearly faster).
lem_status tune_record(lem_handle* h) {
    Tuner& t = h->tune;
    std::vector<lem_kernel_stat> agg;
    lem_status r = profile_collect(h, agg);
    if (r != LEM_OK) return r;
    if (t.step >= 0) {
        const int c = t.step % kTuneCands;
        for (const lem_kernel_stat& st : agg) {
            for (int i = 0; i < kCoopKernels; ++i)
                if (!std::strcmp(st.name, kCoopNames[i])) t.coop_ms[i][c] += st.total_ms;
            if (!std::strcmp(st.name, "k_flowdirs")) t.fd_ms[c] += st.total_ms;
        }
        t.coop_n[c] += 1;
    }
    if (++t.step < t.steps) return LEM_OK;
    const int def = kTuneDefault;
    t.default_ms = t.tuned_ms = 0;
    for (int i = 0; i < kCoopKernels; ++i) {
        int best = def;
        for (int c = 0; c < kTuneCands; ++c)
            if (t.coop_ms[i][c] / t.coop_n[c] < t.coop_ms[i][best] / t.coop_n[best]) best = c;
        if (t.coop_ms[i][best] / t.coop_n[best] > kTuneMargin * t.coop_ms[i][def] / t.coop_n[def]) best = def;
        h->s.coop_blocks[i] = coop_blocks_of(h, i, best);
        t.default_ms += t.coop_ms[i][def] / t.coop_n[def];
        t.tuned_ms += t.coop_ms[i][best] / t.coop_n[best];
    }
    // the flow-direction tile shape: the fastest, unless the default is within the margin
    int fbest = def;
    for (int c = 0; c < kTuneCands; ++c)
        if (t.fd_ms[c] / t.coop_n[c] < t.fd_ms[fbest] / t.coop_n[fbest]) fbest = c;
    if (t.fd_ms[fbest] / t.coop_n[fbest] > kTuneMargin * t.fd_ms[def] / t.coop_n[def]) fbest = def;
    h->s.fd_rows = kTuneFdShape[fbest];
    t.default_ms += t.fd_ms[def] / t.coop_n[def];
    t.tuned_ms += t.fd_ms[fbest] / t.coop_n[fbest];
    t.state = 2;
    h->profiling = false;
    if (h->gexec) {  // captured with other launch arguments
        cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
    }
    return LEM_OK;
}

lem_status run_stage(lem_handle* h, int stage, uint32_t flags) {
    lem_status r = prepare(h);
    if (r != LEM_OK) return r;
    const Launch L = h->launch();
    if (stage == 0) return launch_flow_direction(h->s, h->k, L);
    if (stage == 1) {
        uint32_t f = flags & ~LEM_STEP_SET_OUTLET_FROM_FA;
        if (any_flag(h, LEM_STEP_SET_OUTLET_FROM_FA)) f |= LEM_STEP_SET_OUTLET_FROM_FA;
        return launch_flow_accumulation(h->s, h->k, f, L);
    }
    return launch_erosion(h->s, h->k, flags, L);
}

// A whole timestep as one graph launch.  The per-DEM inputs are uploaded first
// (the kernels read them from device memory); the step's launches are captured
// once per launch configuration (chunk count, visited tiles, step flags) and
// replayed while it holds.  Every loop decision of a step is taken on the
// device, so a replay runs exactly the kernels an eager step runs.
lem_status graph_step(lem_handle* h, uint32_t flags) {
    lem_status r = prepare(h);
    if (r != LEM_OK) return r;
    uint32_t f = flags & ~LEM_STEP_SET_OUTLET_FROM_FA;
    if (any_flag(h, LEM_STEP_SET_OUTLET_FROM_FA)) f |= LEM_STEP_SET_OUTLET_FROM_FA;
    const int32_t key[3] = {h->s.n_chunks, h->s.n_live, (int32_t)f};
    if (!h->gexec || std::memcmp(key, h->gkey, sizeof key) != 0) {
        if (h->gexec) {
            cudaGraphExecDestroy(h->gexec);
            h->gexec = nullptr;
        }
        LEM_CUDA_TRY(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
        uint64_t n = 0;
        const Launch L{h->st, &n, nullptr};
        r = launch_flow_direction(h->s, h->k, L);
        if (r == LEM_OK) r = launch_flow_accumulation(h->s, h->k, f, L);
        if (r == LEM_OK) r = launch_erosion(h->s, h->k, flags, L);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->st, &g);
        if (r != LEM_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return r != LEM_OK ? r : cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
        }
        const cudaError_t ei = cudaGraphInstantiate(&h->gexec, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            h->gexec = nullptr;
            return cuda_fail(ei, "cudaGraphInstantiate", __FILE__, __LINE__);
        }
        std::memcpy(h->gkey, key, sizeof key);
        h->glaunches = n;
    }
    LEM_CUDA_TRY(cudaGraphLaunch(h->gexec, h->st));
    h->launches += h->glaunches;
    return LEM_OK;
}

}  // namespace

extern "C" {

lem_status lem_create(const lem_grid_desc* grid, const lem_params* params, double init_rain, double init_temp,
                      lem_handle** out) {
    lem_status r = create_common(grid, params, 1, false, out);
    if (r != LEM_OK) return r;
    HostDem& d = (*out)->dems[0];
    d.x0 = d.y0 = 0;
    d.w = grid->width;
    d.h = grid->height;
    d.rain = d.rain0 = init_rain;
    d.temp = d.temp0 = init_temp;
    d.outlet_set = true;  // cell 0 until lem_set_outlet
    return LEM_OK;
}

lem_status lem_destroy(lem_handle* h) {
    if (!h) return LEM_ERR_INVALID;
    if (h->exports) return LEM_ERR_STATE;  // wait for every export first
    if (h->st) cudaStreamSynchronize(h->st);
    if (h->side) {
        cudaStreamSynchronize(h->side);
        cudaStreamDestroy(h->side);
    }
    for (auto& b : h->pinned_free) cudaFreeHost(b.first);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    for (cudaEvent_t e : h->prof.pool) cudaEventDestroy(e);
    for (cudaEvent_t e : h->events)
        if (e) cudaEventDestroy(e);
    for (void* q : h->allocs) cudaFree(q);
    if (h->staging) cudaFreeHost(h->staging);
    if (h->host_sc) cudaFreeHost(h->host_sc);
    if (h->host_out) cudaFreeHost(h->host_out);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
    return LEM_OK;
}

lem_status lem_set_field(lem_handle* h, lem_field f, const void* host) {
    if (!h || !host || f < 0 || f >= LEM_F_COUNT) return LEM_ERR_INVALID;
    if (h->batch) return LEM_ERR_STATE;
    HostDem& d = h->dems[0];
    lem_status r = set_region_field(h, d, f, host);
    if (r != LEM_OK || f != LEM_F_DEM || h->dem_set) return r;
    // createmask (MEM_kernels/memory.cu:229-238) and the DEM of the initial climate grids
    const double* dem = static_cast<const double*>(host);
    uint8_t* m = static_cast<uint8_t*>(h->staging);
    for (size_t i = 0; i < h->N; ++i) m[i] = (dem[i] == -9999) ? 0 : 1;
    LEM_CUDA_TRY(cudaMemcpyAsync(h->s.mask, m, h->N, cudaMemcpyHostToDevice, h->st));
    LEM_CUDA_TRY(cudaMemcpyAsync(h->s.z_init, dem, sizeof(double) * h->N, cudaMemcpyHostToDevice, h->st));
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    h->dem_set = true;
    d.active = true;
    return LEM_OK;
}

lem_status lem_get_field(lem_handle* h, lem_field f, void* host) {
    if (!h || !host || f < 0 || f >= LEM_F_COUNT) return LEM_ERR_INVALID;
    if (h->batch) return LEM_ERR_STATE;
    return get_region_field(h, h->dems[0], 0, f, host);
}

lem_status lem_set_outlet(lem_handle* h, int32_t cell) {
    if (!h || cell < 0 || (size_t)cell >= h->N) return LEM_ERR_INVALID;
    if (h->batch) return LEM_ERR_STATE;
    LEM_CUDA_TRY(cudaMemcpyAsync(&h->dem_out[0].outlet, &cell, sizeof(int32_t), cudaMemcpyHostToDevice, h->st));
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    return LEM_OK;
}

lem_status lem_set_climate(lem_handle* h, const lem_climate* c) {
    if (!h || !c) return LEM_ERR_INVALID;
    if (h->batch) return LEM_ERR_STATE;
    return set_climate(h->dems[0], c);
}

lem_status lem_flow_direction(lem_handle* h) {
    if (!h) return LEM_ERR_INVALID;
    if (!h->batch && !h->dem_set) return LEM_ERR_STATE;
    return run_stage(h, 0, 0);
}

lem_status lem_flow_accumulation(lem_handle* h, uint32_t flags) {
    if (!h) return LEM_ERR_INVALID;
    if (!h->batch && !h->dem_set) return LEM_ERR_STATE;
    if (!h->batch) h->dems[0].next_flags = flags;
    lem_status r = run_stage(h, 1, flags);
    if (!h->batch) h->dems[0].next_flags = 0;
    return r;
}

lem_status lem_erosion(lem_handle* h, uint32_t flags) {
    if (!h) return LEM_ERR_INVALID;
    if (!h->batch && !h->dem_set) return LEM_ERR_STATE;
    return run_stage(h, 2, flags);
}

lem_status lem_step(lem_handle* h, const lem_climate* c, uint32_t flags) {
    lem_status r;
    if (!h) return LEM_ERR_INVALID;
    if (c && (r = lem_set_climate(h, c)) != LEM_OK) return r;
    if (h->tune.state == 1) {
        if (h->batch || !h->dem_set) return LEM_ERR_STATE;
        tune_apply(h);
        h->dems[0].next_flags = flags;
        if ((r = run_stage(h, 0, 0)) == LEM_OK && (r = run_stage(h, 1, flags)) == LEM_OK) r = run_stage(h, 2, flags);
        h->dems[0].next_flags = 0;
        return r != LEM_OK ? r : tune_record(h);
    }
    if (h->graphs && !h->profiling) {
        if (h->batch || !h->dem_set) return LEM_ERR_STATE;
        h->dems[0].next_flags = flags;
        r = graph_step(h, flags);
        h->dems[0].next_flags = 0;
        return r;
    }
    if ((r = lem_flow_direction(h)) != LEM_OK) return r;
    if ((r = lem_flow_accumulation(h, flags)) != LEM_OK) return r;
    return lem_erosion(h, flags);
}

lem_status lem_synchronize(lem_handle* h) {
    if (!h) return LEM_ERR_INVALID;
    lem_status r = sync_scalars(h);
    if (r != LEM_OK) return r;
    const uint32_t err = h->host_sc->err, first = h->host_sc->err_first;
    if (err) {
        const uint32_t zero[2] = {0, 0};  // err and err_first
        LEM_CUDA_TRY(cudaMemcpy(&h->s.sc->err, zero, sizeof zero, cudaMemcpyHostToDevice));
        // the first error raised; a later one may be its consequence
        if (first == ErrFlags::kNoConverge) return LEM_ERR_NOCONVERGE;
        if (first == ErrFlags::kCapacity) return LEM_ERR_CAPACITY;
        return (err & ErrFlags::kCapacity) ? LEM_ERR_CAPACITY : LEM_ERR_NOCONVERGE;
    }
    return LEM_OK;
}

lem_status lem_get_totals(lem_handle* h, lem_totals* o) {
    if (!h || !o) return LEM_ERR_INVALID;
    if (h->batch) return LEM_ERR_STATE;
    return totals_of(h, 0, o);
}

// ---- batches

lem_status lem_create_batch(const lem_grid_desc* grid, const lem_params* params, int32_t max_dems,
                            lem_handle** out) {
    if (!grid || grid->width % kTile != 0) return LEM_ERR_INVALID;
    return create_common(grid, params, max_dems, true, out);
}

lem_status lem_dem_add(lem_handle* h, int32_t x0, int32_t y0, int32_t width, int32_t height, const double* dem,
                       double init_rain, double init_temp, int32_t* id) {
    if (!h || !dem || !id || !h->batch) return LEM_ERR_INVALID;
    if (x0 < 0 || y0 < 0 || width < 3 || height < 3 || x0 % kTile || y0 % kTile) return LEM_ERR_INVALID;
    if ((int64_t)x0 + width > h->k.W || (int64_t)y0 + height > h->k.H) return LEM_ERR_INVALID;
    // the tiles a DEM occupies belong to it alone
    auto ext = [](int32_t v) { return (v + kTile - 1) / kTile * kTile; };
    int slot = -1;
    for (int d = 0; d < (int)h->dems.size(); ++d) {
        const HostDem& o = h->dems[d];
        if (!o.active) {
            if (slot < 0) slot = d;
            continue;
        }
        if (x0 < o.x0 + ext(o.w) && o.x0 < x0 + ext(width) && y0 < o.y0 + ext(o.h) && o.y0 < y0 + ext(height))
            return LEM_ERR_INVALID;
    }
    if (slot < 0) return LEM_ERR_CAPACITY;
    // a nodata ring: no in-catchment cell of the DEM has a neighbour outside it
    for (int32_t x = 0; x < width; ++x)
        if (dem[x] != -9999 || dem[(size_t)(height - 1) * width + x] != -9999) return LEM_ERR_INVALID;
    for (int32_t y = 0; y < height; ++y)
        if (dem[(size_t)y * width] != -9999 || dem[(size_t)y * width + width - 1] != -9999) return LEM_ERR_INVALID;
    HostDem& d = h->dems[slot];
    d = HostDem{};
    d.x0 = x0;
    d.y0 = y0;
    d.w = width;
    d.h = height;
    d.rain = d.rain0 = init_rain;
    d.temp = d.temp0 = init_temp;
    lem_status r = set_region_field(h, d, LEM_F_DEM, dem);
    if (r != LEM_OK) return r;
    if ((r = region_op(h, d, slot)) != LEM_OK) return r;
    DemOut zero{};
    zero.lowest_key = ~0ull;
    LEM_CUDA_TRY(cudaMemcpyAsync(&h->dem_out[slot], &zero, sizeof zero, cudaMemcpyHostToDevice, h->st));
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    d.active = true;
    h->live_dirty = true;
    *id = slot;
    return LEM_OK;
}

static lem_status dem_check(lem_handle* h, int32_t id) {
    if (!h || !h->batch || id < 0 || id >= (int32_t)h->dems.size() || !h->dems[id].active) return LEM_ERR_INVALID;
    return LEM_OK;
}

lem_status lem_dem_remove(lem_handle* h, int32_t id) {
    lem_status r = dem_check(h, id);
    if (r != LEM_OK) return r;
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    if ((r = region_op(h, h->dems[id], -1)) != LEM_OK) return r;
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    h->dems[id] = HostDem{};
    h->live_dirty = true;
    return LEM_OK;
}

lem_status lem_dem_set_field(lem_handle* h, int32_t id, lem_field f, const void* host) {
    lem_status r = dem_check(h, id);
    if (r != LEM_OK) return r;
    if (!host || f < 0 || f >= LEM_F_COUNT) return LEM_ERR_INVALID;
    return set_region_field(h, h->dems[id], f, host);
}

lem_status lem_dem_get_field(lem_handle* h, int32_t id, lem_field f, void* host) {
    lem_status r = dem_check(h, id);
    if (r != LEM_OK) return r;
    if (!host || f < 0 || f >= LEM_F_COUNT) return LEM_ERR_INVALID;
    return get_region_field(h, h->dems[id], id, f, host);
}

lem_status lem_dem_set_outlet(lem_handle* h, int32_t id, int32_t cell) {
    lem_status r = dem_check(h, id);
    if (r != LEM_OK) return r;
    HostDem& d = h->dems[id];
    if (cell < 0 || cell >= d.w * d.h) return LEM_ERR_INVALID;
    const int32_t g = (d.y0 + cell / d.w) * h->k.W + d.x0 + cell % d.w;
    LEM_CUDA_TRY(cudaMemcpyAsync(&h->dem_out[id].outlet, &g, sizeof g, cudaMemcpyHostToDevice, h->st));
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    d.outlet_set = true;
    return LEM_OK;
}

lem_status lem_dem_set_climate(lem_handle* h, int32_t id, const lem_climate* c) {
    lem_status r = dem_check(h, id);
    if (r != LEM_OK) return r;
    if (!c) return LEM_ERR_INVALID;
    return set_climate(h->dems[id], c);
}

lem_status lem_dem_set_step_flags(lem_handle* h, int32_t id, uint32_t flags) {
    lem_status r = dem_check(h, id);
    if (r != LEM_OK) return r;
    h->dems[id].next_flags = flags;
    return LEM_OK;
}

lem_status lem_dem_get_totals(lem_handle* h, int32_t id, lem_totals* out) {
    lem_status r = dem_check(h, id);
    if (r != LEM_OK) return r;
    if (!out) return LEM_ERR_INVALID;
    return totals_of(h, id, out);
}

lem_status lem_dem_get_totals_n(lem_handle* h, const int32_t* ids, int32_t n, lem_totals* out) {
    if (n < 0 || (n > 0 && (!ids || !out))) return LEM_ERR_INVALID;
    for (int32_t k = 0; k < n; ++k) {
        const lem_status r = dem_check(h, ids[k]);
        if (r != LEM_OK) return r;
    }
    if (n == 0) return LEM_OK;
    lem_status r = totals_of(h, ids[0], out);  // synchronises once
    for (int32_t k = 1; k < n && r == LEM_OK; ++k) r = totals_from_host(h, ids[k], out + k);
    return r;
}

// ---- asynchronous exports of one DEM's fields

namespace {

// Bytes per cell of a field's device representation, or 0 when it cannot be exported.
size_t raw_bytes(lem_field f) {
    switch (f) {
        case LEM_F_DEM: return 8;
        case LEM_F_MASK: case LEM_F_FD: case LEM_F_SFD: case LEM_F_SFD_PASS1: return 1;
        case LEM_F_CONTRIB: case LEM_F_WATERSHED: return 4;
        case LEM_F_SLOPES: return 32;
        case LEM_F_FA: return 8;
        case LEM_F_DEM_ROUTED: return 0;  // which grid holds it depends on the step's sinks
        default: return f >= 0 && f < LEM_F_COUNT ? 4 : 0;
    }
}

const void* raw_source(lem_handle* h, lem_field f) {
    DevState& s = h->s;
    switch (f) {
        case LEM_F_DEM: return s.z;
        case LEM_F_MASK: return s.mask;
        case LEM_F_FD: return s.fd;
        case LEM_F_SFD: return s.sfd;
        case LEM_F_SFD_PASS1: return s.sfd1;
        case LEM_F_CONTRIB: return s.contrib;
        case LEM_F_WATERSHED: return s.ws;
        case LEM_F_SLOPES: return s.slopes;
        case LEM_F_FA: return s.fa;
        default: return float_field(h, f);
    }
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

lem_status lem_dem_export(lem_handle* h, int32_t id, const lem_field* fields, int32_t nfields, lem_export** out) {
    if (!h || !fields || nfields < 1 || !out) return LEM_ERR_INVALID;
    *out = nullptr;
    if (h->batch) {
        if (dem_check(h, id) != LEM_OK) return LEM_ERR_INVALID;
    } else if (id != 0 || !h->dem_set) {
        return LEM_ERR_INVALID;
    }
    const HostDem& r = h->dems[id];
    const size_t n = (size_t)r.w * r.h, W = (size_t)h->k.W, cell0 = (size_t)r.y0 * W + r.x0;
    lem_export* e = new lem_export();
    e->h = h;
    e->x0 = r.x0;
    e->y0 = r.y0;
    e->w = r.w;
    e->hgt = r.h;
    bool codes = false;
    for (int32_t k = 0; k < nfields; ++k) {
        const size_t b = raw_bytes(fields[k]);
        if (!b || !raw_source(h, fields[k])) {
            delete e;
            return LEM_ERR_INVALID;
        }
        codes |= fields[k] == LEM_F_FD || fields[k] == LEM_F_SFD || fields[k] == LEM_F_SFD_PASS1;
        e->fields.push_back(fields[k]);
        e->off.push_back(e->bytes);
        e->bytes = align256(e->bytes + n * b);
    }
    e->mask_off = e->bytes;  // the mask gives codes outside the catchment their -9999
    if (codes) e->bytes = align256(e->bytes + n);
    e->out_off = e->bytes;
    e->bytes = align256(e->bytes + sizeof(DemOut));
    lem_status st = LEM_OK;
    void* dstage = nullptr;
    auto fail = [&](lem_status x) {
        if (e->done) cudaEventDestroy(e->done);
        if (e->host) h->pinned_free.emplace_back(e->host, e->host_cap);
        delete e;
        return x;
    };
    // pinned host staging, reused from earlier exports: the smallest free
    // buffer that is large enough (exports of DEMs of many sizes keep theirs)
    size_t best = h->pinned_free.size();
    for (size_t k = 0; k < h->pinned_free.size(); ++k)
        if (h->pinned_free[k].second >= e->bytes &&
            (best == h->pinned_free.size() || h->pinned_free[k].second < h->pinned_free[best].second))
            best = k;
    if (best < h->pinned_free.size()) {
        e->host = h->pinned_free[best].first;
        e->host_cap = h->pinned_free[best].second;
        h->pinned_free.erase(h->pinned_free.begin() + best);
    }
    if (!e->host) {
        if (cudaHostAlloc(&e->host, e->bytes, cudaHostAllocDefault) != cudaSuccess) return fail(LEM_ERR_NOMEM);
        e->host_cap = e->bytes;
    }
    if (!h->side && cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "cudaStreamCreate", __FILE__, __LINE__));
    cudaEvent_t copied = nullptr;
    cudaError_t ce = cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&copied, cudaEventDisableTiming);
    // a snapshot on the handle's stream (ordered after the steps enqueued so far,
    // and before any later step or removal touches the region) ...
    if (ce == cudaSuccess) ce = cudaMallocAsync(&dstage, e->bytes, h->st);
    for (size_t k = 0; ce == cudaSuccess && k < e->fields.size(); ++k) {
        const size_t b = raw_bytes(e->fields[k]);
        const char* src = static_cast<const char*>(raw_source(h, e->fields[k])) + cell0 * b;
        ce = cudaMemcpy2DAsync(static_cast<char*>(dstage) + e->off[k], r.w * b, src, W * b, r.w * b, r.h,
                               cudaMemcpyDeviceToDevice, h->st);
    }
    if (ce == cudaSuccess && codes)
        ce = cudaMemcpy2DAsync(static_cast<char*>(dstage) + e->mask_off, r.w, h->s.mask + cell0, W, r.w, r.h,
                               cudaMemcpyDeviceToDevice, h->st);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(static_cast<char*>(dstage) + e->out_off, h->dem_out + id, sizeof(DemOut),
                             cudaMemcpyDeviceToDevice, h->st);
    if (ce == cudaSuccess) ce = cudaEventRecord(copied, h->st);
    // ... then the device-to-host copy on the side stream, overlapping later steps
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(h->side, copied, 0);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(e->host, dstage, e->bytes, cudaMemcpyDeviceToHost, h->side);
    if (ce == cudaSuccess) ce = cudaFreeAsync(dstage, h->side);
    if (ce == cudaSuccess) ce = cudaEventRecord(e->done, h->side);
    if (copied) cudaEventDestroy(copied);  // released once its record completes
    if (ce != cudaSuccess) {
        st = cuda_fail(ce, "lem_dem_export", __FILE__, __LINE__);
        if (e->done) cudaEventSynchronize(e->done);
        cudaStreamSynchronize(h->side);
        return fail(st);
    }
    ++h->exports;
    *out = e;
    return LEM_OK;
}

lem_status lem_export_ready(lem_export* e, int32_t* ready) {
    if (!e || !ready) return LEM_ERR_INVALID;
    const cudaError_t q = cudaEventQuery(e->done);
    if (q == cudaErrorNotReady) {
        *ready = 0;
        return LEM_OK;
    }
    if (q != cudaSuccess) return cuda_fail(q, "cudaEventQuery", __FILE__, __LINE__);
    *ready = 1;
    return LEM_OK;
}

lem_status lem_export_wait(lem_export* e, void* const* host) {
    if (!e || !host) return LEM_ERR_INVALID;
    lem_handle* h = e->h;
    const cudaError_t ce = cudaEventSynchronize(e->done);
    lem_status st = ce == cudaSuccess ? LEM_OK : cuda_fail(ce, "cudaEventSynchronize", __FILE__, __LINE__);
    const size_t n = (size_t)e->w * e->hgt;
    const char* base = static_cast<const char*>(e->host);
    if (st == LEM_OK) {
        // the outlet (a grid cell in the staged DemOut) as an index of the DEM's own grid
        DemOut o;
        std::memcpy(&o, base + e->out_off, sizeof o);
        const int64_t W = h->k.W;
        const int64_t ol = ((int64_t)o.outlet / W - e->y0) * e->w + ((int64_t)o.outlet % W - e->x0);
        for (size_t k = 0; k < e->fields.size(); ++k) {
            const lem_field f = e->fields[k];
            const char* src = base + e->off[k];
            if (!host[k]) continue;
            switch (f) {
                case LEM_F_DEM:
                    std::memcpy(host[k], src, n * 8);
                    break;
                case LEM_F_MASK: {
                    int32_t* out = static_cast<int32_t*>(host[k]);
                    for (size_t i = 0; i < n; ++i) out[i] = static_cast<const uint8_t*>((const void*)src)[i];
                    break;
                }
                case LEM_F_FD:
                case LEM_F_SFD:
                case LEM_F_SFD_PASS1: {
                    const uint8_t* c = reinterpret_cast<const uint8_t*>(src);
                    const uint8_t* m = reinterpret_cast<const uint8_t*>(base + e->mask_off);
                    int32_t* out = static_cast<int32_t*>(host[k]);
                    for (size_t i = 0; i < n; ++i) {
                        int32_t v = m[i] ? (int32_t)c[i] : -9999;          // newflow.cu:74
                        if (f == LEM_F_FD && (int64_t)i == ol) v = 16;     // routeflow.cu:953
                        out[i] = v;
                    }
                    break;
                }
                case LEM_F_CONTRIB:
                case LEM_F_WATERSHED:
                    std::memcpy(host[k], src, n * 4);
                    break;
                case LEM_F_SLOPES: {
                    const float* t = reinterpret_cast<const float*>(src);
                    double* out = static_cast<double*>(host[k]);
                    for (size_t i = 0; i < 8 * n; ++i) out[i] = t[i];
                    break;
                }
                case LEM_F_FA: {
                    const float2* t = reinterpret_cast<const float2*>(src);
                    double* out = static_cast<double*>(host[k]);
                    for (size_t i = 0; i < n; ++i) out[i] = (double)t[i].x + (double)t[i].y;
                    break;
                }
                default: {
                    const float* t = reinterpret_cast<const float*>(src);
                    double* out = static_cast<double*>(host[k]);
                    for (size_t i = 0; i < n; ++i) out[i] = t[i];
                    break;
                }
            }
        }
    }
    cudaEventDestroy(e->done);
    h->pinned_free.emplace_back(e->host, e->host_cap);
    --h->exports;
    delete e;
    return st;
}

size_t lem_device_bytes(lem_handle* h) { return h ? h->device_bytes : 0; }

// ---- restart snapshots of one DEM's resident state

namespace {
struct SnapHeader {
    uint32_t magic, version;
    int32_t w, h;
    double rain, temp, rain0, temp0;
    int32_t from_current, outlet;  // outlet: index of the DEM's own grid
    uint32_t pad[2];
};
constexpr uint32_t kSnapMagic = 0x534d454cu;  // "LEMS"
struct SnapField {
    void* dev;
    size_t elem;  // bytes per cell
};
void snap_fields(lem_handle* h, SnapField* f) {
    DevState& s = h->s;
    f[0] = {s.z, 8};
    f[1] = {s.z_init, 8};
    f[2] = {s.mask, 1};
    f[3] = {s.slopes, 32};
    f[4] = {s.stone, 4};
    f[5] = {s.fines, 4};
    f[6] = {s.soilT, 4};
    f[7] = {s.soilM, 4};
    f[8] = {s.soilB, 4};
    f[9] = {s.nut, 4};
    f[10] = {s.totB, 4};
}
constexpr int kSnapFields = 11;
size_t snap_bytes(const HostDem& r) { return sizeof(SnapHeader) + (size_t)r.w * r.h * (8 + 8 + 1 + 32 + 7 * 4); }
lem_status snap_target(lem_handle* h, int32_t id, HostDem** r) {
    if (!h) return LEM_ERR_INVALID;
    if (h->batch) {
        lem_status st = dem_check(h, id);
        if (st != LEM_OK) return st;
    } else if (id != 0) {
        return LEM_ERR_INVALID;
    }
    *r = &h->dems[id];
    return LEM_OK;
}
}  // namespace

size_t lem_snapshot_bytes(lem_handle* h, int32_t id) {
    HostDem* r = nullptr;
    if (snap_target(h, id, &r) != LEM_OK) return 0;
    return snap_bytes(*r);
}

lem_status lem_snapshot_save(lem_handle* h, int32_t id, void* host, size_t bytes) {
    HostDem* r = nullptr;
    lem_status st = snap_target(h, id, &r);
    if (st != LEM_OK) return st;
    if (!host || bytes < snap_bytes(*r)) return LEM_ERR_INVALID;
    if (!h->batch && !h->dem_set) return LEM_ERR_STATE;
    if ((st = sync_scalars(h)) != LEM_OK) return st;
    SnapHeader hd{};
    hd.magic = kSnapMagic;
    hd.version = 1;
    hd.w = r->w;
    hd.h = r->h;
    hd.rain = r->rain;
    hd.temp = r->temp;
    hd.rain0 = r->rain0;
    hd.temp0 = r->temp0;
    hd.from_current = r->from_current ? 1 : 0;
    const int64_t o = h->host_out[id].outlet;
    hd.outlet = (int32_t)((o / h->k.W - r->y0) * r->w + (o % h->k.W - r->x0));
    unsigned char* p = static_cast<unsigned char*>(host);
    std::memcpy(p, &hd, sizeof hd);
    p += sizeof hd;
    SnapField f[kSnapFields];
    snap_fields(h, f);
    const size_t W = (size_t)h->k.W, off = (size_t)r->y0 * W + r->x0;
    for (const SnapField& q : f) {
        const unsigned char* src = static_cast<const unsigned char*>(q.dev) + off * q.elem;
        LEM_CUDA_TRY(cudaMemcpy2D(p, r->w * q.elem, src, W * q.elem, r->w * q.elem, r->h, cudaMemcpyDeviceToHost));
        p += (size_t)r->w * r->h * q.elem;
    }
    return LEM_OK;
}

lem_status lem_snapshot_load(lem_handle* h, int32_t id, const void* host, size_t bytes) {
    HostDem* r = nullptr;
    lem_status st = snap_target(h, id, &r);
    if (st != LEM_OK) return st;
    if (!host || bytes < sizeof(SnapHeader)) return LEM_ERR_INVALID;
    SnapHeader hd;
    std::memcpy(&hd, host, sizeof hd);
    if (hd.magic != kSnapMagic || hd.version != 1 || hd.w != r->w || hd.h != r->h || bytes < snap_bytes(*r) ||
        hd.outlet < 0 || hd.outlet >= r->w * r->h)
        return LEM_ERR_INVALID;
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    const unsigned char* p = static_cast<const unsigned char*>(host) + sizeof hd;
    SnapField f[kSnapFields];
    snap_fields(h, f);
    const size_t W = (size_t)h->k.W, off = (size_t)r->y0 * W + r->x0;
    for (const SnapField& q : f) {
        unsigned char* dst = static_cast<unsigned char*>(q.dev) + off * q.elem;
        LEM_CUDA_TRY(cudaMemcpy2D(dst, W * q.elem, p, r->w * q.elem, r->w * q.elem, r->h, cudaMemcpyHostToDevice));
        p += (size_t)r->w * r->h * q.elem;
    }
    r->rain = hd.rain;
    r->temp = hd.temp;
    r->rain0 = hd.rain0;
    r->temp0 = hd.temp0;
    r->from_current = hd.from_current != 0;
    const int32_t g = (r->y0 + hd.outlet / r->w) * h->k.W + r->x0 + hd.outlet % r->w;
    LEM_CUDA_TRY(cudaMemcpy(&h->dem_out[id].outlet, &g, sizeof g, cudaMemcpyHostToDevice));
    r->outlet_set = true;
    if (!h->batch) {
        h->dem_set = true;
        r->active = true;
    }
    return LEM_OK;
}

lem_status lem_step_batch(lem_handle* h, uint32_t flags) {
    if (!h || !h->batch) return LEM_ERR_INVALID;
    lem_status r;
    if (h->tune.state == 1) {
        tune_apply(h);
        if ((r = run_stage(h, 0, 0)) == LEM_OK && (r = run_stage(h, 1, flags)) == LEM_OK) r = run_stage(h, 2, flags);
        if (r == LEM_OK) r = tune_record(h);
    } else if (h->graphs && !h->profiling) {
        r = graph_step(h, flags);
    } else {
        if ((r = run_stage(h, 0, 0)) != LEM_OK) return r;
        if ((r = run_stage(h, 1, flags)) != LEM_OK) return r;
        r = run_stage(h, 2, flags);
    }
    for (HostDem& d : h->dems) d.next_flags = 0;
    return r;
}

lem_status lem_autotune(lem_handle* h, int32_t cycles) {
    if (!h || cycles < 1 || cycles > 1000) return LEM_ERR_INVALID;
    if (h->profiling || h->tune.state == 1) return LEM_ERR_STATE;
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    h->tune = Tuner{};
    h->tune.state = 1;
    h->tune.steps = kTuneCands * cycles;
    h->profiling = true;  // the tuning steps time every kernel
    h->prof.recs.clear();
    h->prof.used = 0;
    return LEM_OK;
}

lem_status lem_get_tuning(lem_handle* h, lem_tuning* out) {
    if (!h || !out) return LEM_ERR_INVALID;
    std::memset(out, 0, sizeof *out);
    out->state = h->tune.state;
    out->steps_left = h->tune.state == 1 ? h->tune.steps - h->tune.step : 0;
    for (int i = 0; i < kCoopKernels; ++i) out->coop_blocks[i] = h->s.coop_blocks[i];
    out->default_ms = h->tune.default_ms;
    out->tuned_ms = h->tune.tuned_ms;
    out->flowdirs_tile_rows = h->s.fd_tma ? kFdRows[h->s.fd_rows] : 0;
    return LEM_OK;
}

lem_status lem_set_graphs(lem_handle* h, int32_t on) {
    if (!h) return LEM_ERR_INVALID;
    h->graphs = on != 0;
    if (!h->graphs && h->gexec) {
        LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
        cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
    }
    return LEM_OK;
}

lem_status lem_set_limits(lem_handle* h, const lem_limits* l) {
    if (!h || !l || l->max_rounds < 0 || l->edge_table_log2 < 0 || l->edge_table_log2 > 40) return LEM_ERR_INVALID;
    static_assert(offsetof(DevScalars, edge_log_cap) == offsetof(DevScalars, round_cap) + sizeof(int32_t),
                  "the two limits are adjacent");
    const int32_t v[2] = {l->max_rounds, l->edge_table_log2};
    LEM_CUDA_TRY(cudaMemcpyAsync(&h->s.sc->round_cap, v, sizeof v, cudaMemcpyHostToDevice, h->st));
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    return LEM_OK;
}

void* lem_stream(lem_handle* h) { return h ? (void*)h->st : nullptr; }

lem_status lem_select_device(int32_t device) {
    LEM_CUDA_TRY(cudaSetDevice(device));
    return LEM_OK;
}

lem_status lem_event_record(lem_handle* h, int32_t slot) {
    if (!h || slot < 0 || slot >= 16) return LEM_ERR_INVALID;
    if (!h->events[slot]) LEM_CUDA_TRY(cudaEventCreate(&h->events[slot]));
    LEM_CUDA_TRY(cudaEventRecord(h->events[slot], h->st));
    return LEM_OK;
}

lem_status lem_event_elapsed(lem_handle* h, int32_t from, int32_t to, float* ms) {
    if (!h || !ms || from < 0 || from >= 16 || to < 0 || to >= 16 || !h->events[from] || !h->events[to])
        return LEM_ERR_INVALID;
    LEM_CUDA_TRY(cudaEventSynchronize(h->events[to]));
    LEM_CUDA_TRY(cudaEventElapsedTime(ms, h->events[from], h->events[to]));
    return LEM_OK;
}

lem_status lem_set_profiling(lem_handle* h, int32_t on) {
    if (!h) return LEM_ERR_INVALID;
    if (h->tune.state == 1) return LEM_ERR_STATE;
    LEM_CUDA_TRY(cudaStreamSynchronize(h->st));
    h->profiling = on != 0;
    h->prof.recs.clear();
    h->prof.used = 0;
    return LEM_OK;
}

lem_status lem_profile_read(lem_handle* h, lem_kernel_stat* out, int32_t cap, int32_t* count) {
    if (!h || !count || (cap > 0 && !out)) return LEM_ERR_INVALID;
    if (h->tune.state == 1) return LEM_ERR_STATE;
    std::vector<lem_kernel_stat> agg;
    lem_status r = profile_collect(h, agg);
    if (r != LEM_OK) return r;
    *count = (int32_t)agg.size();
    for (int32_t i = 0; i < cap && i < (int32_t)agg.size(); ++i) out[i] = agg[i];
    return LEM_OK;
}

uint64_t lem_launch_count(lem_handle* h) { return h ? h->launches : 0; }

}  // extern "C"
