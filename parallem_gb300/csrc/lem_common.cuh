// lem_common.cuh -- shared device helpers of the GB300 landscape-evolution path.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/lem_gb300.h"

namespace lem {

// Direction index d = 0..7 is N, NE, E, SE, S, SW, W, NW (routeflow.cu:701-702);
// its MFD bit follows newflow.cu:99-106.
__host__ __device__ constexpr int dir_dx(int d) { return (d == 1 || d == 2 || d == 3) ? 1 : (d == 5 || d == 6 || d == 7) ? -1 : 0; }
__host__ __device__ constexpr int dir_dy(int d) { return (d == 0 || d == 1 || d == 7) ? -1 : (d == 3 || d == 4 || d == 5) ? 1 : 0; }
__host__ __device__ constexpr uint32_t dir_bit(int d) { return d == 0 ? 64u : d == 1 ? 128u : (1u << (d - 2)); }
// direction index of a single-bit code (bit b of the byte maps to d = (b + 2) % 8)
__host__ __device__ inline int bit_dir(uint32_t code) {
    if (code == 0 || (code & (code - 1))) return -1;
#ifdef __CUDA_ARCH__
    const int b = __ffs((int)code) - 1;
#else
    const int b = __builtin_ctz(code);
#endif
    return (b + 2) & 7;
}
// Donor scan order of CalcMFD / MFDsedbud (mfd_simple.cu:95-165): neighbours E, SE,
// S, SW, W, NW, N, NE; the neighbour in direction d donates when its code has the
// bit of the opposite direction (d + 4) % 8.  The scan order is d = 2,3,4,5,6,7,0,1.
__host__ __device__ constexpr int scan_dir(int k) { return (k + 2) & 7; }
__host__ __device__ constexpr int scan_index(int d) { return (d + 6) & 7; }  // k with scan_dir(k) == d

// The int32 code of a masked cell is -9999 (newflow.cu:74); only its low byte 0xF1
// (bits E, W, NW, N, NE) takes part in the bit tests of the accumulation kernels.
constexpr uint8_t kMaskedCode = 0xF1;
constexpr double kNoData = -9999.0;

// Order-preserving map of a double to uint64 (exact comparisons without the FP64
// pipe).  NaN maps to 0, which callers treat as "unordered": every comparison of
// the reference involving a NaN elevation is false.
__device__ __forceinline__ uint64_t dkey(double z) {
    uint64_t b = (uint64_t)__double_as_longlong(z);
    if ((b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull) return 0;  // NaN
    if (b == 0x8000000000000000ull) b = 0;  // -0.0 == +0.0
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(uint64_t k) {
    uint64_t b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    return __longlong_as_double((long long)b);
}

// Split of a double into an fp32 head (mantissa truncated to 24 bits) and an fp32
// tail holding the next 24 bits, with integer operations only.  |z - hi - lo| <=
// 2^-47 |z| for normal fp32-range magnitudes; tiny magnitudes collapse to zero.
__device__ __forceinline__ void dsplit(double z, float& hi, float& lo) {
    uint64_t b = (uint64_t)__double_as_longlong(z);
    uint32_t sign = (uint32_t)(b >> 63);
    int e = (int)((b >> 52) & 0x7FF);
    uint64_t m = b & 0x000FFFFFFFFFFFFFull;
    int fe = e - 1023 + 127;
    if (fe <= 0 || e == 0) { hi = 0.0f; lo = 0.0f; return; }
    if (fe >= 255) { hi = sign ? -3.0e38f : 3.0e38f; lo = 0.0f; return; }
    uint32_t hb = (sign << 31) | ((uint32_t)fe << 23) | (uint32_t)(m >> 29);
    hi = __uint_as_float(hb);
    uint32_t rest = (uint32_t)(m & 0x1FFFFFFFull);  // 29 bits, value rest * 2^(e-1075)
    int pe = e - 1075 + 127;                          // exponent of 2^(e-1075) as fp32
    if (pe <= 0 || rest == 0) { lo = 0.0f; return; }
    float scale = __uint_as_float((uint32_t)pe << 23);
    float r = __uint2float_rn(rest) * scale;
    lo = sign ? -r : r;
}

struct ErrFlags {  // bits of the device error word
    static constexpr uint32_t kCapacity = 1u;
    static constexpr uint32_t kNoConverge = 2u;
};

// Raises an error flag.  `err` is DevScalars::err; the word after it keeps the
// first flag raised, which the host reports: a loop that stops at its round
// cap leaves later tables inconsistent, and an overflow those raise is a
// consequence, not the cause.
__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t flag) {
    atomicOr(err, flag);
    atomicCAS(err + 1, 0u, flag);
}

// Device-side scalars of one handle (one allocation, read back only on request).
struct DevScalars {
    int32_t sinkcount_pass1;         // masked-in SFD == 0 after the first plateau pass, all DEMs
    int32_t plateau_sweeps;
    int32_t n_cand;                  // plateau candidates
    int32_t n_sinks;                 // sink cells of the flooding
    int32_t n_edges;                 // distinct basin pairs
    int32_t n_basins;
    int32_t flood_sweeps, label_rounds, spill_rounds;
    uint32_t err;                    // ErrFlags raised since the host last read them
    uint32_t err_first;              // the first of them (a later one may be its consequence)
    int32_t round_id;                // monotonic id of worklist rounds (de-duplication marks)
    int32_t flag[4];                 // convergence flags of the cooperative loops
    int32_t counters[8];
    int32_t tiled_ok;                // 1: this step's accumulation may take the tiled path
    int32_t tile_src;                // tile outlets with no pending inflow (coarse sources)
    int32_t sed_tiled_ok;            // 1: this step's sediment routing may take the tiled path
    int32_t epoch;                   // flow-direction stages run so far (first-seen marks of basin labels)
    int32_t round_cap;               // rounds of every device loop before it gives up (0: kDefaultRoundCap)
    int32_t edge_log_cap;            // log2 slots the basin-pair table may use (0: sized per step)
};

// Every device loop (grid-barrier rounds, worklist waves) stops after this
// many rounds and raises ErrFlags::kNoConverge; lem_set_limits lowers it.
constexpr int kDefaultRoundCap = 1 << 16;
// Read once at kernel start, so every block of a cooperative launch sees the
// same value (the host writes it before the launch, in stream order).
__device__ __forceinline__ int round_cap_of(const DevScalars* sc) {
    const int c = *((const volatile int32_t*)&sc->round_cap);
    return c > 0 ? c : kDefaultRoundCap;
}

static_assert(offsetof(DevScalars, err_first) == offsetof(DevScalars, err) + sizeof(uint32_t),
              "raise_error keeps the first flag in the word after err");

// The DEMs of a handle.  A single grid is one DEM covering the whole grid; a
// batch packs several DEMs into one grid, each in its own region (32-aligned,
// with a nodata ring, so no in-catchment cell of one DEM sees another DEM).
constexpr uint16_t kNoDem = 0xFFFF;  // a cell outside every DEM's region

// Per-DEM inputs owned by the host, uploaded before each stage: the region and
// the climate scalars of the step (SetClimateMatrices, Data.cpp:211-303).
struct DemIn {
    int32_t x0, y0, w, h;            // region in the grid
    int32_t active;
    int32_t from_current_dem;        // temperature from the DEM at step start (1) or the initial DEM (0)
    int32_t outlet_from_fa;          // this step moves the outlet to the largest accumulation
    int32_t pad;
    double rain, temp, rain_inc;     // rain row gradient (2R - R) / h
    double rain0, temp0, rain0_inc;  // initial ("last") scalars
};

// Per-DEM results kept on the device.
struct DemOut {
    unsigned long long lowest_key;   // min masked-in DEM key (testoutletislowest)
    unsigned long long fa_max_key;   // FA_max as an ordered key of hi+lo
    double base_level;               // update_newSurface base (updates.cu:151)
    double outlet_z_clim;            // z[outlet] as seen by the climate grids ...
    double tot_e, tot_i, tot_g, tot_d, tot_wc, tot_wp, tot_bio;
    int32_t outlet;                  // grid cell index
    int32_t sink_counter, flat_counter;
    int32_t sinkcount_pass1;         // this DEM's share of DevScalars::sinkcount_pass1
    int32_t sinkcount;               // Data.sinkcount
    int32_t fa_done, sed_done, n_active;
    int32_t argmax;                  // first cell holding FA_max
    int32_t zero_seen;               // epoch of the last sinkcount that counted basin 0
    int32_t outlet_clim;             // ... for this cell: the outlet when the step's directions were
                                     //   computed (the accumulation stage may move the outlet)
};

struct DemCtx {
    const uint16_t* of;  // DEM of each cell; null: every cell belongs to DEM 0
    const DemIn* in;
    DemOut* out;
    int32_t n;           // DEM slots
};
__device__ __forceinline__ int dem_at(const DemCtx& dc, size_t cell) { return dc.of ? (int)dc.of[cell] : 0; }

}  // namespace lem

#define LEM_CUDA_TRY(expr)                                            \
    do {                                                              \
        cudaError_t _e = (expr);                                      \
        if (_e != cudaSuccess) return ::lem::cuda_fail(_e, #expr, __FILE__, __LINE__); \
    } while (0)

namespace lem {
lem_status cuda_fail(cudaError_t e, const char* what, const char* file, int line);
}
