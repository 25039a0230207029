// lem_ctx.cuh -- resident device state of one grid and the stage launchers.
#pragma once

#include <cuda.h>

#include "lem_common.cuh"

namespace lem {

constexpr int kTile = 32;     // edge of the accumulation tiles
constexpr int kTileEnt = 136; // inflow slots per tile (inflows come from the 132 halo ring cells)
constexpr int kTilePool = 1280; // sediment node inputs per tile: one per waiting in-tile edge (< 1024) or inflow (< 132)

// Dreybrodt temperature response table (see lem_mod.cu): log10 of
// K1*KC*KH / (4*K2*gammaCa*gammaHCO3^2) sampled every kTabStep degrees.
constexpr int kTabN = 3841;
constexpr float kTabT0 = -60.0f;
constexpr float kTabStep = 1.0f / 32.0f;

struct ModelConsts {  // per-handle constants derived on the host in double
    int32_t W, H;
    int32_t csize;          // (int)cellsize, routeflow.cu:716
    int32_t flow_type;      // Data.flowdirectiontype
    int32_t mfd_props;      // calcprops instead of calcpropsSFD
    int32_t soil_struct, profile_permeability;
    float inv_len[8];       // 1 / (float)((float)csize * dc)
    double len[8];          // (double)(float)((float)csize * dc)
    float q_threshold, g_slope, kappa, g_flowlim, flow_a, flow_b, max_incision;
    float ddk, dck, dgk, temp_inflex, temp_sens;
    float rescale_conc;     // 1 / (10000 / cs^2)          eroincidep.cu:310
    float rescale_conc_lo;  //   its fp32 tail (rescale_conc + rescale_conc_lo = the fp64 value)
    float q_threshold_lo;   //   fp32 tail of Qthreshold
    float g_flowlim_lo;     //   fp32 tail of Gflowlim
    float rescale_weather;  // 10000 * (10000 / cs^2)      eroincidep.cu:628
    float rescale_veg;      // 10000 / cs^2                Data.cpp:124
    float erod_const;       // 0.043*(struct-2) + 0.033*(perm-3)
};

// The cooperative kernels whose block count the autotuner sets (the order of
// lem_tuning's array).
enum CoopKernel { kCkPlateau = 0, kCkMerge, kCkJump, kCkSpill, kCkFatCoarse, kCkFaWalk, kCkSedCoarse, kCkSedWalk,
                  kCoopKernels };


// Tile shapes of the TMA flow-direction kernel (rows of a 32-column strip),
// chosen per handle by the autotuner.
constexpr int kFdShapes = 3;
constexpr int kFdRows[kFdShapes] = {8, 16, 32};

// Tensor maps of the TMA flow-direction kernel, one set per tile shape: the
// elevations of both passes, the mask and the persistent slopes (host memory
// of the handle; passed to the kernels by value).
struct FdTmaMaps {
    CUtensorMap z[kFdShapes], zf[kFdShapes], mask[kFdShapes], slopes[kFdShapes];
    int blocks[kFdShapes];  // co-resident blocks of each shape's kernel on the device
};

struct DevState {
    // grids
    double* z;          // Data.dem
    double* zf;         // DEM of the second flow-direction pass (raised)
    double* z_init;     // DEM the run-in climate grids were built from
    uint8_t* mask;
    float* slopes;      // 8 per cell
    uint8_t* sfd;       // SFD code (low byte; masked = 0xF1)
    uint8_t* mfd;       // MFD code
    uint8_t* fd;        // final code after the epilogue
    uint8_t* sfd1;      // SFD code after the first plateau pass (the basis of the basin labels)
    float* sp;          // plateau distances
    int32_t* ws;        // basin labels / pointers
    int32_t* pending;   // wave in-degrees
    int32_t* list_a;    // worklists
    int32_t* list_b;
    int32_t* mark;      // worklist de-duplication epochs
    uint8_t* eqm;       // per plateau candidate: directions of its equal-height neighbours
    int32_t* tq;        // the plateau routing's tile queue: entries and slot sequence numbers
    int32_t tq_cap;     //   its slots (more than the plateau tiles)
    float2* fa;         // accumulation as an unevaluated fp32 pair (hi, lo)
    float* w;           // runoff weight
    float* slopeptr;
    float* stone; float* fines; float* soilT; float* soilM; float* soilB; float* nut; float* totB;
    float* ero; float* inci; float* geli; float* depo;
    float* dz; float* wc; float* wp;  // diagnostics
    float* prop;        // 8 per cell, MFD proportions (calcprops mode only)
    int32_t* contrib;
    // tiled accumulation (32x32 tiles): per cell, used at tile entries / outlets
    int32_t* t_dst;     // entry cell: the outlet of its tile its path reaches, or -1
    int32_t* t_pend;    // outlet: inflows still to arrive (kBlocked: never completes)
    int32_t* t_orng;    // outlet: (first << 16) | count of its inflows in t_ent
    float2* t_la;       // outlet: accumulation from inside its tile only
    int32_t* t_ent;     // per tile, kTileEnt inflow cells (outlets of neighbours) grouped by outlet
    // tiled sediment routing: per tile, the cells that wait on other tiles as
    // programs (one per outlet, kTile*kTile slots per tile)
    float4* p_abc;      // node: stone mix coefficients A, B, the settled donors' sum C, inputs and flags
    int32_t* p_ref;     // per tile, kPool node inputs: the feeding node (program slot) or cell
                        //   (the accumulation's program uses the same slots earlier in the step)
    float4* p_map;      // per tile, kPool node inputs: the map through the cells in between
    float* p_val;       // slot: the value of every program node once the coarse wave has run
    uint8_t* t_stat;    // cell: 1 settled inside its tile, 2 waits on another tile, 0 neither
                        //   (written for the tiles whose waiting cells are routed by a second wave)
    // per tile, kTile*kTile slots: the waiting cells the final pass stores.
    // Sediment: each as its outlet, the program node that feeds it and the
    // map from that node's value to its own stone.  Accumulation (earlier in
    // the step, same slots): each as its node and its local accumulation.
    int4* f_idx;        // cell, p_val slot of the feeding node, outlet cell, flags | cell, node, flags
    float4* f_map;      // clamp map: feeding node's value -> the cell's stone
    float2* f_ds;       // the cell's deposition and new soil thickness | its local accumulation
    int32_t* t_fcnt;    // tile: number of such cells (accumulation: | nodes << 16); -1: the second wave
    int32_t* n_meta;    // accumulation, per tile kTile*kTile nodes: first input in p_ref | count << 11
    // flooding tables
    unsigned long long* ekey;   // hash keys (label pair)
    unsigned long long* ewt;    // min boundary height key
    int64_t ecap;               // capacity (power of two)
    int32_t* edge_a; int32_t* edge_b; unsigned long long* edge_w;
    unsigned long long* raise;  // per label (label = cell + 1), ordered keys
    int32_t* label_seen;
    int32_t* comp;              // component label of basins that never reach basin 0
    unsigned long long* cdist;  //   their minimax distance to the component's label basin
    unsigned long long* cmaxw;  //   the component's largest spanning-tree edge
    // the basin graph with basins numbered 0..n_basins-1 per step
    int32_t* bid;               // per label: its basin number
    int32_t* blab;              // per basin: its label
    int32_t* boff;              // per basin: the spill round that last lowered it
    unsigned long long* bdist;  // per basin: minimax distance to basin 0 (ordered key)
    int32_t* adj_v;             // per edge: its two basin numbers
    DevScalars* sc;
    DemCtx dems;                // the DEMs of the grid
    int32_t* chunk_start;       // streaming passes: first chunk of each DEM (n + 1 entries)
    int32_t n_chunks;
    int32_t* live;              // batch grids: the tiles holding a DEM's region, ascending
    int32_t n_live;             // tiles the canvas-wide kernels visit
    float* temp_tab;
    int32_t max_coop_blocks;    // co-resident blocks of the cooperative kernels
    int32_t coop_blocks[kCoopKernels];  // blocks each cooperative kernel launches with (<= its coop_cap)
    int32_t coop_cap[kCoopKernels];     // co-resident blocks of each cooperative kernel
    const FdTmaMaps* fd_tma;    // host: the TMA flow-direction kernel's maps (null: rows TMA cannot address)
    int32_t fd_rows;            // its tile shape, an index into kFdRows
};

// The tiles a canvas-wide kernel visits: in a batch grid the 32x32 tiles that
// hold a DEM's region (every other cell is nodata outside every DEM and keeps
// the values its region was emptied with; no in-catchment cell has such a
// neighbour), in a single grid every tile.  Position v of a visit is cell
// v & 1023 of the (v >> 10)-th visited tile, row by row, so a warp covers one
// 32-cell row of one tile and never two DEMs.
static_assert(kTile == 32, "visit positions hold a 32x32 tile in 10 bits");
struct TileSet {
    const int32_t* id;  // visited tile ids; null: tiles 0 .. n-1
    int n;
    int tw;             // tiles per grid row
    __device__ __forceinline__ int tile(int i) const { return id ? __ldg(id + i) : i; }
    __host__ __device__ __forceinline__ size_t span() const { return (size_t)n << 10; }
    // the cell at visit position v; false where an edge tile of a single grid
    // extends past the grid
    __device__ __forceinline__ bool cell(size_t v, int W, int H, int& x, int& y) const {
        const int t = tile((int)(v >> 10));
        const int o = (int)(v & 1023);
        x = (t % tw) * kTile + (o & (kTile - 1));
        y = (t / tw) * kTile + o / kTile;
        return x < W && y < H;
    }
};
inline TileSet tiles_of(const DevState& s, int W) {
    return TileSet{s.live, s.n_live, (W + kTile - 1) / kTile};
}

// Streaming passes over the DEMs' regions run one block per chunk of kChunk
// cells, every chunk inside one DEM, so block sums go to that DEM's totals.
constexpr int kChunk = 4096;
struct Chunk {
    int d;          // DEM
    int64_t first;  // first region-linear cell of the chunk
    int64_t end;    // one past the last
};
__device__ __forceinline__ Chunk chunk_of(const int32_t* chunk_start, int n, const DemIn* in) {
    // the DEM whose chunk range holds blockIdx.x (n is small: binary search)
    int lo = 0, hi = n;
    const int b = blockIdx.x;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (chunk_start[mid] <= b) lo = mid; else hi = mid;
    }
    Chunk c;
    c.d = lo;
    c.first = (int64_t)(b - chunk_start[lo]) * kChunk;
    const int64_t cells = (int64_t)in[lo].w * in[lo].h;
    c.end = c.first + kChunk < cells ? c.first + kChunk : cells;
    return c;
}
// grid index of region-linear cell i of DEM region r
__device__ __forceinline__ size_t region_cell(const DemIn& r, int64_t i, int W, int* x, int* y) {
    const uint32_t u = (uint32_t)i, rw = (uint32_t)r.w;  // a region holds fewer than 2^31 cells: 32-bit division
    const int ry = (int)(u / rw), rx = (int)(u - (uint32_t)ry * rw);
    *x = r.x0 + rx;
    *y = r.y0 + ry;
    return (size_t)(*y) * W + *x;
}

// Optional per-kernel timing with CUDA events on the handle's stream.
struct Profiler;
void profiler_begin(Profiler* p, const char* name, cudaStream_t st);
void profiler_end(Profiler* p, cudaStream_t st);

// Where and how a stage launches: the handle's stream, its launch counter and
// (when enabled) the profiler that brackets every launch with events.
struct Launch {
    cudaStream_t st;
    uint64_t* count;
    Profiler* prof;
    void pre(const char* name) const {
        if (prof) profiler_begin(prof, name, st);
    }
    void post() const {
        if (prof) profiler_end(prof, st);
        ++*count;
    }
};

// A slot in a list counted in shared memory, one atomic per warp; every lane
// of the warp calls it.  -1 where pred is false.
__device__ __forceinline__ int warp_slot(bool pred, int* s_count) {
    const unsigned b = __ballot_sync(0xffffffffu, pred);
    if (!b) return -1;
    const int lane = threadIdx.x & 31, leader = __ffs(b) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(s_count, __popc(b));
    base = __shfl_sync(0xffffffffu, base, leader);
    return pred ? base + __popc(b & ((1u << lane) - 1)) : -1;
}

// Append with one atomic per block: every thread of the block calls it, and
// s_cnt holds (threads of the block) / 32 + 1 ints.  block_reserve returns the
// list position of a thread with pred set (-1 otherwise).  Kernels whose every block appends to
// one list (sinks, plateau candidates, ready tile outlets) use it, so the
// blocks of a launch do not queue on one counter warp by warp.
__device__ __forceinline__ int block_reserve(bool pred, int32_t* count, int* s_cnt) {
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;  // warps are runs of 32 linear thread ids
    const int lane = tid & 31, wid = tid >> 5, nw = (blockDim.x * blockDim.y) >> 5;
    const unsigned ballot = __ballot_sync(0xffffffffu, pred);
    if (lane == 0) s_cnt[wid] = __popc(ballot);
    __syncthreads();
    if (tid == 0) {
        int tot = 0;
        for (int w = 0; w < nw; ++w) {
            const int c = s_cnt[w];
            s_cnt[w] = tot;
            tot += c;
        }
        s_cnt[nw] = tot ? atomicAdd(count, tot) : 0;
    }
    __syncthreads();
    return pred ? s_cnt[nw] + s_cnt[wid] + __popc(ballot & ((1u << lane) - 1)) : -1;
}
__device__ __forceinline__ void block_append(bool pred, int32_t value, int32_t* list, int32_t* count, int cap,
                                             uint32_t* err, int* s_cnt) {
    const int pos = block_reserve(pred, count, s_cnt);
    if (pos >= 0) {
        if (pos < cap)
            list[pos] = value;
        else
            raise_error(err, ErrFlags::kCapacity);
    }
}

// A cooperative launch (grid-wide barriers) of 256-thread blocks, as a launch
// attribute so that it can be captured into a CUDA graph.
inline cudaError_t coop_launch(const void* fn, int blocks, void** args, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

#define LEM_LAUNCH(L, kern, grid, block, ...)                  \
    do {                                                       \
        (L).pre(#kern);                                        \
        kern<<<(grid), (block), 0, (L).st>>>(__VA_ARGS__);     \
        (L).post();                                            \
    } while (0)

// stage launchers (stream-ordered, no host synchronisation)
lem_status launch_flow_direction(const DevState& s, const ModelConsts& k, const Launch& L);
lem_status launch_flow_accumulation(const DevState& s, const ModelConsts& k, uint32_t flags,
                                    const Launch& L);
lem_status launch_erosion(const DevState& s, const ModelConsts& k, uint32_t flags,
                          const Launch& L);
int coop_blocks_for(const void* kernel, int threads, size_t smem);
// Encodes the TMA flow-direction kernel's tensor maps for the state's grids
// (rows must be multiples of 16 bytes: width a multiple of 16).
lem_status fd_tma_setup(const DevState& s, const ModelConsts& k, FdTmaMaps* maps);

}  // namespace lem
