/*
 * lem_gb300.h -- C ABI of the GB300 per-timestep landscape-evolution path.
 *
 * One handle holds one DEM and its whole model state resident in HBM.  A step
 * is the reference's three host calls in its timestep loop (lem.cpp:83-97):
 *   flow direction    cuFlowDirection          FD_kernels/routeflow.cu:686-975
 *   flow accumulation computeRunOffWeights     MOD_kernels/runoffweight.cu:61-113
 *                     calcpropsSFD / calcprops MOD_kernels/runoffweight.cu:115-354
 *                     correctmfdflow           FA_kernels/mfd_simple.cu:238-384
 *   process update    erosionGPU               MOD_kernels/erosion.cu:69-186
 * The per-stage buffers that the reference mallocs, uploads, downloads and frees
 * around every call (MEM_kernels/memory_dev.cu:33-240) stay on the device for
 * the life of the handle; host mirrors are filled only by lem_get_field.
 *
 * Every entry point returns lem_status and never exits the process.  Calls on
 * one handle are issued on the handle's own CUDA stream; they are asynchronous
 * unless stated otherwise.  One handle must not be used from two host threads
 * at once.
 */
#ifndef LEM_GB300_H
#define LEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lem_status {
    LEM_OK = 0,
    LEM_ERR_INVALID = 1,     /* bad argument or unsupported combination            */
    LEM_ERR_CAPACITY = 2,    /* a fixed-capacity table or worklist overflowed      */
    LEM_ERR_NOCONVERGE = 3,  /* a sweep or worklist hit its iteration cap          */
    LEM_ERR_CUDA = 4,        /* a CUDA runtime call failed                         */
    LEM_ERR_NOMEM = 5,       /* device or host allocation failed                   */
    LEM_ERR_STATE = 6        /* call out of order (e.g. step before the DEM is set) */
} lem_status;

/* Grid geometry: MapInfo (headers/MapInfo.h:4-12).  cellsize is the ESRI
 * header value; the direction kernels use (int)cellsize like routeflow.cu:716. */
typedef struct lem_grid_desc {
    int32_t width;      /* ncols */
    int32_t height;     /* nrows */
    double cellsize;
} lem_grid_desc;

/* Model coefficients: default.par lines 11 and 16-35 as read by readinpar
 * (MEM_kernels/io.cpp:469-568).  Field names follow the Data members. */
typedef struct lem_params {
    int32_t flow_direction_type;  /* Data.flowdirectiontype: 0 = SFD, 1 = MFD            */
    int32_t mfd_proportions;      /* 0 = calcpropsSFD (prop 1 on every direction),
                                     1 = calcprops (slope-proportional MFD partition)      */
    int32_t soil_struct;          /* Data.soil_struct                                    */
    int32_t profile_permeability; /* Data.profile_permeability                           */
    double q_threshold;           /* Data.Qthreshold                                     */
    double g_slope;               /* Data.Gslope                                         */
    double kappa;                 /* Data.kappa                                          */
    double g_flowlim;             /* Data.Gflowlim                                       */
    double flow_a;                /* Data.Flow_A                                         */
    double flow_b;                /* Data.Flow_B                                         */
    double max_incision;          /* Data.max_incision                                   */
    double ddk;                   /* Data.ddk (clamped to 0.95 as mfd_accum.cu:406)      */
    double dck;                   /* Data.dck (clamped to 0.9 as mfd_accum.cu:407)       */
    double dgk;                   /* Data.dgk                                            */
    double temp_inflex;           /* Data.temp_inflex                                    */
    double temp_sens;             /* Data.temp_sens                                      */
} lem_params;

/* Climate of one step.  recompute = 1 is SetClimateMatrices(data, i) before the
 * step (MEM_kernels/Data.cpp:211-303, lem.cpp:79-81): rain and temperature
 * grids are rebuilt from these scalars and the DEM at the start of the step.
 * recompute = 0 keeps the grids of the previous call; before any recompute the
 * grids are the ones built at lem_create from the initial rain/temperature and
 * the DEM first uploaded (the run-in of lem.cpp:71).  A recompute = 0 step after
 * a recompute = 1 step is rejected with LEM_ERR_STATE. */
typedef struct lem_climate {
    double rain;
    double temp;
    int32_t recompute;
} lem_climate;

/* Per-step totals: the budgets CSV row (MEM_kernels/io.cpp:233-263). */
typedef struct lem_totals {
    double tot_e;            /* Data.totE, sum of diffuse erosion            */
    double tot_i;            /* Data.totI, sum of concentrated erosion       */
    double tot_g;            /* Data.totG, sum of gelifluction               */
    double tot_d;            /* Data.totD, sum of deposition                 */
    double tot_weather_c;    /* Data.totweatherC                             */
    double tot_weather_p;    /* Data.totweatherP                             */
    double tot_bio;          /* Data.totbio                                  */
    double fa_max;           /* Data.FA_max                                  */
    double rain;             /* Data.rain of the step                        */
    double temp;             /* Data.temp of the step                        */
    int32_t sinkcount;       /* Data.sinkcount                               */
    int32_t outlet;          /* Data.outletcellidx after the step            */
    int32_t initial_sinks;   /* FlowDirs sink counter (routeflow.cu:778)     */
    int32_t initial_flats;   /* FlowDirs flat counter (routeflow.cu:779)     */
    int32_t plateau_sweeps;  /* 32x32 tile visits of the plateau routing     */
    int32_t flood_edges;     /* distinct basin pairs of the sink flooding    */
    int32_t fa_uncomputed;   /* masked-in cells left out of accumulation     */
    int32_t sed_uncomputed;  /* masked-in cells left out of sediment routing */
    int32_t merge_rounds;    /* sink flooding: rounds of the equal-height label merge   */
    int32_t label_rounds;    /*   rounds of the basin labelling (pointer jumping)       */
    int32_t spill_rounds;    /*   rounds of the minimax spill relaxation                */
    int32_t pad;
} lem_totals;

/* Grid fields.  Element type per field: D = double[W*H], I = int32[W*H],
 * D8 = double[8*W*H] (cell-major, direction index 0..7 = N,NE,E,SE,S,SW,W,NW
 * as newflow.cu:71,99-106). */
typedef enum lem_field {
    LEM_F_DEM = 0,        /* D  Data.dem (nodata = -9999)                          */
    LEM_F_MASK = 1,       /* I  Data.mask (1 in catchment, 0 outside); read only   */
    LEM_F_FD = 2,         /* I  Data.fd after the FD epilogue (routeflow.cu:938-953) */
    LEM_F_SFD = 3,        /* I  Data.SFD                                            */
    LEM_F_SLOPES = 4,     /* D8 Data.Slopes                                         */
    LEM_F_SLOPEPTR = 5,   /* D  Data.SlopePtr (aveslope)                            */
    LEM_F_FA = 6,         /* D  Data.fa                                             */
    LEM_F_RUNOFF = 7,     /* D  Data.runoffweight                                   */
    LEM_F_STONE = 8,      /* D  Data.stonePtr                                       */
    LEM_F_FINES = 9,      /* D  Data.finesPtr                                       */
    LEM_F_SOILT = 10,     /* D  Data.soilTPtr                                       */
    LEM_F_SOILM = 11,     /* D  Data.soilMPtr                                       */
    LEM_F_SOILB = 12,     /* D  Data.soilBPtr                                       */
    LEM_F_NUT = 13,       /* D  Data.nutPtr                                         */
    LEM_F_TOTB = 14,      /* D  Data.TotBPtr                                        */
    LEM_F_ERO = 15,       /* D  Data.eroPtr                                         */
    LEM_F_INCI = 16,      /* D  Data.inciPtr                                        */
    LEM_F_GELI = 17,      /* D  Data.geliPtr                                        */
    LEM_F_DEPO = 18,      /* D  Data.depoPtr                                        */
    LEM_F_DZ = 19,        /* D  Data.dz        (needs LEM_STEP_KEEP_DIAGNOSTICS)    */
    LEM_F_WEATHER_C = 20, /* D  Data.weatherC  (needs LEM_STEP_KEEP_DIAGNOSTICS)    */
    LEM_F_WEATHER_P = 21, /* D  Data.weatherP  (needs LEM_STEP_KEEP_DIAGNOSTICS)    */
    LEM_F_CONTRIB = 22,   /* I  contributing cells incl. self along the SFD codes
                                (needs LEM_STEP_CONTRIB)                             */
    LEM_F_WATERSHED = 23, /* I  basin label of the last sink flooding (0 = drains
                                off the grid or to nodata)                           */
    LEM_F_DEM_ROUTED = 24,/* D  the DEM the final codes were computed on: the stage's
                                DEM raised to the spill heights; read only           */
    LEM_F_SFD_PASS1 = 25, /* I  SFD codes after the first plateau pass, the codes the
                                basins of the sink flooding follow; read only        */
    LEM_F_COUNT = 26
} lem_field;

/* Step flags. */
#define LEM_STEP_SET_OUTLET_FROM_FA  0x1u  /* correctmfdflow's first-iteration branch
                                              (mfd_simple.cu:336-349): the outlet moves
                                              to the cell of largest accumulation       */
#define LEM_STEP_KEEP_DIAGNOSTICS    0x2u  /* store dz, weatherC, weatherP             */
#define LEM_STEP_CONTRIB             0x4u  /* also count contributing cells (int32)    */

typedef struct lem_handle lem_handle;

/* Allocates the resident state of one grid on the current CUDA device.
 * init_rain / init_temp are the run-in scalars of default.par lines 12-13; they
 * also serve as the "last" climate of grow_vegetation (updates.cu:90-92). */
lem_status lem_create(const lem_grid_desc* grid, const lem_params* params,
                      double init_rain, double init_temp, lem_handle** out);
lem_status lem_destroy(lem_handle* h);

/* Host <-> device copies of one field (synchronous).  The first LEM_F_DEM upload
 * also fixes the mask (dem != -9999, createmask in MEM_kernels/memory.cu:217-242)
 * and the DEM that the initial climate grids were built from.  LEM_F_FD and
 * LEM_F_SFD may be set (int32 codes, -9999 outside the catchment) to run the
 * later stages from given directions; MASK, CONTRIB and WATERSHED are read only. */
lem_status lem_set_field(lem_handle* h, lem_field f, const void* host);
lem_status lem_get_field(lem_handle* h, lem_field f, void* host);
lem_status lem_set_outlet(lem_handle* h, int32_t cell);  /* init_setoutletcell result */

/* One stage each; the argument order follows the reference calls. */
lem_status lem_flow_direction(lem_handle* h);                          /* cuFlowDirection */
lem_status lem_flow_accumulation(lem_handle* h, uint32_t flags);       /* runoff + props + correctmfdflow */
lem_status lem_erosion(lem_handle* h, uint32_t flags);                 /* erosionGPU */
lem_status lem_set_climate(lem_handle* h, const lem_climate* c);       /* SetClimateMatrices */

/* One whole timestep: lem_set_climate + the three stages. */
lem_status lem_step(lem_handle* h, const lem_climate* c, uint32_t flags);

/* Blocks until the handle's stream is idle; returns the first device-side error
 * (capacity, convergence) raised since the previous call. */
lem_status lem_synchronize(lem_handle* h);
lem_status lem_get_totals(lem_handle* h, lem_totals* out);            /* synchronous */

/* The handle's cudaStream_t, for callers that order their own work after it. */
void* lem_stream(lem_handle* h);

/* Makes `device` current for the calling host thread in this library (its CUDA
 * runtime is linked statically, so the caller's own runtime state is not
 * shared).  Handles are created on the device current at lem_create. */
lem_status lem_select_device(int32_t device);

/* Device timing on the handle's stream: lem_event_record places event `slot`
 * (0..15) on the stream; lem_event_elapsed waits for event `to` and returns the
 * milliseconds between the two records. */
lem_status lem_event_record(lem_handle* h, int32_t slot);
lem_status lem_event_elapsed(lem_handle* h, int32_t from, int32_t to, float* ms);

/* Per-kernel timing: when enabled every kernel launch of the handle is
 * bracketed by two events on its stream.  lem_profile_read synchronises,
 * returns launches and summed device milliseconds per kernel name since the
 * previous read (or since enabling) and starts a new interval. */
typedef struct lem_kernel_stat {
    char name[48];
    uint32_t launches;
    double total_ms;
} lem_kernel_stat;
lem_status lem_set_profiling(lem_handle* h, int32_t on);
lem_status lem_profile_read(lem_handle* h, lem_kernel_stat* out, int32_t cap, int32_t* count);

/* Kernel launches issued by this handle since creation (for launch accounting). */
uint64_t lem_launch_count(lem_handle* h);

const char* lem_status_string(lem_status s);

/* ---- Batches: many DEMs of uneven sizes stepped together.
 * No counterpart in the reference, which runs one grid per process
 * (lem.cpp:67-97).  A batch handle owns one grid (the canvas); each DEM lives
 * in its own region of it, placed by the caller at multiples of 32 cells, and
 * must carry a nodata ring (all its border cells -9999), so no in-catchment
 * cell of one DEM sees another.  One lem_step_batch runs the three stages of
 * every active DEM with one launch per kernel; each DEM keeps its own outlet,
 * climate and budget totals, and its grids equal those of the same DEM run
 * alone.  Cell indices of a DEM (outlet, totals) are indices of the DEM's own
 * grid.  The canvas width must be a multiple of 32; max_dems < 65535. */
lem_status lem_create_batch(const lem_grid_desc* canvas, const lem_params* params, int32_t max_dems,
                            lem_handle** out);
/* Adds a DEM at (x0, y0) of the canvas (x0, y0 multiples of 32; the 32-rounded
 * extents of two DEMs may not overlap).  Its other fields start at zero; set
 * the soil state with lem_dem_set_field and the outlet with lem_dem_set_outlet
 * before the next step.  LEM_ERR_CAPACITY: no free DEM slot. */
lem_status lem_dem_add(lem_handle* h, int32_t x0, int32_t y0, int32_t width, int32_t height, const double* dem,
                       double init_rain, double init_temp, int32_t* id);
lem_status lem_dem_remove(lem_handle* h, int32_t id);       /* its region returns to nodata */
lem_status lem_dem_set_field(lem_handle* h, int32_t id, lem_field f, const void* host);  /* width*height */
lem_status lem_dem_get_field(lem_handle* h, int32_t id, lem_field f, void* host);
lem_status lem_dem_set_outlet(lem_handle* h, int32_t id, int32_t cell);
lem_status lem_dem_set_climate(lem_handle* h, int32_t id, const lem_climate* c);
/* Flags for this DEM's next step only (LEM_STEP_SET_OUTLET_FROM_FA for its first). */
lem_status lem_dem_set_step_flags(lem_handle* h, int32_t id, uint32_t flags);
lem_status lem_dem_get_totals(lem_handle* h, int32_t id, lem_totals* out);  /* synchronous */
/* The budget rows of n DEMs after one synchronisation (out[k] for ids[k]);
 * the per-step loop of a batch reads all its rows with it. */
lem_status lem_dem_get_totals_n(lem_handle* h, const int32_t* ids, int32_t n, lem_totals* out);
/* One timestep of every active DEM; flags as lem_step, for all DEMs. */
lem_status lem_step_batch(lem_handle* h, uint32_t flags);

/* CUDA-graph steps (off by default; no counterpart in the reference, which
 * launches every kernel from the host).  When on, lem_step and lem_step_batch
 * upload the per-DEM inputs and then launch the whole timestep as one graph,
 * captured on first use and again whenever the launch configuration changes
 * (a DEM joins or leaves, other step flags); results equal eager steps bit for
 * bit.  While per-kernel profiling (lem_set_profiling) is on, steps launch
 * eagerly.  The single-stage calls (lem_flow_direction ...) are always eager. */
lem_status lem_set_graphs(lem_handle* h, int32_t on);

/* Caps of the device loops and tables.  The reference's loops run until their
 * change flags clear, with no bound (plateau sweeps routeflow.cu:854-872, label
 * and merge loops routeflow.cu:285-302,314-338, accumulation mfd_simple.cu:
 * 204-226), and its basin-pair hash table overflows silently
 * (newflow.cu:860-872).  Here every loop stops after max_rounds rounds and the
 * next lem_synchronize returns LEM_ERR_NOCONVERGE; the basin-pair table holds
 * at most 2^edge_table_log2 pairs and a full table makes lem_synchronize return
 * LEM_ERR_CAPACITY.  After either error the step's results are incomplete but
 * the handle stays usable.  0 in a field restores its default (65536 rounds;
 * a table of 8 slots per sink, at least 1024).  Lowering them serves tests of
 * the error paths and callers that bound a step's device time. */
typedef struct lem_limits {
    int32_t max_rounds;       /* rounds of every device loop; 0: 65536                   */
    int32_t edge_table_log2;  /* log2 of the basin-pair table's slots (1..40); 0: sized per step */
} lem_limits;
lem_status lem_set_limits(lem_handle* h, const lem_limits* limits);

/* Autotuner of the launch schedule (no counterpart in the reference).  The
 * handle's next 1 + 4 * cycles steps (lem_step or lem_step_batch; real steps
 * of the model, launched eagerly) run the cooperative kernels with 1, 2 and 4
 * blocks per SM and with all their co-resident blocks in turn, and the
 * flow-direction kernel with TMA tiles of 8, 32, 16 (the default) and 8 rows, and time them
 * with events; afterwards each keeps the block count (the tile shape) with the
 * lowest mean time if it beats the default by more than 3 %.  The default, also before
 * any tuning, is the block count every cooperative kernel can hold at once.  Results are the same under every block count.  LEM_ERR_STATE while
 * profiling is on (and lem_set_profiling and lem_profile_read return it while
 * tuning). */
#define LEM_TUNE_COOP 8   /* k_plateau_relax, k_flood_merge, k_flood_jump, k_flood_spill,
                             k_fat_coarse, k_fa_walk, k_sedt_coarse, k_sed_walk */
typedef struct lem_tuning {
    int32_t state;                          /* 0 default schedule, 1 tuning, 2 tuned            */
    int32_t steps_left;                     /* tuning steps still to run                        */
    int32_t coop_blocks[LEM_TUNE_COOP];     /* blocks each cooperative kernel launches with    */
    double default_ms;                      /* ms per step of these kernels, default schedule  */
    double tuned_ms;                        /*   and with the schedule kept (as measured)       */
    int32_t flowdirs_tile_rows;             /* rows of the flow-direction kernel's 32-column TMA
                                               tiles (8, 16 or 32); 0: plain loads (grid width
                                               not a multiple of 16)                             */
    int32_t pad;
} lem_tuning;
lem_status lem_autotune(lem_handle* h, int32_t cycles);
lem_status lem_get_tuning(lem_handle* h, lem_tuning* out);

/* Asynchronous export of finished grids.  No counterpart in the reference,
 * whose writegrids (MEM_kernels/io.cpp:201-230) reads host arrays that every
 * stage copied back synchronously.  lem_dem_export snapshots the given fields
 * of DEM `id` (0 for a single-grid handle) on the handle's stream -- after the
 * steps enqueued so far, before any later step or lem_dem_remove changes the
 * region -- and copies the snapshot to pinned host memory on a second stream,
 * so the copy overlaps the handle's next steps; it returns at once.
 * lem_export_ready says whether the copy has finished; lem_export_wait waits
 * for it, writes field k into host[k] in the types of lem_get_field (a NULL
 * host[k] skips the field) and releases the export.  Every export must be
 * waited for, and before lem_destroy (which refuses with LEM_ERR_STATE while
 * exports are open).  LEM_F_DEM_ROUTED cannot be exported. */
typedef struct lem_export lem_export;
lem_status lem_dem_export(lem_handle* h, int32_t id, const lem_field* fields, int32_t nfields, lem_export** out);
lem_status lem_export_ready(lem_export* e, int32_t* ready);
lem_status lem_export_wait(lem_export* e, void* const* host);

/* Bytes of device memory the handle holds for its resident state (what an
 * admission budget counts; exports add their snapshot while in flight).  No
 * counterpart in the reference. */
size_t lem_device_bytes(lem_handle* h);

/* Restart snapshot of one DEM's resident state: the DEM, the DEM of the
 * initial climate grids, the mask, the persistent slopes (whose stale entries
 * the next steps read), the seven soil and vegetation fields, the outlet and
 * the climate scalars -- what the reference's restart rereads
 * (retriveProcessMatrices, MEM_kernels/ioGDAL.cpp:662+), as one binary block
 * instead of rasters.  id: 0 for a single-grid handle, a DEM of a batch.
 * Loading needs a DEM of the same size (a new single-grid handle may load
 * before any lem_set_field); the steps after a load equal the steps after the
 * save. */
size_t lem_snapshot_bytes(lem_handle* h, int32_t id);
lem_status lem_snapshot_save(lem_handle* h, int32_t id, void* host, size_t bytes);
lem_status lem_snapshot_load(lem_handle* h, int32_t id, const void* host, size_t bytes);

/* Flow accumulation that allocates nothing.  No counterpart in the reference.
 * It serves callers that must not allocate device memory themselves or through
 * this library: a host program that hands the path only buffers carved from its
 * own device arena, or a memory-budgeted service that may not call cudaMalloc
 * on its request path (cudaMalloc synchronises the whole device and can fail
 * under fragmentation).
 * Inputs and the output are the caller's device arrays, width*height each:
 *   d_fd      int32 direction codes, one bit per receiving neighbour (N 64,
 *             NE 128, E 1, SE 2, S 4, SW 8, W 16, NW 32), -9999 outside;
 *   d_weight  the runoff weight of every cell;
 *   d_dem     the elevations; cells equal to -9999 are outside the catchment,
 *             pass no flow and output 0;
 *   d_fa      receives, for every cell inside, its weight plus the full
 *             accumulation of every neighbour whose code points at it (a donor
 *             passes its whole flow to every receiver bit), donors summed in the
 *             order E, SE, S, SW, W, NW, N, NE.
 * Cells that no chain of finished donors reaches (a cycle in the codes, or
 * everything below one) output their own weight and the call returns
 * LEM_ERR_NOCONVERGE after writing d_fa.
 * Intermediate data lives in one statically allocated device array sized for
 * LEM_NOALLOC_MAX_CELLS cells (about 27 MB, held by every GPU that loads the
 * library until the process exits); larger grids are rejected with
 * LEM_ERR_CAPACITY before any work.  The call looks up that array's device
 * address on the current device; the first call on a device must come before
 * any stream capture on it (later calls inside a capture reuse the address of
 * the previous call).  All calls share the array and each starts by clearing
 * what it counts: calls whose work overlaps on the GPU (other threads or
 * streams) race, so serialise them.  The call is stream-ordered on `stream`
 * (NULL: the default stream) and returns after its work has finished. */
#define LEM_NOALLOC_MAX_CELLS (1 << 20)
lem_status lem_accumulate_flow_noalloc(const int32_t* d_fd, const double* d_weight, const double* d_dem,
                                       double* d_fa, int32_t width, int32_t height, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LEM_GB300_H */
