// lem_refshim.cpp -- PARALLEM's stage entry points on the resident-state C ABI.
//
// Each reference call keeps its name, signature and place in the driver loop
// (lem.cpp:51-57,83-97,114) and becomes the matching lem_gb300 call on one
// handle per Data, created by createDeviceSpace and destroyed by
// clearDeviceSpace.  State stays in HBM between calls; after each stage the
// shim writes the host arrays that the driver and its writers read
// (writeSummaryDataToFile MEM_kernels/io.cpp:233-263, writegrids :201-230).
// Nothing here exits the process: failures are logged and kept for
// lem_refshim_status().

#include "lem_refshim.h"

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>

namespace {

struct Shim {
    lem_handle* h = nullptr;
    int iter = 0;  // the iteration cuFlowDirection was called with (the step's)
};

std::mutex g_mu;
std::map<const Data*, Shim> g_shims;
lem_status g_status = LEM_OK;

Shim* shim_of(const Data* data) {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_shims.find(data);
    return it == g_shims.end() ? nullptr : &it->second;
}

bool ok(Data* data, const char* what, lem_status s) {
    if (s == LEM_OK) return true;
    std::fprintf(stderr, "lem_refshim: %s: %s\n", what, lem_status_string(s));
    if (data && data->outlog) std::fprintf(data->outlog, "lem_refshim: %s: %s\n", what, lem_status_string(s));
    std::lock_guard<std::mutex> lock(g_mu);
    g_status = s;
    return false;
}

// the handle of `data`, or a logged LEM_ERR_STATE when createDeviceSpace has not run
Shim* need(Data* data, const char* what) {
    Shim* sh = data ? shim_of(data) : nullptr;
    if (!sh || !sh->h) ok(data, what, LEM_ERR_STATE);
    return sh && sh->h ? sh : nullptr;
}

// one host mirror (skipped when the driver did not allocate it)
bool pull(Data* data, Shim* sh, lem_field f, void* host, const char* what) {
    return !host || ok(data, what, lem_get_field(sh->h, f, host));
}

bool push(Data* data, Shim* sh, lem_field f, const void* host, const char* what) {
    return !host || ok(data, what, lem_set_field(sh->h, f, host));
}

long cells(const Data* data) { return (long)data->mapInfo.width * data->mapInfo.height; }

// correctmfdflow's first iteration (mfd_simple.cu:335-336)
bool first_iteration(const Data* data, int iter) { return iter == data->start_iter - data->runiniter; }

}  // namespace

// ---- MEM_kernels/memory_dev.cu ------------------------------------------------

void createDeviceSpace(Data* data, Data* device) {
    if (!data) return;
    {
        Shim* old = shim_of(data);
        if (old && old->h) {
            lem_destroy(old->h);
            old->h = nullptr;
        }
    }
    lem_grid_desc g{data->mapInfo.width, data->mapInfo.height, data->mapInfo.cellsize};
    // the driver sets proportions with calcpropsSFD (lem.cpp:91)
    lem_params p{data->flowdirectiontype, 0, data->soil_struct, data->profile_permeability, data->Qthreshold,
                 data->Gslope, data->kappa, data->Gflowlim, data->Flow_A, data->Flow_B, data->max_incision,
                 data->ddk, data->dck, data->dgk, data->temp_inflex, data->temp_sens};
    lem_handle* h = nullptr;
    // the run-in climate SetClimateMatrices(data, -10000) built the grids from (lem.cpp:50)
    if (!ok(data, "createDeviceSpace: lem_create", lem_create(&g, &p, data->rain, data->temp, &h))) return;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        g_shims[data] = Shim{h, 0};
    }
    Shim* sh = shim_of(data);
    push(data, sh, LEM_F_DEM, data->dem, "createDeviceSpace: dem") &&
        ok(data, "createDeviceSpace: outlet", lem_set_outlet(h, data->outletcellidx)) &&
        push(data, sh, LEM_F_STONE, data->stonePtr, "createDeviceSpace: stone") &&
        push(data, sh, LEM_F_FINES, data->finesPtr, "createDeviceSpace: fines") &&
        push(data, sh, LEM_F_SOILT, data->soilTPtr, "createDeviceSpace: soilT") &&
        push(data, sh, LEM_F_SOILM, data->soilMPtr, "createDeviceSpace: soilM") &&
        push(data, sh, LEM_F_SOILB, data->soilBPtr, "createDeviceSpace: soilB") &&
        push(data, sh, LEM_F_NUT, data->nutPtr, "createDeviceSpace: nut") &&
        push(data, sh, LEM_F_TOTB, data->TotBPtr, "createDeviceSpace: TotB") &&
        push(data, sh, LEM_F_SLOPES, data->Slopes, "createDeviceSpace: Slopes");
    if (device) {
        // the driver frees these two device pointers at exit (lem.cpp:120-121)
        device->mask = nullptr;
        device->Flow_C = nullptr;
    }
}

int clearDeviceSpace(Data* data, Data* device) {
    (void)device;
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_shims.find(data);
    if (it != g_shims.end()) {
        if (it->second.h) lem_destroy(it->second.h);
        g_shims.erase(it);
    }
    return 0;
}

int copyMask(Data* data, Data* device) {
    // the mask follows the DEM on the device (createmask semantics); the
    // driver's count of active cells is kept
    if (device) device->mask = nullptr;
    if (!data || !data->mask) return 0;
    int active = 0;
    for (long i = 0; i < cells(data); ++i) active += data->mask[i] == 1;
    data->activecells = active;
    return 0;
}

// The initial climate is the handle's "last" climate (grow_vegetation's
// reference climate, updates.cu:90-92); it is fixed at createDeviceSpace.
int copylastclimate(Data* data, Data* device) {
    (void)data;
    (void)device;
    return 0;
}

// The driver disables this call (lem.cpp:102); the handle keeps the initial
// climate as its "last" climate, so moving it is refused.
int copytolastclimate(Data* data, Data* device) {
    (void)device;
    ok(data, "copytolastclimate", LEM_ERR_INVALID);
    return 1;
}

// The reference clears sizeof(pointer) bytes of each grid (memset with
// sizeof(data->eroPtr), memory_dev.cu:349-360): the first cell only.  Kept as is.
int zerogrids(Data* data) {
    if (!data) return 0;
    double* grids[] = {data->eroPtr, data->geliPtr, data->inciPtr, data->depoPtr, data->fa, data->runoffweight};
    for (double* g : grids)
        if (g) std::memset(g, 0, sizeof(double*));
    return 0;
}

// Stage buffers stay resident: nothing to allocate, upload or free per stage.
void setslopesspace(Data*, Data*) {}
void setdevicespace_FD(Data*, Data*) {}
void setdevicespace_FA(Data*, Data*) {}
void setdevicespace_Process(Data*, Data*) {}
void cleardevicespace_FD(Data*, Data*) {}
void cleardevicespace_Process(Data*, Data*) {}

void cleardevicespace_FA(Data* data, Data* device) {
    (void)device;
    // the codes of this step become prevfd (memory_dev.cu:137)
    if (data && data->prevfd && data->fd) std::memcpy(data->prevfd, data->fd, sizeof(int) * cells(data));
}

// ---- FD_kernels/routeflow.cu ---------------------------------------------------

void cuFlowDirection(Data* data, Data* device, int iter) {
    (void)device;
    Shim* sh = need(data, "cuFlowDirection");
    if (!sh) return;
    sh->iter = iter;
    if (iter >= 0) {
        // lem.cpp:79-81 called SetClimateMatrices(data, i): grids from this step's scalars
        lem_climate c{data->rain, data->temp, 1};
        if (!ok(data, "cuFlowDirection: climate", lem_set_climate(sh->h, &c))) return;
    }
    if (!ok(data, "cuFlowDirection", lem_flow_direction(sh->h))) return;
    if (!ok(data, "cuFlowDirection", lem_synchronize(sh->h))) return;
    lem_totals t;
    pull(data, sh, LEM_F_FD, data->fd, "cuFlowDirection: fd") &&
        pull(data, sh, LEM_F_SFD, data->SFD, "cuFlowDirection: SFD") &&
        pull(data, sh, LEM_F_SLOPES, data->Slopes, "cuFlowDirection: Slopes") &&
        pull(data, sh, LEM_F_DEM, data->dem, "cuFlowDirection: dem") &&
        ok(data, "cuFlowDirection: totals", lem_get_totals(sh->h, &t)) && (data->sinkcount = t.sinkcount, true);
}

// ---- MOD_kernels/runoffweight.cu, FA_kernels/mfd_simple.cu ---------------------

int computeRunOffWeights(Data* data, Data* device) {
    (void)device;
    Shim* sh = need(data, "computeRunOffWeights");
    if (!sh) return 0;
    // the whole accumulation stage runs here (runoff weights, proportions,
    // correctmfdflow), so that calcwater sees this step's weights
    const uint32_t flags = first_iteration(data, sh->iter) ? LEM_STEP_SET_OUTLET_FROM_FA : 0u;
    if (!ok(data, "computeRunOffWeights", lem_flow_accumulation(sh->h, flags))) return 0;
    if (!ok(data, "computeRunOffWeights", lem_synchronize(sh->h))) return 0;
    pull(data, sh, LEM_F_RUNOFF, data->runoffweight, "computeRunOffWeights: runoffweight") &&
        pull(data, sh, LEM_F_SOILM, data->soilMPtr, "computeRunOffWeights: soilM");
    return 1;
}

void calcwater(Data* data) {
    if (!data || !data->mask || !data->runoffweight) return;
    double sumwater = 0.0;
    for (long i = 0; i < cells(data); ++i)
        if (data->mask[i] == 1) sumwater += data->runoffweight[i];
    std::printf("Total amount of water in grid for runoff = %lf \n", sumwater);
    if (data->outlog) std::fprintf(data->outlog, "Total amount of water in grid for runoff = %lf \n", sumwater);
}

void calcpropsSFD(Data* data, Data* device) {
    (void)device;
    // the device proportions are calcpropsSFD's (lem_params.mfd_proportions = 0);
    // the host array gets the same values (runoffweight.cu:127-133)
    if (!data || !data->prop || !data->mask) return;
    for (long i = 0; i < cells(data); ++i)
        for (int k = 0; k < 8; ++k) data->prop[8 * i + k] = data->mask[i] == 1 ? 1.0 : 0.0;
}

// calcprops' slope-proportional partition is a handle property fixed at
// creation (lem_params.mfd_proportions = 1); the shim's handles use
// calcpropsSFD's, as the driver does, so this call is refused.
void calcprops(Data* data) { ok(data, "calcprops", LEM_ERR_INVALID); }

void correctmfdflow(Data* data, Data* device, int iter) {
    (void)device;
    Shim* sh = need(data, "correctmfdflow");
    if (!sh) return;
    lem_totals t;
    if (!data->fa || !pull(data, sh, LEM_F_FA, data->fa, "correctmfdflow: fa")) return;
    if (!ok(data, "correctmfdflow: totals", lem_get_totals(sh->h, &t))) return;
    // FA_max: the largest accumulation, from 0 up (mfd_simple.cu:338-354); the
    // device derives it later, in the erosion stage, so it is taken here from
    // the mirror
    double fa_max = 0.0;
    for (long i = 0; i < cells(data); ++i)
        if (data->fa[i] > fa_max) fa_max = data->fa[i];
    data->FA_max = fa_max;
    // the first iteration's outlet, which the stage moved to the first cell
    // holding that maximum (mfd_simple.cu:336-349)
    if (first_iteration(data, iter)) data->outletcellidx = t.outlet;
    if (data->outlog) {
        std::fprintf(data->outlog, "Number of actual cells not computed = %d\n", t.fa_uncomputed);
        std::fprintf(data->outlog, "FA: Maximum FA is  %.6f \n\n", data->FA_max);
        std::fprintf(data->outlog, "FA: Outletcell index is  %d \n\n", data->outletcellidx);
    }
}

// ---- MOD_kernels/erosion.cu ------------------------------------------------------

void erosionGPU(Data* data, Data* device, int iter) {
    (void)device;
    (void)iter;
    Shim* sh = need(data, "erosionGPU");
    if (!sh) return;
    const bool diag = data->dz && data->weatherC && data->weatherP;
    if (!ok(data, "erosionGPU", lem_erosion(sh->h, diag ? LEM_STEP_KEEP_DIAGNOSTICS : 0u))) return;
    if (!ok(data, "erosionGPU", lem_synchronize(sh->h))) return;
    const struct {
        lem_field f;
        double* host;
        const char* name;
    } grids[] = {
        {LEM_F_DEM, data->dem, "erosionGPU: dem"},         {LEM_F_SLOPEPTR, data->SlopePtr, "erosionGPU: SlopePtr"},
        {LEM_F_FINES, data->finesPtr, "erosionGPU: fines"}, {LEM_F_STONE, data->stonePtr, "erosionGPU: stone"},
        {LEM_F_SOILT, data->soilTPtr, "erosionGPU: soilT"}, {LEM_F_SOILM, data->soilMPtr, "erosionGPU: soilM"},
        {LEM_F_SOILB, data->soilBPtr, "erosionGPU: soilB"}, {LEM_F_NUT, data->nutPtr, "erosionGPU: nut"},
        {LEM_F_TOTB, data->TotBPtr, "erosionGPU: TotB"},    {LEM_F_ERO, data->eroPtr, "erosionGPU: ero"},
        {LEM_F_INCI, data->inciPtr, "erosionGPU: inci"},    {LEM_F_GELI, data->geliPtr, "erosionGPU: geli"},
        {LEM_F_DEPO, data->depoPtr, "erosionGPU: depo"},    {LEM_F_DZ, diag ? data->dz : nullptr, "erosionGPU: dz"},
        {LEM_F_WEATHER_C, diag ? data->weatherC : nullptr, "erosionGPU: weatherC"},
        {LEM_F_WEATHER_P, diag ? data->weatherP : nullptr, "erosionGPU: weatherP"},
    };
    for (const auto& g : grids)
        if (!pull(data, sh, g.f, g.host, g.name)) return;
    lem_totals t;
    if (!ok(data, "erosionGPU: totals", lem_get_totals(sh->h, &t))) return;
    data->totE = t.tot_e;
    data->totI = t.tot_i;
    data->totG = t.tot_g;
    data->totD = t.tot_d;
    data->totweatherC = t.tot_weather_c;
    data->totweatherP = t.tot_weather_p;
    data->totbio = t.tot_bio;
}

// ---- no counterpart in the reference ---------------------------------------------

extern "C" lem_status lem_refshim_status(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    const lem_status s = g_status;
    g_status = LEM_OK;
    return s;
}

extern "C" lem_handle* lem_refshim_handle(const Data* data) {
    Shim* sh = shim_of(data);
    return sh ? sh->h : nullptr;
}
