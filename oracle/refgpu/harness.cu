// harness.cu -- PARALLEM's own CUDA code run the way lem.cpp runs it, with
// arrays in place of its par, ASCII and climate files, and every stage timed.
//
// TEST AND MEASUREMENT INFRASTRUCTURE: built by oracle/refgpu_build.py together
// with the reference's sources (copied from the reference tree into
// oracle/_ref/gpu), never linked into the product.  The set-up calls are
// lem.cpp:45-57's (createmask, init_setoutletcell, createSoilTfromformula,
// copyMask, SetClimateMatrices(-10000), copylastclimate,
// createProcessMatrices, setProcessMatrices, createDeviceSpace); the given
// initial soil and vegetation state then replaces the par-file values, so both
// implementations start from the same state.  The loop is lem.cpp:67-101.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "Data.h"
#include "erosion.h"
#include "lem_gb300.h"
#include "memory.h"
#include "memory_dev.h"
#include "mfd_simple.h"
#include "routeflow.h"
#include "runoffweight.h"

namespace {
double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}
}  // namespace

// soil: stone, fines, soilT, soilM, soilB, nut, TotB (7 * N).  out: dem, fa,
// runoffweight, SlopePtr, stone, fines, soilT, soilM, soilB, nut, TotB, ero,
// inci, geli, depo, dz (16 * N).  codes: fd, SFD (2 * N).  rows: per step
// totE, totI, totG, totD, totweatherC, totweatherP, totbio, FA_max, sinkcount,
// outletcellidx.  stage_ms: per step cuFlowDirection, accumulation
// (computeRunOffWeights .. correctmfdflow), erosionGPU and the whole step,
// each with its setdevicespace_* / cleardevicespace_* calls, wall clock.
extern "C" int refgpu_run(int W, int H, double cellsize, const double* dem, const double* soil,
                          const lem_params* p, double init_rain, double init_temp, int first_iter, int steps,
                          const double* rain, const double* temp, double* out, int* codes, double* rows,
                          double* stage_ms, const char* logpath) {
    const long N = (long)W * H;
    static Data data;  // lem.cpp keeps both on main's stack; static keeps 5 KB off the caller's
    static Data device;
    std::memset(&data, 0, sizeof data);
    std::memset(&device, 0, sizeof device);
    data.outlog = std::fopen(logpath ? logpath : "/dev/null", "w");
    if (!data.outlog) return 1;
    data.mapInfo.width = W;
    data.mapInfo.height = H;
    data.mapInfo.cellsize = cellsize;
    data.mapInfo.nodata = -9999;
    data.dem = (double*)std::malloc(sizeof(double) * N);
    std::memcpy(data.dem, dem, sizeof(double) * N);
    data.flowdirectiontype = p->flow_direction_type;
    data.soil_struct = p->soil_struct;
    data.profile_permeability = p->profile_permeability;
    data.Qthreshold = p->q_threshold;
    data.Gslope = p->g_slope;
    data.kappa = p->kappa;
    data.Gflowlim = p->g_flowlim;
    data.Flow_A = p->flow_a;
    data.Flow_B = p->flow_b;
    data.max_incision = p->max_incision;
    data.ddk = p->ddk;
    data.dck = p->dck;
    data.dgk = p->dgk;
    data.temp_inflex = p->temp_inflex;
    data.temp_sens = p->temp_sens;
    // the climate series as ReadClimateDataFromFile leaves it: one entry per iteration >= 0
    const int last = first_iter + steps;
    const int nclim = last > 0 ? last : 1;
    data.rainchange = (double*)std::calloc(nclim, sizeof(double));
    data.tempchange = (double*)std::calloc(nclim, sizeof(double));
    for (int k = 0; k < steps; ++k)
        if (first_iter + k >= 0) {
            data.rainchange[first_iter + k] = rain[k];
            data.tempchange[first_iter + k] = temp[k];
        }
    data.rain = init_rain;
    data.temp = init_temp;

    createmask(&data);
    init_setoutletcell(&data);
    createSoilTfromformula(&data);
    copyMask(&data, &device);
    SetClimateMatrices(&data, -10000);
    copylastclimate(&data, &device);
    createProcessMatrices(&data);
    setProcessMatrices(&data);
    double* state[] = {data.stonePtr, data.finesPtr, data.soilTPtr, data.soilMPtr, data.soilBPtr, data.nutPtr,
                       data.TotBPtr};
    for (int f = 0; f < 7; ++f) std::memcpy(state[f], soil + f * N, sizeof(double) * N);
    createDeviceSpace(&data, &device);
    data.start_iter = first_iter;
    data.runiniter = 0;

    for (int k = 0; k < steps; ++k) {
        const int i = first_iter + k;
        checkCudaErrors(cudaDeviceSynchronize());
        const double t0 = now_ms();
        if (i >= 0) SetClimateMatrices(&data, i);
        setdevicespace_FD(&data, &device);
        cuFlowDirection(&data, &device, i);
        cleardevicespace_FD(&data, &device);
        checkCudaErrors(cudaDeviceSynchronize());
        const double t1 = now_ms();
        setdevicespace_FA(&data, &device);
        computeRunOffWeights(&data, &device);
        calcwater(&data);
        calcpropsSFD(&data, &device);
        correctmfdflow(&data, &device, i);
        cleardevicespace_FA(&data, &device);
        checkCudaErrors(cudaDeviceSynchronize());
        const double t2 = now_ms();
        setdevicespace_Process(&data, &device);
        erosionGPU(&data, &device, i);
        cleardevicespace_Process(&data, &device);
        checkCudaErrors(cudaDeviceSynchronize());
        const double t3 = now_ms();
        stage_ms[4 * k + 0] = t1 - t0;
        stage_ms[4 * k + 1] = t2 - t1;
        stage_ms[4 * k + 2] = t3 - t2;
        stage_ms[4 * k + 3] = t3 - t0;
        double* r = rows + 10 * k;
        r[0] = data.totE;
        r[1] = data.totI;
        r[2] = data.totG;
        r[3] = data.totD;
        r[4] = data.totweatherC;
        r[5] = data.totweatherP;
        r[6] = data.totbio;
        r[7] = data.FA_max;
        r[8] = data.sinkcount;
        r[9] = data.outletcellidx;
        if (k + 1 < steps) zerogrids(&data);
    }
    const double* grids[] = {data.dem, data.fa, data.runoffweight, data.SlopePtr, data.stonePtr, data.finesPtr,
                             data.soilTPtr, data.soilMPtr, data.soilBPtr, data.nutPtr, data.TotBPtr, data.eroPtr,
                             data.inciPtr, data.geliPtr, data.depoPtr, data.dz};
    for (int g = 0; g < 16; ++g) std::memcpy(out + g * N, grids[g], sizeof(double) * N);
    std::memcpy(codes, data.fd, sizeof(int) * N);
    std::memcpy(codes + N, data.SFD, sizeof(int) * N);
    clearDeviceSpace(&data, &device);
    std::fclose(data.outlog);
    return 0;
}
