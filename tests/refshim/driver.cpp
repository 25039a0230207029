// driver.cpp -- the timestep loop of PARALLEM's driver (lem.cpp:45-97,114) on a
// Data struct, calling the reference's stage entry points in the driver's
// order; linked against liblem_refshim.so by tests/test_refshim.py.
//
// TEST INFRASTRUCTURE.  Inputs come as arrays instead of the par, ASCII and
// climate files lem.cpp reads; everything between reading and writing follows
// lem.cpp: copyMask, copylastclimate, createDeviceSpace, then per iteration
// (SetClimateMatrices scalars for i >= 0) setdevicespace_FD, cuFlowDirection,
// cleardevicespace_FD, setdevicespace_FA, computeRunOffWeights, calcwater,
// calcpropsSFD, correctmfdflow, cleardevicespace_FA, setdevicespace_Process,
// erosionGPU, cleardevicespace_Process, the summary row, zerogrids; finally
// clearDeviceSpace.
#include <chrono>
#include <cstdlib>
#include <cstring>

#include "lem_refshim.h"

namespace {
double* dup(const double* src, long n) {
    double* p = (double*)std::malloc(sizeof(double) * n);
    std::memcpy(p, src, sizeof(double) * n);
    return p;
}
double* zeros(long n) { return (double*)std::calloc(n, sizeof(double)); }
double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}
}  // namespace

// soil: stone, fines, soilT, soilM, soilB, nut, TotB (7 * N).  out: dem, fa,
// runoffweight, SlopePtr, stone, fines, soilT, soilM, soilB, nut, TotB, ero,
// inci, geli, depo, dz (16 * N).  codes: fd, SFD (2 * N).  rows: per step
// totE, totI, totG, totD, totweatherC, totweatherP, totbio, FA_max, sinkcount,
// outletcellidx (10 per step).  stage_ms (optional): per step the flow-direction,
// accumulation and erosion calls with their device-space calls, and the whole
// step, wall clock.  Returns lem_refshim_status().
extern "C" int refshim_run(int W, int H, double cellsize, const double* dem, const double* soil, int outlet,
                           const lem_params* p, double init_rain, double init_temp, int first_iter, int steps,
                           const double* rain, const double* temp, double* out, int* codes, double* rows,
                           double* stage_ms) {
    const long N = (long)W * H;
    Data data;
    Data device;
    std::memset(&data, 0, sizeof data);
    std::memset(&device, 0, sizeof device);
    data.mapInfo.width = W;
    data.mapInfo.height = H;
    data.mapInfo.cellsize = cellsize;
    data.mapInfo.nodata = -9999;
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
    data.start_iter = first_iter;
    data.runiniter = 0;
    data.rain = data.last_rain = init_rain;
    data.temp = data.last_temp = init_temp;
    data.outletcellidx = outlet;
    data.dem = dup(dem, N);
    data.mask = (int*)std::malloc(sizeof(int) * N);
    for (long i = 0; i < N; ++i) data.mask[i] = dem[i] != -9999 ? 1 : 0;  // createmask
    data.fd = (int*)std::calloc(N, sizeof(int));
    data.SFD = (int*)std::calloc(N, sizeof(int));
    data.prevfd = (int*)std::calloc(N, sizeof(int));
    data.fa = zeros(N);
    data.runoffweight = zeros(N);
    data.SlopePtr = zeros(N);
    data.Slopes = zeros(8 * N);
    data.prop = zeros(8 * N);
    data.stonePtr = dup(soil + 0 * N, N);
    data.finesPtr = dup(soil + 1 * N, N);
    data.soilTPtr = dup(soil + 2 * N, N);
    data.soilMPtr = dup(soil + 3 * N, N);
    data.soilBPtr = dup(soil + 4 * N, N);
    data.nutPtr = dup(soil + 5 * N, N);
    data.TotBPtr = dup(soil + 6 * N, N);
    data.eroPtr = zeros(N);
    data.inciPtr = zeros(N);
    data.geliPtr = zeros(N);
    data.depoPtr = zeros(N);
    data.dz = zeros(N);
    data.weatherC = zeros(N);
    data.weatherP = zeros(N);

    copyMask(&data, &device);
    copylastclimate(&data, &device);
    createDeviceSpace(&data, &device);
    for (int k = 0; k < steps; ++k) {
        const int i = first_iter + k;
        if (i >= 0) {  // SetClimateMatrices(&data, i): this step's scalars
            data.rain = rain[k];
            data.temp = temp[k];
        }
        const double t0 = now_ms();
        setdevicespace_FD(&data, &device);
        cuFlowDirection(&data, &device, i);
        cleardevicespace_FD(&data, &device);
        const double t1 = now_ms();
        setdevicespace_FA(&data, &device);
        computeRunOffWeights(&data, &device);
        calcwater(&data);
        calcpropsSFD(&data, &device);
        correctmfdflow(&data, &device, i);
        cleardevicespace_FA(&data, &device);
        const double t2 = now_ms();
        setdevicespace_Process(&data, &device);
        erosionGPU(&data, &device, i);
        cleardevicespace_Process(&data, &device);
        const double t3 = now_ms();  // every shim call returns after its device work
        if (stage_ms) {
            stage_ms[4 * k + 0] = t1 - t0;
            stage_ms[4 * k + 1] = t2 - t1;
            stage_ms[4 * k + 2] = t3 - t2;
            stage_ms[4 * k + 3] = t3 - t0;
        }
        double* r = rows + 10 * k;  // writeSummaryDataToFile's fields (io.cpp:233-263)
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
        if (k + 1 < steps) zerogrids(&data);  // lem.cpp:101 (cell 0 of six grids; the last step's grids are returned)
    }
    const double* grids[] = {data.dem, data.fa, data.runoffweight, data.SlopePtr, data.stonePtr, data.finesPtr,
                             data.soilTPtr, data.soilMPtr, data.soilBPtr, data.nutPtr, data.TotBPtr, data.eroPtr,
                             data.inciPtr, data.geliPtr, data.depoPtr, data.dz};
    for (int g = 0; g < 16; ++g) std::memcpy(out + g * N, grids[g], sizeof(double) * N);
    std::memcpy(codes, data.fd, sizeof(int) * N);
    std::memcpy(codes + N, data.SFD, sizeof(int) * N);
    clearDeviceSpace(&data, &device);
    for (void* q : {(void*)data.dem, (void*)data.mask, (void*)data.fd, (void*)data.SFD, (void*)data.prevfd,
                    (void*)data.fa, (void*)data.runoffweight, (void*)data.SlopePtr, (void*)data.Slopes,
                    (void*)data.prop, (void*)data.stonePtr, (void*)data.finesPtr, (void*)data.soilTPtr,
                    (void*)data.soilMPtr, (void*)data.soilBPtr, (void*)data.nutPtr, (void*)data.TotBPtr,
                    (void*)data.eroPtr, (void*)data.inciPtr, (void*)data.geliPtr, (void*)data.depoPtr,
                    (void*)data.dz, (void*)data.weatherC, (void*)data.weatherP})
        std::free(q);
    return (int)lem_refshim_status();
}
