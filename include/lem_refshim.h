/*
 * lem_refshim.h -- PARALLEM's own stage entry points, defined on top of the C
 * ABI of include/lem_gb300.h (parallem_gb300/refshim/lem_refshim.cpp, built
 * into liblem_refshim.so).
 *
 * Same names, signatures and C++ linkage as the reference's declarations, so
 * its driver loop (lem.cpp:51-57,83-97,114) links against liblem_refshim.so in
 * place of the objects of FD_kernels/, FA_kernels/, MOD_kernels/runoffweight.cu,
 * MOD_kernels/erosion.cu and MEM_kernels/memory_dev.cu.  Compile with the
 * reference's headers/ on the include path (the reference's Data type).
 *
 * Semantics.  The reference mallocs, uploads, downloads and frees every grid
 * around every stage; here one lem_handle per Data keeps the state resident in
 * HBM from createDeviceSpace to clearDeviceSpace, the setdevicespace_* and
 * cleardevicespace_* calls move nothing, and each stage call refreshes the host
 * arrays the driver reads after it (the host-mirror post-conditions):
 *   cuFlowDirection   fd, SFD, Slopes, dem (outlet lowered by
 *                     testoutletislowest), sinkcount
 *   computeRunOffWeights  runoffweight, soilMPtr (runs the whole
 *                     accumulation stage: runoff, proportions, correctmfdflow)
 *   correctmfdflow    fa, FA_max (from the fa mirror), and on the first
 *                     iteration outletcellidx
 *   erosionGPU        dem, SlopePtr, the seven soil and vegetation grids,
 *                     eroPtr, inciPtr, geliPtr, depoPtr, dz, weatherC, weatherP
 *                     (when allocated) and the tot* budget scalars
 * The host arrays are mirrors: a caller that edits one between steps must
 * write it through lem_set_field on lem_refshim_handle(data).
 * Errors never exit the process (the reference's checkCudaErrors does): a
 * failed call is reported on data->outlog and stderr, and its status is kept
 * for lem_refshim_status().
 */
#ifndef LEM_REFSHIM_H
#define LEM_REFSHIM_H

#include "Data.h"
#include "lem_gb300.h"

/* memory_dev.h:37-57 (MEM_kernels/memory_dev.cu) */
void setslopesspace(Data* data, Data* device);
void setdevicespace_FD(Data* data, Data* device);
void setdevicespace_FA(Data* data, Data* device);
void setdevicespace_Process(Data* data, Data* device);
void cleardevicespace_FD(Data* data, Data* device);
void cleardevicespace_FA(Data* data, Data* device);
void cleardevicespace_Process(Data* data, Data* device);
void createDeviceSpace(Data* data, Data* device);
int clearDeviceSpace(Data* data, Data* device);
int copyMask(Data* data, Data* device);
int copylastclimate(Data* data, Data* device);
int zerogrids(Data* data);
int copytolastclimate(Data* data, Data* device);
/* routeflow.h:34 (FD_kernels/routeflow.cu:686) */
void cuFlowDirection(Data* data, Data* device, int iter);
/* runoffweight.h:27-30 (MOD_kernels/runoffweight.cu:61,115,141,356) */
int computeRunOffWeights(Data* data, Data* device);
void calcpropsSFD(Data* data, Data* device);
void calcprops(Data* data);
void calcwater(Data* data);
/* mfd_simple.h:28 (FA_kernels/mfd_simple.cu:238) */
void correctmfdflow(Data* data, Data* device, int iter);
/* erosion.h:15 (MOD_kernels/erosion.cu:69) */
void erosionGPU(Data* data, Data* device, int iter);

#ifdef __cplusplus
extern "C" {
#endif
/* No counterpart in the reference: the status of the last failed shim call
 * (LEM_OK when none failed since the previous read; reading clears it), and
 * the handle that holds `data`'s state (NULL before createDeviceSpace). */
lem_status lem_refshim_status(void);
lem_handle* lem_refshim_handle(const Data* data);
#ifdef __cplusplus
}
#endif

#endif /* LEM_REFSHIM_H */
