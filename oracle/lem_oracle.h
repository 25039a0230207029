/*
 * lem_oracle.h -- FP64 CPU restatement of the PARALLEM per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA path is compared
 * against (tests/, __graft_entry__.smoke, bench.py's cpu_baseline and
 * --impl reference legs).  Nothing in the product links or calls it.
 *
 * State mirrors the reference's host Data struct (headers/Data.h:15-187): fp64
 * row-major grids, int32 direction codes, Slopes/prop as 8 doubles per cell.
 * Every array is owned by the caller and updated in place.
 */
#ifndef LEM_ORACLE_H
#define LEM_ORACLE_H

#include <stdint.h>
#include "../include/lem_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_state {
    int32_t W, H;
    double cellsize;
    double* dem;           /* N   Data.dem                                  */
    int32_t* mask;         /* N   Data.mask                                 */
    double* slopes;        /* 8N  Data.Slopes (persistent, stale entries kept) */
    double* prop;          /* 8N  device prop (persistent)                  */
    int32_t* fd;           /* N   Data.fd                                   */
    int32_t* sfd;          /* N   Data.SFD                                  */
    double* fa;            /* N                                             */
    double* runoff;        /* N   Data.runoffweight                         */
    double* slopeptr;      /* N   Data.SlopePtr                             */
    double* stone;
    double* fines;
    double* soilT;
    double* soilM;
    double* soilB;
    double* nut;
    double* totB;
    double* ero;
    double* inci;
    double* geli;
    double* depo;
    double* dz;
    double* wC;
    double* wP;
    double* rainmat;       /* N   Data.rainmat                              */
    double* tempmat;       /* N   Data.tempmat                              */
    double* last_rainmat;  /* N   device last_rainmat                       */
    double* last_tempmat;  /* N   device last_tempmat                       */
    float* shortest_paths; /* N   optional: final plateau distances (NULL ok) */
    int32_t* watershed;    /* N   optional: basin labels of the flooding (NULL ok) */
    int32_t* contrib;      /* N   optional: SFD contributing-cell counts (NULL ok) */
    double* dem_routed;    /* N   optional: the DEM the final codes were computed on (raised) */
    int32_t* sfd_pass1;    /* N   optional: SFD codes after the first plateau pass */
    int32_t outlet;        /* Data.outletcellidx                            */
    double rain, temp;     /* Data.rain / Data.temp of the step             */
    double last_rain, last_temp;
    /* outputs of the step */
    double totE, totI, totG, totD, totWC, totWP, totbio, FA_max;
    int32_t sinkcount, init_sinks, init_flats, plateau_sweeps, flood_basins;
    int32_t fa_uncomputed, sed_uncomputed;
} oracle_state;

/* SetClimateMatrices (MEM_kernels/Data.cpp:211-303).  init != 0 is the
 * iteration == -10000 call that also fills the last_* grids. */
void oracle_set_climate(oracle_state* s, int init);

/* setProcessMatrices + createSoilTfromformula-free initial fields
 * (MEM_kernels/Data.cpp:115-209): fills every process grid for a new run. */
void oracle_init_process(oracle_state* s, double stoneval, double fineval, double soilMval,
                         double nutval, double soilBval);

/* createmask (MEM_kernels/memory.cu:217-242) + init_setoutletcell (Data.cpp:38-66). */
void oracle_init_mask_outlet(oracle_state* s);

/* cuFlowDirection (FD_kernels/routeflow.cu:686-975). */
int oracle_flow_direction(oracle_state* s, const lem_params* p);

/* computeRunOffWeights + calcpropsSFD/calcprops + correctmfdflow
 * (MOD_kernels/runoffweight.cu:21-354, FA_kernels/mfd_simple.cu:33-384). */
int oracle_flow_accumulation(oracle_state* s, const lem_params* p, uint32_t flags);

/* erosionGPU (MOD_kernels/erosion.cu:69-186) with its kernels. */
int oracle_erosion(oracle_state* s, lem_params* p);

/* One timestep of lem.cpp:79-97. */
int oracle_step(oracle_state* s, lem_params* p, const lem_climate* c, uint32_t flags);

/* Sizes used by the timing leg. */
int oracle_num_threads(void);
void oracle_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
