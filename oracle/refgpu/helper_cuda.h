// helper_cuda.h -- the one helper the reference's sources take from the CUDA
// Samples (not part of the toolkit): checkCudaErrors, which reports a failed
// runtime call and ends the process, as the Samples' version does.
// TEST INFRASTRUCTURE: used only to build the reference's own CUDA code.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>

#define checkCudaErrors(call)                                                                  \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            std::fprintf(stderr, "CUDA error %s at %s:%d: %s\n", cudaGetErrorName(e_), __FILE__, \
                         __LINE__, #call);                                                     \
            std::exit(EXIT_FAILURE);                                                           \
        }                                                                                      \
    } while (0)
