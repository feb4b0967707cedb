// Stand-in for the CUDA samples' helper_cuda.h, which the reference's sources include but
// which is not part of the CUDA toolkit: the two error-check macros they use.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>
#define checkCudaErrors(x)                                                  \
    do {                                                                    \
        cudaError_t e_ = (x);                                               \
        if (e_ != cudaSuccess) {                                            \
            fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(e_));    \
            exit(1);                                                        \
        }                                                                   \
    } while (0)
#define getLastCudaError(m)                                                 \
    do {                                                                    \
        cudaError_t e_ = cudaGetLastError();                                \
        if (e_ != cudaSuccess) {                                            \
            fprintf(stderr, "%s: %s\n", (m), cudaGetErrorString(e_));       \
            exit(1);                                                        \
        }                                                                   \
    } while (0)
