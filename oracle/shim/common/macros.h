// Headless stand-in for the reference's libs/common/include/common/macros.h, used only to compile the
// reference's own PBF.cu / MPM.cu unmodified into cubins for the parity tests. The reference's CUDACHECK
// reports through the Windows debugger (macros.h:8-26); here it prints and aborts. Only host code uses it,
// and the cubin build keeps device code only.
#pragma once
#include <cstdio>
#include <cstdlib>

#define CUDACHECK(x)                                                                                       \
    do {                                                                                                   \
        cudaError_t gpe_shim_err = (x);                                                                    \
        if (gpe_shim_err != cudaSuccess) {                                                                 \
            std::fprintf(stderr, "%s:%d %s -> %s\n", __FILE__, __LINE__, #x,                               \
                         cudaGetErrorString(gpe_shim_err));                                                \
            std::abort();                                                                                  \
        }                                                                                                  \
    } while (0)
