// common/macros.h of the headless engine: CUDACHECK for code written against the reference's interface.
// The reference's version reports through the Windows debugger (libs/common/include/common/macros.h:8-26);
// here a failing call prints the call, the error and the location, then aborts.
#pragma once
#include <cstdio>
#include <cstdlib>

#define CUDACHECK(x)                                                                                       \
    do {                                                                                                   \
        cudaError_t gpe_check_err_ = (x);                                                                  \
        if (gpe_check_err_ != cudaSuccess) {                                                               \
            std::fprintf(stderr, "%s:%d %s -> %s\n", __FILE__, __LINE__, #x,                               \
                         cudaGetErrorString(gpe_check_err_));                                              \
            std::abort();                                                                                  \
        }                                                                                                  \
    } while (0)
