// capi.cu — error plumbing shared by every C-ABI entry point. The codes follow the reference's render C ABI
// (libs/render/source/cuda-render.cu:23-27 records the cudaError_t in last_error and returns -1), with the
// detail kept per host thread.
#include <cstdarg>
#include <cstdio>

#include "gpe_internal.h"

namespace gpe {

namespace {
thread_local int32_t t_last_cuda = 0;
thread_local char t_msg[512]     = {0};
} // namespace

void set_error(int32_t status, const char* fmt, ...)
{
    (void)status;
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(t_msg, sizeof(t_msg), fmt, ap);
    va_end(ap);
}

void set_cuda_error(cudaError_t e, const char* what)
{
    t_last_cuda = (int32_t)e;
    std::snprintf(t_msg, sizeof(t_msg), "%s -> %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

void clear_error() { t_msg[0] = 0; }

int32_t current_device(int* dev)
{
    int count        = 0;
    cudaError_t e    = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        set_cuda_error(e == cudaSuccess ? cudaErrorNoDevice : e, "cudaGetDeviceCount");
        return GPE_ERR_DEVICE;
    }
    e = cudaGetDevice(dev);
    if (e != cudaSuccess) {
        set_cuda_error(e, "cudaGetDevice");
        return GPE_ERR_DEVICE;
    }
    return GPE_OK;
}

int32_t sm_count()
{
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { return 1; }
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) { return 1; }
    return n > 0 ? n : 1;
}

} // namespace gpe

extern "C" {

const char* gpe_error_name(int32_t status)
{
    switch (status) {
        case GPE_OK: return "GPE_OK";
        case GPE_ERR_CUDA: return "GPE_ERR_CUDA";
        case GPE_ERR_DEVICE: return "GPE_ERR_DEVICE";
        case GPE_ERR_NOT_READY: return "GPE_ERR_NOT_READY";
        case GPE_ERR_BAD_ARG: return "GPE_ERR_BAD_ARG";
        case GPE_ERR_ALREADY: return "GPE_ERR_ALREADY";
        case GPE_ERR_CAPACITY: return "GPE_ERR_CAPACITY";
        case GPE_ERR_NONFINITE: return "GPE_ERR_NONFINITE";
        case GPE_ERR_TIMEOUT: return "GPE_ERR_TIMEOUT";
        default: return "GPE_ERR_UNKNOWN";
    }
}

int32_t gpe_last_cuda_error(void) { return gpe::t_last_cuda; }

const char* gpe_last_error_message(void) { return gpe::t_msg; }

int32_t gpe_version(void) { return 100; }

} // extern "C"
