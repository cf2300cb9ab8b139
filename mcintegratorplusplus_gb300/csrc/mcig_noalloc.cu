// mcig_noalloc.cu -- MJBlocker error estimate that allocates no device memory.
//
// mcig_estimate() copies the caller's host array to the device and allocates
// the blocking scratch (a double copy of the data) with cudaMalloc on every
// call.  Some callers cannot do that: code whose device memory is owned
// entirely by its own pool, hosts that forbid device allocation after start-up,
// and loops that must not synchronize the device (cudaMalloc/cudaFree can
// synchronize).  mcig_mjblocker_estimate_noalloc takes device pointers for the
// input and the outputs and uses the file-scope array below as scratch.
//
// The scratch array is MCIG_NOALLOC_MAX_VALUES doubles (16 MiB) held by every
// GPU that loads this library until the process exits.  Every call shares it
// and it keeps the last call's contents; the kernel writes each scratch entry
// before reading it, so nothing needs clearing between calls.  Calls that
// overlap on the GPU (different streams, or several host threads) race on the
// array: the caller must order them.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/mcig.h"
#include "mcig_estimators.cuh"

int mcig_set_last_error(int code, const char *msg); // mcig_capi.cu

static __device__ __align__(256) double g_noalloc_scratch[MCIG_NOALLOC_MAX_VALUES];

// Device address of the scratch array, looked up once per device with that
// device current.  In host code the array's name is only a host-side stand-in,
// never a device address, so it is not handed to a kernel directly.
static std::mutex g_noalloc_mutex;
static double *g_noalloc_ptr[MCIG_NOALLOC_MAX_DEVICES] = {nullptr};

static int noalloc_scratch(int dev, double **out, const char **msg)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            *msg = cudaGetErrorString(e);
            return MCIG_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = (double *)p;
    }
    *out = g_noalloc_ptr[dev];
    return MCIG_OK;
}

extern "C" int mcig_mjblocker_estimate_noalloc(const double *d_x, int64_t n, int ndim, double *d_avg, double *d_err,
                                               void *stream)
{
    static thread_local char err[256];
    if (!d_x || !d_avg || !d_err || ndim < 1) {
        snprintf(err, sizeof(err), "mcig_mjblocker_estimate_noalloc: null pointer or ndim < 1");
        return mcig_set_last_error(MCIG_ERR_INVALID_ARGUMENT, err);
    }
    if (n <= 0 || (n & (n - 1)) != 0) {
        return mcig_set_last_error(MCIG_ERR_INVALID_ARGUMENT, "[MJBlocker] ndata must be a power of two.");
    }
    if (n > (int64_t)MCIG_NOALLOC_MAX_VALUES / ndim) {
        snprintf(err, sizeof(err),
                 "mcig_mjblocker_estimate_noalloc: n*ndim = %lld exceeds the static scratch of %d values; "
                 "use mcig_estimate for larger arrays",
                 (long long)n * ndim, (int)MCIG_NOALLOC_MAX_VALUES);
        return mcig_set_last_error(MCIG_ERR_INVALID_ARGUMENT, err);
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { return mcig_set_last_error(MCIG_ERR_CUDA, cudaGetErrorString(e)); }
    if (dev < 0 || dev >= MCIG_NOALLOC_MAX_DEVICES) {
        return mcig_set_last_error(MCIG_ERR_UNSUPPORTED, "mcig_mjblocker_estimate_noalloc: device ordinal too large");
    }
    double *scratch = nullptr;
    const char *msg = nullptr;
    const int rc = noalloc_scratch(dev, &scratch, &msg);
    if (rc) { return mcig_set_last_error(rc, msg); }
    EstArgs a;
    a.data = d_x;
    a.is_float = 0;
    a.n = n;
    a.nv = ndim;
    a.nchains = 1;
    a.avg = d_avg;
    a.err = d_err;
    a.ldo = ndim;
    a.off = 0;
    a.scratch = scratch;
    a.one_d = (ndim == 1);
    const int block = 128;
    est_mj_kernel<<<(ndim + block - 1) / block, block, 0, (cudaStream_t)stream>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) { return mcig_set_last_error(MCIG_ERR_CUDA, cudaGetErrorString(e)); }
    return MCIG_OK;
}
