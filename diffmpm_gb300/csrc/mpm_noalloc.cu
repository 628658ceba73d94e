// mpm_volume_setup_noalloc: the particle volume set-up without device allocation.
//
// Some callers cannot call cudaMalloc: a JAX/XLA FFI handler receives its input
// and output buffers from XLA's allocator and must not allocate device memory
// of its own, and an application that embeds this library inside a framework
// owning the device memory pool has the same constraint.  This entry point
// serves them: the caller passes the particle positions and densities and the
// three output arrays, and the per-element particle counters the computation
// needs live in a file-scope __device__ array of fixed size instead of memory
// allocated per call.
//
// The counter array holds kMaxElements ints (4 MiB) and stays resident on every
// GPU that loads this library until the process exits.  Its device address is
// looked up once per device with cudaGetSymbolAddress, by the first call made
// while that device is current; make that first call before any stream capture
// on the device.  Every call uses the same array: each call clears the counters
// it needs before counting, and calls whose work overlaps on the GPU (two
// streams, or two host threads) race on the counters, so such calls must be
// ordered by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/diffmpm_gb300.h"
#include "mpm_device.cuh"
#include "mpm_kernels.h"

// The per-element counters.  In host code this name is only a stand-in for the
// device symbol, not a device address: kernels receive the address that
// cudaGetSymbolAddress returns for the current device.
static __device__ __align__(256) int g_element_count[MPM_NOALLOC_MAX_ELEMENTS];

namespace {

constexpr int kMaxElements = MPM_NOALLOC_MAX_ELEMENTS;
constexpr int kMaxDevices = 64;

std::mutex g_mutex;
int* g_count_addr[kMaxDevices] = {};

// Failures are reported through mpm_last_error(NULL), like mpm_create's.
int noalloc_fail(int code, const std::string& msg) {
    mpm::set_thread_error(msg);
    return code;
}

// Device address of g_element_count on the current device (set up once per device).
int counters(int** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(MPM_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(MPM_ERR_UNSUPPORTED, "device index too large");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_count_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_element_count);
        if (e != cudaSuccess)
            return noalloc_fail(MPM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_count_addr[dev] = static_cast<int*>(p);
    }
    *out = g_count_addr[dev];
    return MPM_OK;
}

__global__ void k_noalloc_count(const float* __restrict__ loc, int n, int nx, int ny, float hx,
                                float hy, int* __restrict__ count, int32_t* __restrict__ eid) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int i = mpm::locate_axis(loc[2 * (size_t)p], hx, nx);
    const int j = mpm::locate_axis(loc[2 * (size_t)p + 1], hy, ny);
    int e = -1;
    if (i >= 0 && i < nx && j >= 0 && j < ny) {
        e = j * nx + i;
        atomicAdd(&count[e], 1);
    }
    eid[p] = e;
}

__global__ void k_noalloc_volume(int n, const int32_t* __restrict__ eid,
                                 const int* __restrict__ count, float vol_el,
                                 const float* __restrict__ density, float* __restrict__ volume,
                                 float* __restrict__ mass) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int e = eid[p];
    const int c = e >= 0 ? count[e] : 0;
    const float V = c ? mpm::fdv(vol_el, (float)c) : 0.0f;
    volume[p] = V;
    mass[p] = mpm::fm(V, density[p]);
}

}  // namespace

extern "C" int mpm_volume_setup_noalloc(int nx, int ny, double hx, double hy, int64_t n,
                                        const float* loc, const float* density,
                                        int32_t* element_id, float* volume, float* mass,
                                        void* stream) {
    if (nx < 1 || ny < 1) return noalloc_fail(MPM_ERR_INVALID, "nx and ny must be positive");
    if ((int64_t)nx * ny > kMaxElements) {
        char buf[160];
        snprintf(buf, sizeof buf, "mesh of %lld elements exceeds the no-allocation limit of %d elements",
                 (long long)nx * ny, kMaxElements);
        return noalloc_fail(MPM_ERR_INVALID, buf);
    }
    if (!(hx > 0) || !(hy > 0)) return noalloc_fail(MPM_ERR_INVALID, "element lengths must be positive");
    if (n < 0 || n > 0x7fffffff) return noalloc_fail(MPM_ERR_INVALID, "particle count out of range");
    if (n == 0) return MPM_OK;
    if (!loc || !density || !element_id || !volume || !mass)
        return noalloc_fail(MPM_ERR_INVALID, "null buffer");
    int* count = nullptr;
    int r = counters(&count);
    if (r != MPM_OK) return r;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int) * (size_t)nx * ny, s);
    if (e != cudaSuccess) return noalloc_fail(MPM_ERR_CUDA, cudaGetErrorString(e));
    const float fhx = (float)hx, fhy = (float)hy;
    const int blocks = (int)((n + 255) / 256);
    k_noalloc_count<<<blocks, 256, 0, s>>>(loc, (int)n, nx, ny, fhx, fhy, count, element_id);
    k_noalloc_volume<<<blocks, 256, 0, s>>>((int)n, element_id, count, mpm::element_volume(fhx, fhy),
                                            density, volume, mass);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(MPM_ERR_CUDA, cudaGetErrorString(e));
    return MPM_OK;
}
