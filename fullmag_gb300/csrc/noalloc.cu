// noalloc.cu -- magnetization upload that allocates no memory.
//
// The regular upload (fullmag_fdm_backend_upload_magnetization_f64) stages the host
// AoS doubles in a device buffer that the handle allocates with cudaMalloc on first
// use.  Some callers cannot allow that: a solver loop that edits the state while other
// streams run on the device (cudaMalloc / cudaFree may synchronise the whole device
// and stall them), or a process whose device memory is fully reserved up front.  This
// variant stages through a fixed file-scope device array instead, so it never calls
// an allocating routine.
//
// Limits and rules:
//  * at most kNoAllocMaxCells cells (the scratch is 3 * kNoAllocMaxCells doubles,
//    6 MiB); larger grids are rejected and must use the regular upload;
//  * the scratch is resolved with cudaGetSymbolAddress once per device, on the first
//    call for a handle on that device, with that device made current for the lookup.
//    With lazy module loading (the CUDA 12+ default) that first call also loads this
//    file's module and its 6 MiB array, which can synchronise the device once; later
//    calls do not.  Make the first call before any stream capture and before the
//    latency-critical part of a run;
//  * nothing in the scratch has to start at zero: the kernel reads only the 3n doubles
//    the same call copied in;
//  * all handles on one device share the scratch, so calls that overlap in time (for
//    example from several host threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "noalloc.h"

namespace fm {

namespace {

static __device__ __align__(256) double g_upload_scratch[3 * kNoAllocMaxCells];

constexpr int kMaxDevices = 64;
// Resolved addresses, one per device, kept for the life of the process.  They belong to
// the device's primary context: a caller that destroys that context (cudaDeviceReset)
// invalidates them, and must not use this upload afterwards in the same process.
double *g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

// AoS double -> SoA float conversion reading the static scratch (the converter of the
// regular upload reads the handle's staging buffer instead).
__global__ void noalloc_aos_to_soa_kernel(const double *__restrict__ in, float *__restrict__ out,
                                          const uint8_t *__restrict__ mask, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const bool act = mask == nullptr || mask[i] != 0;
        for (int c = 0; c < 3; ++c) out[c * n + i] = act ? (float)in[3 * i + c] : 0.f;
    }
}

cudaError_t scratch_for(int device, double **out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        int prev = -1;
        cudaError_t rc = cudaGetDevice(&prev);
        if (rc != cudaSuccess) return rc;
        if (prev != device && (rc = cudaSetDevice(device)) != cudaSuccess) return rc;
        void *p = nullptr;
        rc = cudaGetSymbolAddress(&p, g_upload_scratch);
        if (prev != device) {
            const cudaError_t r2 = cudaSetDevice(prev);
            if (rc == cudaSuccess) rc = r2;
        }
        if (rc != cudaSuccess) return rc;
        g_scratch_addr[device] = static_cast<double *>(p);
    }
    *out = g_scratch_addr[device];
    return cudaSuccess;
}

}  // namespace

cudaError_t noalloc_upload_f64(int device, const double *m_xyz, long long n, float *dst_soa, const uint8_t *mask,
                               cudaStream_t stream) {
    if (n <= 0 || n > kNoAllocMaxCells) return cudaErrorInvalidValue;
    double *scratch = nullptr;
    cudaError_t rc = scratch_for(device, &scratch);
    if (rc != cudaSuccess) return rc;
    rc = cudaMemcpyAsync(scratch, m_xyz, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, stream);
    if (rc != cudaSuccess) return rc;
    noalloc_aos_to_soa_kernel<<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, stream>>>(scratch, dst_soa,
                                                                                                      mask, n);
    rc = cudaGetLastError();
    if (rc != cudaSuccess) return rc;
    return cudaStreamSynchronize(stream);
}

}  // namespace fm
