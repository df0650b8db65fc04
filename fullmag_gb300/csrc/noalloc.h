// noalloc.h -- allocation-free magnetization upload (noalloc.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fm {

// Largest grid the allocation-free upload accepts (cells); its staging scratch is a
// file-scope device array of 3 * kNoAllocMaxCells doubles (6 MiB).
constexpr long long kNoAllocMaxCells = 1LL << 18;

// Copies n AoS double triples from host memory into the static scratch of `device`,
// converts them to SoA float in dst_soa (inactive cells of `mask` set to zero) and
// synchronises `stream`.  Allocates nothing; n must be in [1, kNoAllocMaxCells].
cudaError_t noalloc_upload_f64(int device, const double *m_xyz, long long n, float *dst_soa, const uint8_t *mask,
                               cudaStream_t stream);

}  // namespace fm
