// columns.cu -- y/z transforms of the demag convolution and the tensor multiply,
// plus the deterministic final reduction of the per-block statistics.
//
// Reference behaviour restated (paths in mzrptu/fullmag):
//   tensor multiply H(k) = -N(k) M(k)          native/backends/fdm/src/demag_fp32.cu:138-164
//                                              crates/fullmag-engine/src/fdm_fields.rs:560-588
//   multi-pass FP64 reductions                 native/backends/fdm/src/reductions_fp64.cu:30-84,354-393
// Here the kernel is real and octant-unique (6 floats per octant frequency), the
// multiply sits between the forward and inverse z (3-D) or y (thin film)
// transforms of one CTA, and the y-frequencies ky and py-ky share one CTA so
// every octant kernel value is read from HBM once per evaluation.
#include "engine.h"

namespace fm {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ void kernel_mirror(int k, int p, int &km, float &sg) {
    if (k > p / 2) {
        km = p - k;
        sg = -1.f;
    } else {
        km = k;
        sg = 1.f;
    }
}

// X[c][z][y<ny][kx] -> Y[c][z][ky<py][kx] (forward along y, zero rows pruned)
__global__ void __launch_bounds__(kThreads) y_forward_kernel(const ColPass p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = blockIdx.x * tx, ncol = min(tx, g.nkx - kx0);
    const int z = blockIdx.y, c = blockIdx.z;
    const int ls = skewed_len(g.py);
    float2 *a = reinterpret_cast<float2 *>(smem);
    float2 *b = a + tx * ls;
    const float2 *src = p.in + ((size_t)c * g.nz + z) * g.ny * g.nkx;
    batched_copy<8>(
        g.ny * tx,
        [&](int idx) {
            const int y = p.fd_tx.div(idx), col = idx - y * tx;
            return col < ncol ? src[(size_t)y * g.nkx + kx0 + col] : make_float2(0.f, 0.f);
        },
        [&](int idx, float2 v) {
            const int y = p.fd_tx.div(idx), col = idx - y * tx;
            a[col * ls + sk(y)] = v;
        });
    for (int line = threadIdx.x >> 5; line < tx; line += blockDim.x >> 5)  // zero padding rows
        for (int y = g.ny + (threadIdx.x & 31); y < g.py; y += 32) a[line * ls + sk(y)] = make_float2(0.f, 0.f);
    __syncthreads();
    float2 *r = fft_lines(a, b, tx, ls, p.plan, false);
    float2 *dst = p.out + ((size_t)c * g.nz + z) * g.py * g.nkx;
    for (int idx = threadIdx.x; idx < g.py * tx; idx += blockDim.x) {
        const int y = p.fd_tx.div(idx), col = idx - y * tx;
        if (col < ncol) dst[(size_t)y * g.nkx + kx0 + col] = r[col * ls + sk(y)];
    }
}

// Y[c][z][ky][kx] -> X[c][z][y<ny][kx] (inverse along y, only physical rows kept)
__global__ void __launch_bounds__(kThreads) y_inverse_kernel(const ColPass p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = blockIdx.x * tx, ncol = min(tx, g.nkx - kx0);
    const int z = blockIdx.y, c = blockIdx.z;
    const int ls = skewed_len(g.py);
    float2 *a = reinterpret_cast<float2 *>(smem);
    float2 *b = a + tx * ls;
    const float2 *src = p.in + ((size_t)c * g.nz + z) * g.py * g.nkx;
    batched_copy<8>(
        g.py * tx,
        [&](int idx) {
            const int y = p.fd_tx.div(idx), col = idx - y * tx;
            return col < ncol ? src[(size_t)y * g.nkx + kx0 + col] : make_float2(0.f, 0.f);
        },
        [&](int idx, float2 v) {
            const int y = p.fd_tx.div(idx), col = idx - y * tx;
            a[col * ls + sk(y)] = v;
        });
    __syncthreads();
    float2 *r = fft_lines(a, b, tx, ls, p.plan, true);
    float2 *dst = p.out + ((size_t)c * g.nz + z) * g.ny * g.nkx;
    for (int idx = threadIdx.x; idx < g.ny * tx; idx += blockDim.x) {
        const int y = p.fd_tx.div(idx), col = idx - y * tx;
        if (col < ncol) dst[(size_t)y * g.nkx + kx0 + col] = r[col * ls + sk(y)];
    }
}

// Number of y-frequencies a CTA handles: ky and py - ky (1 for ky = 0 and the Nyquist row).
__device__ __forceinline__ int ky_pair(int kya, int py, int &kyb) {
    kyb = py - kya;
    return (kya == 0 || kyb == kya) ? 1 : 2;
}

// 3-D: for y-frequencies (ky, py-ky) and a tile of kx, forward z-transform of the
// nz physical planes (zero-padded to pz), multiply by -N(k), inverse, keep nz planes.
__global__ void __launch_bounds__(kThreads) z_convolve_kernel(const ColPass p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = blockIdx.x * tx, ncol = min(tx, g.nkx - kx0);
    const int kya = blockIdx.y;
    int kyb;
    const int np = ky_pair(kya, g.py, kyb);
    const int ls = skewed_len(g.pz);
    const int nl = np * 3 * tx;  // line (q, c, col) at ((q*3 + c)*tx + col)
    float2 *a = reinterpret_cast<float2 *>(smem);
    float2 *b = a + (size_t)2 * 3 * tx * ls;
    const size_t cstride = (size_t)g.nz * g.py * g.nkx;  // component stride of Y
    const size_t zstride = (size_t)g.py * g.nkx;
    batched_copy<8>(
        np * 3 * g.nz * tx,
        [&](int idx) {
            const int r1 = p.fd_tx.div(idx), col = idx - r1 * tx;
            const int r2 = g.fd_nz.div(r1), z = r1 - r2 * g.nz;
            const int q = r2 / 3, c = r2 - 3 * q;
            const int ky = q ? kyb : kya;
            return col < ncol ? p.in[c * cstride + z * zstride + (size_t)ky * g.nkx + kx0 + col] : make_float2(0.f, 0.f);
        },
        [&](int idx, float2 v) {
            const int r1 = p.fd_tx.div(idx), col = idx - r1 * tx;
            const int r2 = g.fd_nz.div(r1), z = r1 - r2 * g.nz;
            a[(r2 * tx + col) * ls + sk(z)] = v;
        });
    // zero the padded planes z in [nz, pz): one warp per line
    for (int line = threadIdx.x >> 5; line < nl; line += blockDim.x >> 5)
        for (int z = g.nz + (threadIdx.x & 31); z < g.pz; z += 32) a[line * ls + sk(z)] = make_float2(0.f, 0.f);
    __syncthreads();
    float2 *r = fft_lines(a, b, nl, ls, p.plan, false);
    float2 *o = (r == a) ? b : a;
    const size_t kc = (size_t)g.nkz * g.nky * g.nkx;
    for (int idx = threadIdx.x; idx < g.pz * tx; idx += blockDim.x) {
        const int kz = p.fd_tx.div(idx), col = idx - kz * tx;
        const int kx = min(kx0 + col, g.nkx - 1);
        int kzm;
        float sz;
        kernel_mirror(kz, g.pz, kzm, sz);
        const float *K = p.kern + ((size_t)kzm * g.nky + kya) * g.nkx + kx;
        const float kxx = __ldg(K), kyy = __ldg(K + kc), kzz = __ldg(K + 2 * kc);
        const float kxy0 = __ldg(K + 3 * kc), kxz = sz * __ldg(K + 4 * kc), kyz0 = sz * __ldg(K + 5 * kc);
        for (int q = 0; q < np; ++q) {
            // the second frequency of the pair is the y-mirror: odd-in-y components flip sign
            const float sy = q ? -1.f : 1.f;
            const float kxy = sy * kxy0, kyz = sy * kyz0;
            float2 *lx = r + ((q * 3 + 0) * tx + col) * ls + sk(kz);
            float2 *ly = r + ((q * 3 + 1) * tx + col) * ls + sk(kz);
            float2 *lz = r + ((q * 3 + 2) * tx + col) * ls + sk(kz);
            const float2 mx = *lx, my = *ly, mz = *lz;
            *lx = make_float2(-(kxx * mx.x + kxy * my.x + kxz * mz.x), -(kxx * mx.y + kxy * my.y + kxz * mz.y));
            *ly = make_float2(-(kxy * mx.x + kyy * my.x + kyz * mz.x), -(kxy * mx.y + kyy * my.y + kyz * mz.y));
            *lz = make_float2(-(kxz * mx.x + kyz * my.x + kzz * mz.x), -(kxz * mx.y + kyz * my.y + kzz * mz.y));
        }
    }
    __syncthreads();
    float2 *qb = fft_lines(r, o, nl, ls, p.plan, true);
    for (int idx = threadIdx.x; idx < np * 3 * g.nz * tx; idx += blockDim.x) {
        const int r1 = p.fd_tx.div(idx), col = idx - r1 * tx;
        const int r2 = g.fd_nz.div(r1), z = r1 - r2 * g.nz;
        const int q = r2 / 3, c = r2 - 3 * q;
        const int ky = q ? kyb : kya;
        if (col < ncol)
            p.out[c * cstride + z * zstride + (size_t)ky * g.nkx + kx0 + col] = qb[((q * 3 + c) * tx + col) * ls + sk(z)];
    }
}

// 3-D grids whose (y, z) plane fits in shared memory: forward y-transform of the nz
// physical planes, in-smem transpose, forward z, multiply, inverse z, transpose back,
// inverse y -- X -> X in place, one pass instead of three and no Y round trip.
// Lines: y-lines (c, col, z) at ((c*tx + col)*nz + z), z-lines (c, col, ky) at
// ((c*tx + col)*py + ky); both layouts share two ping-pong buffers of `half_buf`.
__device__ __forceinline__ void yz_convolve_body(const ColPass &p, const int tile) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const FftPlan &plan_z = p.plan2;
    const int tx = p.tx, kx0 = tile * tx, ncol = min(tx, g.nkx - kx0);
    const int lsy = skewed_len(g.py), lsz = skewed_len(g.pz);
    const int nly = 3 * tx * g.nz, nlz = 3 * tx * g.py;
    const int half_buf = max(nly * lsy, nlz * lsz);
    float2 *P = reinterpret_cast<float2 *>(smem);
    float2 *Q = P + half_buf;
    const size_t cstride = (size_t)g.nz * g.ny * g.nkx;
    batched_copy<8>(
        3 * g.nz * g.ny * tx,
        [&](int idx) {
            const int r = p.fd_tx.div(idx), col = idx - r * tx;
            const int r2 = g.fd_ny.div(r), y = r - r2 * g.ny;
            const int c = g.fd_nz.div(r2), z = r2 - c * g.nz;
            return col < ncol ? p.in[c * cstride + ((size_t)z * g.ny + y) * g.nkx + kx0 + col] : make_float2(0.f, 0.f);
        },
        [&](int idx, float2 v) {
            const int r = p.fd_tx.div(idx), col = idx - r * tx;
            const int r2 = g.fd_ny.div(r), y = r - r2 * g.ny;
            const int c = g.fd_nz.div(r2), z = r2 - c * g.nz;
            P[((c * tx + col) * g.nz + z) * lsy + sk(y)] = v;
        });
    for (int line = threadIdx.x >> 5; line < nly; line += blockDim.x >> 5)
        for (int y = g.ny + (threadIdx.x & 31); y < g.py; y += 32) P[line * lsy + sk(y)] = make_float2(0.f, 0.f);
    __syncthreads();
    float2 *R = fft_lines(P, Q, nly, lsy, p.plan, false);
    float2 *O = (R == P) ? Q : P;
    // transpose to z-lines, zero planes z >= nz
    for (int idx = threadIdx.x; idx < nlz * g.pz; idx += blockDim.x) {
        const int lz = g.fd_pz.div(idx), z = idx - lz * g.pz;
        const int cc = g.fd_py.div(lz), ky = lz - cc * g.py;
        O[lz * lsz + sk(z)] = z < g.nz ? R[(cc * g.nz + z) * lsy + sk(ky)] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *R2 = fft_lines(O, R, nlz, lsz, plan_z, false);
    const size_t kc = (size_t)g.nkz * g.nky * g.nkx;
    for (int idx = threadIdx.x; idx < tx * g.py * g.pz; idx += blockDim.x) {
        const int r = g.fd_pz.div(idx), kz = idx - r * g.pz;
        const int col = g.fd_py.div(r), ky = r - col * g.py;
        const int kx = min(kx0 + col, g.nkx - 1);
        int kym, kzm;
        float sy, sz;
        kernel_mirror(ky, g.py, kym, sy);
        kernel_mirror(kz, g.pz, kzm, sz);
        const float *K = p.kern + ((size_t)kzm * g.nky + kym) * g.nkx + kx;
        const float kxx = __ldg(K), kyy = __ldg(K + kc), kzz = __ldg(K + 2 * kc);
        const float kxy = sy * __ldg(K + 3 * kc), kxz = sz * __ldg(K + 4 * kc), kyz = sy * sz * __ldg(K + 5 * kc);
        float2 *lx = R2 + ((0 * tx + col) * g.py + ky) * lsz + sk(kz);
        float2 *ly = R2 + ((1 * tx + col) * g.py + ky) * lsz + sk(kz);
        float2 *lz = R2 + ((2 * tx + col) * g.py + ky) * lsz + sk(kz);
        const float2 mx = *lx, my = *ly, mz = *lz;
        *lx = make_float2(-(kxx * mx.x + kxy * my.x + kxz * mz.x), -(kxx * mx.y + kxy * my.y + kxz * mz.y));
        *ly = make_float2(-(kxy * mx.x + kyy * my.x + kyz * mz.x), -(kxy * mx.y + kyy * my.y + kyz * mz.y));
        *lz = make_float2(-(kxz * mx.x + kyz * my.x + kzz * mz.x), -(kxz * mx.y + kyz * my.y + kzz * mz.y));
    }
    __syncthreads();
    float2 *R3 = fft_lines(R2, (R2 == P) ? Q : P, nlz, lsz, plan_z, true);
    float2 *O3 = (R3 == P) ? Q : P;
    // transpose back to y-lines, keeping the physical planes z < nz
    for (int idx = threadIdx.x; idx < nly * g.py; idx += blockDim.x) {
        const int ly = g.fd_py.div(idx), ky = idx - ly * g.py;
        const int cc = g.fd_nz.div(ly), z = ly - cc * g.nz;
        O3[ly * lsy + sk(ky)] = R3[(cc * g.py + ky) * lsz + sk(z)];
    }
    __syncthreads();
    float2 *R4 = fft_lines(O3, R3, nly, lsy, p.plan, true);
    for (int idx = threadIdx.x; idx < 3 * g.nz * g.ny * tx; idx += blockDim.x) {
        const int r = p.fd_tx.div(idx), col = idx - r * tx;
        const int r2 = g.fd_ny.div(r), y = r - r2 * g.ny;
        const int c = g.fd_nz.div(r2), z = r2 - c * g.nz;
        if (col < ncol)
            p.out[c * cstride + ((size_t)z * g.ny + y) * g.nkx + kx0 + col] = R4[((c * tx + col) * g.nz + z) * lsy + sk(y)];
    }
}

// Thin film: forward y-transform of ny physical rows (zero-padded to py), multiply by
// the 2-D kernel, inverse, keep ny rows.  X -> X in place.
__device__ __forceinline__ void y_convolve_2d_body(const ColPass &p, const int tile) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = tile * tx, ncol = min(tx, g.nkx - kx0);
    const int ls = skewed_len(g.py);
    const int nl = 3 * tx;
    float2 *a = reinterpret_cast<float2 *>(smem);
    float2 *b = a + nl * ls;
    const size_t cstride = (size_t)g.ny * g.nkx;
    batched_copy<8>(
        3 * g.ny * tx,
        [&](int idx) {
            const int r1 = p.fd_tx.div(idx), col = idx - r1 * tx;
            const int c = g.fd_ny.div(r1), y = r1 - c * g.ny;
            return col < ncol ? p.in[c * cstride + (size_t)y * g.nkx + kx0 + col] : make_float2(0.f, 0.f);
        },
        [&](int idx, float2 v) {
            const int r1 = p.fd_tx.div(idx), col = idx - r1 * tx;
            const int c = g.fd_ny.div(r1), y = r1 - c * g.ny;
            a[(c * tx + col) * ls + sk(y)] = v;
        });
    for (int line = threadIdx.x >> 5; line < nl; line += blockDim.x >> 5)  // zero padding rows
        for (int y = g.ny + (threadIdx.x & 31); y < g.py; y += 32) a[line * ls + sk(y)] = make_float2(0.f, 0.f);
    __syncthreads();
    float2 *r = fft_lines(a, b, nl, ls, p.plan, false);
    float2 *o = (r == a) ? b : a;
    const size_t kc = (size_t)g.nky * g.nkx;
    for (int idx = threadIdx.x; idx < g.py * tx; idx += blockDim.x) {
        const int ky = p.fd_tx.div(idx), col = idx - ky * tx;
        const int kx = min(kx0 + col, g.nkx - 1);
        int kym;
        float sy;
        kernel_mirror(ky, g.py, kym, sy);
        const float *K = p.kern + (size_t)kym * g.nkx + kx;
        const float kxx = __ldg(K), kyy = __ldg(K + kc), kzz = __ldg(K + 2 * kc), kxy = sy * __ldg(K + 3 * kc);
        float2 *lx = r + (0 * tx + col) * ls + sk(ky);
        float2 *ly = r + (1 * tx + col) * ls + sk(ky);
        float2 *lz = r + (2 * tx + col) * ls + sk(ky);
        const float2 mx = *lx, my = *ly, mz = *lz;
        *lx = make_float2(-(kxx * mx.x + kxy * my.x), -(kxx * mx.y + kxy * my.y));
        *ly = make_float2(-(kxy * mx.x + kyy * my.x), -(kxy * mx.y + kyy * my.y));
        *lz = make_float2(-(kzz * mz.x), -(kzz * mz.y));
    }
    __syncthreads();
    float2 *q = fft_lines(r, o, nl, ls, p.plan, true);
    for (int idx = threadIdx.x; idx < 3 * g.ny * tx; idx += blockDim.x) {
        const int r1 = p.fd_tx.div(idx), col = idx - r1 * tx;
        const int c = g.fd_ny.div(r1), y = r1 - c * g.ny;
        if (col < ncol) p.out[c * cstride + (size_t)y * g.nkx + kx0 + col] = q[(c * tx + col) * ls + sk(y)];
    }
}

__global__ void __launch_bounds__(kThreads) yz_convolve_kernel(const ColPass p) { yz_convolve_body(p, blockIdx.x); }
__global__ void __launch_bounds__(kThreads) y_convolve_2d_kernel(const ColPass p) { y_convolve_2d_body(p, blockIdx.x); }

// One launch for many problems: work[blockIdx.x] = (problem, kx tile); kind 0 thin
// film, 1 fused y+z.
__global__ void __launch_bounds__(kThreads) col_batched_kernel(const ColPass *__restrict__ ps,
                                                               const int2 *__restrict__ work, int kind) {
    __shared__ __align__(16) unsigned char desc[sizeof(ColPass)];  // descriptor staged once per CTA
    const int2 w = work[blockIdx.x];
    const int *src = reinterpret_cast<const int *>(ps + w.x);
    for (int i = threadIdx.x; i < (int)(sizeof(ColPass) / sizeof(int)); i += blockDim.x)
        reinterpret_cast<int *>(desc)[i] = src[i];
    __syncthreads();
    const ColPass &p = *reinterpret_cast<const ColPass *>(desc);
    if (kind == 0) y_convolve_2d_body(p, w.y);
    else yz_convolve_body(p, w.y);
}

// Deterministic final reduction of the per-block partials (layout [stat][block] of
// float-float pairs): 1024 threads stride over the blocks with compensated TwoSum
// accumulation for the energies and max for the norms, then a fixed-order tree
// combines the threads.  GB300's FP64 rate is a small fraction of its FP32 rate, so
// the compensation runs on FP32 pipes; only the final hi + lo is formed in FP64.
constexpr int kFinThreads = 1024;

__device__ __forceinline__ void finalize_body(const float2 *__restrict__ partials, int nblocks, double *__restrict__ out) {
    __shared__ float2 sh[kFinThreads];
    for (int s = 0; s < kNumStats; ++s) {
        const bool is_sum = s < 5;
        const float2 *src = partials + (size_t)s * nblocks;
        float h = 0.f, l = 0.f;
        for (int b = threadIdx.x; b < nblocks; b += kFinThreads) {
            const float2 v = src[b];
            if (is_sum) {
                ff_add(h, l, v.x);
                l += v.y;
            } else {
                h = fmaxf(h, v.x);
            }
        }
        sh[threadIdx.x] = make_float2(h, l);
        __syncthreads();
        for (int w = kFinThreads / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) {
                float2 a = sh[threadIdx.x];
                const float2 b = sh[threadIdx.x + w];
                if (is_sum) {
                    ff_add(a.x, a.y, b.x);
                    a.y += b.y;
                } else {
                    a.x = fmaxf(a.x, b.x);
                }
                sh[threadIdx.x] = a;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) out[s] = (double)sh[0].x + (double)sh[0].y;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kFinThreads) finalize_stats_kernel(const float2 *__restrict__ partials, int nblocks,
                                                                     double *__restrict__ out) {
    finalize_body(partials, nblocks, out);
}

// One block per problem; statistics land in out[problem * kNumStats + s].
__global__ void __launch_bounds__(kFinThreads) finalize_batched_kernel(const FinDesc *__restrict__ fd, double *__restrict__ out) {
    const FinDesc d = fd[blockIdx.x];
    finalize_body(d.partials, d.nblocks, out + (size_t)blockIdx.x * kNumStats);
}

cudaError_t ensure_smem(const void *fn, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

unsigned tiles(const ColPass &p) { return (unsigned)((p.g.nkx + p.tx - 1) / p.tx); }

}  // namespace

int col_tile(const Grid &g, int lines_per_col, int len) {
    // largest tile (<= 8 kx columns) whose two ping-pong buffers fit in 200 KB
    int tx = 8;
    while (tx > 1 && (size_t)2 * lines_per_col * tx * skewed_len(len) * sizeof(float2) > 200u * 1024u) tx >>= 1;
    return tx;
}

cudaError_t launch_y_forward(const ColPass &p, cudaStream_t s) {
    const size_t sm = 2 * sizeof(float2) * (size_t)p.tx * skewed_len(p.g.py);
    cudaError_t e = ensure_smem((const void *)y_forward_kernel, sm);
    if (e != cudaSuccess) return e;
    y_forward_kernel<<<dim3(tiles(p), p.g.nz, 3), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_y_inverse(const ColPass &p, cudaStream_t s) {
    const size_t sm = 2 * sizeof(float2) * (size_t)p.tx * skewed_len(p.g.py);
    cudaError_t e = ensure_smem((const void *)y_inverse_kernel, sm);
    if (e != cudaSuccess) return e;
    y_inverse_kernel<<<dim3(tiles(p), p.g.nz, 3), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_z_convolve(const ColPass &p, cudaStream_t s) {
    // room for a y-frequency pair: 2 x 3 lines per kx column, two ping-pong buffers
    const size_t sm = 2 * sizeof(float2) * (size_t)2 * 3 * p.tx * skewed_len(p.g.pz);
    cudaError_t e = ensure_smem((const void *)z_convolve_kernel, sm);
    if (e != cudaSuccess) return e;
    z_convolve_kernel<<<dim3(tiles(p), p.g.nky), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

size_t yz_convolve_smem(const Grid &g, int tx) {
    const size_t a = (size_t)3 * tx * g.nz * skewed_len(g.py);
    const size_t b = (size_t)3 * tx * g.py * skewed_len(g.pz);
    return 2 * sizeof(float2) * (a > b ? a : b);
}

cudaError_t launch_yz_convolve(const ColPass &p, cudaStream_t s) {
    const size_t sm = yz_convolve_smem(p.g, p.tx);
    cudaError_t e = ensure_smem((const void *)yz_convolve_kernel, sm);
    if (e != cudaSuccess) return e;
    yz_convolve_kernel<<<tiles(p), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

size_t y_convolve_2d_smem(const Grid &g, int tx) { return 2 * sizeof(float2) * (size_t)3 * tx * skewed_len(g.py); }

cudaError_t launch_col_batched(const ColPass *ps, const int2 *work, int nwork, int kind, size_t smem, cudaStream_t s) {
    cudaError_t e = ensure_smem((const void *)col_batched_kernel, smem);
    if (e != cudaSuccess) return e;
    col_batched_kernel<<<nwork, kThreads, smem, s>>>(ps, work, kind);
    return cudaGetLastError();
}

cudaError_t launch_finalize_batched(const FinDesc *fd, int nproblems, double *out, cudaStream_t s) {
    finalize_batched_kernel<<<nproblems, kFinThreads, 0, s>>>(fd, out);
    return cudaGetLastError();
}

cudaError_t launch_y_convolve_2d(const ColPass &p, cudaStream_t s) {
    const size_t sm = 2 * sizeof(float2) * (size_t)3 * p.tx * skewed_len(p.g.py);
    cudaError_t e = ensure_smem((const void *)y_convolve_2d_kernel, sm);
    if (e != cudaSuccess) return e;
    y_convolve_2d_kernel<<<tiles(p), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_finalize_stats(const float2 *partials, int nblocks, double *out, cudaStream_t s) {
    finalize_stats_kernel<<<1, kFinThreads, 0, s>>>(partials, nblocks, out);
    return cudaGetLastError();
}

}  // namespace fm
