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
#include "fft_pair.cuh"

#include <algorithm>

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

// H = -K M with the complex kernel of a periodic grid: K points at component xx of one
// frequency, the other components follow at stride kc (xx yy zz xy xz yz; 2-D: the
// first four, xz = yz = 0).
__device__ __forceinline__ float2 cmadd(float2 k, float2 m, float2 acc) {
    return make_float2(acc.x + k.x * m.x - k.y * m.y, acc.y + k.x * m.y + k.y * m.x);
}
__device__ __forceinline__ void multiply_periodic(const float2 *K, size_t kc, bool thin, float2 *lx, float2 *ly,
                                                  float2 *lz) {
    const float2 kxx = __ldg(K), kyy = __ldg(K + kc), kzz = __ldg(K + 2 * kc), kxy = __ldg(K + 3 * kc);
    const float2 z0 = make_float2(0.f, 0.f);
    const float2 kxz = thin ? z0 : __ldg(K + 4 * kc), kyz = thin ? z0 : __ldg(K + 5 * kc);
    const float2 mx = *lx, my = *ly, mz = *lz;
    const float2 hx = cmadd(kxz, mz, cmadd(kxy, my, cmadd(kxx, mx, z0)));
    const float2 hy = cmadd(kyz, mz, cmadd(kyy, my, cmadd(kxy, mx, z0)));
    const float2 hz = cmadd(kzz, mz, cmadd(kyz, my, cmadd(kxz, mx, z0)));
    *lx = make_float2(-hx.x, -hx.y);
    *ly = make_float2(-hy.x, -hy.y);
    *lz = make_float2(-hz.x, -hz.y);
}

// X[c][z][y<ny][kx] -> Y[c][z][ky<py][kx] (forward along y, zero rows pruned)
__global__ void __launch_bounds__(kThreads) y_forward_kernel(const ColPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
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
    pdl_wait();
    if (p.early) pdl_trigger();
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

// Work item `it` of a kx tile -> (row, col), col fastest over the tile's ncol live
// columns.  nkx = px/2 + 1 is odd, so the last tile of a grid usually holds one live
// column; iterating rows * ncol items (not rows * tx) lets it skip the padding columns
// instead of computing them.  Only the last tile can be partial, so the divider is
// either the tile width's or the last tile's (fd_last, precomputed on the host).
// Shared-memory lines stay indexed by col within tx.
__device__ __forceinline__ void tile_item(const ColPass &p, int ncol, int it, int &row, int &col) {
    const FastDiv &fd = ncol == p.tx ? p.fd_tx : p.fd_last;
    row = fd.div(it);
    col = it - row * ncol;
}

// Number of y-frequencies a CTA handles: ky and py - ky (1 for ky = 0 and the Nyquist row).
__device__ __forceinline__ int ky_pair(int kya, int py, int &kyb) {
    kyb = py - kya;
    return (kya == 0 || kyb == kya) ? 1 : 2;
}

// 3-D: for y-frequencies (ky, py-ky) and a tile of kx, forward z-transform of the
// nz physical planes (zero-padded to pz), multiply by -N(k), inverse, keep nz planes.
__global__ void __launch_bounds__(kThreads) z_convolve_kernel(const ColPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
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
    if (g.per) {  // complex kernel K[c][kz][ky][kx]
        const size_t kcp = (size_t)g.pz * g.py * g.nkx;
        for (int idx = threadIdx.x; idx < np * g.pz * tx; idx += blockDim.x) {
            const int r1 = p.fd_tx.div(idx), col = idx - r1 * tx;
            const int q = r1 >= g.pz ? 1 : 0, kz = r1 - q * g.pz;
            const int kx = min(kx0 + col, g.nkx - 1), ky = q ? kyb : kya;
            const float2 *K = reinterpret_cast<const float2 *>(p.kern) + ((size_t)kz * g.py + ky) * g.nkx + kx;
            multiply_periodic(K, kcp, false, r + ((q * 3 + 0) * tx + col) * ls + sk(kz), r + ((q * 3 + 1) * tx + col) * ls + sk(kz),
                              r + ((q * 3 + 2) * tx + col) * ls + sk(kz));
        }
    }
    const size_t kc = (size_t)g.nkz * g.nky * g.nkx;
    for (int idx = threadIdx.x; idx < (g.per ? 0 : g.pz * tx); idx += blockDim.x) {
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

// ---- pruned two-level transforms (half_dft_store / half_idft_load in fft_smem.cuh) ----

// X[c][z][y<ny][kx] -> Y[c][z][ky<py][kx], py = N1 * N2: half-input outer pass from
// global memory, inner N2-point pass straight to global memory, one barrier.
template <int N1, int N2>
__global__ void __launch_bounds__(kThreads, 2) y_forward_fused_kernel(const ColPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
    constexpr int N = N1 * N2, H1 = N1 / 2;
    constexpr int ls = skewed_len(N);
    extern __shared__ __align__(16) unsigned char smem[];
    float2 *buf = reinterpret_cast<float2 *>(smem);
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = blockIdx.x * tx, ncol = min(tx, g.nkx - kx0);
    const int z = blockIdx.y, c = blockIdx.z;
    const float2 *__restrict__ tw = p.plan.tw;
    const float2 *src = p.in + ((size_t)c * g.nz + z) * g.ny * g.nkx + kx0;
    for (int it = threadIdx.x; it < N2 * ncol; it += blockDim.x) {
        int n2, col;
        tile_item(p, ncol, it, n2, col);
        float2 e[H1];
#pragma unroll
        for (int n1 = 0; n1 < H1; ++n1) {
            const int y = N2 * n1 + n2;
            e[n1] = y < g.ny ? src[(size_t)y * g.nkx + col] : make_float2(0.f, 0.f);
        }
        half_dft_store<N1, N2>(e, n2, buf + col * ls, tw);
    }
    __syncthreads();
    float2 *dst = p.out + ((size_t)c * g.nz + z) * g.py * g.nkx + kx0;
    for (int it = threadIdx.x; it < N1 * ncol; it += blockDim.x) {
        int k1, col;
        tile_item(p, ncol, it, k1, col);
        const float2 *line = buf + col * ls;
        float2 v[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) v[n2] = line[sk(k1 * N2 + n2)];
        dft_small<N2>(v, false);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) dst[(size_t)(k1 + N1 * k2) * g.nkx + col] = v[k2];
    }
}

// Y[c][z][ky][kx] -> X[c][z][y<ny][kx]: inner inverse N2-point pass from global memory,
// half-output outer pass straight to global memory, one barrier.
template <int N1, int N2>
__global__ void __launch_bounds__(kThreads, 2) y_inverse_fused_kernel(const ColPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
    constexpr int N = N1 * N2, H1 = N1 / 2;
    constexpr int ls = skewed_len(N);
    extern __shared__ __align__(16) unsigned char smem[];
    float2 *buf = reinterpret_cast<float2 *>(smem);
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = blockIdx.x * tx, ncol = min(tx, g.nkx - kx0);
    const int z = blockIdx.y, c = blockIdx.z;
    const float2 *__restrict__ tw = p.plan.tw;
    const float2 *src = p.in + ((size_t)c * g.nz + z) * g.py * g.nkx + kx0;
    for (int it = threadIdx.x; it < N1 * ncol; it += blockDim.x) {
        int k1, col;
        tile_item(p, ncol, it, k1, col);
        float2 v[N2];
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) v[k2] = src[(size_t)(k1 + N1 * k2) * g.nkx + col];
        dft_small<N2>(v, true);
        float2 *line = buf + col * ls;
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2)
            line[sk(k1 * N2 + n2)] = (n2 && k1) ? cmul(v[n2], cconj(__ldg(tw + n2 * k1))) : v[n2];
    }
    __syncthreads();
    float2 *dst = p.out + ((size_t)c * g.nz + z) * g.ny * g.nkx + kx0;
    for (int it = threadIdx.x; it < N2 * ncol; it += blockDim.x) {
        int n2, col;
        tile_item(p, ncol, it, n2, col);
        float2 e[H1];
        half_idft_load<N1, N2>(e, n2, buf + col * ls, tw);
#pragma unroll
        for (int n1 = 0; n1 < H1; ++n1) {
            const int y = N2 * n1 + n2;
            if (y < g.ny) dst[(size_t)y * g.nkx + col] = e[n1];
        }
    }
}

// Pruned two-level z convolution for power-of-two pz = N1 * N2.  With z = N2 z1 + z2 and
// k = k1 + N1 k2 the transform of one z line is
//   X[k1 + N1 k2] = sum_z2 W_N2^{z2 k2} W_pz^{z2 k1} sum_z1 x[N2 z1 + z2] W_N1^{z1 k1}
// and its inverse runs the same factors backwards.  Inputs vanish for z >= pz/2 (z1 >=
// N1/2) and only z < nz <= pz/2 is kept, so the outer N1-point passes work on half
// lines: a half-input DFT is two N1/2-point DFTs (even and odd outputs), a half-output
// inverse is two N1/2-point inverses.  Phase 1 (line, z2): global loads straight into
// registers, half-input DFT, twiddle, one shared-memory write.  Phase 2 (ky of the pair,
// column, k1; all three components): N2-point DFTs, the tensor multiply, inverse
// N2-point DFTs, conjugate twiddle, in place.  Phase 3 (line, z2): half-output inverse
// straight to global memory.  Two barriers per tile, one buffer.
template <int N1, int N2>
__global__ void __launch_bounds__(kThreads, (N1 * N2 <= 128) ? 3 : 1) z_convolve_fused_kernel(const ColPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
    constexpr int N = N1 * N2, H1 = N1 / 2;
    constexpr int ls = skewed_len(N);
    extern __shared__ __align__(16) unsigned char smem[];
    float2 *buf = reinterpret_cast<float2 *>(smem);  // line (q, c, col) at ((q*3 + c)*tx + col)*ls
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = blockIdx.x * tx, ncol = min(tx, g.nkx - kx0);
    const int kya = blockIdx.y;
    int kyb;
    const int np = ky_pair(kya, g.py, kyb);
    const int nz = g.nz;
    const size_t cstride = (size_t)nz * g.py * g.nkx;  // component stride of Y
    const size_t zstride = (size_t)g.py * g.nkx;
    const float2 *__restrict__ tw = p.plan.tw;        // e^{-2 pi i e / N}

    // phase 1: item (r2, z2, col), col fastest
    const int n13 = np * 3 * N2 * ncol;
    for (int it = threadIdx.x; it < n13; it += blockDim.x) {
        int rz, col;
        tile_item(p, ncol, it, rz, col);
        const int z2 = rz & (N2 - 1), r2 = rz / N2;
        const int q = r2 >= 3, c = r2 - 3 * q;
        const int ky = q ? kyb : kya;
        const float2 *src = p.in + c * cstride + (size_t)ky * g.nkx + kx0 + col;
        float2 e[H1];
#pragma unroll
        for (int z1 = 0; z1 < H1; ++z1) {
            const int z = N2 * z1 + z2;
            e[z1] = z < nz ? src[(size_t)z * zstride] : make_float2(0.f, 0.f);
        }
        half_dft_store<N1, N2>(e, z2, buf + (r2 * tx + col) * ls, tw);
    }
    __syncthreads();

    // phase 2: item (q, k1, col), col fastest; all three components of one frequency column
    const size_t kc = (size_t)g.nkz * g.nky * g.nkx;
    const int n2 = np * N1 * ncol;
    for (int it = threadIdx.x; it < n2; it += blockDim.x) {
        int qk, col;
        tile_item(p, ncol, it, qk, col);
        const int k1 = qk & (N1 - 1), q = qk / N1;
        float2 m[3][N2];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 *line = buf + ((q * 3 + c) * tx + col) * ls;
#pragma unroll
            for (int z2 = 0; z2 < N2; ++z2) m[c][z2] = line[sk(k1 * N2 + z2)];
            dft_small<N2>(m[c], false);
        }
        const int kx = min(kx0 + col, g.nkx - 1);
        // the second frequency of the pair is the y-mirror: odd-in-y components flip sign
        const float sy = q ? -1.f : 1.f;
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) {
            int kzm;
            float sz;
            kernel_mirror(k1 + N1 * k2, N, kzm, sz);
            const float *K = p.kern + ((size_t)kzm * g.nky + kya) * g.nkx + kx;
            const float kxx = __ldg(K), kyy = __ldg(K + kc), kzz = __ldg(K + 2 * kc);
            const float kxy = sy * __ldg(K + 3 * kc), kxz = sz * __ldg(K + 4 * kc), kyz = sy * sz * __ldg(K + 5 * kc);
            const float2 mx = m[0][k2], my = m[1][k2], mz = m[2][k2];
            m[0][k2] = make_float2(-(kxx * mx.x + kxy * my.x + kxz * mz.x), -(kxx * mx.y + kxy * my.y + kxz * mz.y));
            m[1][k2] = make_float2(-(kxy * mx.x + kyy * my.x + kyz * mz.x), -(kxy * mx.y + kyy * my.y + kyz * mz.y));
            m[2][k2] = make_float2(-(kxz * mx.x + kyz * my.x + kzz * mz.x), -(kxz * mx.y + kyz * my.y + kzz * mz.y));
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            dft_small<N2>(m[c], true);
            float2 *line = buf + ((q * 3 + c) * tx + col) * ls;
#pragma unroll
            for (int z2 = 0; z2 < N2; ++z2)
                line[sk(k1 * N2 + z2)] = (z2 && k1) ? cmul(m[c][z2], cconj(__ldg(tw + z2 * k1))) : m[c][z2];
        }
    }
    __syncthreads();

    // phase 3: item (r2, z2, col), col fastest; outputs z1 < N1/2 with z < nz
    for (int it = threadIdx.x; it < n13; it += blockDim.x) {
        int rz, col;
        tile_item(p, ncol, it, rz, col);
        const int z2 = rz & (N2 - 1), r2 = rz / N2;
        const int q = r2 >= 3, c = r2 - 3 * q;
        const int ky = q ? kyb : kya;
        float2 e[H1];
        half_idft_load<N1, N2>(e, z2, buf + (r2 * tx + col) * ls, tw);
        float2 *dst = p.out + c * cstride + (size_t)ky * g.nkx + kx0 + col;
#pragma unroll
        for (int z1 = 0; z1 < H1; ++z1) {
            const int z = N2 * z1 + z2;
            if (z < nz) dst[(size_t)z * zstride] = e[z1];
        }
    }
}

// The pruned two-level z convolution on y-frequency pairs in packed FP32x2 form: lane A
// is ky, lane B is py - ky (the two share every twiddle and, up to the sign of the
// odd-in-y components xy and yz, every kernel value).  Tiles of 8 kx columns; phase 1
// item (c, z2, col), phase 2 item (k1, col) with all three components of both lanes,
// phase 3 item (c, z2, col).  Shared memory holds pair elements (float4), so the
// buffer is the size of the unpaired kernel's.  For ky = 0 and ky = py/2 (no partner)
// lane B repeats lane A and is not stored.
template <int N1, int N2>
__global__ void __launch_bounds__(3 * N2 * 8, 2) z_convolve_pair_kernel(const ColPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
    constexpr int N = N1 * N2, H1 = N1 / 2, TX = 8;
    constexpr int ls = skewed_len(N);
    extern __shared__ __align__(16) unsigned char smem[];
    float4 *buf = reinterpret_cast<float4 *>(smem);  // line (c, col) at (c*TX + col)*ls
    const Grid &g = p.g;
    const int kx0 = blockIdx.x * TX, ncol = min(TX, g.nkx - kx0);
    const int kya = blockIdx.y;
    int kyb;
    const int np = ky_pair(kya, g.py, kyb);
    const int kyB = np == 2 ? kyb : kya;
    const int nz = g.nz;
    const size_t cstride = (size_t)nz * g.py * g.nkx;  // component stride of Y
    const size_t zstride = (size_t)g.py * g.nkx;
    const float2 *__restrict__ tw = p.plan.tw;        // e^{-2 pi i e / N}

    // phase 1: item (c, z2, col), col fastest
    for (int it = threadIdx.x; it < 3 * N2 * TX; it += blockDim.x) {
        const int col = it & (TX - 1), cz = it >> 3;
        if (col >= ncol) continue;
        const int z2 = cz & (N2 - 1), c = cz / N2;
        const float2 *srcA = p.in + c * cstride + (size_t)kya * g.nkx + kx0 + col;
        const float2 *srcB = p.in + c * cstride + (size_t)kyB * g.nkx + kx0 + col;
        cp2 e[H1];
#pragma unroll
        for (int z1 = 0; z1 < H1; ++z1) {
            const int z = N2 * z1 + z2;
            e[z1] = z < nz ? ppack(srcA[(size_t)z * zstride], srcB[(size_t)z * zstride]) : pzero();
        }
        phalf_dft_store<N1, N2>(e, z2, buf + (c * TX + col) * ls, tw);
    }
    __syncthreads();

    // phase 2: item (k1, col); inner DFTs, the tensor multiply, inverse inner DFTs
    const size_t kc = (size_t)g.nkz * g.nky * g.nkx;
    for (int it = threadIdx.x; it < N1 * TX; it += blockDim.x) {
        const int col = it & (TX - 1), k1 = it >> 3;
        if (col >= ncol) continue;
        cp2 m[3][N2];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float4 *line = buf + (c * TX + col) * ls;
#pragma unroll
            for (int z2 = 0; z2 < N2; ++z2) m[c][z2] = pload(line[sk(k1 * N2 + z2)]);
            pdft<N2>(m[c], false);
        }
        const int kx = kx0 + col;
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) {
            int kzm;
            float sz;
            kernel_mirror(k1 + N1 * k2, N, kzm, sz);
            const float *K = p.kern + ((size_t)kzm * g.nky + kya) * g.nkx + kx;
            const float kxx = __ldg(K), kyy = __ldg(K + kc), kzz = __ldg(K + 2 * kc);
            const float kxy = __ldg(K + 3 * kc), kxz = sz * __ldg(K + 4 * kc), kyz = sz * __ldg(K + 5 * kc);
            // H = -N M; lane B (py - ky) flips the odd-in-y components xy and yz
            const float2 Nxx = pb(-kxx), Nyy = pb(-kyy), Nzz = pb(-kzz), Nxz = pb(-kxz);
            const float2 Nxy = make_float2(-kxy, kxy), Nyz = make_float2(-kyz, kyz);
            const cp2 mx = m[0][k2], my = m[1][k2], mz = m[2][k2];
            m[0][k2] = {__ffma2_rn(Nxz, mz.re, __ffma2_rn(Nxy, my.re, __fmul2_rn(Nxx, mx.re))),
                        __ffma2_rn(Nxz, mz.im, __ffma2_rn(Nxy, my.im, __fmul2_rn(Nxx, mx.im)))};
            m[1][k2] = {__ffma2_rn(Nyz, mz.re, __ffma2_rn(Nyy, my.re, __fmul2_rn(Nxy, mx.re))),
                        __ffma2_rn(Nyz, mz.im, __ffma2_rn(Nyy, my.im, __fmul2_rn(Nxy, mx.im)))};
            m[2][k2] = {__ffma2_rn(Nzz, mz.re, __ffma2_rn(Nyz, my.re, __fmul2_rn(Nxz, mx.re))),
                        __ffma2_rn(Nzz, mz.im, __ffma2_rn(Nyz, my.im, __fmul2_rn(Nxz, mx.im)))};
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            pdft<N2>(m[c], true);
            float4 *line = buf + (c * TX + col) * ls;
#pragma unroll
            for (int z2 = 0; z2 < N2; ++z2)
                line[sk(k1 * N2 + z2)] = pstore((z2 && k1) ? pmulw(m[c][z2], __ldg(tw + z2 * k1), true) : m[c][z2]);
        }
    }
    __syncthreads();

    // phase 3: item (c, z2, col); outputs z1 < N1/2 with z < nz
    for (int it = threadIdx.x; it < 3 * N2 * TX; it += blockDim.x) {
        const int col = it & (TX - 1), cz = it >> 3;
        if (col >= ncol) continue;
        const int z2 = cz & (N2 - 1), c = cz / N2;
        cp2 e[H1];
        phalf_idft_load<N1, N2>(e, z2, buf + (c * TX + col) * ls, tw);
        float2 *dstA = p.out + c * cstride + (size_t)kya * g.nkx + kx0 + col;
        float2 *dstB = p.out + c * cstride + (size_t)kyb * g.nkx + kx0 + col;
#pragma unroll
        for (int z1 = 0; z1 < H1; ++z1) {
            const int z = N2 * z1 + z2;
            if (z < nz) {
                dstA[(size_t)z * zstride] = plane_a(e[z1]);
                if (np == 2) dstB[(size_t)z * zstride] = plane_b(e[z1]);
            }
        }
    }
}

// Register-resident z convolution of one (kx column, ky) for pz <= 8: forward z DFT of
// the nz physical planes (zero above), -N(k) multiply, inverse DFT, planes z < nz
// written back.  Component c, plane z of the column sits at line[(c*nz + z)*lstride].
template <int PZ>
__device__ __forceinline__ void z_small_convolve(float2 *line, size_t lstride, int nz, const float *__restrict__ kern,
                                                 size_t kc, int nky, int nkx, int ky, int py, int kx) {
    float2 v[3][PZ];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
        for (int z = 0; z < PZ; ++z) v[c][z] = z < nz ? line[(c * nz + z) * lstride] : make_float2(0.f, 0.f);
        dft_small<PZ>(v[c], false);
    }
    int kym;
    float sy;
    kernel_mirror(ky, py, kym, sy);
#pragma unroll
    for (int kz = 0; kz < PZ; ++kz) {
        int kzm;
        float sz;
        kernel_mirror(kz, PZ, kzm, sz);
        const float *K = kern + ((size_t)kzm * nkx + kx) * nky + kym;  // ky-fastest layout
        const float kxx = __ldg(K), kyy = __ldg(K + kc), kzz = __ldg(K + 2 * kc);
        const float kxy = sy * __ldg(K + 3 * kc), kxz = sz * __ldg(K + 4 * kc), kyz = sy * sz * __ldg(K + 5 * kc);
        const float2 mx = v[0][kz], my = v[1][kz], mz = v[2][kz];
        v[0][kz] = make_float2(-(kxx * mx.x + kxy * my.x + kxz * mz.x), -(kxx * mx.y + kxy * my.y + kxz * mz.y));
        v[1][kz] = make_float2(-(kxy * mx.x + kyy * my.x + kyz * mz.x), -(kxy * mx.y + kyy * my.y + kyz * mz.y));
        v[2][kz] = make_float2(-(kxz * mx.x + kyz * my.x + kzz * mz.x), -(kxz * mx.y + kyz * my.y + kzz * mz.y));
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        dft_small<PZ>(v[c], true);
#pragma unroll
        for (int z = 0; z < PZ; ++z)
            if (z < nz) line[(c * nz + z) * lstride] = v[c][z];
    }
}

__host__ __device__ __forceinline__ bool yz_fused_ok(const Grid &g) {
    const int py = g.py, pz = g.pz;
    return g.per == 0 && (py == 16 || py == 32 || py == 64 || py == 128 || py == 256) && 2 * g.ny <= py &&
           (pz == 2 || pz == 4 || pz == 8) && 2 * g.nz <= pz;
}

// Small 3-D grids, py = N1 * N2 and pz <= 8: the pruned two-level y transforms of
// the nz physical planes around a register-resident z convolution.  Lines (c, z, col)
// at L = (c*nz + z)*tx + col in two buffers: A holds the outer-pass slots, B the
// natural-order y spectrum.  Phases: outer half-input DFT from global memory -> A;
// inner DFTs A -> B; per (col, ky) z convolution in B; inner inverse B -> A; outer
// half-output inverse A -> global memory.
template <int N1, int N2>
__device__ __forceinline__ void yz_convolve_fused_body(const ColPass &p, const int tile) {
    constexpr int N = N1 * N2, H1 = N1 / 2;
    constexpr int ls = skewed_len(N);
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = tile * tx, ncol = min(tx, g.nkx - kx0);
    const int nz = g.nz, nl = 3 * nz * tx, nlive = 3 * nz * ncol;  // lines in the buffers / live lines
    float2 *A = reinterpret_cast<float2 *>(smem);
    float2 *B = A + (size_t)nl * ls;
    const size_t zstride = (size_t)g.ny * g.nkx, cstride = (size_t)nz * zstride;
    const float2 *__restrict__ tw = p.plan.tw;
    for (int it = threadIdx.x; it < nlive * N2; it += blockDim.x) {
        int rest, col;
        tile_item(p, ncol, it, rest, col);
        const int n2 = rest & (N2 - 1), cz = rest / N2;  // cz = c*nz + z
        const float2 *src = p.in + cz * zstride + kx0 + col;
        float2 e[H1];
#pragma unroll
        for (int y1 = 0; y1 < H1; ++y1) {
            const int y = N2 * y1 + n2;
            e[y1] = y < g.ny ? src[(size_t)y * g.nkx] : make_float2(0.f, 0.f);
        }
        half_dft_store<N1, N2>(e, n2, A + (cz * tx + col) * ls, tw);
    }
    __syncthreads();
    for (int it = threadIdx.x; it < nlive * N1; it += blockDim.x) {
        int rest, col;
        tile_item(p, ncol, it, rest, col);
        const int k1 = rest & (N1 - 1), cz = rest / N1;
        const float2 *sl = A + (cz * tx + col) * ls;
        float2 v[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) v[n2] = sl[sk(k1 * N2 + n2)];
        dft_small<N2>(v, false);
        float2 *bl = B + (cz * tx + col) * ls;
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) bl[sk(k1 + N1 * k2)] = v[k2];
    }
    __syncthreads();
    const size_t kc = (size_t)g.nkz * g.nky * g.nkx;
    for (int it = threadIdx.x; it < N * ncol; it += blockDim.x) {
        int ky, col;
        tile_item(p, ncol, it, ky, col);
        const int kx = min(kx0 + col, g.nkx - 1);
        float2 *line = B + (size_t)col * ls + sk(ky);
        const size_t lstride = (size_t)tx * ls;
        if (g.pz == 2) z_small_convolve<2>(line, lstride, nz, p.kern, kc, g.nky, g.nkx, ky, N, kx);
        else if (g.pz == 4) z_small_convolve<4>(line, lstride, nz, p.kern, kc, g.nky, g.nkx, ky, N, kx);
        else z_small_convolve<8>(line, lstride, nz, p.kern, kc, g.nky, g.nkx, ky, N, kx);
    }
    __syncthreads();
    for (int it = threadIdx.x; it < nlive * N1; it += blockDim.x) {
        int rest, col;
        tile_item(p, ncol, it, rest, col);
        const int k1 = rest & (N1 - 1), cz = rest / N1;
        const float2 *bl = B + (cz * tx + col) * ls;
        float2 v[N2];
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) v[k2] = bl[sk(k1 + N1 * k2)];
        dft_small<N2>(v, true);
        float2 *sl = A + (cz * tx + col) * ls;
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) sl[sk(k1 * N2 + n2)] = (n2 && k1) ? cmul(v[n2], cconj(__ldg(tw + n2 * k1))) : v[n2];
    }
    __syncthreads();
    for (int it = threadIdx.x; it < nlive * N2; it += blockDim.x) {
        int rest, col;
        tile_item(p, ncol, it, rest, col);
        const int n2 = rest & (N2 - 1), cz = rest / N2;
        float2 e[H1];
        half_idft_load<N1, N2>(e, n2, A + (cz * tx + col) * ls, tw);
        if (col < ncol) {
            float2 *dst = p.out + cz * zstride + kx0 + col;
#pragma unroll
            for (int y1 = 0; y1 < H1; ++y1) {
                const int y = N2 * y1 + n2;
                if (y < g.ny) dst[(size_t)y * g.nkx] = e[y1];
            }
        }
    }
    (void)cstride;
}

__device__ __forceinline__ void yz_convolve_general_body(const ColPass &p, const int tile);

__device__ __forceinline__ void yz_convolve_fused_dispatch(const ColPass &p, const int tile) {
    switch (p.g.py) {
        case 16: yz_convolve_fused_body<4, 4>(p, tile); return;
        case 32: yz_convolve_fused_body<8, 4>(p, tile); return;
        case 64: yz_convolve_fused_body<8, 8>(p, tile); return;
        case 128: yz_convolve_fused_body<16, 8>(p, tile); return;
        default: yz_convolve_fused_body<16, 16>(p, tile); return;
    }
}

__device__ __forceinline__ void yz_convolve_body(const ColPass &p, const int tile) {
    if (yz_fused_ok(p.g)) yz_convolve_fused_dispatch(p, tile);
    else yz_convolve_general_body(p, tile);
}

// 3-D grids whose (y, z) plane fits in shared memory: forward y-transform of the nz
// physical planes, in-smem transpose, forward z, multiply, inverse z, transpose back,
// inverse y -- X -> X in place, one pass instead of three and no Y round trip.
// Lines: y-lines (c, col, z) at ((c*tx + col)*nz + z), z-lines (c, col, ky) at
// ((c*tx + col)*py + ky); both layouts share two ping-pong buffers of `half_buf`.
__device__ __forceinline__ void yz_convolve_general_body(const ColPass &p, const int tile) {
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
        const float *K = p.kern + ((size_t)kzm * g.nkx + kx) * g.nky + kym;  // ky-fastest layout
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
// Thin film, power-of-two py = N1 * N2 (2 ny <= py): the pruned two-level form of the
// y convolution -- half-input outer pass from global memory, inner passes with the
// 4-component multiply in registers, half-output outer inverse to global memory.
template <int N1, int N2>
__device__ __forceinline__ void y_convolve_2d_fused_body(const ColPass &p, const int tile) {
    constexpr int N = N1 * N2, H1 = N1 / 2;
    constexpr int ls = skewed_len(N);
    extern __shared__ __align__(16) unsigned char smem[];
    float2 *buf = reinterpret_cast<float2 *>(smem);  // line (c, col) at (c*tx + col)*ls
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = tile * tx, ncol = min(tx, g.nkx - kx0);
    const size_t cstride = (size_t)g.ny * g.nkx;
    const float2 *__restrict__ tw = p.plan.tw;
    const int n13 = 3 * N2 * ncol;
    for (int it = threadIdx.x; it < n13; it += blockDim.x) {
        int rz, col;
        tile_item(p, ncol, it, rz, col);
        const int n2 = rz & (N2 - 1), c = rz / N2;
        const float2 *src = p.in + c * cstride + kx0 + col;
        float2 e[H1];
#pragma unroll
        for (int n1 = 0; n1 < H1; ++n1) {
            const int y = N2 * n1 + n2;
            e[n1] = y < g.ny ? src[(size_t)y * g.nkx] : make_float2(0.f, 0.f);
        }
        half_dft_store<N1, N2>(e, n2, buf + (c * tx + col) * ls, tw);
    }
    __syncthreads();
    const size_t kc = (size_t)g.nky * g.nkx;
    for (int it = threadIdx.x; it < N1 * ncol; it += blockDim.x) {
        int k1, col;
        tile_item(p, ncol, it, k1, col);
        float2 m[3][N2];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 *line = buf + (c * tx + col) * ls;
#pragma unroll
            for (int n2 = 0; n2 < N2; ++n2) m[c][n2] = line[sk(k1 * N2 + n2)];
            dft_small<N2>(m[c], false);
        }
        const int kx = min(kx0 + col, g.nkx - 1);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) {
            int kym;
            float sy;
            kernel_mirror(k1 + N1 * k2, N, kym, sy);
            const float *K = p.kern + (size_t)kym * g.nkx + kx;
            const float kxx = __ldg(K), kyy = __ldg(K + kc), kzz = __ldg(K + 2 * kc), kxy = sy * __ldg(K + 3 * kc);
            const float2 mx = m[0][k2], my = m[1][k2], mz = m[2][k2];
            m[0][k2] = make_float2(-(kxx * mx.x + kxy * my.x), -(kxx * mx.y + kxy * my.y));
            m[1][k2] = make_float2(-(kxy * mx.x + kyy * my.x), -(kxy * mx.y + kyy * my.y));
            m[2][k2] = make_float2(-(kzz * mz.x), -(kzz * mz.y));
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            dft_small<N2>(m[c], true);
            float2 *line = buf + (c * tx + col) * ls;
#pragma unroll
            for (int n2 = 0; n2 < N2; ++n2)
                line[sk(k1 * N2 + n2)] = (n2 && k1) ? cmul(m[c][n2], cconj(__ldg(tw + n2 * k1))) : m[c][n2];
        }
    }
    __syncthreads();
    for (int it = threadIdx.x; it < n13; it += blockDim.x) {
        int rz, col;
        tile_item(p, ncol, it, rz, col);
        const int n2 = rz & (N2 - 1), c = rz / N2;
        float2 e[H1];
        half_idft_load<N1, N2>(e, n2, buf + (c * tx + col) * ls, tw);
        if (col < ncol) {
            float2 *dst = p.out + c * cstride + kx0 + col;
#pragma unroll
            for (int n1 = 0; n1 < H1; ++n1) {
                const int y = N2 * n1 + n2;
                if (y < g.ny) dst[(size_t)y * g.nkx] = e[n1];
            }
        }
    }
}

// (py = 512 takes y_convolve_2d_p512_kernel, a kernel of its own: its inner pass holds
// 3 x 16 complex values a thread)
__host__ __device__ __forceinline__ bool y2d_fused_ok(const Grid &g) {
    const int py = g.py;
    return g.per == 0 && (py == 16 || py == 32 || py == 64 || py == 128 || py == 256) && 2 * g.ny <= py;
}

__device__ __forceinline__ void y_convolve_2d_general_body(const ColPass &p, const int tile);

__device__ __forceinline__ void y_convolve_2d_fused_dispatch(const ColPass &p, const int tile) {
    switch (p.g.py) {
        case 16: y_convolve_2d_fused_body<4, 4>(p, tile); return;
        case 32: y_convolve_2d_fused_body<8, 4>(p, tile); return;
        case 64: y_convolve_2d_fused_body<8, 8>(p, tile); return;
        case 128: y_convolve_2d_fused_body<16, 8>(p, tile); return;
        default: y_convolve_2d_fused_body<32, 8>(p, tile); return;
    }
}

__device__ __forceinline__ void y_convolve_2d_body(const ColPass &p, const int tile) {
    if (y2d_fused_ok(p.g)) y_convolve_2d_fused_dispatch(p, tile);
    else y_convolve_2d_general_body(p, tile);
}

__device__ __forceinline__ void y_convolve_2d_general_body(const ColPass &p, const int tile) {
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
    if (g.per) {  // complex kernel K[c][ky][kx]
        const size_t kcp = (size_t)g.py * g.nkx;
        for (int idx = threadIdx.x; idx < g.py * tx; idx += blockDim.x) {
            const int ky = p.fd_tx.div(idx), col = idx - ky * tx;
            const int kx = min(kx0 + col, g.nkx - 1);
            const float2 *K = reinterpret_cast<const float2 *>(p.kern) + (size_t)ky * g.nkx + kx;
            multiply_periodic(K, kcp, true, r + (0 * tx + col) * ls + sk(ky), r + (1 * tx + col) * ls + sk(ky),
                              r + (2 * tx + col) * ls + sk(ky));
        }
    }
    const size_t kc = (size_t)g.nky * g.nkx;
    for (int idx = threadIdx.x; idx < (g.per ? 0 : g.py * tx); idx += blockDim.x) {
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

__global__ void __launch_bounds__(kThreads) yz_convolve_kernel(const ColPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
    yz_convolve_body(p, blockIdx.x);
}
__global__ void __launch_bounds__(kThreads) y_convolve_2d_kernel(const ColPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
    y_convolve_2d_body(p, blockIdx.x);
}
// py = 512 (films of 129..256 rows): the two-level 32 x 16 form, whose inner pass holds
// 3 x 16 complex values a thread; a kernel of its own so that its registers do not weigh
// on the other lengths
__global__ void __launch_bounds__(kThreads, 2) y_convolve_2d_p512_kernel(const ColPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
    y_convolve_2d_fused_body<32, 16>(p, blockIdx.x);
}

// One launch for many problems: work[blockIdx.x] = (problem, kx tile).  KIND (see
// col_batched_kind): 0 thin film pruned, 1 fused y+z pruned, 2 thin film general,
// 3 fused y+z general -- one kernel per kind, so each gets its own register allocation.
template <int KIND>
__global__ void __launch_bounds__(kThreads, KIND < 2 ? 2 : 4) col_batched_kernel(const ColPass *__restrict__ ps,
                                                               const int2 *__restrict__ work) {
    __shared__ __align__(16) unsigned char desc[sizeof(ColPass)];  // descriptor staged once per CTA
    const int2 w = work[blockIdx.x];
    // a finished problem (step size 0) keeps its tiles in the table until the round is
    // rebuilt; the whole CTA leaves before its first barrier
    const double *skip = ps[w.x].skip_dt;
    if (skip && *skip <= 0.0) return;
    const int *src = reinterpret_cast<const int *>(ps + w.x);
    for (int i = threadIdx.x; i < (int)(sizeof(ColPass) / sizeof(int)); i += blockDim.x)
        reinterpret_cast<int *>(desc)[i] = src[i];
    __syncthreads();
    const ColPass &p = *reinterpret_cast<const ColPass *>(desc);
    if constexpr (KIND == 0) y_convolve_2d_fused_dispatch(p, w.y);
    else if constexpr (KIND == 1) yz_convolve_fused_dispatch(p, w.y);
    else if constexpr (KIND == 2) y_convolve_2d_general_body(p, w.y);
    else yz_convolve_general_body(p, w.y);
}

// Deterministic final reduction of the per-block partials (layout [stat][block] of
// float-float pairs): the threads stride over the blocks with compensated TwoSum
// accumulation for the energies and max for the norms, all nine statistics at once;
// warp butterflies and one barrier combine the threads in a fixed order.  GB300's FP64
// rate is a small fraction of its FP32 rate, so the compensation runs on FP32 pipes;
// only the final hi + lo is formed in FP64.
constexpr int kFinThreads = 1024;

// One butterfly level: float-float sums combined in lane order (every lane ends with
// the same bits), maxima by fmaxf.
__device__ __forceinline__ void fin_level(float (&h)[kNumStats], float (&l)[kNumStats], int o) {
    const bool low = (threadIdx.x & o) == 0;
#pragma unroll
    for (int s = 0; s < kNumStats; ++s) {
        const float oh = __shfl_xor_sync(0xffffffffu, h[s], o);
        const float ol = __shfl_xor_sync(0xffffffffu, l[s], o);
        if (s < 5) {
            float ah = low ? h[s] : oh, al = low ? l[s] : ol;
            ff_add(ah, al, low ? oh : h[s]);
            al += low ? ol : l[s];
            h[s] = ah;
            l[s] = al;
        } else {
            h[s] = fmaxf(h[s], oh);
        }
    }
}

__device__ __forceinline__ void finalize_body(const float2 *__restrict__ partials, int nblocks, double *__restrict__ out) {
    __shared__ float2 sh[kFinThreads / 32][kNumStats];
    float h[kNumStats], l[kNumStats];
#pragma unroll
    for (int s = 0; s < kNumStats; ++s) h[s] = l[s] = 0.f;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
        for (int s = 0; s < kNumStats; ++s) {
            const float2 v = partials[(size_t)s * nblocks + b];
            if (s < 5) {
                ff_add(h[s], l[s], v.x);
                l[s] += v.y;
            } else {
                h[s] = fmaxf(h[s], v.x);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) fin_level(h, l, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
#pragma unroll
        for (int s = 0; s < kNumStats; ++s) sh[wid][s] = make_float2(h[s], l[s]);
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int s = 0; s < kNumStats; ++s) {
            const float2 v = lane < nw ? sh[lane][s] : make_float2(0.f, 0.f);
            h[s] = v.x;
            l[s] = v.y;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) fin_level(h, l, o);
        if (lane == 0) {
#pragma unroll
            for (int s = 0; s < kNumStats; ++s) out[s] = (double)h[s] + (double)l[s];
        }
    }
}

__global__ void __launch_bounds__(kFinThreads) finalize_stats_kernel(const float2 *__restrict__ partials, int nblocks,
                                                                     double *__restrict__ out, int early) {
    pdl_wait();
    if (early) pdl_trigger();
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

namespace {
// power-of-two py with every physical row in the lower half: the pruned two-level y passes
bool y_fused_ok(const Grid &g) {
    const int py = g.py;
    return (py == 16 || py == 32 || py == 64 || py == 128 || py == 256 || py == 512) && 2 * g.ny <= py;
}
template <int N1, int N2, bool INV>
cudaError_t launch_y_fused(const ColPass &p, cudaStream_t s) {
    const size_t sm = sizeof(float2) * (size_t)p.tx * skewed_len(N1 * N2);
    const void *fn = INV ? (const void *)y_inverse_fused_kernel<N1, N2> : (const void *)y_forward_fused_kernel<N1, N2>;
    cudaError_t e = ensure_smem(fn, sm);
    if (e != cudaSuccess) return e;
    if (INV) return launch_pdl(y_inverse_fused_kernel<N1, N2>, dim3(tiles(p), p.g.nz, 3), dim3(kThreads), sm, s, p);
    return launch_pdl(y_forward_fused_kernel<N1, N2>, dim3(tiles(p), p.g.nz, 3), dim3(kThreads), sm, s, p);
}
// Radix split N = N1 x N2 of the two-level passes: split 0 is the default, split 1 the
// alternative the autotuner times against it (512 has one split: a 64-point outer pass
// would not fit the registers).
template <bool INV>
cudaError_t launch_y_dispatch(const ColPass &p, cudaStream_t s) {
    const bool alt = p.split != 0;
    switch (p.g.py) {
        case 16: return alt ? launch_y_fused<8, 2, INV>(p, s) : launch_y_fused<4, 4, INV>(p, s);
        case 32: return alt ? launch_y_fused<4, 8, INV>(p, s) : launch_y_fused<8, 4, INV>(p, s);
        case 64: return alt ? launch_y_fused<16, 4, INV>(p, s) : launch_y_fused<8, 8, INV>(p, s);
        case 128: return alt ? launch_y_fused<32, 4, INV>(p, s) : launch_y_fused<16, 8, INV>(p, s);
        case 256: return alt ? launch_y_fused<32, 8, INV>(p, s) : launch_y_fused<16, 16, INV>(p, s);
        default: return launch_y_fused<32, 16, INV>(p, s);
    }
}
}  // namespace

size_t y_pass_smem(const Grid &g, int tx) {
    const size_t one = sizeof(float2) * (size_t)tx * skewed_len(g.py);
    return y_fused_ok(g) ? one : 2 * one;
}

cudaError_t launch_y_forward(const ColPass &p, cudaStream_t s) {
    if (y_fused_ok(p.g)) return launch_y_dispatch<false>(p, s);
    const size_t sm = 2 * sizeof(float2) * (size_t)p.tx * skewed_len(p.g.py);
    cudaError_t e = ensure_smem((const void *)y_forward_kernel, sm);
    if (e != cudaSuccess) return e;
    return launch_pdl(y_forward_kernel, dim3(tiles(p), p.g.nz, 3), dim3(kThreads), sm, s, p);
}

cudaError_t launch_y_inverse(const ColPass &p, cudaStream_t s) {
    if (y_fused_ok(p.g)) return launch_y_dispatch<true>(p, s);
    const size_t sm = 2 * sizeof(float2) * (size_t)p.tx * skewed_len(p.g.py);
    cudaError_t e = ensure_smem((const void *)y_inverse_kernel, sm);
    if (e != cudaSuccess) return e;
    return launch_pdl(y_inverse_kernel, dim3(tiles(p), p.g.nz, 3), dim3(kThreads), sm, s, p);
}

namespace {
template <int N1, int N2>
cudaError_t launch_z_fused(const ColPass &p, cudaStream_t s) {
    const size_t sm = sizeof(float2) * (size_t)2 * 3 * p.tx * skewed_len(N1 * N2);
    cudaError_t e = ensure_smem((const void *)z_convolve_fused_kernel<N1, N2>, sm);
    if (e != cudaSuccess) return e;
    return launch_pdl(z_convolve_fused_kernel<N1, N2>, dim3(tiles(p), p.g.nky), dim3(kThreads), sm, s, p);
}
// power-of-two pz with every physical plane in the lower half: the pruned fused kernel
bool z_fused_ok(const Grid &g) {
    const int pz = g.pz;
    return g.per == 0 && (pz == 16 || pz == 32 || pz == 64 || pz == 128 || pz == 256 || pz == 512) && 2 * g.nz <= pz;
}
}  // namespace

size_t z_convolve_smem(const Grid &g, int tx) {
    const size_t one = sizeof(float2) * (size_t)2 * 3 * tx * skewed_len(g.pz);
    return z_fused_ok(g) ? one : 2 * one;
}

namespace {

// the packed ky-pair z pass: tile 8, pz = N1 * N2 with an inner radix of 8
bool z_pair_ok(const Grid &g, int tx) { return tx == 8 && z_fused_ok(g) && (g.pz == 64 || g.pz == 128); }

template <int N1, int N2>
cudaError_t launch_z_pair(const ColPass &p, cudaStream_t s) {
    const void *fn = (const void *)z_convolve_pair_kernel<N1, N2>;
    const size_t sm = sizeof(float4) * (size_t)3 * 8 * skewed_len(N1 * N2);
    cudaError_t e = ensure_smem(fn, sm);
    if (e != cudaSuccess) return e;
    return launch_pdl(z_convolve_pair_kernel<N1, N2>, dim3(tiles(p), p.g.nky), dim3(3 * N2 * 8), sm, s, p);
}
}  // namespace

bool z_convolve_pair_ok(const Grid &g, int tx) { return z_pair_ok(g, tx); }

cudaError_t launch_z_convolve(const ColPass &p, cudaStream_t s) {
    if (p.pipe) {
        if (!z_pair_ok(p.g, p.tx)) return cudaErrorInvalidValue;
        return p.g.pz == 64 ? launch_z_pair<8, 8>(p, s) : launch_z_pair<16, 8>(p, s);
    }
    if (z_fused_ok(p.g)) {
        const bool alt = p.split != 0;  // radix split, as launch_y_dispatch
        switch (p.g.pz) {
            case 16: return alt ? launch_z_fused<8, 2>(p, s) : launch_z_fused<4, 4>(p, s);
            case 32: return alt ? launch_z_fused<4, 8>(p, s) : launch_z_fused<8, 4>(p, s);
            case 64: return alt ? launch_z_fused<16, 4>(p, s) : launch_z_fused<8, 8>(p, s);
            case 128: return alt ? launch_z_fused<32, 4>(p, s) : launch_z_fused<16, 8>(p, s);
            case 256: return alt ? launch_z_fused<32, 8>(p, s) : launch_z_fused<16, 16>(p, s);
            default: return launch_z_fused<32, 16>(p, s);
        }
    }
    // room for a y-frequency pair: 2 x 3 lines per kx column, two ping-pong buffers
    const size_t sm = 2 * sizeof(float2) * (size_t)2 * 3 * p.tx * skewed_len(p.g.pz);
    cudaError_t e = ensure_smem((const void *)z_convolve_kernel, sm);
    if (e != cudaSuccess) return e;
    return launch_pdl(z_convolve_kernel, dim3(tiles(p), p.g.nky), dim3(kThreads), sm, s, p);
}

size_t yz_convolve_smem(const Grid &g, int tx) {
    const size_t a = (size_t)3 * tx * g.nz * skewed_len(g.py);
    if (yz_fused_ok(g)) return 2 * sizeof(float2) * a;
    const size_t b = (size_t)3 * tx * g.py * skewed_len(g.pz);
    return 2 * sizeof(float2) * (a > b ? a : b);
}

cudaError_t launch_yz_convolve(const ColPass &p, cudaStream_t s) {
    if (p.g.per) return cudaErrorInvalidValue;  // the fused y+z pass reads the octant kernel only
    const size_t sm = yz_convolve_smem(p.g, p.tx);
    cudaError_t e = ensure_smem((const void *)yz_convolve_kernel, sm);
    if (e != cudaSuccess) return e;
    return launch_pdl(yz_convolve_kernel, dim3(tiles(p)), dim3(kThreads), sm, s, p);
}

int col_batched_kind(const Grid &g) {
    if (g.thin) return y2d_fused_ok(g) ? 0 : 2;
    return yz_fused_ok(g) ? 1 : 3;
}

size_t y_convolve_2d_smem(const Grid &g, int tx) {
    const size_t one = sizeof(float2) * (size_t)3 * tx * skewed_len(g.py);
    const bool p512 = g.per == 0 && g.py == 512 && 2 * g.ny <= 512;
    return (y2d_fused_ok(g) || p512) ? one : 2 * one;
}

cudaError_t launch_col_batched(const ColPass *ps, const int2 *work, int nwork, int kind, size_t smem, cudaStream_t s) {
    const void *fns[4] = {(const void *)col_batched_kernel<0>, (const void *)col_batched_kernel<1>,
                          (const void *)col_batched_kernel<2>, (const void *)col_batched_kernel<3>};
    if (kind < 0 || kind > 3) return cudaErrorInvalidValue;
    cudaError_t e = ensure_smem(fns[kind], smem);
    if (e != cudaSuccess) return e;
    switch (kind) {
        case 0: col_batched_kernel<0><<<nwork, kThreads, smem, s>>>(ps, work); break;
        case 1: col_batched_kernel<1><<<nwork, kThreads, smem, s>>>(ps, work); break;
        case 2: col_batched_kernel<2><<<nwork, kThreads, smem, s>>>(ps, work); break;
        default: col_batched_kernel<3><<<nwork, kThreads, smem, s>>>(ps, work); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_finalize_batched(const FinDesc *fd, int nproblems, double *out, cudaStream_t s) {
    finalize_batched_kernel<<<nproblems, kFinThreads, 0, s>>>(fd, out);
    return cudaGetLastError();
}

cudaError_t launch_y_convolve_2d(const ColPass &p, cudaStream_t s) {
    const size_t sm = y_convolve_2d_smem(p.g, p.tx);
    const bool p512 = p.g.per == 0 && p.g.py == 512 && 2 * p.g.ny <= 512;
    const auto fn = p512 ? y_convolve_2d_p512_kernel : y_convolve_2d_kernel;
    cudaError_t e = ensure_smem((const void *)fn, sm);
    if (e != cudaSuccess) return e;
    return launch_pdl(fn, dim3(tiles(p)), dim3(kThreads), sm, s, p);
}

cudaError_t launch_finalize_stats(const float2 *partials, int nblocks, double *out, cudaStream_t s, int early) {
    return launch_pdl(finalize_stats_kernel, dim3(1), dim3(kFinThreads), 0, s, partials, nblocks, out, early);
}

namespace {
// [c][kz][ky][kx] -> [c][kz][kx][ky]; one launch at setup
__global__ void kern_ky_fast_kernel(const float *__restrict__ in, float *__restrict__ out, long long planes, int nky,
                                    int nkx) {
    const long long per = (long long)nky * nkx;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < planes * per; i += (long long)gridDim.x * blockDim.x) {
        const long long pl = i / per;
        const int r = (int)(i - pl * per), ky = r / nkx, kx = r - ky * nkx;
        out[pl * per + (long long)kx * nky + ky] = in[i];
    }
}
}  // namespace

cudaError_t launch_kern_ky_fast(const float *in, float *out, int ncomp, int nkz, int nky, int nkx, cudaStream_t s) {
    const long long total = (long long)ncomp * nkz * nky * nkx;
    const int blocks = (int)std::min<long long>((total + 255) / 256, 4096);
    kern_ky_fast_kernel<<<blocks, 256, 0, s>>>(in, out, (long long)ncomp * nkz, nky, nkx);
    return cudaGetLastError();
}

}  // namespace fm
