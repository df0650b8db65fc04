// fp64.cu -- the double-precision state path (plan precision FULLMAG_FDM_PRECISION_DOUBLE).
//
// State, stage derivatives, fields, the FFT convolution and every reduction are FP64.
// The structure is one kernel per operation, like the reference's FP64 backend, with
// this engine's own pieces: a mixed-radix FP64 FFT on lines in shared memory (no
// cuFFT), the real, octant-unique demag kernel of the FP32 path held in FP64, and the
// FP64 GPU Newell builder when the caller passes no spectra.  This path exists for
// accuracy, not speed: GB300 issues FP64 at a small fraction of its FP32 rate.
//
// Reference behaviour restated (paths in mzrptu/fullmag):
//   precision switch, plan validation          native/backends/fdm/src/api.cpp:97,324-395,533
//   exchange: mask clamp, region table          native/backends/fdm/src/exchange_fp64.cu:23-130
//   boundary tier T0 (face-link exchange)       native/backends/fdm/src/exchange_t0_fp64.cu:27-164
//   boundary tier T1 (boundary stencil)         native/backends/fdm/src/exchange_t1_fp64.cu:38-204
//   tier dispatch                               native/backends/fdm/src/exchange_fp64.cu:162-231
//   demag input phi Ms m, sparse correction      native/backends/fdm/src/demag_fp64.cu:55-90,440-545,
//                                               demag_boundary_fp64.cu:23-76
//   local terms, LLG right-hand side            native/backends/fdm/src/llg_fp64.cu
//   Heun / RK4 / DP45 / RK23 / ABM3 in FP64       llg_fp64.cu, llg_rk4_fp64.cu, llg_dp45_fp64.cu,
//                                               llg_rk23_fp64.cu, llg_abm3_fp64.cu
//   phi-weighted energies                        native/backends/fdm/src/reductions_fp64.cu:123-260,415-520
// Two kept differences from those kernels, both where the reference contradicts its own
// stated intent ("interior cells (phi = 1, f = 1) produce the standard exchange"):
//   * without region ids the T0 and T1 kernels scale by 2A/(mu0 Ms) and also weight
//     every face by A, so A enters twice; here A enters once, as in the standard kernel;
//   * cells with phi <= 0 (or m = 0) return before writing H there; here H = 0 there.
#include "fp64.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"

namespace fm {

namespace {

constexpr int kT = 256;
constexpr double kMu0d = 4.0 * M_PI * 1e-7;
constexpr int kMaxRadixStages = 32;
constexpr int kStats = 9;  // e_ex e_d e_ext e_uni e_cub | max|Heff|^2 max|Hd|^2 max|k|^2 max err^2
constexpr int kRedBlocks = 1024;

struct Plan64 {
    int n;
    int ns;
    int radix[kMaxRadixStages];
    const double2 *tw;  // n entries, e^{-2 pi i e / n}
};

__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 ztw(const double2 *tw, int e, bool inv) {
    const double2 w = tw[e];
    return inv ? zconj(w) : w;
}

// One line of length p.n in shared memory, transformed by the whole CTA with Stockham
// stages (natural order in and out); returns the buffer holding the result.  Radix 4
// and 2 have their own butterflies; any other radix R is an O(R^2) DFT read from the
// table at stride n / R.  Contains __syncthreads: every thread of the CTA calls it.
__device__ double2 *fft_line64(double2 *a, double2 *b, const Plan64 &p, bool inv) {
    int Ns = 1;
    const int n = p.n;
    for (int s = 0; s < p.ns; ++s) {
        const int R = p.radix[s], nb = n / R, tws = n / (Ns * R), rs = n / R;
        for (int j = threadIdx.x; j < nb; j += blockDim.x) {
            const int k = j % Ns, o = (j / Ns) * Ns * R + k;
            if (R == 2) {
                double2 v0 = a[j], v1 = a[j + nb];
                if (Ns > 1) v1 = zmul(v1, ztw(p.tw, k * tws, inv));
                b[o] = zadd(v0, v1);
                b[o + Ns] = zsub(v0, v1);
            } else if (R == 4) {
                double2 v[4];
                for (int t = 0; t < 4; ++t) {
                    v[t] = a[j + t * nb];
                    if (Ns > 1 && t) v[t] = zmul(v[t], ztw(p.tw, t * k * tws, inv));
                }
                const double2 a0 = zadd(v[0], v[2]), a1 = zsub(v[0], v[2]), b0 = zadd(v[1], v[3]);
                const double2 d = zsub(v[1], v[3]);
                const double2 b1 = inv ? make_double2(-d.y, d.x) : make_double2(d.y, -d.x);
                b[o] = zadd(a0, b0);
                b[o + 2 * Ns] = zsub(a0, b0);
                b[o + Ns] = zadd(a1, b1);
                b[o + 3 * Ns] = zsub(a1, b1);
            } else {
                for (int q = 0; q < R; ++q) {
                    double2 acc = make_double2(0.0, 0.0);
                    for (int t = 0; t < R; ++t) {
                        double2 x = a[j + t * nb];
                        if (Ns > 1 && t) x = zmul(x, ztw(p.tw, t * k * tws, inv));
                        acc = zadd(acc, zmul(x, ztw(p.tw, ((t * q) % R) * rs, inv)));
                    }
                    b[o + q * Ns] = acc;
                }
            }
        }
        __syncthreads();
        double2 *t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

__device__ __forceinline__ void mirror(int k, int p, int &km, double &sg) {
    if (k > p / 2) {
        km = p - k;
        sg = -1.0;
    } else {
        km = k;
        sg = 1.0;
    }
}

struct Conv64 {
    int nx, ny, nz, px, py, pz, nkx, nky, nkz, thin;
    long long n;
    Plan64 plx, ply, plz;
    const double *kern;    // octant kernel scaled by Ms / P
    const double2 *kernc;  // periodic grids: complex kernel K[c][kz][ky][kx] (full ky, kz), else NULL
};

// row (y, z) and component c: phi m along x, zero padded to px -> X[c][row][kx < nkx]
__global__ void x_forward64(const Conv64 C, const double *__restrict__ m, const double *__restrict__ phi,
                            double2 *__restrict__ X) {
    extern __shared__ double2 sm64[];
    double2 *a = sm64, *b = sm64 + C.px;
    const int row = blockIdx.x, c = blockIdx.y, nrows = C.ny * C.nz;
    const long long base = (long long)row * C.nx;
    for (int x = threadIdx.x; x < C.px; x += blockDim.x) {
        double v = 0.0;
        if (x < C.nx) {
            v = m[c * C.n + base + x];
            if (phi) v *= phi[base + x];
        }
        a[x] = make_double2(v, 0.0);
    }
    __syncthreads();
    const double2 *r = fft_line64(a, b, C.plx, false);
    for (int k = threadIdx.x; k < C.nkx; k += blockDim.x) X[((long long)c * nrows + row) * C.nkx + k] = r[k];
}

// X[c][row][kx] -> H_d along x (real part of the inverse of the Hermitian-completed line);
// zero at cells outside the body (mask, or phi <= 0 with a boundary tier)
__global__ void x_inverse64(const Conv64 C, const double2 *__restrict__ X, double *__restrict__ hd,
                            const uint8_t *__restrict__ mask, const double *__restrict__ phi) {
    extern __shared__ double2 sm64[];
    double2 *a = sm64, *b = sm64 + C.px;
    const int row = blockIdx.x, c = blockIdx.y, nrows = C.ny * C.nz;
    const double2 *src = X + ((long long)c * nrows + row) * C.nkx;
    for (int k = threadIdx.x; k < C.px; k += blockDim.x) a[k] = k < C.nkx ? src[k] : zconj(src[C.px - k]);
    __syncthreads();
    const double2 *r = fft_line64(a, b, C.plx, true);
    for (int x = threadIdx.x; x < C.nx; x += blockDim.x) {
        const long long i = (long long)row * C.nx + x;
        const bool act = (mask == nullptr || mask[i] != 0) && (phi == nullptr || phi[i] > 0.0);
        hd[c * C.n + i] = act ? r[x].x : 0.0;
    }
}

// (c, z, kx): y < ny zero padded to py, forward -> Y[c][z][ky][kx]
__global__ void y_forward64(const Conv64 C, const double2 *__restrict__ X, double2 *__restrict__ Y) {
    extern __shared__ double2 sm64[];
    double2 *a = sm64, *b = sm64 + C.py;
    const int kx = blockIdx.x, z = blockIdx.y, c = blockIdx.z;
    const double2 *src = X + (((long long)c * C.nz + z) * C.ny) * C.nkx + kx;
    for (int y = threadIdx.x; y < C.py; y += blockDim.x) a[y] = y < C.ny ? src[(long long)y * C.nkx] : make_double2(0.0, 0.0);
    __syncthreads();
    const double2 *r = fft_line64(a, b, C.ply, false);
    double2 *dst = Y + (((long long)c * C.nz + z) * C.py) * C.nkx + kx;
    for (int ky = threadIdx.x; ky < C.py; ky += blockDim.x) dst[(long long)ky * C.nkx] = r[ky];
}

// (c, z, kx): inverse over ky, rows y < ny back into X
__global__ void y_inverse64(const Conv64 C, const double2 *__restrict__ Y, double2 *__restrict__ X) {
    extern __shared__ double2 sm64[];
    double2 *a = sm64, *b = sm64 + C.py;
    const int kx = blockIdx.x, z = blockIdx.y, c = blockIdx.z;
    const double2 *src = Y + (((long long)c * C.nz + z) * C.py) * C.nkx + kx;
    for (int ky = threadIdx.x; ky < C.py; ky += blockDim.x) a[ky] = src[(long long)ky * C.nkx];
    __syncthreads();
    const double2 *r = fft_line64(a, b, C.ply, true);
    double2 *dst = X + (((long long)c * C.nz + z) * C.ny) * C.nkx + kx;
    for (int y = threadIdx.x; y < C.ny; y += blockDim.x) dst[(long long)y * C.nkx] = r[y];
}

__device__ __forceinline__ double2 zmadd(double2 k, double2 m, double2 acc) {
    return make_double2(acc.x + k.x * m.x - k.y * m.y, acc.y + k.x * m.y + k.y * m.x);
}

// H(k) = -N(k) M(k) on three lines a[0..2] at (kx, ky, kz) of the octant kernel, or of the
// complex kernel of a periodic grid (components xx yy zz xy xz yz; 2-D: the first four)
__device__ __forceinline__ void multiply3(const Conv64 &C, double2 *mx, double2 *my, double2 *mz, int kx, int ky, int kz) {
    if (C.kernc) {
        const long long kc = (long long)C.pz * C.py * C.nkx;
        const double2 *K = C.kernc + ((long long)kz * C.py + ky) * C.nkx + kx;
        const double2 z0 = make_double2(0.0, 0.0);
        const double2 kxx = K[0], kyy = K[kc], kzz = K[2 * kc], kxy = K[3 * kc];
        const double2 kxz = C.thin ? z0 : K[4 * kc], kyz = C.thin ? z0 : K[5 * kc];
        const double2 a = *mx, b = *my, d = *mz;
        const double2 hx = zmadd(kxz, d, zmadd(kxy, b, zmadd(kxx, a, z0)));
        const double2 hy = zmadd(kyz, d, zmadd(kyy, b, zmadd(kxy, a, z0)));
        const double2 hz = zmadd(kzz, d, zmadd(kyz, b, zmadd(kxz, a, z0)));
        *mx = make_double2(-hx.x, -hx.y);
        *my = make_double2(-hy.x, -hy.y);
        *mz = make_double2(-hz.x, -hz.y);
        return;
    }
    int kym, kzm;
    double sy, sz;
    mirror(ky, C.py, kym, sy);
    if (C.thin) {
        const long long kc = (long long)C.nky * C.nkx;
        const double *K = C.kern + (long long)kym * C.nkx + kx;
        const double kxx = K[0], kyy = K[kc], kzz = K[2 * kc], kxy = sy * K[3 * kc];
        const double2 a = *mx, b = *my, d = *mz;
        *mx = make_double2(-(kxx * a.x + kxy * b.x), -(kxx * a.y + kxy * b.y));
        *my = make_double2(-(kxy * a.x + kyy * b.x), -(kxy * a.y + kyy * b.y));
        *mz = make_double2(-kzz * d.x, -kzz * d.y);
        return;
    }
    mirror(kz, C.pz, kzm, sz);
    const long long kc = (long long)C.nkz * C.nky * C.nkx;
    const double *K = C.kern + ((long long)kzm * C.nky + kym) * C.nkx + kx;
    const double kxx = K[0], kyy = K[kc], kzz = K[2 * kc];
    const double kxy = sy * K[3 * kc], kxz = sz * K[4 * kc], kyz = sy * sz * K[5 * kc];
    const double2 a = *mx, b = *my, d = *mz;
    *mx = make_double2(-(kxx * a.x + kxy * b.x + kxz * d.x), -(kxx * a.y + kxy * b.y + kxz * d.y));
    *my = make_double2(-(kxy * a.x + kyy * b.x + kyz * d.x), -(kxy * a.y + kyy * b.y + kyz * d.y));
    *mz = make_double2(-(kxz * a.x + kyz * b.x + kzz * d.x), -(kxz * a.y + kyz * b.y + kzz * d.y));
}

// 3-D: (kx, ky): forward z of the three components, multiply, inverse, planes z < nz
__global__ void z_convolve64(const Conv64 C, double2 *__restrict__ Y) {
    extern __shared__ double2 sm64[];
    const int kx = blockIdx.x, ky = blockIdx.y, L = C.pz;
    double2 *a[3], *b[3];
    for (int c = 0; c < 3; ++c) {
        a[c] = sm64 + 2 * c * L;
        b[c] = a[c] + L;
    }
    const long long zs = (long long)C.py * C.nkx, cs = (long long)C.nz * zs;
    for (int c = 0; c < 3; ++c)
        for (int z = threadIdx.x; z < L; z += blockDim.x)
            a[c][z] = z < C.nz ? Y[c * cs + z * zs + (long long)ky * C.nkx + kx] : make_double2(0.0, 0.0);
    __syncthreads();
    double2 *r[3];
    for (int c = 0; c < 3; ++c) r[c] = fft_line64(a[c], b[c], C.plz, false);
    for (int kz = threadIdx.x; kz < L; kz += blockDim.x) multiply3(C, r[0] + kz, r[1] + kz, r[2] + kz, kx, ky, kz);
    __syncthreads();
    double2 *q[3];
    for (int c = 0; c < 3; ++c) q[c] = fft_line64(r[c], r[c] == a[c] ? b[c] : a[c], C.plz, true);
    for (int c = 0; c < 3; ++c)
        for (int z = threadIdx.x; z < C.nz; z += blockDim.x) Y[c * cs + z * zs + (long long)ky * C.nkx + kx] = q[c][z];
}

// thin film: (kx): forward y of the three components, 2-D multiply, inverse, rows y < ny
__global__ void y_convolve64(const Conv64 C, double2 *__restrict__ X) {
    extern __shared__ double2 sm64[];
    const int kx = blockIdx.x, L = C.py;
    double2 *a[3], *b[3];
    for (int c = 0; c < 3; ++c) {
        a[c] = sm64 + 2 * c * L;
        b[c] = a[c] + L;
    }
    const long long cs = (long long)C.ny * C.nkx;
    for (int c = 0; c < 3; ++c)
        for (int y = threadIdx.x; y < L; y += blockDim.x)
            a[c][y] = y < C.ny ? X[c * cs + (long long)y * C.nkx + kx] : make_double2(0.0, 0.0);
    __syncthreads();
    double2 *r[3];
    for (int c = 0; c < 3; ++c) r[c] = fft_line64(a[c], b[c], C.ply, false);
    for (int ky = threadIdx.x; ky < L; ky += blockDim.x) multiply3(C, r[0] + ky, r[1] + ky, r[2] + ky, kx, ky, 0);
    __syncthreads();
    double2 *q[3];
    for (int c = 0; c < 3; ++c) q[c] = fft_line64(r[c], r[c] == a[c] ? b[c] : a[c], C.ply, true);
    for (int c = 0; c < 3; ++c)
        for (int y = threadIdx.x; y < C.ny; y += blockDim.x) X[c * cs + (long long)y * C.nkx + kx] = q[c][y];
}

// H_corr(t) = -sum_s dN(t, s) (phi_s Ms m_s), added to H_d at the target cells
// (demag_boundary_fp64.cu:23-76); the tensor row of (t, s) is xx xy xz yy yz zz.
__global__ void demag_correction64(double *__restrict__ hd, const double *__restrict__ m, const double *__restrict__ phi,
                                   const int32_t *__restrict__ tidx, const int32_t *__restrict__ sidx,
                                   const double *__restrict__ tensor, double ms, long long n, uint32_t ntarget,
                                   uint32_t stencil) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntarget; t += gridDim.x * blockDim.x) {
        const int32_t ti = tidx[t];
        if (ti < 0) continue;
        double hx = 0.0, hy = 0.0, hz = 0.0;
        for (uint32_t s = 0; s < stencil; ++s) {
            const int32_t si = sidx[(size_t)t * stencil + s];
            if (si < 0) continue;
            const double *N = tensor + ((size_t)t * stencil + s) * 6;
            const double w = (phi ? phi[si] : 1.0) * ms;
            const double Mx = w * m[si], My = w * m[n + si], Mz = w * m[2 * n + si];
            hx -= N[0] * Mx + N[1] * My + N[2] * Mz;
            hy -= N[1] * Mx + N[3] * My + N[4] * Mz;
            hz -= N[2] * Mx + N[4] * My + N[5] * Mz;
        }
        hd[ti] += hx;
        hd[n + ti] += hy;
        hd[2 * n + ti] += hz;
    }
}

struct Field64 {
    int nx, ny, nz;
    long long n;
    const double *m, *hd;     // hd NULL: no demag
    double *hex, *heff, *k;   // k NULL: not stored
    const uint8_t *mask;
    const uint8_t *region;    // ids (< 256) or NULL
    const double *lut;        // 256 x 256 stiffness table (J/m)
    int tier;                 // 0 none, 1 T0 face links, 2 T1 boundary distances
    const double *phi;        // volume fractions (tiers 1, 2; also weights the energies)
    const double *face[6];    // +x -x +y -y +z -z
    const double *delta[6];
    double phi_floor, delta_min;
    int exchange;
    int per;                  // periodic axes (bit 0 x, 1 y, 2 z): neighbours wrap around
    double a_ex, ms, dx, dy, dz;
    int has_ext;
    double hext[3];
    int has_uni;
    double ku1, ku2, u[3];
    int has_cub;
    double kc1, kc2, kc3, c1[3], c2[3], c3[3];
    double gbar, alpha, prec;
    double *partials;         // [block][kStats] or NULL
};

// exchange field at cell i (x, y, z); the neighbour offsets are +x -x +y -y +z -z
__device__ void exchange64(const Field64 &P, long long i, int x, int y, int z, double e[3]) {
    e[0] = e[1] = e[2] = 0.0;
    if (!P.exchange) return;
    const double *m = P.m;
    const long long n = P.n, nxy = (long long)P.nx * P.ny;
    const bool has[6] = {x + 1 < P.nx, x > 0, y + 1 < P.ny, y > 0, z + 1 < P.nz, z > 0};
    const long long off[6] = {1, -1, P.nx, -(long long)P.nx, nxy, -nxy};
    const double inv2[6] = {1.0 / (P.dx * P.dx), 1.0 / (P.dx * P.dx), 1.0 / (P.dy * P.dy),
                            1.0 / (P.dy * P.dy), 1.0 / (P.dz * P.dz), 1.0 / (P.dz * P.dz)};
    const double c0[3] = {m[i], m[n + i], m[2 * n + i]};
    const int ri = P.region ? P.region[i] : 0;
    if (P.tier == 0) {
        // clamped neighbours: out of range or inactive -> the centre (no contribution); on a
        // periodic axis the neighbour wraps around (fdm_types.rs:126-132)
        const int ext[3] = {P.nx, P.ny, P.nz};
        for (int q = 0; q < 6; ++q) {
            long long j = has[q] ? i + off[q] : ((P.per >> (q >> 1)) & 1) ? i - off[q] * (ext[q >> 1] - 1) : i;
            if (P.mask && P.mask[j] == 0) j = i;
            if (j == i) continue;
            const double w = (P.region ? P.lut[ri * FULLMAG_FDM_MAX_EXCHANGE_REGIONS + P.region[j]] : P.a_ex) * inv2[q];
            for (int c = 0; c < 3; ++c) e[c] += w * (m[c * n + j] - c0[c]);
        }
    } else if (P.tier == 1) {
        // T0: face-link weights f
        for (int q = 0; q < 6; ++q) {
            if (q >= 4 && P.nz <= 1) continue;
            const double f = P.face[q][i];
            if (!(f > 0.0) || !has[q]) continue;
            const long long j = i + off[q];
            const double w = (P.region ? P.lut[ri * FULLMAG_FDM_MAX_EXCHANGE_REGIONS + P.region[j]] : P.a_ex) * f * inv2[q];
            for (int c = 0; c < 3; ++c) e[c] += w * (m[c * n + j] - c0[c]);
        }
    } else {
        // T1: neighbour at distance d across the face, boundary at the opposite distance
        // delta: 2 / (d (d + delta_opposite)) per face
        const double d[6] = {P.dx, P.dx, P.dy, P.dy, P.dz, P.dz};
        for (int q = 0; q < 6; ++q) {
            if (q >= 4 && P.nz <= 1) continue;
            const double dopp = fmax(P.delta[q ^ 1][i], P.delta_min);
            const double dsel = fmax(P.delta[q][i], P.delta_min);
            if (!has[q] || !(dsel > 0.0)) continue;
            const long long j = i + off[q];
            const double mj[3] = {m[j], m[n + j], m[2 * n + j]};
            if (mj[0] == 0.0 && mj[1] == 0.0 && mj[2] == 0.0) continue;
            const double w = (P.region ? P.lut[ri * FULLMAG_FDM_MAX_EXCHANGE_REGIONS + P.region[j]] : P.a_ex) * 2.0 /
                             (d[q] * (d[q] + dopp));
            for (int c = 0; c < 3; ++c) e[c] += w * (mj[c] - c0[c]);
        }
    }
    double s = 2.0 / (kMu0d * P.ms);
    if (P.tier > 0) s /= fmax(P.phi[i], P.phi_floor);
    for (int c = 0; c < 3; ++c) e[c] *= s;
}

// exchange energy pairs of cell i with its forward neighbours (reductions_fp64.cu:123-210)
__device__ double exchange_pairs64(const Field64 &P, long long i, int x, int y, int z, double phi_i) {
    if (!P.exchange) return 0.0;
    const double *m = P.m;
    const long long n = P.n, nxy = (long long)P.nx * P.ny;
    const bool has[3] = {x + 1 < P.nx, y + 1 < P.ny, z + 1 < P.nz};
    const long long off[3] = {1, P.nx, nxy};
    const int ext[3] = {P.nx, P.ny, P.nz};
    const double inv2[3] = {1.0 / (P.dx * P.dx), 1.0 / (P.dy * P.dy), 1.0 / (P.dz * P.dz)};
    const int ri = P.region ? P.region[i] : 0;
    double e = 0.0;
    for (int a = 0; a < 3; ++a) {
        // forward pairs; on a periodic axis the last cell pairs with the first
        const bool wrap = !has[a] && ((P.per >> a) & 1);
        if (!has[a] && !wrap) continue;
        const long long j = has[a] ? i + off[a] : i - off[a] * (ext[a] - 1);
        if (j == i) continue;
        if (P.mask && P.mask[j] == 0) continue;
        if (P.phi && !(P.phi[j] > 0.0)) continue;
        const double A = P.region ? P.lut[ri * FULLMAG_FDM_MAX_EXCHANGE_REGIONS + P.region[j]] : P.a_ex;
        double s2 = 0.0;
        for (int c = 0; c < 3; ++c) {
            const double dm = m[c * n + j] - m[c * n + i];
            s2 += dm * dm;
        }
        e += A * phi_i * s2 * inv2[a];
    }
    return e;
}

__device__ __forceinline__ void block_stats(double (&v)[kStats], double *out) {
    __shared__ double red[kT / 32][kStats];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int s = 0; s < kStats; ++s)
        for (int o = 16; o > 0; o >>= 1) {
            const double w = __shfl_xor_sync(0xffffffffu, v[s], o);
            v[s] = s < 5 ? v[s] + w : fmax(v[s], w);
        }
    if (lane == 0)
        for (int s = 0; s < kStats; ++s) red[wid][s] = v[s];
    __syncthreads();
    if (threadIdx.x < kStats) {
        const int s = threadIdx.x;
        double acc = 0.0;
        for (int w = 0; w < kT / 32; ++w) acc = s < 5 ? acc + red[w][s] : fmax(acc, red[w][s]);
        out[blockIdx.x * kStats + s] = acc;
    }
}

// H_eff, the right-hand side and (optionally) the statistics of one evaluation
__global__ void __launch_bounds__(kT) field64(const Field64 P) {
    double st[kStats] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const long long n = P.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % P.nx), y = (int)((i / P.nx) % P.ny), z = (int)(i / ((long long)P.nx * P.ny));
        const double phi_i = P.phi ? P.phi[i] : 1.0;
        const bool act = (P.mask == nullptr || P.mask[i] != 0) && (P.tier == 0 || phi_i > 0.0);
        double h[3] = {0, 0, 0}, ex[3] = {0, 0, 0}, hd[3] = {0, 0, 0}, k[3] = {0, 0, 0};
        if (act) {
            const double m0[3] = {P.m[i], P.m[n + i], P.m[2 * n + i]};
            exchange64(P, i, x, y, z, ex);
            if (P.hd)
                for (int c = 0; c < 3; ++c) hd[c] = P.hd[c * n + i];
            for (int c = 0; c < 3; ++c) h[c] = ex[c] + hd[c] + (P.has_ext ? P.hext[c] : 0.0);
            double e_uni = 0.0, e_cub = 0.0;
            const double inv_mu0ms = 1.0 / (kMu0d * P.ms);
            if (P.has_uni) {
                const double mu = m0[0] * P.u[0] + m0[1] * P.u[1] + m0[2] * P.u[2];
                const double cf = 2.0 * inv_mu0ms * (P.ku1 * mu + 2.0 * P.ku2 * mu * mu * mu);
                for (int c = 0; c < 3; ++c) h[c] += cf * P.u[c];
                e_uni = P.ku1 * mu * mu + P.ku2 * mu * mu * mu * mu;
            }
            if (P.has_cub) {
                const double a1 = m0[0] * P.c1[0] + m0[1] * P.c1[1] + m0[2] * P.c1[2];
                const double a2 = m0[0] * P.c2[0] + m0[1] * P.c2[1] + m0[2] * P.c2[2];
                const double a3 = m0[0] * P.c3[0] + m0[1] * P.c3[1] + m0[2] * P.c3[2];
                const double s1 = a1 * a1, s2 = a2 * a2, s3 = a3 * a3;
                const double sig = s1 * s2 + s2 * s3 + s1 * s3;
                const double k1c = -2.0 * P.kc1 * inv_mu0ms, k2c = -2.0 * P.kc2 * inv_mu0ms, k3c = -4.0 * P.kc3 * inv_mu0ms;
                const double g1 = k1c * a1 * (s2 + s3) + k2c * a1 * s2 * s3 + k3c * sig * a1 * (s2 + s3);
                const double g2 = k1c * a2 * (s1 + s3) + k2c * a2 * s1 * s3 + k3c * sig * a2 * (s1 + s3);
                const double g3 = k1c * a3 * (s1 + s2) + k2c * a3 * s1 * s2 + k3c * sig * a3 * (s1 + s2);
                for (int c = 0; c < 3; ++c) h[c] += g1 * P.c1[c] + g2 * P.c2[c] + g3 * P.c3[c];
                e_cub = P.kc1 * sig + P.kc2 * s1 * s2 * s3 + P.kc3 * sig * sig;
            }
            const double p0 = m0[1] * h[2] - m0[2] * h[1], p1 = m0[2] * h[0] - m0[0] * h[2], p2 = m0[0] * h[1] - m0[1] * h[0];
            const double q0 = m0[1] * p2 - m0[2] * p1, q1 = m0[2] * p0 - m0[0] * p2, q2 = m0[0] * p1 - m0[1] * p0;
            k[0] = -P.gbar * (P.prec * p0 + P.alpha * q0);
            k[1] = -P.gbar * (P.prec * p1 + P.alpha * q1);
            k[2] = -P.gbar * (P.prec * p2 + P.alpha * q2);
            if (P.partials) {
                st[0] += exchange_pairs64(P, i, x, y, z, phi_i);
                st[1] += phi_i * (m0[0] * hd[0] + m0[1] * hd[1] + m0[2] * hd[2]);
                if (P.has_ext) st[2] += phi_i * (m0[0] * P.hext[0] + m0[1] * P.hext[1] + m0[2] * P.hext[2]);
                st[3] += phi_i * e_uni;
                st[4] += phi_i * e_cub;
                st[5] = fmax(st[5], h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
                st[6] = fmax(st[6], hd[0] * hd[0] + hd[1] * hd[1] + hd[2] * hd[2]);
                st[7] = fmax(st[7], k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
            }
        }
        for (int c = 0; c < 3; ++c) {
            P.hex[c * n + i] = ex[c];
            P.heff[c * n + i] = h[c];
            if (P.k) P.k[c * n + i] = k[c];
        }
    }
    if (P.partials) block_stats(st, P.partials);
}

// out = N(m0 + dt sum_j c_j k_j) (a zero vector stays zero)
struct Comb64 {
    long long n;
    const double *m0;
    int nk;
    const double *k[8];
    double c[8];
    double dt;
    double *out;
};
__global__ void combine64(const Comb64 C) {
    const long long n = C.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double v[3];
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int t = 0; t < C.nk; ++t) s += C.c[t] * C.k[t][c * n + i];
            v[c] = C.m0[c * n + i] + C.dt * s;
        }
        const double nn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        const double inv = nn > 0.0 ? 1.0 / nn : 0.0;
        for (int c = 0; c < 3; ++c) C.out[c * n + i] = v[c] * inv;
    }
}

// max over cells of |dt sum_j e_j k_j|^2 into partials[block * kStats + 8]
__global__ void __launch_bounds__(kT) error64(const Comb64 C, double *partials) {
    double st[kStats] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const long long n = C.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double e2 = 0.0;
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int t = 0; t < C.nk; ++t) s += C.c[t] * C.k[t][c * n + i];
            s *= C.dt;
            e2 += s * s;
        }
        st[8] = fmax(st[8], e2);
    }
    block_stats(st, partials);
}

// sums / maxima of the block partials in a fixed order (one CTA)
__global__ void finalize64(const double *partials, int nblocks, double *out, int with_err) {
    __shared__ double sh[kT][kStats];
    for (int s = 0; s < kStats; ++s) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
            const double v = partials[b * kStats + s];
            acc = s < 5 ? acc + v : fmax(acc, v);
        }
        sh[threadIdx.x][s] = acc;
    }
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int s = 0; s < kStats; ++s)
                sh[threadIdx.x][s] = s < 5 ? sh[threadIdx.x][s] + sh[threadIdx.x + o][s] : fmax(sh[threadIdx.x][s], sh[threadIdx.x + o][s]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int s = 0; s < kStats; ++s)
            if (s < 8 || with_err) out[s] = sh[0][s];
}

__global__ void aos_to_soa64(const double *__restrict__ in, double *__restrict__ out, const uint8_t *__restrict__ mask,
                             const double *__restrict__ phi, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const bool act = (mask == nullptr || mask[i] != 0) && (phi == nullptr || phi[i] > 0.0);
        for (int c = 0; c < 3; ++c) out[c * n + i] = act ? in[3 * i + c] : 0.0;
    }
}

__global__ void soa_to_aos64(const double *__restrict__ in, double *__restrict__ out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        for (int c = 0; c < 3; ++c) out[3 * i + c] = in[c * n + i];
}

unsigned blocks_for(long long n) { return (unsigned)std::min<long long>((n + kT - 1) / kT, kRedBlocks); }

// radices 4, 2, 3, 5, 7, then any remaining prime
bool make_plan64(int n, std::vector<double2> &tw, std::vector<size_t> &off, Plan64 &p) {
    p.n = n;
    p.ns = 0;
    int r = n;
    for (int f : {4, 2, 3, 5, 7}) {
        while (r % f == 0) {
            if (p.ns >= kMaxRadixStages) return false;
            p.radix[p.ns++] = f;
            r /= f;
        }
    }
    for (int f = 11; r > 1; f += 2) {
        while (r % f == 0) {
            if (p.ns >= kMaxRadixStages) return false;
            p.radix[p.ns++] = f;
            r /= f;
        }
    }
    off.push_back(tw.size());
    for (int e = 0; e < n; ++e) {
        const double a = 2.0 * M_PI * (double)e / (double)n;
        tw.push_back(make_double2(cos(a), -sin(a)));
    }
    p.tw = nullptr;
    return true;
}

// One FP64 line of length p per CTA along an axis of layout [outer][p][inner] (real
// input in_re with zero imaginary part, or complex c_in), forward transform
// e^{-2 pi i k a / p}, the first nout outputs written to out[outer][nout][inner].
__global__ void fft_axis64_kernel(const double *__restrict__ in_re, const double2 *__restrict__ c_in,
                                  double2 *__restrict__ out, int p, int nout, int inner, const Plan64 plan) {
    extern __shared__ double2 sm64[];
    double2 *a = sm64, *b = sm64 + p;
    const long long line = blockIdx.x;
    const long long o = line / inner, q = line - o * inner;
    const long long base = o * p * inner + q;
    for (int i = threadIdx.x; i < p; i += blockDim.x)
        a[i] = in_re ? make_double2(in_re[base + (long long)i * inner], 0.0) : c_in[base + (long long)i * inner];
    __syncthreads();
    const double2 *r = fft_line64(a, b, plan, false);
    for (int k = threadIdx.x; k < nout; k += blockDim.x) out[(o * nout + k) * inner + q] = r[k];
}

}  // namespace

bool fft64_axis(const double *in_re, const double2 *c_in, double2 *out, long long outer, int p, int nout, int inner,
                cudaStream_t s, std::string &err) {
    std::vector<double2> tw;
    std::vector<size_t> off;
    Plan64 plan;
    if (!make_plan64(p, tw, off, plan)) return err = "FFT length has too many factors", false;
    const size_t smem = sizeof(double2) * 2 * (size_t)p;
    if (smem > 227 * 1024) return err = "FFT length too large for the double-precision lines", false;
    double2 *dtw = nullptr;
    cudaError_t e = cudaMalloc(&dtw, sizeof(double2) * tw.size());
    if (e == cudaSuccess) e = cudaMemcpyAsync(dtw, tw.data(), sizeof(double2) * tw.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute((const void *)fft_axis64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) {
        plan.tw = dtw;
        const long long lines = outer * inner;
        fft_axis64_kernel<<<(unsigned)lines, 128, smem, s>>>(in_re, c_in, out, p, nout, inner, plan);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(dtw);
    if (e != cudaSuccess) return err = std::string("fft64_axis: ") + cudaGetErrorString(e), false;
    return true;
}

struct Fp64Engine {
    // configuration
    int nx = 0, ny = 0, nz = 0;
    long long n = 0;
    double dx = 0, dy = 0, dz = 0, ms = 0, a_ex = 0, alpha = 0, gamma = 0;
    int integrator = FULLMAG_FDM_INTEGRATOR_HEUN;
    bool exchange = false, demag = false, has_ext = false, has_uni = false, has_cub = false, prec = true;
    double hext[3] = {0, 0, 0};
    double ku1 = 0, ku2 = 0, u[3] = {0, 0, 1}, kc1 = 0, kc2 = 0, kc3 = 0, c1[3] = {1, 0, 0}, c2[3] = {0, 1, 0}, c3[3] = {0, 0, 1};
    double max_error = 1e-5, dt_min = 1e-18, dt_max = 1e-10, headroom = 0.8;
    int tier = 0;
    double phi_floor = 0.0, delta_min = 0.0;
    int per = 0;                     // periodic axes (bit 0 x, 1 y, 2 z)
    uint32_t images[3] = {10, 10, 10};
    bool has_mask = false;
    std::vector<uint8_t> mask_host;
    uint32_t corr_targets = 0, corr_stencil = 0;
    // device
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    double *S[2] = {nullptr, nullptr}, *K[7] = {}, *A[2] = {nullptr, nullptr};
    double *hex = nullptr, *hd = nullptr, *heff = nullptr, *staging = nullptr;
    double *partials = nullptr, *dstats = nullptr, *hstats = nullptr;
    uint8_t *mask = nullptr, *region = nullptr;
    double *lut = nullptr, *phi = nullptr, *face[6] = {}, *delta[6] = {};
    int32_t *ctidx = nullptr, *csidx = nullptr;
    double *ctensor = nullptr;
    Conv64 conv{};
    double2 *X = nullptr, *Y = nullptr;
    double *kern = nullptr;
    double2 *kernc = nullptr;  // periodic grids: the complex image-sum kernel
    double2 *twid = nullptr;
    // state
    int cur = 0;
    double time = 0.0;
    uint64_t step_count = 0;
    bool k1_valid = false;
    bool fields_ok = false;  // hex / hd / heff hold the fields of the committed state
    fullmag_fdm_step_stats cur_stats{};
    double raw[kStats] = {};
    // ABM3 history (indices into K, rotated)
    int abm_startup = 0;
    double abm_last_dt = 0.0;
    int abm_hist[3] = {1, 2, 3}, abm_kf = 4;
    std::string err;

    ~Fp64Engine() {
        if (stream) cudaStreamSynchronize(stream);
        for (void *p : allocs) cudaFree(p);
        if (hstats) cudaFreeHost(hstats);
        if (stream) cudaStreamDestroy(stream);
    }

    bool fail(const char *what, cudaError_t e) {
        if (e == cudaSuccess) return false;
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return true;
    }
    template <typename T>
    bool alloc(T *&p, size_t count) {
        void *q = nullptr;
        if (fail("cudaMalloc", cudaMalloc(&q, sizeof(T) * std::max<size_t>(count, 1)))) return false;
        allocs.push_back(q);
        p = static_cast<T *>(q);
        return true;
    }
    template <typename T>
    bool put(T *&p, const T *src, size_t count) {
        return alloc(p, count) &&
               !fail("cudaMemcpy", cudaMemcpyAsync(p, src, sizeof(T) * count, cudaMemcpyHostToDevice, stream));
    }

    bool setup(const fullmag_fdm_plan_desc *plan);
    bool upload(const double *m_xyz);

    // ---- one evaluation: H_d by the FFT convolution, then the field kernel ----
    bool demag_field(const double *m) {
        if (!demag) return true;
        const Conv64 &C = conv;
        const int nrows = ny * nz;
        const size_t smx = sizeof(double2) * 2 * C.px, smy = sizeof(double2) * 2 * C.py;
        x_forward64<<<dim3(nrows, 3), kT, smx, stream>>>(C, m, tier > 0 ? phi : nullptr, X);
        if (C.thin) {
            y_convolve64<<<C.nkx, kT, 3 * smy, stream>>>(C, X);
        } else {
            y_forward64<<<dim3(C.nkx, nz, 3), kT, smy, stream>>>(C, X, Y);
            z_convolve64<<<dim3(C.nkx, C.py), kT, sizeof(double2) * 6 * C.pz, stream>>>(C, Y);
            y_inverse64<<<dim3(C.nkx, nz, 3), kT, smy, stream>>>(C, Y, X);
        }
        x_inverse64<<<dim3(nrows, 3), kT, smx, stream>>>(C, X, hd, mask, tier > 0 ? phi : nullptr);
        // the correction's source weights phi_s are the volume fractions whenever the plan has them
        if (corr_targets > 0)
            demag_correction64<<<std::max(1u, std::min(1024u, (corr_targets + kT - 1) / kT)), kT, 0, stream>>>(
                hd, m, phi, ctidx, csidx, ctensor, ms, n, corr_targets, corr_stencil);
        return !fail("demag kernels", cudaGetLastError());
    }

    Field64 field_base() const {
        Field64 P{};
        P.nx = nx;
        P.ny = ny;
        P.nz = nz;
        P.n = n;
        P.hd = demag ? hd : nullptr;
        P.hex = hex;
        P.heff = heff;
        P.mask = mask;
        P.region = region;
        P.lut = lut;
        P.tier = tier;
        P.phi = (tier > 0) ? phi : nullptr;
        for (int q = 0; q < 6; ++q) {
            P.face[q] = face[q];
            P.delta[q] = delta[q];
        }
        P.phi_floor = phi_floor;
        P.delta_min = delta_min;
        P.exchange = exchange;
        P.per = per;
        P.a_ex = a_ex;
        P.ms = ms;
        P.dx = dx;
        P.dy = dy;
        P.dz = dz;
        P.has_ext = has_ext;
        for (int c = 0; c < 3; ++c) {
            P.hext[c] = hext[c];
            P.u[c] = u[c];
            P.c1[c] = c1[c];
            P.c2[c] = c2[c];
            P.c3[c] = c3[c];
        }
        P.has_uni = has_uni;
        P.ku1 = ku1;
        P.ku2 = ku2;
        P.has_cub = has_cub;
        P.kc1 = kc1;
        P.kc2 = kc2;
        P.kc3 = kc3;
        P.gbar = gamma / (1.0 + alpha * alpha);
        P.alpha = alpha;
        P.prec = prec ? 1.0 : 0.0;
        return P;
    }

    // RHS at m into k (when non-null); with stats the statistics land in dstats[0..7]
    bool eval(const double *m, double *k, bool stats) {
        fields_ok = false;
        if (!demag_field(m)) return false;
        Field64 P = field_base();
        P.m = m;
        P.k = k;
        P.partials = stats ? partials : nullptr;
        const unsigned nb = blocks_for(n);
        field64<<<nb, kT, 0, stream>>>(P);
        if (stats) finalize64<<<1, kT, 0, stream>>>(partials, (int)nb, dstats, 0);
        return !fail("field kernels", cudaGetLastError());
    }

    bool combine(const double *m0, int nk, const int *kidx, const double *coef, const double *kcur, double dt, double *out) {
        Comb64 C{};
        C.n = n;
        C.m0 = m0;
        C.nk = nk;
        for (int t = 0; t < nk; ++t) {
            C.k[t] = kidx[t] < 0 ? kcur : K[kidx[t]];
            C.c[t] = coef[t];
        }
        C.dt = dt;
        C.out = out;
        combine64<<<blocks_for(n), kT, 0, stream>>>(C);
        return !fail("combine", cudaGetLastError());
    }

    bool error_norm(int nk, const int *kidx, const double *coef, double dt) {
        Comb64 C{};
        C.n = n;
        C.nk = nk;
        for (int t = 0; t < nk; ++t) {
            C.k[t] = K[kidx[t]];
            C.c[t] = coef[t];
        }
        C.dt = dt;
        const unsigned nb = blocks_for(n);
        error64<<<nb, kT, 0, stream>>>(C, partials);
        finalize64<<<1, kT, 0, stream>>>(partials, (int)nb, dstats + kStats, 1);
        return !fail("error norm", cudaGetLastError());
    }

    bool read_stats() {
        if (fail("stats copy", cudaMemcpyAsync(hstats, dstats, sizeof(double) * 2 * kStats, cudaMemcpyDeviceToHost, stream)) ||
            fail("stream sync", cudaStreamSynchronize(stream)))
            return false;
        return true;
    }

    void fill_stats(const double *d) {
        const double V = dx * dy * dz;
        fullmag_fdm_step_stats &st = cur_stats;
        st.exchange_energy_joules = exchange ? V * d[0] : 0.0;
        st.demag_energy_joules = demag ? -0.5 * kMu0d * ms * V * d[1] : 0.0;
        st.external_energy_joules = has_ext ? -kMu0d * ms * V * d[2] : 0.0;
        st.anisotropy_energy_joules = has_uni ? -V * d[3] : 0.0;
        st.cubic_energy_joules = has_cub ? V * d[4] : 0.0;
        st.dmi_energy_joules = 0.0;
        st.total_energy_joules = st.exchange_energy_joules + st.demag_energy_joules + st.external_energy_joules +
                                 st.anisotropy_energy_joules + st.cubic_energy_joules;
        st.max_effective_field_amplitude = sqrt(d[5]);
        st.max_demag_field_amplitude = demag ? sqrt(d[6]) : 0.0;
        st.max_rhs_amplitude = sqrt(d[7]);
        st.step = step_count;
        st.time_seconds = time;
    }

    // k1 = f(S[cur]) with the statistics and observables of the committed state
    bool eval_state() {
        if (!eval(S[cur], K[0], true) || !read_stats()) return false;
        memcpy(raw, hstats, sizeof(raw));
        fill_stats(raw);
        k1_valid = true;
        fields_ok = true;
        return true;
    }

    bool poll_hit(fullmag_fdm_interrupt_poll_fn poll, void *user) { return poll && poll(user) != 0; }

    void commit(double dt) {
        cur = 1 - cur;
        step_count += 1;
        time += dt;
        memcpy(raw, hstats, sizeof(raw));
        fill_stats(raw);
        cur_stats.dt_seconds = dt;
        cur_stats.suggested_next_dt = 0.0;
        k1_valid = true;
        fields_ok = true;
    }

    // explicit Runge-Kutta stages from S[cur]: stage s input N(m0 + dt sum_j a_sj k_j),
    // k_s into K[s]; the proposal into S[1-cur]; its derivative into K[kfinal] with stats
    int rk_fixed(double dt, fullmag_fdm_interrupt_poll_fn poll, void *user) {
        const int nxt = 1 - cur;
        if (integrator == FULLMAG_FDM_INTEGRATOR_RK4) {
            const int k0[1] = {0}, k1[1] = {1}, k2[1] = {2}, kall[4] = {0, 1, 2, 3};
            const double h[1] = {0.5}, one[1] = {1.0}, b[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
            if (!combine(S[cur], 1, k0, h, nullptr, dt, A[0]) || !eval(A[0], K[1], false)) return -1;
            if (poll_hit(poll, user)) return 1;
            if (!combine(S[cur], 1, k1, h, nullptr, dt, A[1]) || !eval(A[1], K[2], false)) return -1;
            if (poll_hit(poll, user)) return 1;
            if (!combine(S[cur], 1, k2, one, nullptr, dt, A[0]) || !eval(A[0], K[3], false)) return -1;
            if (poll_hit(poll, user)) return 1;
            if (!combine(S[cur], 4, kall, b, nullptr, dt, S[nxt])) return -1;
        } else {  // Heun
            const int k0[1] = {0}, kb[2] = {0, 1};
            const double one[1] = {1.0}, half[2] = {0.5, 0.5};
            if (!combine(S[cur], 1, k0, one, nullptr, dt, A[0]) || !eval(A[0], K[1], false)) return -1;
            if (poll_hit(poll, user)) return 1;
            if (!combine(S[cur], 2, kb, half, nullptr, dt, S[nxt])) return -1;
        }
        // k1 of the next step (the combination above was the last reader of K[0])
        k1_valid = false;
        if (!eval(S[nxt], K[0], true) || !read_stats()) return -1;
        commit(dt);
        return 0;
    }

    // Dormand-Prince 5(4) or Bogacki-Shampine 3(2) attempt; 1 accepted, 0 rejected, -1 error, 2 interrupted
    int rk_adaptive_attempt(double dt, double &next_dt, fullmag_fdm_interrupt_poll_fn poll, void *user) {
        const int nxt = 1 - cur;
        int kfin;
        if (integrator == FULLMAG_FDM_INTEGRATOR_RK23) {
            static const double a2[1] = {0.5}, a3[1] = {0.75};
            static const double b[3] = {2.0 / 9.0, 1.0 / 3.0, 4.0 / 9.0};
            static const double e[4] = {-5.0 / 72.0, 1.0 / 12.0, 1.0 / 9.0, -1.0 / 8.0};
            const int k0[1] = {0}, k1[1] = {1}, kb[3] = {0, 1, 2}, ke[4] = {0, 1, 2, 3};
            if (!combine(S[cur], 1, k0, a2, nullptr, dt, A[0]) || !eval(A[0], K[1], false)) return -1;
            if (poll_hit(poll, user)) return 2;
            if (!combine(S[cur], 1, k1, a3, nullptr, dt, A[1]) || !eval(A[1], K[2], false)) return -1;
            if (poll_hit(poll, user)) return 2;
            if (!combine(S[cur], 3, kb, b, nullptr, dt, S[nxt]) || !eval(S[nxt], K[3], true)) return -1;
            if (!error_norm(4, ke, e, dt)) return -1;
            kfin = 3;
        } else {
            static const double a21[1] = {1.0 / 5.0};
            static const double a3[2] = {3.0 / 40.0, 9.0 / 40.0};
            static const double a4[3] = {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0};
            static const double a5[4] = {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0};
            static const double a6[5] = {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0};
            static const double b[5] = {35.0 / 384.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0};
            static const double e[6] = {71.0 / 57600.0, -71.0 / 16695.0, 71.0 / 1920.0, -17253.0 / 339200.0, 22.0 / 525.0,
                                        -1.0 / 40.0};
            const int k1[1] = {0}, k2[2] = {0, 1}, k3[3] = {0, 1, 2}, k4[4] = {0, 1, 2, 3}, k5[5] = {0, 1, 2, 3, 4};
            const int kb[5] = {0, 2, 3, 4, 5}, ke[6] = {0, 2, 3, 4, 5, 6};
            if (!combine(S[cur], 1, k1, a21, nullptr, dt, A[0]) || !eval(A[0], K[1], false)) return -1;
            if (poll_hit(poll, user)) return 2;
            if (!combine(S[cur], 2, k2, a3, nullptr, dt, A[1]) || !eval(A[1], K[2], false)) return -1;
            if (poll_hit(poll, user)) return 2;
            if (!combine(S[cur], 3, k3, a4, nullptr, dt, A[0]) || !eval(A[0], K[3], false)) return -1;
            if (poll_hit(poll, user)) return 2;
            if (!combine(S[cur], 4, k4, a5, nullptr, dt, A[1]) || !eval(A[1], K[4], false)) return -1;
            if (poll_hit(poll, user)) return 2;
            if (!combine(S[cur], 5, k5, a6, nullptr, dt, A[0]) || !eval(A[0], K[5], false)) return -1;
            if (poll_hit(poll, user)) return 2;
            if (!combine(S[cur], 5, kb, b, nullptr, dt, S[nxt]) || !eval(S[nxt], K[6], true)) return -1;
            if (!error_norm(6, ke, e, dt)) return -1;
            kfin = 6;
        }
        if (!read_stats()) return -1;
        const double er = sqrt(hstats[kStats + 8]);
        const double ex = integrator == FULLMAG_FDM_INTEGRATOR_RK23 ? 1.0 / 3.0 : 0.2;
        if (er <= max_error || dt <= dt_min) {
            double dtn = dt_max;
            if (er > 0.0) dtn = std::min(std::max(headroom * dt * pow(max_error / er, ex), dt_min), dt_max);
            if (fail("fsal copy", cudaMemcpyAsync(K[0], K[kfin], sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, stream)))
                return -1;
            commit(dt);
            cur_stats.suggested_next_dt = dtn;
            next_dt = dtn;
            return 1;
        }
        next_dt = std::min(std::max(headroom * dt * pow(max_error / er, ex), dt_min), dt_max);
        return 0;
    }

    // Adams-Bashforth-Moulton 3 as in the FP32 path: Heun steps build the history
    int abm3(double dt, fullmag_fdm_interrupt_poll_fn poll, void *user) {
        if (abm_last_dt > 0.0 && std::fabs(dt - abm_last_dt) / abm_last_dt > 0.1) abm_startup = 0;
        const int nxt = 1 - cur;
        if (abm_startup < 3) {
            const int saved = integrator;
            integrator = FULLMAG_FDM_INTEGRATOR_HEUN;
            const int rc = rk_fixed(dt, poll, user);
            integrator = saved;
            if (rc != 0) return rc;
            const int slot = abm_hist[2];
            abm_hist[2] = abm_hist[1];
            abm_hist[1] = abm_hist[0];
            abm_hist[0] = slot;
            if (fail("history copy", cudaMemcpyAsync(K[slot], K[0], sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, stream)))
                return -1;
            abm_startup += 1;
        } else {
            const int kp[3] = {abm_hist[0], abm_hist[1], abm_hist[2]};
            const double cp[3] = {23.0 / 12.0, -16.0 / 12.0, 5.0 / 12.0};
            if (!combine(S[cur], 3, kp, cp, nullptr, dt, A[0]) || !eval(A[0], K[abm_kf], false)) return -1;
            if (poll_hit(poll, user)) return 1;
            const int kc[3] = {abm_kf, abm_hist[0], abm_hist[1]};
            const double cc[3] = {5.0 / 12.0, 8.0 / 12.0, -1.0 / 12.0};
            if (!combine(S[cur], 3, kc, cc, nullptr, dt, S[nxt])) return -1;
            if (poll_hit(poll, user)) return 1;
            if (!eval(S[nxt], K[0], true) || !read_stats()) return -1;
            const int freed = abm_hist[2];
            abm_hist[2] = abm_hist[1];
            abm_hist[1] = abm_hist[0];
            abm_hist[0] = abm_kf;
            abm_kf = freed;
            commit(dt);
        }
        abm_last_dt = dt;
        return 0;
    }
};

bool Fp64Engine::setup(const fullmag_fdm_plan_desc *plan) {
    nx = (int)plan->grid.nx;
    ny = (int)plan->grid.ny;
    nz = (int)plan->grid.nz;
    n = (long long)nx * ny * nz;
    dx = plan->grid.dx;
    dy = plan->grid.dy;
    dz = plan->grid.dz;
    ms = plan->material.saturation_magnetisation;
    a_ex = plan->material.exchange_stiffness;
    alpha = plan->material.damping;
    gamma = plan->material.gyromagnetic_ratio;
    integrator = plan->integrator;
    exchange = plan->enable_exchange != 0;
    demag = plan->enable_demag != 0;
    prec = plan->disable_precession == 0;
    has_ext = plan->has_external_field != 0;
    for (int c = 0; c < 3; ++c) hext[c] = has_ext ? plan->external_field_am[c] : 0.0;
    max_error = plan->adaptive_max_error > 0 ? plan->adaptive_max_error : 1e-5;
    dt_min = plan->adaptive_dt_min > 0 ? plan->adaptive_dt_min : 1e-18;
    dt_max = plan->adaptive_dt_max > 0 ? plan->adaptive_dt_max : 1e-10;
    headroom = plan->adaptive_headroom > 0 ? plan->adaptive_headroom : 0.8;

    if (n == 0) return err = "grid has zero cells", false;
    if (plan->initial_magnetization_xyz == nullptr || plan->initial_magnetization_len != 3 * (uint64_t)n)
        return err = "initial_magnetization_len mismatch: expected " + std::to_string(3 * (uint64_t)n) + ", got " +
                     std::to_string(plan->initial_magnetization_len),
               false;
    if (plan->region_mask && plan->region_mask_len != (uint64_t)n)
        return err = "region_mask_len mismatch: expected " + std::to_string(n) + ", got " + std::to_string(plan->region_mask_len),
               false;
    if (plan->active_mask && plan->active_mask_len != (uint64_t)n)
        return err = "active_mask_len mismatch: expected " + std::to_string(n) + ", got " + std::to_string(plan->active_mask_len),
               false;
    if (!(dx > 0 && dy > 0 && dz > 0)) return err = "cell sizes must be positive", false;
    if (!(ms > 0)) return err = "saturation_magnetisation must be positive", false;
    if (integrator != FULLMAG_FDM_INTEGRATOR_HEUN && integrator != FULLMAG_FDM_INTEGRATOR_RK4 &&
        integrator != FULLMAG_FDM_INTEGRATOR_DP45 && integrator != FULLMAG_FDM_INTEGRATOR_RK23 &&
        integrator != FULLMAG_FDM_INTEGRATOR_ABM3)
        return err = "unsupported integrator", false;
    struct Feat {
        bool on;
        const char *what;
    };
    const Feat rejected[] = {
        {plan->has_interfacial_dmi != 0 || plan->has_bulk_dmi != 0, "DMI"},
        {plan->has_magnetoelastic != 0, "magnetoelastic coupling"},
        {plan->temperature > 0.0, "thermal noise"},
        {plan->current_density_x != 0.0 || plan->current_density_y != 0.0 || plan->current_density_z != 0.0,
         "spin-transfer torque"},
        {plan->has_sot != 0, "spin-orbit torque"},
        {plan->has_oersted_cylinder != 0, "Oersted field"},
        {plan->ku1_field || plan->ku2_field || plan->kc1_field || plan->kc2_field || plan->kc3_field,
         "per-cell anisotropy maps"},
    };
    for (const Feat &f : rejected)
        if (f.on) return err = std::string(f.what) + " is not available with double-precision state (use SINGLE)", false;

    has_uni = plan->has_uniaxial_anisotropy != 0;
    ku1 = plan->uniaxial_anisotropy_constant;
    ku2 = plan->uniaxial_anisotropy_k2;
    has_cub = plan->has_cubic_anisotropy != 0;
    kc1 = plan->cubic_Kc1;
    kc2 = plan->cubic_Kc2;
    kc3 = plan->cubic_Kc3;
    if (has_uni) {
        const double *a = plan->anisotropy_axis;
        const double nn = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        if (!(nn > 0)) return err = "anisotropy_axis must be non-zero", false;
        for (int c = 0; c < 3; ++c) u[c] = a[c] / nn;
    }
    if (has_cub) {
        const double *a = plan->cubic_axis1, *b = plan->cubic_axis2;
        const double na = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]), nb = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        if (!(na > 0 && nb > 0)) return err = "cubic axes must be non-zero", false;
        for (int c = 0; c < 3; ++c) {
            c1[c] = a[c] / na;
            c2[c] = b[c] / nb;
        }
        c3[0] = c1[1] * c2[2] - c1[2] * c2[1];
        c3[1] = c1[2] * c2[0] - c1[0] * c2[2];
        c3[2] = c1[0] * c2[1] - c1[1] * c2[0];
    }

    // boundary tiers (exchange_fp64.cu:162-231): T0 needs the volume and face-link
    // fractions, T1 the volume fractions and boundary distances; without them the tier
    // falls back to the binary-mask exchange, as the reference's dispatch does
    tier = 0;
    if (plan->boundary_correction != FULLMAG_FDM_BOUNDARY_NONE && plan->volume_fraction) {
        if (plan->volume_fraction_len != (uint64_t)n)
            return err = "volume_fraction_len mismatch: expected " + std::to_string(n), false;
        if (plan->boundary_correction == FULLMAG_FDM_BOUNDARY_VOLUME && plan->face_link_xp && plan->face_link_xm &&
            plan->face_link_yp && plan->face_link_ym && plan->face_link_zp && plan->face_link_zm)
            tier = 1;
        else if (plan->boundary_correction == FULLMAG_FDM_BOUNDARY_FULL && plan->delta_xp && plan->delta_xm &&
                 plan->delta_yp && plan->delta_ym && plan->delta_zp && plan->delta_zm)
            tier = 2;
    }
    phi_floor = plan->boundary_phi_floor;
    delta_min = plan->boundary_delta_min;
    if (per && (tier > 0 || (plan->has_demag_boundary_corr && plan->demag_corr_target_count > 0)))
        return err = "boundary correction is not available with periodic boundaries", false;
    if (plan->has_demag_boundary_corr && plan->demag_corr_target_count > 0) {
        if (!plan->demag_corr_target_idx || !plan->demag_corr_source_idx || !plan->demag_corr_tensor ||
            plan->demag_corr_stencil_size == 0)
            return err = "demag boundary correction arrays are incomplete", false;
        corr_targets = plan->demag_corr_target_count;
        corr_stencil = plan->demag_corr_stencil_size;
        const size_t ns = (size_t)corr_targets * corr_stencil;
        for (uint32_t t = 0; t < corr_targets; ++t)
            if (plan->demag_corr_target_idx[t] >= (int64_t)n) return err = "demag correction target index out of range", false;
        for (size_t s = 0; s < ns; ++s)
            if (plan->demag_corr_source_idx[s] >= (int64_t)n) return err = "demag correction source index out of range", false;
    }

    // ---- device ----
    if (fail("cudaGetDevice", cudaGetDevice(&device))) return false;
    if (fail("cudaStreamCreate", cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking))) return false;
    const size_t v3 = 3 * (size_t)n;
    for (int s = 0; s < 2; ++s)
        if (!alloc(S[s], v3) || !alloc(A[s], v3)) return false;
    for (int s = 0; s < 7; ++s)
        if (!alloc(K[s], v3)) return false;
    if (!alloc(hex, v3) || !alloc(hd, v3) || !alloc(heff, v3) || !alloc(staging, v3) || !alloc(partials, kRedBlocks * kStats) ||
        !alloc(dstats, 2 * kStats))
        return false;
    if (fail("cudaMemsetAsync", cudaMemsetAsync(hd, 0, sizeof(double) * v3, stream))) return false;
    if (fail("cudaMallocHost", cudaMallocHost((void **)&hstats, sizeof(double) * 2 * kStats))) return false;
    if (plan->active_mask) {
        has_mask = true;
        mask_host.assign(plan->active_mask, plan->active_mask + n);
        if (!put(mask, plan->active_mask, (size_t)n)) return false;
    }
    if (plan->region_mask) {
        std::vector<uint8_t> r((size_t)n);
        for (long long i = 0; i < n; ++i) {
            if (plan->region_mask[i] >= FULLMAG_FDM_MAX_EXCHANGE_REGIONS)
                return err = "region_mask ids must be below " + std::to_string(FULLMAG_FDM_MAX_EXCHANGE_REGIONS), false;
            r[i] = (uint8_t)plan->region_mask[i];
        }
        // the caller's table when it has 256 x 256 entries, else A on the diagonal (api.cpp:405-420)
        const size_t R = FULLMAG_FDM_MAX_EXCHANGE_REGIONS, R2 = R * R;
        std::vector<double> table(R2, 0.0);
        if (plan->exchange_lut && plan->exchange_lut_len == R2) std::copy(plan->exchange_lut, plan->exchange_lut + R2, table.begin());
        else
            for (size_t q = 0; q < R; ++q) table[q * R + q] = a_ex;
        if (!put(region, r.data(), r.size()) || !put(lut, table.data(), R2)) return false;
    }
    if (tier > 0 || corr_targets > 0) {
        if (plan->volume_fraction && plan->volume_fraction_len == (uint64_t)n) {
            if (!put(phi, plan->volume_fraction, (size_t)n)) return false;
        }
    }
    if (tier == 1) {
        const double *f[6] = {plan->face_link_xp, plan->face_link_xm, plan->face_link_yp,
                              plan->face_link_ym, plan->face_link_zp, plan->face_link_zm};
        for (int q = 0; q < 6; ++q)
            if (!put(face[q], f[q], (size_t)n)) return false;
    } else if (tier == 2) {
        const double *d[6] = {plan->delta_xp, plan->delta_xm, plan->delta_yp, plan->delta_ym, plan->delta_zp, plan->delta_zm};
        for (int q = 0; q < 6; ++q)
            if (!put(delta[q], d[q], (size_t)n)) return false;
    }
    if (corr_targets > 0) {
        const size_t ns = (size_t)corr_targets * corr_stencil;
        if (!put(ctidx, plan->demag_corr_target_idx, corr_targets) || !put(csidx, plan->demag_corr_source_idx, ns) ||
            !put(ctensor, plan->demag_corr_tensor, 6 * ns))
            return false;
    }

    // ---- demag: padded geometry P = 2n per axis (thin film: 2-D when nz == 1) ----
    if (demag) {
        Conv64 &C = conv;
        C.nx = nx;
        C.ny = ny;
        C.nz = nz;
        C.n = n;
        // periodic axes (fdm_fft.rs:140-160): unpadded, and the backend builds the tensor
        C.px = (per & 1) ? nx : 2 * nx;
        C.py = (per & 2) ? ny : 2 * ny;
        if (per && plan->demag_kernel_spectrum_len != 0)
            return err = "periodic boundaries: the backend builds the image-sum demag tensor, the plan must carry no spectra",
                   false;
        const uint64_t len3 = 2ull * (uint64_t)(2 * nx) * (2 * ny) * (2 * nz);
        const uint64_t len2 = 2ull * (uint64_t)(2 * nx) * (2 * ny);
        const bool given = plan->demag_kernel_spectrum_len != 0;
        bool thin = false;
        if (!given) {
            thin = nz == 1;
        } else {
            if (!plan->demag_kernel_xx_spectrum || !plan->demag_kernel_yy_spectrum || !plan->demag_kernel_zz_spectrum ||
                !plan->demag_kernel_xy_spectrum || !plan->demag_kernel_xz_spectrum || !plan->demag_kernel_yz_spectrum)
                return err = "demag kernel spectra pointers must all be present when demag_kernel_spectrum_len is set", false;
            if (nz == 1 && plan->demag_kernel_spectrum_len == len2) thin = true;
            else if (plan->demag_kernel_spectrum_len != len3)
                return err = "demag_kernel_spectrum_len mismatch: expected " + std::to_string(len3) + " (3D)" +
                             (nz == 1 ? " or " + std::to_string(len2) + " (thin-film 2D)" : std::string()) + ", got " +
                             std::to_string(plan->demag_kernel_spectrum_len),
                       false;
        }
        C.thin = thin;
        C.pz = thin ? 1 : (per & 4) ? nz : 2 * nz;
        C.nkx = C.px / 2 + 1;
        C.nky = C.py / 2 + 1;
        C.nkz = C.pz / 2 + 1;
        std::vector<double2> tw;
        std::vector<size_t> off;
        if (!make_plan64(C.px, tw, off, C.plx) || !make_plan64(C.py, tw, off, C.ply) ||
            (!thin && !make_plan64(C.pz, tw, off, C.plz)))
            return err = "FFT length has too many factors", false;
        if (!put(twid, tw.data(), tw.size())) return false;
        C.plx.tw = twid + off[0];
        C.ply.tw = twid + off[1];
        if (!thin) C.plz.tw = twid + off[2];
        const int ncomp = thin ? 4 : 6;
        const size_t kper = per ? (size_t)C.pz * C.py * C.nkx : (size_t)C.nkz * C.nky * C.nkx;
        if (per ? !alloc(kernc, ncomp * kper) : !alloc(kern, ncomp * kper)) return false;
        if (!alloc(X, 3 * (size_t)nz * ny * C.nkx)) return false;
        if (!thin && !alloc(Y, 3 * (size_t)nz * C.py * C.nkx)) return false;
        const size_t smz = sizeof(double2) * 6 * std::max(C.pz, thin ? C.py : 1);
        const size_t smx = sizeof(double2) * 2 * std::max(C.px, C.py);
        if (smz > 227 * 1024 || smx > 227 * 1024) return err = "grid too large for the double-precision FFT lines", false;
        const void *big[] = {(const void *)z_convolve64, (const void *)y_convolve64, (const void *)x_forward64,
                             (const void *)x_inverse64, (const void *)y_forward64, (const void *)y_inverse64};
        for (const void *f : big)
            if (fail("cudaFuncSetAttribute", cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024)))
                return false;
        if (given) {
            const double *src[6] = {plan->demag_kernel_xx_spectrum, plan->demag_kernel_yy_spectrum, plan->demag_kernel_zz_spectrum,
                                    plan->demag_kernel_xy_spectrum, plan->demag_kernel_xz_spectrum, plan->demag_kernel_yz_spectrum};
            const double scale = ms / ((double)C.px * C.py * C.pz);
            std::vector<double> h(ncomp * kper);
            for (int c = 0; c < ncomp; ++c)
                for (int kz = 0; kz < C.nkz; ++kz)
                    for (int ky = 0; ky < C.nky; ++ky)
                        for (int kx = 0; kx < C.nkx; ++kx) {
                            const size_t s = (size_t)kx + (size_t)C.px * (ky + (size_t)C.py * kz);
                            h[(size_t)c * kper + ((size_t)kz * C.nky + ky) * C.nkx + kx] = src[c][2 * s] * scale;
                        }
            if (fail("cudaMemcpy(kernel)", cudaMemcpyAsync(kern, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, stream)) ||
                fail("kernel sync", cudaStreamSynchronize(stream)))
                return false;
        } else {
            Grid g{};
            g.nx = nx;
            g.ny = ny;
            g.nz = nz;
            g.n = n;
            g.px = C.px;
            g.py = C.py;
            g.pz = C.pz;
            g.half = C.px / 2;
            g.nkx = C.nkx;
            g.nky = C.nky;
            g.nkz = C.nkz;
            g.thin = thin;
            g.per = per;
            if (per ? !newell_periodic_spectrum_gpu(g, dx, dy, dz, ms, images, nullptr, kernc, stream, err)
                    : !newell_spectrum_gpu64(g, dx, dy, dz, ms, kern, stream, err))
                return false;
        }
        C.kern = kern;
        C.kernc = kernc;
    }
    return true;
}

bool Fp64Engine::upload(const double *m_xyz) {
    if (fail("cudaMemcpy(state)", cudaMemcpyAsync(staging, m_xyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, stream)))
        return false;
    aos_to_soa64<<<blocks_for(n), kT, 0, stream>>>(staging, S[cur], mask, tier > 0 ? phi : nullptr, n);
    if (fail("upload convert", cudaGetLastError())) return false;
    k1_valid = false;
    abm_startup = 0;
    abm_last_dt = 0.0;
    return eval_state();
}

bool fp64_refresh(Fp64Engine *e, std::string &err);

Fp64Engine *fp64_create(const fullmag_fdm_plan_desc *plan, std::string &err, int periodic, const uint32_t *images) {
    Fp64Engine *e = new (std::nothrow) Fp64Engine();
    if (!e) {
        err = "out of host memory";
        return nullptr;
    }
    e->per = periodic;
    if (images)
        for (int a = 0; a < 3; ++a) e->images[a] = images[a];
    if (!e->setup(plan) || !e->upload(plan->initial_magnetization_xyz)) {
        err = e->err;
        delete e;
        return nullptr;
    }
    e->cur_stats.step = 0;
    e->cur_stats.time_seconds = 0.0;
    return e;
}

void fp64_destroy(Fp64Engine *e) { delete e; }

int fp64_step(Fp64Engine *e, double dt, fullmag_fdm_step_stats *out, fullmag_fdm_interrupt_poll_fn poll, void *user,
              std::string &err) {
    const auto t0 = std::chrono::steady_clock::now();
    e->err.clear();
    int rc = 0;
    if (!e->k1_valid && !e->eval_state()) rc = -1;
    else if (e->poll_hit(poll, user)) rc = 1;
    else if (e->integrator == FULLMAG_FDM_INTEGRATOR_DP45 || e->integrator == FULLMAG_FDM_INTEGRATOR_RK23) {
        for (;;) {
            double next = dt;
            const int a = e->rk_adaptive_attempt(dt, next, poll, user);
            if (a < 0) {
                rc = -1;
                break;
            }
            if (a == 2) {
                rc = 1;
                break;
            }
            if (a == 1) break;
            dt = next;
        }
    } else if (e->integrator == FULLMAG_FDM_INTEGRATOR_ABM3) {
        rc = e->abm3(dt, poll, user);
    } else {
        rc = e->rk_fixed(dt, poll, user);
    }
    err = e->err;
    if (rc < 0) return FULLMAG_FDM_ERR_CUDA;
    *out = e->cur_stats;
    if (rc == 1) {
        out->dt_seconds = 0.0;
        out->wall_time_ns = 0;
        err = "interrupted";
        return FULLMAG_FDM_ERR_INTERRUPTED;
    }
    out->wall_time_ns =
        (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
    e->cur_stats.wall_time_ns = out->wall_time_ns;
    return FULLMAG_FDM_OK;
}

bool fp64_download(Fp64Engine *e, int obs, double *out, std::string &err) {
    const long long n = e->n;
    if (obs == FULLMAG_FDM_OBSERVABLE_H_EXT) {
        for (long long i = 0; i < n; ++i) {
            const bool act = !e->has_mask || e->mask_host[i] != 0;
            for (int c = 0; c < 3; ++c) out[3 * i + c] = (e->has_ext && act) ? e->hext[c] : 0.0;
        }
        return true;
    }
    const double *src = nullptr;
    switch (obs) {
        case FULLMAG_FDM_OBSERVABLE_M: src = e->S[e->cur]; break;
        case FULLMAG_FDM_OBSERVABLE_H_EX: src = e->hex; break;
        case FULLMAG_FDM_OBSERVABLE_H_DEMAG: src = e->hd; break;
        case FULLMAG_FDM_OBSERVABLE_H_EFF: src = e->heff; break;
        default: err = "unknown observable " + std::to_string(obs); return false;
    }
    // the field buffers hold the last evaluation: after an interrupted step or a rejected
    // attempt that is not the committed state, which is evaluated again
    if (obs != FULLMAG_FDM_OBSERVABLE_M && !e->fields_ok && !fp64_refresh(e, err)) return false;
    soa_to_aos64<<<blocks_for(n), kT, 0, e->stream>>>(src, e->staging, n);
    if (e->fail("download convert", cudaGetLastError()) ||
        e->fail("cudaMemcpy(field)", cudaMemcpyAsync(out, e->staging, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->stream)) ||
        e->fail("download sync", cudaStreamSynchronize(e->stream))) {
        err = e->err;
        return false;
    }
    return true;
}

bool fp64_upload(Fp64Engine *e, const double *m_xyz, std::string &err) {
    const bool ok = e->upload(m_xyz);
    if (!ok) err = e->err;
    return ok;
}

bool fp64_refresh(Fp64Engine *e, std::string &err) {
    const fullmag_fdm_step_stats keep = e->cur_stats;
    const bool ok = e->eval_state();
    if (!ok) {
        err = e->err;
        return false;
    }
    e->cur_stats.dt_seconds = keep.dt_seconds;
    e->cur_stats.suggested_next_dt = keep.suggested_next_dt;
    e->cur_stats.wall_time_ns = keep.wall_time_ns;
    return true;
}

void fp64_stats(const Fp64Engine *e, fullmag_fdm_step_stats *out) { *out = e->cur_stats; }

void fp64_grid(const Fp64Engine *e, int &nx, int &ny, int &nz) {
    nx = e->nx;
    ny = e->ny;
    nz = e->nz;
}

int fp64_device(const Fp64Engine *e) { return e->device; }

void fp64_fft_shape(const Fp64Engine *e, uint32_t &px, uint32_t &py, uint32_t &pz) {
    px = e->demag ? (uint32_t)e->conv.px : 0;
    py = e->demag ? (uint32_t)e->conv.py : 0;
    pz = e->demag ? (uint32_t)e->conv.pz : 0;
}

}  // namespace fm
