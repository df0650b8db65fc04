// newell.cu -- FP64 Newell demagnetisation tensor and its spectrum, built on the GPU.
//
// Follows the algorithm of crates/fullmag-fdm-demag/src/newell.rs:
//   f, g base functions with log1p/atan forms            newell.rs:21-131
//   Kahan-Neumaier 27-point second difference / (4 pi V) newell.rs:133-210
//   point-dipole asymptotics beyond 40 cells             newell.rs:212-231, 356-373
//   octant placement with even/odd parity                newell.rs:393-425
// and the spectrum of crates/fullmag-engine/src/fdm_fft.rs:334-437 (2-D thin-film
// variant: the z = 0 plane of the nz = 1 tensor).  The reference's CUDA version
// (native/backends/fdm/src/newell_gpu_fp64.cu:384-484) computed the tensor and then
// discarded it; here it becomes the engine's kernel.
//
// Because each placed component is even or odd along every axis, its DFT is real
// and separable: along an even axis sum_i w_i N(i) cos(2 pi k i / p) with w_0 = 1,
// w_i = 2; along an odd axis -i * sum_i 2 N(i) sin(2 pi k i / p).  Two odd axes give
// the overall factor -1 of the off-diagonal components.  Evaluating these direct
// real transforms in FP64 for the octant k in [0, p/2] yields exactly the stored
// kernel, with no padded complex array and no FP64 FFT.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "engine.h"
#include "fp64.h"

namespace fm {

namespace {

constexpr int kAsym = 40;

__device__ double newell_f(double x, double y, double z) {
    const double x2 = x * x, y2 = y * y, z2 = z * z;
    const double r2 = x2 + y2 + z2;
    if (r2 < 1e-300) return 0.0;
    const double r = sqrt(r2);
    double acc = (2.0 * x2 - y2 - z2) * r / 6.0;
    const double sxz = x2 + z2;
    if (sxz > 1e-300) {
        const double t = 2.0 * y * (y + r) / sxz;
        if (t > -1.0) acc += y * (z2 - x2) / 4.0 * log1p(t);
    }
    const double sxy = x2 + y2;
    if (sxy > 1e-300) {
        const double t = 2.0 * z * (z + r) / sxy;
        if (t > -1.0) acc += z * (y2 - x2) / 4.0 * log1p(t);
    }
    if (fabs(x) > 1e-300) acc -= x * y * z * atan(y * z / (x * r));
    return acc;
}

__device__ double newell_g(double x, double y, double z) {
    const double x2 = x * x, y2 = y * y, z2 = z * z;
    const double r2 = x2 + y2 + z2;
    if (r2 < 1e-300) return 0.0;
    const double r = sqrt(r2);
    double acc = -x * y * r / 3.0;
    const double sxy = x2 + y2;
    if (sxy > 1e-300) {
        const double t = 2.0 * z * (z + r) / sxy;
        if (t > -1.0) acc += x * y * z * log1p(t) / 2.0;
    }
    const double syz = y2 + z2;
    if (syz > 1e-300) {
        const double t = 2.0 * x * (x + r) / syz;
        if (t > -1.0) acc += y * (3.0 * z2 - y2) * log1p(t) / 12.0;
    }
    const double sxz = x2 + z2;
    if (sxz > 1e-300) {
        const double t = 2.0 * y * (y + r) / sxz;
        if (t > -1.0) acc += x * (3.0 * z2 - x2) * log1p(t) / 12.0;
    }
    if (fabs(z) > 1e-300) acc -= z2 * z / 6.0 * atan(x * y / (z * r));
    if (fabs(y) > 1e-300) acc -= y2 * z / 2.0 * atan(x * z / (y * r));
    if (fabs(x) > 1e-300) acc -= x2 * z / 2.0 * atan(y * z / (x * r));
    return acc;
}

// T[f][c][b][a]: f in {fxx, fyy, fzz, gxy, gxz, gyz} at signed offsets (a-1, b-1, c-1) cells.
__global__ void fg_table_kernel(double *T, int sx, int sy, int sz, double dx, double dy, double dz) {
    const long long len = (long long)sx * sy * sz;
    for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < len; id += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(id % sx);
        const int b = (int)((id / sx) % sy);
        const int c = (int)(id / ((long long)sx * sy));
        const double x = (a - 1) * dx, y = (b - 1) * dy, z = (c - 1) * dz;
        T[0 * len + id] = newell_f(x, y, z);
        T[1 * len + id] = newell_f(y, x, z);
        T[2 * len + id] = newell_f(z, y, x);
        T[3 * len + id] = newell_g(x, y, z);
        T[4 * len + id] = newell_g(x, z, y);
        T[5 * len + id] = newell_g(y, z, x);
    }
}

__device__ double stencil27(const double *t, int i, int j, int k, int sx, int sy, double inv4piv) {
    double s = 0.0, comp = 0.0;
    for (int dc = -1; dc <= 1; ++dc)
        for (int db = -1; db <= 1; ++db)
            for (int da = -1; da <= 1; ++da) {
                const double w = (da == 0 ? 2.0 : -1.0) * (db == 0 ? 2.0 : -1.0) * (dc == 0 ? 2.0 : -1.0);
                const double v = w * t[(long long)(k + 1 + dc) * sy * sx + (long long)(j + 1 + db) * sx + (i + 1 + da)];
                const double u = s + v;
                if (fabs(s) >= fabs(v)) comp += (s - u) + v;
                else comp += (v - u) + s;
                s = u;
            }
    return (s + comp) * inv4piv;
}

__device__ double asym_diag(double x, double y, double z, double vol) {
    const double r2 = x * x + y * y + z * z, r = sqrt(r2), r3 = r2 * r;
    return (1.0 / r3 - 3.0 * x * x / (r3 * r2)) / (4.0 * M_PI) * vol;
}
__device__ double asym_off(double x, double y, double z, double vol) {
    const double r2 = x * x + y * y + z * z, r = sqrt(r2), r5 = r2 * r2 * r;
    return -3.0 * x * y / (4.0 * M_PI * r5) * vol;
}

// First-octant tensor R[c][k][j][i], i < nx, j < ny, k < nz.
__global__ void tensor_kernel(double *R, const double *T, int nx, int ny, int nz, int sx, int sy, int sz, double dx,
                              double dy, double dz) {
    const long long n = (long long)nx * ny * nz;
    const long long tl = (long long)sx * sy * sz;
    const double vol = dx * dy * dz;
    const double inv = 1.0 / (4.0 * M_PI * vol);
    for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < n; id += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(id % nx);
        const int j = (int)((id / nx) % ny);
        const int k = (int)(id / ((long long)nx * ny));
        const long long d2 = (long long)i * i + (long long)j * j + (long long)k * k;
        double v[6];
        if (i >= kAsym || j >= kAsym || k >= kAsym || d2 >= (long long)kAsym * kAsym) {
            const double x = i * dx, y = j * dy, z = k * dz;
            v[0] = asym_diag(x, y, z, vol);
            v[1] = asym_diag(y, x, z, vol);
            v[2] = asym_diag(z, y, x, vol);
            v[3] = asym_off(x, y, z, vol);
            v[4] = asym_off(x, z, y, vol);
            v[5] = asym_off(y, z, x, vol);
        } else {
#pragma unroll 1
            for (int c = 0; c < 6; ++c) v[c] = stencil27(T + c * tl, i, j, k, sx, sy, inv);
        }
        for (int c = 0; c < 6; ++c) R[c * n + id] = v[c];
    }
}

// Direct real transform along one axis of layout [comp][outer][axis][inner]:
// out[c][o][kk][b] = sum_i w_i trig(kk*i) in[c][o][i][b]; the odd flag of each
// component selects sine (i >= 1) instead of cosine.  tw holds cos/sin of 2 pi e / p.
__global__ void axis_transform_kernel(const double *__restrict__ in, double *__restrict__ out, int ncomp, int outer,
                                      int nin, int nout, int inner, int p, const double2 *__restrict__ tw,
                                      unsigned odd_mask) {
    const long long per_out = (long long)outer * nout * inner;
    const long long total = per_out * ncomp;
    for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < total; id += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(id / per_out);
        long long r = id - c * per_out;
        const int b = (int)(r % inner);
        r /= inner;
        const int kk = (int)(r % nout);
        const int o = (int)(r / nout);
        const double *src = in + (((long long)c * outer + o) * nin) * inner + b;
        const bool odd = (odd_mask >> c) & 1u;
        double acc = odd ? 0.0 : src[0];
        int e = 0;  // (kk * i) mod p, advanced incrementally
        for (int i = 1; i < nin; ++i) {
            e += kk;
            if (e >= p) e -= p;
            const double2 w = tw[e];
            acc += 2.0 * (odd ? w.y : w.x) * src[(long long)i * inner];
        }
        out[(((long long)c * outer + o) * nout + kk) * inner + b] = acc;
    }
}

template <typename T>
__global__ void to_float_kernel(const double *__restrict__ in, T *__restrict__ out, long long per, int ncomp,
                                double scale, unsigned neg_mask) {
    const long long total = per * ncomp;
    for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < total; id += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(id / per);
        const double s = ((neg_mask >> c) & 1u) ? -scale : scale;
        out[id] = (T)(in[id] * s);
    }
}

unsigned grid_for(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152LL * 64); }

}  // namespace

static bool ck(cudaError_t e, const char *what, std::string &err) {
    if (e == cudaSuccess) return true;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

// Builds the octant kernel (layout of engine.h) scaled by ms / P into `kern` (FP32) or
// `kern64` (FP64, for the double-precision state path); exactly one of them is non-null.
static bool newell_build(const Grid &g, double dx, double dy, double dz, double ms, float *kern, double *kern64,
                         cudaStream_t s, std::string &err) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int sx = std::min(nx, kAsym) + 2, sy = std::min(ny, kAsym) + 2, sz = std::min(nz, kAsym) + 2;
    const long long tl = (long long)sx * sy * sz;
    const long long n = (long long)nx * ny * nz;
    const int ncomp = g.thin ? 4 : 6;
    // parity bits per component (xx yy zz xy xz yz)
    const unsigned oddx = (1u << 3) | (1u << 4), oddy = (1u << 3) | (1u << 5), oddz = (1u << 4) | (1u << 5);
    const unsigned neg = (1u << 3) | (1u << 4) | (1u << 5);

    std::vector<double2> tw;
    std::vector<size_t> off;
    for (int p : {g.px, g.py, g.pz}) {
        off.push_back(tw.size());
        for (int e = 0; e < p; ++e) {
            const double a = 2.0 * M_PI * (double)e / (double)p;
            tw.push_back(make_double2(cos(a), sin(a)));
        }
    }
    const long long sizeA = 6LL * nz * ny * g.nkx;
    const long long sizeB = 6LL * nz * g.nky * g.nkx;
    const long long sizeC = 6LL * g.nkz * g.nky * g.nkx;
    double *T = nullptr, *R = nullptr, *Ab = nullptr, *Bb = nullptr, *Cb = nullptr;
    double2 *dtw = nullptr;
    bool ok = ck(cudaMalloc(&T, sizeof(double) * 6 * tl), "cudaMalloc(newell table)", err) &&
              ck(cudaMalloc(&R, sizeof(double) * 6 * n), "cudaMalloc(newell tensor)", err) &&
              ck(cudaMalloc(&Ab, sizeof(double) * sizeA), "cudaMalloc(newell x)", err) &&
              ck(cudaMalloc(&Bb, sizeof(double) * sizeB), "cudaMalloc(newell y)", err) &&
              ck(cudaMalloc(&Cb, sizeof(double) * sizeC), "cudaMalloc(newell z)", err) &&
              ck(cudaMalloc(&dtw, sizeof(double2) * tw.size()), "cudaMalloc(newell twiddles)", err);
    if (ok) ok = ck(cudaMemcpyAsync(dtw, tw.data(), sizeof(double2) * tw.size(), cudaMemcpyHostToDevice, s), "twiddle copy", err);
    if (ok) {
        fg_table_kernel<<<grid_for(tl), 256, 0, s>>>(T, sx, sy, sz, dx, dy, dz);
        tensor_kernel<<<grid_for(n), 256, 0, s>>>(R, T, nx, ny, nz, sx, sy, sz, dx, dy, dz);
        // x: [c][(k,j)][i] -> [c][(k,j)][kx]
        axis_transform_kernel<<<grid_for(sizeA), 256, 0, s>>>(R, Ab, 6, nz * ny, nx, g.nkx, 1, g.px, dtw + off[0], oddx);
        // y: [c][k][j][kx] -> [c][k][ky][kx]
        axis_transform_kernel<<<grid_for(sizeB), 256, 0, s>>>(Ab, Bb, 6, nz, ny, g.nky, g.nkx, g.py, dtw + off[1], oddy);
        if (g.thin) {
            // thin film: the k = 0 plane of (xx, yy, zz, xy); P = px * py
            const long long per = (long long)g.nky * g.nkx;
            const double scale = ms / ((double)g.px * g.py);
            // components 0..3 of Bb are contiguous blocks of nz*nky*nkx = per (nz == 1)
            if (kern64) to_float_kernel<<<grid_for(per * 4), 256, 0, s>>>(Bb, kern64, per, 4, scale, 1u << 3);
            else to_float_kernel<<<grid_for(per * 4), 256, 0, s>>>(Bb, kern, per, 4, scale, 1u << 3);
        } else {
            // z: [c][k][(ky,kx)] -> [c][kz][(ky,kx)]
            axis_transform_kernel<<<grid_for(sizeC), 256, 0, s>>>(Bb, Cb, 6, 1, nz, g.nkz, g.nky * g.nkx, g.pz, dtw + off[2],
                                                                  oddz);
            const long long per = (long long)g.nkz * g.nky * g.nkx;
            const double scale = ms / ((double)g.px * g.py * g.pz);
            if (kern64) to_float_kernel<<<grid_for(per * 6), 256, 0, s>>>(Cb, kern64, per, 6, scale, neg);
            else to_float_kernel<<<grid_for(per * 6), 256, 0, s>>>(Cb, kern, per, 6, scale, neg);
        }
        ok = ck(cudaGetLastError(), "newell kernels", err) && ck(cudaStreamSynchronize(s), "newell sync", err);
    }
    (void)ncomp;
    cudaFree(T);
    cudaFree(R);
    cudaFree(Ab);
    cudaFree(Bb);
    cudaFree(Cb);
    cudaFree(dtw);
    return ok;
}

bool newell_spectrum_gpu(const Grid &g, double dx, double dy, double dz, double ms, float *kern, cudaStream_t s,
                         std::string &err) {
    return newell_build(g, dx, dy, dz, ms, kern, nullptr, s, err);
}

bool newell_spectrum_gpu64(const Grid &g, double dx, double dy, double dz, double ms, double *kern, cudaStream_t s,
                           std::string &err) {
    return newell_build(g, dx, dy, dz, ms, nullptr, kern, s, err);
}

}  // namespace fm

// ---- periodic boundaries: truncated image sums (fdm_fft.rs:140-233, 614-717) ----
namespace fm {
namespace {

// Open-boundary tensor component values at the signed offset (i, j, k) cells: the
// first-octant value at (|i|, |j|, |k|) (table stencil or point-dipole asymptotics, the
// criterion on the absolute offsets) with the parity sign of each off-diagonal
// component (newell.rs:393-425).  The f/g table covers offsets up to kAsym + 1.
__device__ void open_tensor_at(const double *T, int sx, int sy, long long tl, int i, int j, int k, double dx, double dy,
                               double dz, double vol, double inv4piv, double v[6]) {
    const int ai = i < 0 ? -i : i, aj = j < 0 ? -j : j, ak = k < 0 ? -k : k;
    const long long d2 = (long long)ai * ai + (long long)aj * aj + (long long)ak * ak;
    if (ai >= kAsym || aj >= kAsym || ak >= kAsym || d2 >= (long long)kAsym * kAsym) {
        // the point-dipole forms of asym_diag / asym_off with 1/r^3 and 1/r^5 formed once
        // for the six components (the image sums evaluate millions of far offsets)
        const double x = ai * dx, y = aj * dy, z = ak * dz;
        const double r2 = x * x + y * y + z * z, r = sqrt(r2);
        const double w = vol / (4.0 * M_PI), i3 = 1.0 / (r2 * r), i5 = i3 / r2;
        v[0] = (i3 - 3.0 * x * x * i5) * w;
        v[1] = (i3 - 3.0 * y * y * i5) * w;
        v[2] = (i3 - 3.0 * z * z * i5) * w;
        v[3] = -3.0 * x * y * i5 * w;
        v[4] = -3.0 * x * z * i5 * w;
        v[5] = -3.0 * y * z * i5 * w;
    } else {
#pragma unroll 1
        for (int c = 0; c < 6; ++c) v[c] = stencil27(T + c * tl, ai, aj, ak, sx, sy, inv4piv);
    }
    const double sxg = i < 0 ? -1.0 : 1.0, syg = j < 0 ? -1.0 : 1.0, szg = k < 0 ? -1.0 : 1.0;
    v[3] *= sxg * syg;
    v[4] *= sxg * szg;
    v[5] *= syg * szg;
}

struct PerAxis {
    int n, p, images, periodic;
};

// Signed offset of padded index i on an open axis, or a flag for the empty gap.
__device__ __forceinline__ bool open_offset(const PerAxis &a, int i, int &o) {
    if (i < a.n) {
        o = i;
        return true;
    }
    if (i > a.p - a.n) {
        o = i - a.p;
        return true;
    }
    return false;
}

// S[c][k][j][i] over the padded grid (px, py, qz): on a periodic axis index i stands for
// the offsets i + m n, |m| <= I, summed image by image in the order z, y, x (outer to
// inner); on an open axis for its one signed offset.  qz = 1 on the thin-film path
// (the z = 0 plane, with z images when z is periodic).
__global__ void periodic_tensor_kernel(double *S, const double *T, int sx, int sy, long long tl, PerAxis ax, PerAxis ay,
                                       PerAxis az, int qz, double dx, double dy, double dz) {
    const long long len = (long long)ax.p * ay.p * qz;
    const double vol = dx * dy * dz, inv = 1.0 / (4.0 * M_PI * vol);
    for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < len; id += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(id % ax.p);
        const int j = (int)((id / ax.p) % ay.p);
        const int k = (int)(id / ((long long)ax.p * ay.p));
        double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        int oi = i, oj = j, ok = k;
        const bool live = (ax.periodic || open_offset(ax, i, oi)) && (ay.periodic || open_offset(ay, j, oj)) &&
                          (az.periodic || qz == 1 || open_offset(az, k, ok));
        if (live) {
            const int iz = az.periodic ? az.images : 0, iy = ay.periodic ? ay.images : 0, ix = ax.periodic ? ax.images : 0;
            for (int mz = -iz; mz <= iz; ++mz)
                for (int my = -iy; my <= iy; ++my)
                    for (int mx = -ix; mx <= ix; ++mx) {
                        double v[6];
                        open_tensor_at(T, sx, sy, tl, oi + mx * ax.n, oj + my * ay.n, ok + mz * az.n, dx, dy, dz, vol, inv, v);
                        for (int c = 0; c < 6; ++c) acc[c] += v[c];
                    }
        }
        for (int c = 0; c < 6; ++c) S[c * len + id] = acc[c];
    }
}

__global__ void scale_complex_kernel(const double2 *__restrict__ in, float2 *__restrict__ out32, double2 *__restrict__ out64,
                                     long long total, double scale) {
    for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < total; id += (long long)gridDim.x * blockDim.x) {
        if (out64) out64[id] = make_double2(in[id].x * scale, in[id].y * scale);
        else out32[id] = make_float2((float)(in[id].x * scale), (float)(in[id].y * scale));
    }
}

}  // namespace

bool newell_periodic_spectrum_gpu(const Grid &g, double dx, double dy, double dz, double ms, const uint32_t images[3],
                                  float2 *kern, double2 *kern64, cudaStream_t s, std::string &err) {
    const int per = g.per;
    const PerAxis ax{g.nx, g.px, (int)images[0], (per & 1) ? 1 : 0};
    const PerAxis ay{g.ny, g.py, (int)images[1], (per & 2) ? 1 : 0};
    const PerAxis az{g.nz, g.thin ? 1 : g.pz, (int)images[2], (per & 4) ? 1 : 0};
    const int qz = g.thin ? 1 : g.pz;
    const int ncomp = g.thin ? 4 : 6;
    // f/g table over the offsets the sums reach (at most the asymptotic distance)
    auto reach = [](const PerAxis &a) { return a.periodic ? (long long)a.n * (2LL * a.images + 1) : (long long)a.n; };
    const int sx = (int)std::min<long long>(reach(ax), kAsym) + 2, sy = (int)std::min<long long>(reach(ay), kAsym) + 2,
              sz = (int)std::min<long long>(reach(az), kAsym) + 2;
    const long long tl = (long long)sx * sy * sz;
    const long long len = (long long)g.px * g.py * qz;
    const long long nA = (long long)6 * qz * g.py * g.nkx;  // after x
    double *T = nullptr, *S = nullptr;
    double2 *A = nullptr, *B = nullptr;
    bool ok = ck(cudaMalloc(&T, sizeof(double) * 6 * tl), "cudaMalloc(newell table)", err) &&
              ck(cudaMalloc(&S, sizeof(double) * 6 * len), "cudaMalloc(periodic tensor)", err) &&
              ck(cudaMalloc(&A, sizeof(double2) * nA), "cudaMalloc(periodic x)", err) &&
              ck(cudaMalloc(&B, sizeof(double2) * nA), "cudaMalloc(periodic y)", err);
    if (ok) {
        fg_table_kernel<<<grid_for(tl), 256, 0, s>>>(T, sx, sy, sz, dx, dy, dz);
        periodic_tensor_kernel<<<grid_for(len), 256, 0, s>>>(S, T, sx, sy, tl, ax, ay, az, qz, dx, dy, dz);
        ok = ck(cudaGetLastError(), "periodic newell tensor", err);
        // FP64 FFTs: x [c][(k,j)][i] real -> [c][(k,j)][kx < nkx]; y [c][k][j][kx] ->
        // [c][k][ky][kx]; z [c][k][(ky,kx)] -> [c][kz][(ky,kx)]
        ok = ok && fft64_axis(S, nullptr, A, 6LL * qz * g.py, g.px, g.nkx, 1, s, err) &&
             fft64_axis(nullptr, A, B, 6LL * qz, g.py, g.py, g.nkx, s, err);
        const double2 *R = B;
        if (ok && qz > 1) {
            ok = fft64_axis(nullptr, B, A, 6, qz, qz, g.py * g.nkx, s, err);
            R = A;
        }
        if (ok) {
            // components xx yy zz xy (xz yz) are the first ncomp blocks of R, scaled by Ms / P
            const double scale = ms / ((double)g.px * g.py * qz);
            scale_complex_kernel<<<grid_for(nA), 256, 0, s>>>(R, kern, kern64, (long long)ncomp * qz * g.py * g.nkx, scale);
            ok = ck(cudaGetLastError(), "periodic newell kernels", err) && ck(cudaStreamSynchronize(s), "periodic newell sync", err);
        }
    }
    cudaFree(T);
    cudaFree(S);
    cudaFree(A);
    cudaFree(B);
    return ok;
}

}  // namespace fm
