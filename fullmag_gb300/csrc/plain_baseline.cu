// plain_baseline.cu -- the "plain" GPU path the fused engine is measured against.
//
// MEASUREMENT BASELINE, NOT PART OF libfullmag_fdm.so.  It restates the per-step kernel
// structure of the reference's CUDA backend with cuFFT and one kernel per operation:
//   exchange field kernel                     native/backends/fdm/src/exchange_fp32.cu:21-156
//   demag: pack Ms*m into three zero-padded complex arrays, 3 forward cuFFT C2C, the
//   6-component tensor multiply, 3 inverse C2C, unpack with 1/P
//                                             native/backends/fdm/src/demag_fp32.cu:50-199,406-502
//   effective field (H_ex + H_d + Zeeman + anisotropy)   demag_fp32.cu:201-402,517-583
//   LLG right-hand side                       native/backends/fdm/src/llg_fp32.cu:32-200
//   RK4 / Heun stage combinations             llg_rk4_fp32.cu:37-232, llg_fp32.cu:204-389
//   post-step diagnostic evaluation, then energies and max norms, each a two-pass FP64
//   reduction ending in a blocking copy of one double
//                                             llg_fp32.cu:336-343, reductions_fp64.cu:123-393
// FP32 state and fields, FP32 complex spectra of the full padded grid (2nx, 2ny, 2nz),
// built from the same FP64 Newell tensor as the engine (newell.cu).  The reference
// build cannot run on the benchmark machine (its sources are not there), so this
// repo-written path stands in for it.  No masks; Heun and RK4 only.
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/fullmag_fdm.h"
#include "engine.h"

namespace fm {
bool newell_spectrum_gpu(const Grid &g, double dx, double dy, double dz, double ms, float *kern, cudaStream_t s,
                         std::string &err);
}

namespace {

using fm::Grid;
constexpr double kMu0 = 4.0 * M_PI * 1e-7;
constexpr int kT = 256;
constexpr int kRedBlocks = 1024;

unsigned blocks_for(long long n) { return (unsigned)std::min<long long>((n + kT - 1) / kT, 152LL * 32); }

struct Params {
    int nx, ny, nz;
    long long n;
    int px, py, pz;
    long long P;
    float ex_pref, idx2, idy2, idz2;
    int has_ext;
    float hext[3];
    int has_uni;
    float ku1c, ku2c, u[3];
    int has_cub;
    float kc1c, kc2c, kc3c, c1[3], c2[3], c3[3];
    float gbar, alpha, prec, ms;
    float ku1f, ku2f, kc1f, kc2f, kc3f;  // raw J/m^3 for the energy densities
};

__global__ void exchange_kernel(Params p, const float *__restrict__ m, float *__restrict__ h) {
    const long long n = p.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % p.nx), y = (int)((i / p.nx) % p.ny), z = (int)(i / ((long long)p.nx * p.ny));
        const long long xm = x > 0 ? i - 1 : i, xp = x < p.nx - 1 ? i + 1 : i;
        const long long ym = y > 0 ? i - p.nx : i, yp = y < p.ny - 1 ? i + p.nx : i;
        const long long zm = z > 0 ? i - (long long)p.nx * p.ny : i, zp = z < p.nz - 1 ? i + (long long)p.nx * p.ny : i;
        for (int c = 0; c < 3; ++c) {
            const float *a = m + c * n;
            const float mc = a[i];
            h[c * n + i] = p.ex_pref * ((a[xp] - 2.f * mc + a[xm]) * p.idx2 + (a[yp] - 2.f * mc + a[ym]) * p.idy2 +
                                        (a[zp] - 2.f * mc + a[zm]) * p.idz2);
        }
    }
}

// Ms * m scattered into the (cleared) padded complex arrays
__global__ void pack_kernel(Params p, const float *__restrict__ m, cufftComplex *__restrict__ M) {
    const long long n = p.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % p.nx), y = (int)((i / p.nx) % p.ny), z = (int)(i / ((long long)p.nx * p.ny));
        const long long d = (long long)x + (long long)p.px * (y + (long long)p.py * z);
        for (int c = 0; c < 3; ++c) M[c * p.P + d] = make_float2(p.ms * m[c * n + i], 0.f);
    }
}

// H(k) = -N(k) M(k) over the full padded grid, in place (N complex, 6 components)
__global__ void multiply_kernel(Params p, cufftComplex *__restrict__ M, const cufftComplex *__restrict__ N) {
    const long long P = p.P;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x) {
        const float2 mx = M[i], my = M[P + i], mz = M[2 * P + i];
        const float2 xx = N[i], yy = N[P + i], zz = N[2 * P + i], xy = N[3 * P + i], xz = N[4 * P + i], yz = N[5 * P + i];
        auto cm = [](float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
        auto add3 = [](float2 a, float2 b, float2 c) { return make_float2(-(a.x + b.x + c.x), -(a.y + b.y + c.y)); };
        M[i] = add3(cm(xx, mx), cm(xy, my), cm(xz, mz));
        M[P + i] = add3(cm(xy, mx), cm(yy, my), cm(yz, mz));
        M[2 * P + i] = add3(cm(xz, mx), cm(yz, my), cm(zz, mz));
    }
}

__global__ void unpack_kernel(Params p, const cufftComplex *__restrict__ H, float *__restrict__ hd) {
    const long long n = p.n;
    const float inv = 1.0f / (float)p.P;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % p.nx), y = (int)((i / p.nx) % p.ny), z = (int)(i / ((long long)p.nx * p.ny));
        const long long d = (long long)x + (long long)p.px * (y + (long long)p.py * z);
        for (int c = 0; c < 3; ++c) hd[c * n + i] = H[c * p.P + d].x * inv;
    }
}

__global__ void effective_field_kernel(Params p, const float *__restrict__ m, const float *__restrict__ hex,
                                       const float *__restrict__ hd, float *__restrict__ heff) {
    const long long n = p.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float mx = m[i], my = m[n + i], mz = m[2 * n + i];
        float h[3] = {hex[i] + hd[i], hex[n + i] + hd[n + i], hex[2 * n + i] + hd[2 * n + i]};
        if (p.has_ext)
            for (int c = 0; c < 3; ++c) h[c] += p.hext[c];
        if (p.has_uni) {
            const float mu = mx * p.u[0] + my * p.u[1] + mz * p.u[2];
            const float cf = p.ku1c * mu + p.ku2c * mu * mu * mu;
            for (int c = 0; c < 3; ++c) h[c] += cf * p.u[c];
        }
        if (p.has_cub) {
            const float a1 = mx * p.c1[0] + my * p.c1[1] + mz * p.c1[2];
            const float a2 = mx * p.c2[0] + my * p.c2[1] + mz * p.c2[2];
            const float a3 = mx * p.c3[0] + my * p.c3[1] + mz * p.c3[2];
            const float s1 = a1 * a1, s2 = a2 * a2, s3 = a3 * a3, sig = s1 * s2 + s2 * s3 + s1 * s3;
            const float g1 = p.kc1c * a1 * (s2 + s3) + p.kc2c * a1 * s2 * s3 + p.kc3c * sig * a1 * (s2 + s3);
            const float g2 = p.kc1c * a2 * (s1 + s3) + p.kc2c * a2 * s1 * s3 + p.kc3c * sig * a2 * (s1 + s3);
            const float g3 = p.kc1c * a3 * (s1 + s2) + p.kc2c * a3 * s1 * s2 + p.kc3c * sig * a3 * (s1 + s2);
            for (int c = 0; c < 3; ++c) h[c] += g1 * p.c1[c] + g2 * p.c2[c] + g3 * p.c3[c];
        }
        for (int c = 0; c < 3; ++c) heff[c * n + i] = h[c];
    }
}

__global__ void llg_rhs_kernel(Params p, const float *__restrict__ m, const float *__restrict__ h, float *__restrict__ k) {
    const long long n = p.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float mx = m[i], my = m[n + i], mz = m[2 * n + i];
        const float hx = h[i], hy = h[n + i], hz = h[2 * n + i];
        const float px = my * hz - mz * hy, py = mz * hx - mx * hz, pz = mx * hy - my * hx;
        const float qx = my * pz - mz * py, qy = mz * px - mx * pz, qz = mx * py - my * px;
        k[i] = -p.gbar * (p.prec * px + p.alpha * qx);
        k[n + i] = -p.gbar * (p.prec * py + p.alpha * qy);
        k[2 * n + i] = -p.gbar * (p.prec * pz + p.alpha * qz);
    }
}

struct Comb {
    const float *k[4];
    float c[4];
    int nk;
};

// out = normalize(m0 + dt * sum c_j k_j)
__global__ void stage_kernel(long long n, const float *__restrict__ m0, Comb cb, float dt, float *__restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float v[3];
        for (int c = 0; c < 3; ++c) {
            float a = 0.f;
            for (int j = 0; j < cb.nk; ++j) a += cb.c[j] * cb.k[j][c * n + i];
            v[c] = m0[c * n + i] + dt * a;
        }
        const float nn = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        const float inv = nn > 0.f ? 1.f / nn : 0.f;
        for (int c = 0; c < 3; ++c) out[c * n + i] = v[c] * inv;
    }
}

// Per-cell quantity of reduction `which`: 0 exchange pair sum, 1 m.H_d, 2 m.H_ext,
// 3 uniaxial density, 4 cubic density (sums); 5 |H_eff|^2, 6 |H_d|^2, 7 |k|^2 (maxima)
__device__ double red_value(const Params &p, int which, long long i, const float *m, const float *hd, const float *heff,
                            const float *k) {
    const long long n = p.n;
    const float mx = m[i], my = m[n + i], mz = m[2 * n + i];
    switch (which) {
        case 0: {
            const int x = (int)(i % p.nx), y = (int)((i / p.nx) % p.ny), z = (int)(i / ((long long)p.nx * p.ny));
            double e = 0.0;
            const long long nb[3] = {x + 1 < p.nx ? i + 1 : -1, y + 1 < p.ny ? i + p.nx : -1,
                                     z + 1 < p.nz ? i + (long long)p.nx * p.ny : -1};
            const float w[3] = {p.idx2, p.idy2, p.idz2};
            for (int a = 0; a < 3; ++a) {
                if (nb[a] < 0) continue;
                const double d0 = m[nb[a]] - mx, d1 = m[n + nb[a]] - my, d2 = m[2 * n + nb[a]] - mz;
                e += (d0 * d0 + d1 * d1 + d2 * d2) * w[a];
            }
            return e;
        }
        case 1: return (double)mx * hd[i] + (double)my * hd[n + i] + (double)mz * hd[2 * n + i];
        case 2: return p.has_ext ? (double)mx * p.hext[0] + (double)my * p.hext[1] + (double)mz * p.hext[2] : 0.0;
        case 3: {
            if (!p.has_uni) return 0.0;
            const double mu = mx * p.u[0] + my * p.u[1] + mz * p.u[2], s = mu * mu;
            return (double)p.ku1f * s + (double)p.ku2f * s * s;
        }
        case 4: {
            if (!p.has_cub) return 0.0;
            const double a1 = mx * p.c1[0] + my * p.c1[1] + mz * p.c1[2];
            const double a2 = mx * p.c2[0] + my * p.c2[1] + mz * p.c2[2];
            const double a3 = mx * p.c3[0] + my * p.c3[1] + mz * p.c3[2];
            const double s1 = a1 * a1, s2 = a2 * a2, s3 = a3 * a3, sig = s1 * s2 + s2 * s3 + s1 * s3;
            return (double)p.kc1f * sig + (double)p.kc2f * s1 * s2 * s3 + (double)p.kc3f * sig * sig;
        }
        case 5: return (double)heff[i] * heff[i] + (double)heff[n + i] * heff[n + i] + (double)heff[2 * n + i] * heff[2 * n + i];
        case 6: return (double)hd[i] * hd[i] + (double)hd[n + i] * hd[n + i] + (double)hd[2 * n + i] * hd[2 * n + i];
        default: return (double)k[i] * k[i] + (double)k[n + i] * k[n + i] + (double)k[2 * n + i] * k[2 * n + i];
    }
}

__global__ void reduce_pass1(Params p, int which, const float *m, const float *hd, const float *heff, const float *k,
                             double *partial) {
    __shared__ double sh[kT];
    const bool is_max = which >= 5;
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < p.n; i += (long long)gridDim.x * blockDim.x) {
        const double v = red_value(p, which, i, m, hd, heff, k);
        acc = is_max ? fmax(acc, v) : acc + v;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kT / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] = is_max ? fmax(sh[threadIdx.x], sh[threadIdx.x + s]) : sh[threadIdx.x] + sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void reduce_pass2(int which, const double *partial, int nb, double *out) {
    __shared__ double sh[kT];
    const bool is_max = which >= 5;
    double acc = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) acc = is_max ? fmax(acc, partial[i]) : acc + partial[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kT / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] = is_max ? fmax(sh[threadIdx.x], sh[threadIdx.x + s]) : sh[threadIdx.x] + sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// full complex spectrum N(k) of one component from the octant kernel of newell.cu
// (scaled back from Ms/P): even components mirror, odd axes flip sign
__global__ void expand_kernel(Grid g, const float *__restrict__ oct, cufftComplex *__restrict__ N, float scale) {
    const long long P = (long long)g.px * g.py * g.pz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x) {
        const int kx = (int)(i % g.px), ky = (int)((i / g.px) % g.py), kz = (int)(i / ((long long)g.px * g.py));
        const int ax = kx > g.px / 2 ? g.px - kx : kx, ay = ky > g.py / 2 ? g.py - ky : ky, az = kz > g.pz / 2 ? g.pz - kz : kz;
        const float sx = kx > g.px / 2 ? -1.f : 1.f, sy = ky > g.py / 2 ? -1.f : 1.f, sz = kz > g.pz / 2 ? -1.f : 1.f;
        const long long o = ((long long)az * g.nky + ay) * g.nkx + ax;
        const long long cs = (long long)g.nkz * g.nky * g.nkx;
        const float sgn[6] = {1.f, 1.f, 1.f, sx * sy, sx * sz, sy * sz};
        for (int c = 0; c < 6; ++c) N[c * P + i] = make_float2(scale * sgn[c] * oct[c * cs + o], 0.f);
    }
}

struct Plain {
    Params p{};
    int integrator = 0;
    double dx = 0, dy = 0, dz = 0, a_ex = 0, ms = 0, ku1 = 0, kc1 = 0;
    bool has_uni = false, has_cub = false, has_ext = false;
    float *m = nullptr, *m0 = nullptr, *mst = nullptr, *k[4] = {}, *hex = nullptr, *hd = nullptr, *heff = nullptr;
    cufftComplex *M = nullptr, *N = nullptr;
    double *partial = nullptr, *red = nullptr;
    cufftHandle plan = 0;
    bool plan_ok = false;
    uint64_t step_count = 0;
    double time = 0.0;
    std::string err;

    ~Plain() {
        if (plan_ok) cufftDestroy(plan);
        for (void *q : {(void *)m, (void *)m0, (void *)mst, (void *)k[0], (void *)k[1], (void *)k[2], (void *)k[3],
                        (void *)hex, (void *)hd, (void *)heff, (void *)M, (void *)N, (void *)partial, (void *)red})
            if (q) cudaFree(q);
    }

    // one field evaluation at state s into k_out (the reference's per-evaluation sequence)
    bool eval(const float *s, float *k_out) {
        const unsigned b = blocks_for(p.n), bP = blocks_for(p.P);
        exchange_kernel<<<b, kT>>>(p, s, hex);
        if (cudaMemsetAsync(M, 0, sizeof(cufftComplex) * 3 * p.P) != cudaSuccess) return false;
        pack_kernel<<<b, kT>>>(p, s, M);
        for (int c = 0; c < 3; ++c)
            if (cufftExecC2C(plan, M + c * p.P, M + c * p.P, CUFFT_FORWARD) != CUFFT_SUCCESS) return false;
        multiply_kernel<<<bP, kT>>>(p, M, N);
        for (int c = 0; c < 3; ++c)
            if (cufftExecC2C(plan, M + c * p.P, M + c * p.P, CUFFT_INVERSE) != CUFFT_SUCCESS) return false;
        unpack_kernel<<<b, kT>>>(p, M, hd);
        effective_field_kernel<<<b, kT>>>(p, s, hex, hd, heff);
        llg_rhs_kernel<<<b, kT>>>(p, s, heff, k_out);
        return cudaGetLastError() == cudaSuccess;
    }

    bool combine(const float *base, int nk, const float *const *ks, const float *cs, double dt, float *out) {
        Comb cb{};
        cb.nk = nk;
        for (int j = 0; j < nk; ++j) {
            cb.k[j] = ks[j];
            cb.c[j] = cs[j];
        }
        stage_kernel<<<blocks_for(p.n), kT>>>(p.n, base, cb, (float)dt, out);
        return cudaGetLastError() == cudaSuccess;
    }

    double reduce(int which, const float *s) {
        reduce_pass1<<<kRedBlocks, kT>>>(p, which, s, hd, heff, k[0], partial);
        reduce_pass2<<<1, kT>>>(which, partial, kRedBlocks, red);
        double v = 0.0;
        cudaMemcpy(&v, red, sizeof(double), cudaMemcpyDeviceToHost);  // blocking, as the reference's reductions
        return v;
    }

    bool step(double dt, fullmag_fdm_step_stats *st) {
        const auto t0 = std::chrono::steady_clock::now();
        const size_t bytes = sizeof(float) * 3 * (size_t)p.n;
        if (cudaMemcpyAsync(m0, m, bytes, cudaMemcpyDeviceToDevice) != cudaSuccess) return false;
        if (integrator == FULLMAG_FDM_INTEGRATOR_RK4) {
            const float h = 0.5f, one = 1.f;
            if (!eval(m0, k[0]) || !combine(m0, 1, &k[0], &h, dt, mst)) return false;
            if (!eval(mst, k[1]) || !combine(m0, 1, &k[1], &h, dt, mst)) return false;
            if (!eval(mst, k[2]) || !combine(m0, 1, &k[2], &one, dt, mst)) return false;
            if (!eval(mst, k[3])) return false;
            const float w[4] = {1.f / 6.f, 1.f / 3.f, 1.f / 3.f, 1.f / 6.f};
            const float *ks[4] = {k[0], k[1], k[2], k[3]};
            if (!combine(m0, 4, ks, w, dt, m)) return false;
        } else {
            const float one = 1.f, half[2] = {0.5f, 0.5f};
            if (!eval(m0, k[0]) || !combine(m0, 1, &k[0], &one, dt, mst)) return false;
            if (!eval(mst, k[1])) return false;
            const float *ks[2] = {k[0], k[1]};
            if (!combine(m0, 2, ks, half, dt, m)) return false;
        }
        // post-step diagnostic evaluation, then the statistics
        if (!eval(m, k[0])) return false;
        double r[8];
        for (int w = 0; w < 8; ++w) r[w] = reduce(w, m);
        if (cudaDeviceSynchronize() != cudaSuccess) return false;
        step_count += 1;
        time += dt;
        if (st) {
            const double V = dx * dy * dz;
            *st = fullmag_fdm_step_stats{};
            st->step = step_count;
            st->time_seconds = time;
            st->dt_seconds = dt;
            st->exchange_energy_joules = a_ex * V * r[0];
            st->demag_energy_joules = -0.5 * kMu0 * ms * V * r[1];
            st->external_energy_joules = has_ext ? -kMu0 * ms * V * r[2] : 0.0;
            st->anisotropy_energy_joules = has_uni ? -V * r[3] : 0.0;
            st->cubic_energy_joules = has_cub ? V * r[4] : 0.0;
            st->total_energy_joules = st->exchange_energy_joules + st->demag_energy_joules + st->external_energy_joules +
                                      st->anisotropy_energy_joules + st->cubic_energy_joules;
            st->max_effective_field_amplitude = sqrt(r[5]);
            st->max_demag_field_amplitude = sqrt(r[6]);
            st->max_rhs_amplitude = sqrt(r[7]);
            st->wall_time_ns = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
                                   std::chrono::steady_clock::now() - t0)
                                   .count();
        }
        return true;
    }
};

std::string g_create_error;

bool setup(Plain &e, const fullmag_fdm_plan_desc *plan) {
    Params &p = e.p;
    p.nx = (int)plan->grid.nx;
    p.ny = (int)plan->grid.ny;
    p.nz = (int)plan->grid.nz;
    p.n = (long long)p.nx * p.ny * p.nz;
    if (p.n <= 0 || !plan->enable_demag || !plan->initial_magnetization_xyz ||
        plan->initial_magnetization_len != 3 * (uint64_t)p.n) {
        e.err = "plain path needs a grid, demag and an initial magnetization";
        return false;
    }
    if (plan->integrator != FULLMAG_FDM_INTEGRATOR_RK4 && plan->integrator != FULLMAG_FDM_INTEGRATOR_HEUN) {
        e.err = "plain path supports HEUN and RK4";
        return false;
    }
    if (plan->active_mask || plan->region_mask) {
        e.err = "plain path has no active or region masks";
        return false;
    }
    e.integrator = plan->integrator;
    e.dx = plan->grid.dx;
    e.dy = plan->grid.dy;
    e.dz = plan->grid.dz;
    e.ms = plan->material.saturation_magnetisation;
    e.a_ex = plan->enable_exchange ? plan->material.exchange_stiffness : 0.0;
    const double alpha = plan->material.damping, gamma = plan->material.gyromagnetic_ratio;
    p.px = 2 * p.nx;
    p.py = 2 * p.ny;
    p.pz = 2 * p.nz;
    p.P = (long long)p.px * p.py * p.pz;
    p.ex_pref = (float)(2.0 * e.a_ex / (kMu0 * e.ms));
    p.idx2 = (float)(1.0 / (e.dx * e.dx));
    p.idy2 = (float)(1.0 / (e.dy * e.dy));
    p.idz2 = (float)(1.0 / (e.dz * e.dz));
    e.has_ext = plan->has_external_field != 0;
    p.has_ext = e.has_ext;
    for (int c = 0; c < 3; ++c) p.hext[c] = (float)plan->external_field_am[c];
    e.has_uni = plan->has_uniaxial_anisotropy != 0;
    p.has_uni = e.has_uni;
    p.ku1c = (float)(2.0 * plan->uniaxial_anisotropy_constant / (kMu0 * e.ms));
    p.ku2c = (float)(4.0 * plan->uniaxial_anisotropy_k2 / (kMu0 * e.ms));
    double un = 0;
    for (int c = 0; c < 3; ++c) un += plan->anisotropy_axis[c] * plan->anisotropy_axis[c];
    un = un > 0 ? sqrt(un) : 1.0;
    for (int c = 0; c < 3; ++c) p.u[c] = (float)(plan->anisotropy_axis[c] / un);
    e.has_cub = plan->has_cubic_anisotropy != 0;
    p.has_cub = e.has_cub;
    p.kc1c = (float)(-2.0 * plan->cubic_Kc1 / (kMu0 * e.ms));
    p.kc2c = (float)(-2.0 * plan->cubic_Kc2 / (kMu0 * e.ms));
    p.kc3c = (float)(-4.0 * plan->cubic_Kc3 / (kMu0 * e.ms));
    double a[3], b[3];
    double na = 0, nb = 0;
    for (int c = 0; c < 3; ++c) {
        a[c] = plan->cubic_axis1[c];
        b[c] = plan->cubic_axis2[c];
        na += a[c] * a[c];
        nb += b[c] * b[c];
    }
    na = na > 0 ? sqrt(na) : 1.0;
    nb = nb > 0 ? sqrt(nb) : 1.0;
    for (int c = 0; c < 3; ++c) {
        a[c] /= na;
        b[c] /= nb;
        p.c1[c] = (float)a[c];
        p.c2[c] = (float)b[c];
    }
    p.c3[0] = (float)(a[1] * b[2] - a[2] * b[1]);
    p.c3[1] = (float)(a[2] * b[0] - a[0] * b[2]);
    p.c3[2] = (float)(a[0] * b[1] - a[1] * b[0]);
    p.gbar = (float)(gamma / (1.0 + alpha * alpha));
    p.alpha = (float)alpha;
    p.prec = plan->disable_precession ? 0.f : 1.f;
    p.ms = (float)e.ms;
    p.ku1f = (float)plan->uniaxial_anisotropy_constant;
    p.ku2f = (float)plan->uniaxial_anisotropy_k2;
    p.kc1f = (float)plan->cubic_Kc1;
    p.kc2f = (float)plan->cubic_Kc2;
    p.kc3f = (float)plan->cubic_Kc3;

    const size_t v3 = sizeof(float) * 3 * (size_t)p.n;
    float **bufs[] = {&e.m, &e.m0, &e.mst, &e.k[0], &e.k[1], &e.k[2], &e.k[3], &e.hex, &e.hd, &e.heff};
    for (float **q : bufs)
        if (cudaMalloc((void **)q, v3) != cudaSuccess) {
            e.err = "cudaMalloc failed";
            return false;
        }
    if (cudaMalloc((void **)&e.M, sizeof(cufftComplex) * 3 * p.P) != cudaSuccess ||
        cudaMalloc((void **)&e.N, sizeof(cufftComplex) * 6 * p.P) != cudaSuccess ||
        cudaMalloc((void **)&e.partial, sizeof(double) * kRedBlocks) != cudaSuccess ||
        cudaMalloc((void **)&e.red, sizeof(double)) != cudaSuccess) {
        e.err = "cudaMalloc failed";
        return false;
    }
    if (cufftPlan3d(&e.plan, p.pz, p.py, p.px, CUFFT_C2C) != CUFFT_SUCCESS) {
        e.err = "cufftPlan3d failed";
        return false;
    }
    e.plan_ok = true;

    // kernel spectra: the engine's FP64 Newell octant kernel (scaled by Ms/P) expanded
    Grid g{};
    g.nx = p.nx;
    g.ny = p.ny;
    g.nz = p.nz;
    g.n = p.n;
    g.px = p.px;
    g.py = p.py;
    g.pz = p.pz;
    g.half = p.px / 2;
    g.nkx = g.half + 1;
    g.nky = p.py / 2 + 1;
    g.nkz = p.pz / 2 + 1;
    g.thin = 0;
    fm::grid_dividers(g);
    float *oct = nullptr;
    const size_t octn = 6ull * g.nkz * g.nky * g.nkx;
    if (cudaMalloc((void **)&oct, sizeof(float) * octn) != cudaSuccess) {
        e.err = "cudaMalloc failed";
        return false;
    }
    if (!fm::newell_spectrum_gpu(g, e.dx, e.dy, e.dz, e.ms, oct, 0, e.err)) {
        cudaFree(oct);
        return false;
    }
    expand_kernel<<<blocks_for(p.P), kT>>>(g, oct, e.N, (float)((double)p.P / e.ms));
    const cudaError_t rc = cudaDeviceSynchronize();
    cudaFree(oct);
    if (rc != cudaSuccess) {
        e.err = std::string("spectrum setup: ") + cudaGetErrorString(rc);
        return false;
    }

    // initial state (AoS doubles -> SoA floats on the host, one copy)
    std::vector<float> soa(3 * (size_t)p.n);
    for (long long i = 0; i < p.n; ++i)
        for (int c = 0; c < 3; ++c) soa[c * p.n + i] = (float)plan->initial_magnetization_xyz[3 * i + c];
    if (cudaMemcpy(e.m, soa.data(), v3, cudaMemcpyHostToDevice) != cudaSuccess) {
        e.err = "initial state copy failed";
        return false;
    }
    return true;
}

}  // namespace

extern "C" {

void *fullmag_fdm_plain_create(const fullmag_fdm_plan_desc *plan) {
    g_create_error.clear();
    if (!plan) return nullptr;
    Plain *e = new (std::nothrow) Plain();
    if (!e) return nullptr;
    if (!setup(*e, plan)) {
        g_create_error = e->err;
        delete e;
        return nullptr;
    }
    return e;
}

const char *fullmag_fdm_plain_create_error(void) { return g_create_error.c_str(); }

int fullmag_fdm_plain_step(void *handle, double dt, fullmag_fdm_step_stats *out) {
    Plain *e = static_cast<Plain *>(handle);
    if (!e || !(dt > 0.0)) return FULLMAG_FDM_ERR_INVALID;
    return e->step(dt, out) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
}

int fullmag_fdm_plain_copy_m(void *handle, double *out_xyz, uint64_t len) {
    Plain *e = static_cast<Plain *>(handle);
    if (!e || !out_xyz || len != 3 * (uint64_t)e->p.n) return FULLMAG_FDM_ERR_INVALID;
    std::vector<float> soa(3 * (size_t)e->p.n);
    if (cudaMemcpy(soa.data(), e->m, sizeof(float) * soa.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
        return FULLMAG_FDM_ERR_CUDA;
    for (long long i = 0; i < e->p.n; ++i)
        for (int c = 0; c < 3; ++c) out_xyz[3 * i + c] = soa[c * e->p.n + i];
    return FULLMAG_FDM_OK;
}

void fullmag_fdm_plain_destroy(void *handle) { delete static_cast<Plain *>(handle); }

}  // extern "C"
