// adjoint.cu -- element-wise kernels of the reverse-mode (adjoint) RK4 step.
//
// Forward step (the fixed-step RK4 of crates/fullmag-engine/src/fdm_integrators.rs:155-262
// with the per-stage normalisation N(v) = v/|v|):
//   k1 = f(y0), y1 = N(y0 + h/2 k1), k2 = f(y1), y2 = N(y0 + h/2 k2), k3 = f(y2),
//   y3 = N(y0 + h k3), k4 = f(y3), m' = N(y0 + h/6 (k1 + 2k2 + 2k3 + k4)),
//   f(m) = -gbar [p + alpha m x p], p = m x H, H = H_lin(m) + H_anis(m) + H_map + H_ext.
// Reverse mode, given the cotangent w of k = f(m) at (m, H):
//   q = prec w + alpha (w x m)
//   lambda_m  = -gbar [H x q + alpha p x w] + (dH_anis/dm)^T lambda_H + H_lin(lambda_H)
//   lambda_H  = -gbar (q x m)          (also the gradient with respect to the field map)
// and through a normalisation u = N(v):  lambda_v = (lambda_u - (u . lambda_u) u) / |v|.
// H_lin (exchange stencil + Newell convolution) is symmetric, so its transpose is
// applied by the forward field passes themselves (engine.cu).
#include "engine.h"

namespace fm {

namespace {

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 ld3(const float *a, long long n, long long i) { return {a[i], a[n + i], a[2 * n + i]}; }
__device__ __forceinline__ void st3(float *a, long long n, long long i, V3 v) {
    a[i] = v.x;
    a[n + i] = v.y;
    a[2 * n + i] = v.z;
}
__device__ __forceinline__ V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 axpy(float s, V3 a, V3 b) { return {s * a.x + b.x, s * a.y + b.y, s * a.z + b.z}; }
__device__ __forceinline__ V3 scl(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }

// lambda_v from lambda_u for u = N(v)
__device__ __forceinline__ V3 norm_vjp(V3 v, V3 lam) {
    const float nn = sqrtf(dot(v, v));
    if (!(nn > 0.f)) return {0.f, 0.f, 0.f};
    const float inv = 1.0f / nn;
    const V3 u = scl(inv, v);
    return scl(inv, axpy(-dot(u, lam), u, lam));
}

__device__ __forceinline__ void ff_acc(float *hi, float *lo, long long n, long long i, V3 v) {
    float h, l;
    h = hi[i], l = lo[i];
    ff_add(h, l, v.x);
    hi[i] = h, lo[i] = l;
    h = hi[n + i], l = lo[n + i];
    ff_add(h, l, v.y);
    hi[n + i] = h, lo[n + i] = l;
    h = hi[2 * n + i], l = lo[2 * n + i];
    ff_add(h, l, v.z);
    hi[2 * n + i] = h, lo[2 * n + i] = l;
}

// Local part of the VJP of f at (m, H) with cotangent w.
__global__ void adj_local_kernel(AdjLocal a) {
    const long long n = a.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const V3 m = ld3(a.m, n, i), H = ld3(a.H, n, i), w = ld3(a.w, n, i);
        const V3 q = axpy(a.alpha, cross(w, m), scl(a.prec, w));
        const V3 p = cross(m, H);
        V3 lm = scl(-a.gbar, axpy(a.alpha, cross(p, w), cross(H, q)));
        const V3 lh = scl(-a.gbar, cross(q, m));
        if (a.has_uni) {
            const V3 u = {a.u[0], a.u[1], a.u[2]};
            const float mu = dot(m, u);
            lm = axpy((a.ku1c + 3.0f * a.ku2c * mu * mu) * dot(u, lh), u, lm);
        }
        st3(a.lam_h, n, i, lh);
        st3(a.lam_m, n, i, lm);
        if (a.g_hi) ff_acc(a.g_hi, a.g_lo, n, i, lh);
    }
}

// Stage update: lambda_y = lambda_m + H_lin(lambda_H); for stage s >= 1 push it through
// y_s = N(y0 + c h k_s) into lambda_y0 and lambda_k_s, for s = 0 add it to lambda_y0.
__global__ void adj_stage_kernel(AdjStage a) {
    const long long n = a.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const V3 ly = axpy(1.0f, ld3(a.lam_m, n, i), ld3(a.lin, n, i));
        V3 y0acc = ld3(a.lam_y0, n, i);
        if (a.k) {
            const V3 v = axpy(a.ch, ld3(a.k, n, i), ld3(a.y0, n, i));
            const V3 mu = norm_vjp(v, ly);
            st3(a.lam_y0, n, i, axpy(1.0f, mu, y0acc));
            st3(a.lam_k, n, i, axpy(a.ch, mu, ld3(a.lam_k, n, i)));
        } else {
            st3(a.lam_y0, n, i, axpy(1.0f, ly, y0acc));
        }
    }
}

// Final normalisation of the step: m' = N(y0 + h/6 (k1 + 2k2 + 2k3 + k4)).
__global__ void adj_final_kernel(AdjFinal a) {
    const long long n = a.n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const V3 k1 = ld3(a.k1, n, i), k2 = ld3(a.k2, n, i), k3 = ld3(a.k3, n, i), k4 = ld3(a.k4, n, i);
        const V3 s = {k1.x + 2.f * k2.x + 2.f * k3.x + k4.x, k1.y + 2.f * k2.y + 2.f * k3.y + k4.y,
                      k1.z + 2.f * k2.z + 2.f * k3.z + k4.z};
        const float h6 = a.h / 6.0f;
        const V3 v = axpy(h6, s, ld3(a.y0, n, i));
        const V3 mu = norm_vjp(v, ld3(a.lam_next, n, i));
        st3(a.lam_y0, n, i, mu);
        st3(a.lk1, n, i, scl(h6, mu));
        st3(a.lk2, n, i, scl(2.f * h6, mu));
        st3(a.lk3, n, i, scl(2.f * h6, mu));
        st3(a.lk4, n, i, scl(h6, mu));
    }
}

unsigned grid_of(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16); }

}  // namespace

cudaError_t launch_adj_local(const AdjLocal &a, cudaStream_t s) {
    adj_local_kernel<<<grid_of(a.n), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_adj_stage(const AdjStage &a, cudaStream_t s) {
    adj_stage_kernel<<<grid_of(a.n), 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_adj_final(const AdjFinal &a, cudaStream_t s) {
    adj_final_kernel<<<grid_of(a.n), 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace fm
