// adjoint.cu -- the reverse-mode (adjoint) RK4 step: equations and the final-combination
// kernel.
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
// applied by the forward field passes themselves.  The local VJP and the stage update
// are fused into the row pass (row_pass.cu, adjoint modes 1 and 2); this file holds the
// step's last normalisation, which starts the reverse sweep of every step.
#include <algorithm>

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

cudaError_t launch_adj_final(const AdjFinal &a, cudaStream_t s) {
    adj_final_kernel<<<grid_of(a.n), 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace fm
