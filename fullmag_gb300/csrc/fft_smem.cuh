// fft_smem.cuh -- shared-memory Stockham FFT used by every demag pass.
//
// A CTA transforms `nlines` complex lines of length n that sit in shared
// memory (line stride `ls` float2), ping-ponging between two buffers.  Each
// stage of radix R is one sweep of n/R butterflies per line; the Stockham
// index map keeps the result in natural order, so no bit reversal pass is
// needed.  Radices 2, 4 and 8 have unrolled butterflies; any other factor
// (3, 5, 7 and larger primes from uneven grid sizes) uses an O(R^2) loop
// over the twiddle table.  Twiddles are FP64-computed host-side and stored
// as float2 e^{-2 pi i e / n}; the inverse conjugates them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fm {

constexpr int kMaxStages = 24;
constexpr int kMaxGenericRadix = 64;

struct FftPlan {
    int n;
    int nstages;
    int radix[kMaxStages];
    const float2 *tw;  // n entries, e^{-2 pi i e / n}
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
__device__ __forceinline__ float2 mul_mi(float2 a, bool inv) {
    return inv ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int R>
__device__ __forceinline__ void dft_small(float2 *v, bool inv);

template <>
__device__ __forceinline__ void dft_small<2>(float2 *v, bool) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <>
__device__ __forceinline__ void dft_small<4>(float2 *v, bool inv) {
    float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    float2 b0 = cadd(v[1], v[3]), b1 = mul_mi(csub(v[1], v[3]), inv);
    v[0] = cadd(a0, b0);
    v[2] = csub(a0, b0);
    v[1] = cadd(a1, b1);
    v[3] = csub(a1, b1);
}

template <>
__device__ __forceinline__ void dft_small<8>(float2 *v, bool inv) {
    // radix-2 decimation in frequency, then two 4-point DFTs
    const float h = 0.70710678118654752440f;
    float2 a[4], b[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        a[t] = cadd(v[t], v[t + 4]);
        b[t] = csub(v[t], v[t + 4]);
    }
    // b[t] *= W8^t  (W8 = e^{-i pi/4} forward, conjugate for inverse)
    {
        float2 x = b[1];
        b[1] = inv ? make_float2(h * (x.x - x.y), h * (x.x + x.y)) : make_float2(h * (x.x + x.y), h * (x.y - x.x));
        b[2] = mul_mi(b[2], inv);
        x = b[3];
        b[3] = inv ? make_float2(-h * (x.x + x.y), h * (x.x - x.y)) : make_float2(h * (x.y - x.x), -h * (x.x + x.y));
    }
    dft_small<4>(a, inv);
    dft_small<4>(b, inv);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        v[2 * q] = a[q];
        v[2 * q + 1] = b[q];
    }
}

template <int R>
__device__ __forceinline__ void stage_fixed(const float2 *__restrict__ in, float2 *__restrict__ out, int nlines, int ls,
                                            int n, int Ns, const float2 *__restrict__ tw, bool inv) {
    const int nb = n / R;
    const int total = nlines * nb;
    const int twstride = n / (Ns * R);
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int l = idx / nb;
        const int j = idx - l * nb;
        const float2 *src = in + (size_t)l * ls;
        float2 *dst = out + (size_t)l * ls;
        const int k = j % Ns;
        float2 v[R];
#pragma unroll
        for (int t = 0; t < R; ++t) v[t] = src[j + t * nb];
        if (Ns > 1) {
#pragma unroll
            for (int t = 1; t < R; ++t) {
                float2 w = __ldg(tw + t * k * twstride);
                if (inv) w.y = -w.y;
                v[t] = cmul(v[t], w);
            }
        }
        dft_small<R>(v, inv);
        const int o = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int t = 0; t < R; ++t) dst[o + t * Ns] = v[t];
    }
}

__device__ __forceinline__ void stage_generic(const float2 *__restrict__ in, float2 *__restrict__ out, int nlines, int ls,
                                              int n, int Ns, int R, const float2 *__restrict__ tw, bool inv) {
    const int nb = n / R;
    const int total = nlines * nb;
    const int twstride = n / (Ns * R);
    const int rstride = n / R;  // W_R^e = tw[e * n / R]
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int l = idx / nb;
        const int j = idx - l * nb;
        const float2 *src = in + (size_t)l * ls;
        float2 *dst = out + (size_t)l * ls;
        const int k = j % Ns;
        const int o = (j / Ns) * Ns * R + k;
        for (int q = 0; q < R; ++q) {
            float2 acc = make_float2(0.f, 0.f);
            for (int t = 0; t < R; ++t) {
                float2 x = src[j + t * nb];
                if (Ns > 1 && t > 0) {
                    float2 w = __ldg(tw + t * k * twstride);
                    if (inv) w.y = -w.y;
                    x = cmul(x, w);
                }
                float2 w = __ldg(tw + ((t * q) % R) * rstride);
                if (inv) w.y = -w.y;
                acc = cadd(acc, cmul(x, w));
            }
            dst[o + q * Ns] = acc;
        }
    }
}

// Runs all stages; returns the buffer that holds the result (a or b).
// Must be called by every thread of the CTA (contains __syncthreads).
__device__ __forceinline__ float2 *fft_lines(float2 *a, float2 *b, int nlines, int ls, const FftPlan &p, bool inv) {
    int Ns = 1;
    for (int s = 0; s < p.nstages; ++s) {
        const int R = p.radix[s];
        if (R == 8) stage_fixed<8>(a, b, nlines, ls, p.n, Ns, p.tw, inv);
        else if (R == 4) stage_fixed<4>(a, b, nlines, ls, p.n, Ns, p.tw, inv);
        else if (R == 2) stage_fixed<2>(a, b, nlines, ls, p.n, Ns, p.tw, inv);
        else stage_generic(a, b, nlines, ls, p.n, Ns, R, p.tw, inv);
        __syncthreads();
        float2 *t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

}  // namespace fm
