// fft_smem.cuh -- shared-memory Stockham FFT used by every demag pass.
//
// A CTA transforms `nlines` complex lines of length n that sit in shared
// memory, ping-ponging between two buffers.  Element e of line l lives at
// buf[l * ls + sk(e)]: one float2 of padding after every 16 elements keeps the
// stride-R writes of the early Stockham stages off a single pair of banks
// (ls >= skewed_len(n)).  Each stage of radix R is one sweep of n/R butterflies
// per line; the Stockham index map keeps the result in natural order.
//
// Power-of-two lengths (every padded extent of the reference's 2n grids when n
// is a power of two) take a compile-time path: radix-16 stages where possible,
// then radix 8 or 4 (pow2_radix: never a lone radix-2 stage), all index
// arithmetic folded to shifts and masks.  Other lengths use the runtime path
// with radices 8, 4, 2 and an O(R^2) loop for any other prime factor.  Twiddles are FP64-computed host-side and stored as
// float2 e^{-2 pi i e / n}; the inverse conjugates them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fm {

constexpr int kMaxStages = 24;
constexpr int kMaxGenericRadix = 64;

struct FftPlan {
    int n;
    int nstages;
    int log2n;  // >= 0 when n is a power of two, else -1
    int radix[kMaxStages];
    const float2 *tw;  // n entries, e^{-2 pi i e / n}
};

// Division by a runtime divisor d >= 1 through a precomputed multiplier
// (round-up reciprocal method: q = (umulhi(n, m) + n) >> s with
// s = ceil(log2 d), m = floor(2^32 (2^s - d) / d) + 1), exact for n < 2^31.
struct FastDiv {
    uint32_t d = 1, m = 1, s = 0;
    FastDiv() = default;
    __host__ explicit FastDiv(uint32_t div) : d(div) {
        s = 0;
        while ((1ull << s) < div) ++s;
        m = (uint32_t)(((1ull << 32) * ((1ull << s) - div)) / div + 1);
    }
    __device__ __forceinline__ int div(int n) const {
        return (int)((__umulhi((uint32_t)n, m) + (uint32_t)n) >> s);
    }
    __device__ __forceinline__ int mod(int n, int q) const { return n - q * (int)d; }
};

__host__ __device__ __forceinline__ int sk(int e) { return e + (e >> 4); }

// Gather `total` elements: B independent loads per thread are issued before any of
// them is consumed, so each thread keeps B requests in flight (the passes are
// latency-bound otherwise: one outstanding load per thread at 2-4 CTAs per SM).
template <int B, typename Load, typename Store>
__device__ __forceinline__ void batched_copy(int total, Load ld, Store st) {
    for (int base = threadIdx.x; base < total; base += B * blockDim.x) {
        float2 v[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int idx = base + u * (int)blockDim.x;
            if (idx < total) v[u] = ld(idx);
        }
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int idx = base + u * (int)blockDim.x;
            if (idx < total) st(idx, v[u]);
        }
    }
}

// Compensated float-float accumulation (Knuth TwoSum): hi + lo carries the sum of
// every added value with error ~ n * eps^2 instead of n * eps, using FP32 pipes only.
__device__ __forceinline__ void ff_add(float &hi, float &lo, float v) {
    const float s = hi + v;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (v - bb);
    hi = s;
    lo += e;
}
__host__ __device__ constexpr int skewed_len(int n) { return n + (n >> 4) + 1; }

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

template <>
__device__ __forceinline__ void dft_small<16>(float2 *v, bool inv) {
    // 16 = 4 x 4: x index 4*n1 + n2, output index k1 + 4*k2
    //   X[k1 + 4 k2] = sum_n2 W4^{n2 k2} W16^{n2 k1} sum_n1 x[4 n1 + n2] W4^{n1 k1}
    // cos / sin of 2 pi e / 16 for e = n2 * k1 in [0, 9]
    const float c16[10] = {1.0f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f, 0.0f,
                           -0.38268343236508977f, -0.70710678118654752f, -0.92387953251128674f, -1.0f,
                           -0.92387953251128674f};
    const float s16[10] = {0.0f, 0.38268343236508977f, 0.70710678118654752f, 0.92387953251128674f, 1.0f,
                           0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f, 0.0f,
                           -0.38268343236508977f};
    float2 t[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
        float2 a[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
        dft_small<4>(a, inv);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            const int e = n2 * k1;
            if (e == 0) {
                t[n2][k1] = a[k1];
            } else {
                // W16^e = cos - i sin (forward), cos + i sin (inverse)
                const float2 w = make_float2(c16[e], inv ? s16[e] : -s16[e]);
                t[n2][k1] = cmul(a[k1], w);
            }
        }
    }
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        float2 b[4] = {t[0][k1], t[1][k1], t[2][k1], t[3][k1]};
        dft_small<4>(b, inv);
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = b[k2];
    }
}

// radix of the next power-of-two stage given the remaining length 2^m:
// radix 16 where possible, never a lone radix-2 stage (2^5 -> 8 x 4, 2^9 -> 16 x 8 x 4)
__host__ __device__ constexpr int pow2_radix(int rem) {
    return rem >= 16 && rem != 32 ? 16 : (rem >= 8 ? 8 : rem);
}

// ---- pruned two-level transforms (power-of-two lengths N = N1 * N2) ----
// With n = N2 n1 + n2 and k = k1 + N1 k2:
//   X[k1 + N1 k2] = sum_n2 W_N2^{n2 k2} W_N^{n2 k1} sum_n1 x[N2 n1 + n2] W_N1^{n1 k1}.
// Inputs vanish for n >= N/2 (n1 >= N1/2) on the forward side and only n < N/2 is kept
// on the inverse side, so the outer N1-point passes run on half lines.  tw holds the N
// twiddles e^{-2 pi i e / N}.

// Half-input N1-point DFT of e[0..N1/2) (two N1/2-point DFTs: even and odd outputs),
// times W_N^{n2 k1}, stored at line[sk(k1 * N2 + n2)].
template <int N1, int N2>
__device__ __forceinline__ void half_dft_store(float2 (&e)[N1 / 2], int n2, float2 *line, const float2 *__restrict__ tw) {
    constexpr int H1 = N1 / 2;
    float2 o[H1];
    o[0] = e[0];
#pragma unroll
    for (int n1 = 1; n1 < H1; ++n1) o[n1] = cmul(e[n1], __ldg(tw + n1 * N2));
    dft_small<H1>(e, false);
    dft_small<H1>(o, false);
#pragma unroll
    for (int u = 0; u < H1; ++u) {
        const int ka = 2 * u, kb = 2 * u + 1;
        line[sk(ka * N2 + n2)] = (n2 && ka) ? cmul(e[u], __ldg(tw + n2 * ka)) : e[u];
        line[sk(kb * N2 + n2)] = n2 ? cmul(o[u], __ldg(tw + n2 * kb)) : o[u];
    }
}

// Half-output inverse N1-point DFT over line[sk(k1 * N2 + n2)], k1 in [0, N1): returns
// y[n1] for n1 < N1/2 in e (two N1/2-point inverses combined with W_N1^{-n1}).
template <int N1, int N2>
__device__ __forceinline__ void half_idft_load(float2 (&e)[N1 / 2], int n2, const float2 *line,
                                               const float2 *__restrict__ tw) {
    constexpr int H1 = N1 / 2;
    float2 o[H1];
#pragma unroll
    for (int u = 0; u < H1; ++u) {
        e[u] = line[sk(2 * u * N2 + n2)];
        o[u] = line[sk((2 * u + 1) * N2 + n2)];
    }
    dft_small<H1>(e, true);
    dft_small<H1>(o, true);
    e[0] = cadd(e[0], o[0]);
#pragma unroll
    for (int n1 = 1; n1 < H1; ++n1) e[n1] = cadd(e[n1], cmul(o[n1], cconj(__ldg(tw + n1 * N2))));
}

// ---- runtime-length path ----

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
        for (int t = 0; t < R; ++t) v[t] = src[sk(j + t * nb)];
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
        for (int t = 0; t < R; ++t) dst[sk(o + t * Ns)] = v[t];
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
                float2 x = src[sk(j + t * nb)];
                if (Ns > 1 && t > 0) {
                    float2 w = __ldg(tw + t * k * twstride);
                    if (inv) w.y = -w.y;
                    x = cmul(x, w);
                }
                float2 w = __ldg(tw + ((t * q) % R) * rstride);
                if (inv) w.y = -w.y;
                acc = cadd(acc, cmul(x, w));
            }
            dst[sk(o + q * Ns)] = acc;
        }
    }
}

// ---- compile-time power-of-two path ----

template <int L, int R, int NS, bool INV>
__device__ __forceinline__ void stage_pow2(const float2 *__restrict__ in, float2 *__restrict__ out, int nlines, int ls,
                                           const float2 *__restrict__ tw) {
    constexpr int NB = L / R;
    constexpr int TWS = L / (NS * R);
    const int total = nlines * NB;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int l = idx / NB;
        const int j = idx % NB;
        const float2 *src = in + l * ls;
        float2 *dst = out + l * ls;
        const int k = j % NS;
        float2 v[R];
#pragma unroll
        for (int t = 0; t < R; ++t) v[t] = src[sk(j + t * NB)];
        if (NS > 1) {
#pragma unroll
            for (int t = 1; t < R; ++t) {
                float2 w = __ldg(tw + t * k * TWS);
                if (INV) w.y = -w.y;
                v[t] = cmul(v[t], w);
            }
        }
        dft_small<R>(v, INV);
        const int o = (j / NS) * NS * R + k;
#pragma unroll
        for (int t = 0; t < R; ++t) dst[sk(o + t * NS)] = v[t];
    }
}

template <int L, int NS, bool INV>
__device__ __forceinline__ float2 *stages_pow2(float2 *a, float2 *b, int nlines, int ls, const float2 *tw) {
    if constexpr (NS >= L) {
        return a;
    } else {
        constexpr int REM = L / NS;
        constexpr int R = pow2_radix(REM);
        stage_pow2<L, R, NS, INV>(a, b, nlines, ls, tw);
        __syncthreads();
        return stages_pow2<L, NS * R, INV>(b, a, nlines, ls, tw);
    }
}

template <bool INV>
__device__ __forceinline__ float2 *fft_pow2_dispatch(int log2n, float2 *a, float2 *b, int nlines, int ls,
                                                     const float2 *tw) {
    switch (log2n) {
        case 1: return stages_pow2<2, 1, INV>(a, b, nlines, ls, tw);
        case 2: return stages_pow2<4, 1, INV>(a, b, nlines, ls, tw);
        case 3: return stages_pow2<8, 1, INV>(a, b, nlines, ls, tw);
        case 4: return stages_pow2<16, 1, INV>(a, b, nlines, ls, tw);
        case 5: return stages_pow2<32, 1, INV>(a, b, nlines, ls, tw);
        case 6: return stages_pow2<64, 1, INV>(a, b, nlines, ls, tw);
        case 7: return stages_pow2<128, 1, INV>(a, b, nlines, ls, tw);
        case 8: return stages_pow2<256, 1, INV>(a, b, nlines, ls, tw);
        case 9: return stages_pow2<512, 1, INV>(a, b, nlines, ls, tw);
        case 10: return stages_pow2<1024, 1, INV>(a, b, nlines, ls, tw);
        case 11: return stages_pow2<2048, 1, INV>(a, b, nlines, ls, tw);
        case 12: return stages_pow2<4096, 1, INV>(a, b, nlines, ls, tw);
        default: return a;
    }
}

// Runs all stages; returns the buffer that holds the result (a or b).
// Must be called by every thread of the CTA (contains __syncthreads).
__device__ __forceinline__ float2 *fft_lines(float2 *a, float2 *b, int nlines, int ls, const FftPlan &p, bool inv) {
    if (p.log2n >= 1 && p.log2n <= 12) {
        return inv ? fft_pow2_dispatch<true>(p.log2n, a, b, nlines, ls, p.tw)
                   : fft_pow2_dispatch<false>(p.log2n, a, b, nlines, ls, p.tw);
    }
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
