// fft_pair.cuh -- FFT butterflies on two independent complex lines at once, in the
// packed FP32x2 instructions of sm_100 and later (FADD2 / FMUL2 / FFMA2 through
// __fadd2_rn, __fmul2_rn, __ffma2_rn).
//
// A pair value cp2 holds element e of line A and element e of line B: lane A in .x and
// lane B in .y of both the real pair and the imaginary pair.  Every complex add of the
// two lines is then two packed instructions instead of four scalar ones, and a multiply
// by a twiddle shared by both lines is four instead of eight.  The passes that use it
// pair lines that share their twiddles (and, in the convolution passes, their kernel
// values): the y-frequencies ky and py - ky of the z pass.  Each packed operation rounds
// every lane exactly like its scalar counterpart (__fadd_rn, __fmul_rn, __fmaf_rn).
//
// In shared memory a pair element is one float4 {re_A, re_B, im_A, im_B}: one 128-bit
// access moves both lines.
#pragma once
#include <cuda_runtime.h>

#include "fft_smem.cuh"

namespace fm {

struct cp2 {
    float2 re, im;
};

__device__ __forceinline__ float2 pb(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 pneg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ cp2 padd(cp2 a, cp2 b) { return {__fadd2_rn(a.re, b.re), __fadd2_rn(a.im, b.im)}; }
__device__ __forceinline__ cp2 psub(cp2 a, cp2 b) { return {__fadd2_rn(a.re, pneg(b.re)), __fadd2_rn(a.im, pneg(b.im))}; }
// a * (c + i s), the same factor in both lanes
__device__ __forceinline__ cp2 pmulw(cp2 a, float c, float s) {
    return {__ffma2_rn(a.im, pb(-s), __fmul2_rn(a.re, pb(c))), __ffma2_rn(a.im, pb(c), __fmul2_rn(a.re, pb(s)))};
}
// a * conj(w) / a * w for a table twiddle w
__device__ __forceinline__ cp2 pmulw(cp2 a, float2 w, bool conj) { return pmulw(a, w.x, conj ? -w.y : w.y); }
// -i a (forward) or +i a (inverse): a swap and a sign
__device__ __forceinline__ cp2 pmul_mi(cp2 a, bool inv) { return inv ? cp2{pneg(a.im), a.re} : cp2{a.im, pneg(a.re)}; }
__device__ __forceinline__ cp2 pzero() { return {make_float2(0.f, 0.f), make_float2(0.f, 0.f)}; }
// pack element values of line A and line B / unpack them
__device__ __forceinline__ cp2 ppack(float2 a, float2 b) { return {make_float2(a.x, b.x), make_float2(a.y, b.y)}; }
__device__ __forceinline__ float2 plane_a(cp2 v) { return make_float2(v.re.x, v.im.x); }
__device__ __forceinline__ float2 plane_b(cp2 v) { return make_float2(v.re.y, v.im.y); }
__device__ __forceinline__ float4 pstore(cp2 v) { return make_float4(v.re.x, v.re.y, v.im.x, v.im.y); }
__device__ __forceinline__ cp2 pload(float4 f) { return {make_float2(f.x, f.y), make_float2(f.z, f.w)}; }

template <int R>
__device__ __forceinline__ void pdft(cp2 *v, bool inv);

template <>
__device__ __forceinline__ void pdft<2>(cp2 *v, bool) {
    const cp2 a = v[0], b = v[1];
    v[0] = padd(a, b);
    v[1] = psub(a, b);
}

template <>
__device__ __forceinline__ void pdft<4>(cp2 *v, bool inv) {
    const cp2 a0 = padd(v[0], v[2]), a1 = psub(v[0], v[2]);
    const cp2 b0 = padd(v[1], v[3]), b1 = pmul_mi(psub(v[1], v[3]), inv);
    v[0] = padd(a0, b0);
    v[2] = psub(a0, b0);
    v[1] = padd(a1, b1);
    v[3] = psub(a1, b1);
}

template <>
__device__ __forceinline__ void pdft<8>(cp2 *v, bool inv) {
    // radix-2 decimation in frequency, then two 4-point DFTs
    const float h = 0.70710678118654752440f;
    cp2 a[4], b[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        a[t] = padd(v[t], v[t + 4]);
        b[t] = psub(v[t], v[t + 4]);
    }
    // b[t] *= W8^t (W8 = e^{-i pi/4} forward, its conjugate inverse)
    b[1] = pmulw(b[1], h, inv ? h : -h);
    b[2] = pmul_mi(b[2], inv);
    b[3] = pmulw(b[3], -h, inv ? h : -h);
    pdft<4>(a, inv);
    pdft<4>(b, inv);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        v[2 * q] = a[q];
        v[2 * q + 1] = b[q];
    }
}

template <>
__device__ __forceinline__ void pdft<16>(cp2 *v, bool inv) {
    // 16 = 4 x 4: x index 4 n1 + n2, output index k1 + 4 k2 (as dft_small<16>)
    const float c16[10] = {1.0f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f, 0.0f,
                           -0.38268343236508977f, -0.70710678118654752f, -0.92387953251128674f, -1.0f,
                           -0.92387953251128674f};
    const float s16[10] = {0.0f, 0.38268343236508977f, 0.70710678118654752f, 0.92387953251128674f, 1.0f,
                           0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f, 0.0f,
                           -0.38268343236508977f};
    cp2 t[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
        cp2 a[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
        pdft<4>(a, inv);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            const int e = n2 * k1;
            if (e == 0) t[n2][k1] = a[k1];
            else if (e == 4) t[n2][k1] = pmul_mi(a[k1], inv);
            else t[n2][k1] = pmulw(a[k1], c16[e], inv ? s16[e] : -s16[e]);
        }
    }
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        cp2 b[4] = {t[0][k1], t[1][k1], t[2][k1], t[3][k1]};
        pdft<4>(b, inv);
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = b[k2];
    }
}

// Pruned two-level forms of half_dft_store / half_idft_load (fft_smem.cuh) on pairs; the
// line holds pair elements as float4 at line[sk(k1 * N2 + n2)].
template <int N1, int N2>
__device__ __forceinline__ void phalf_dft_store(cp2 (&e)[N1 / 2], int n2, float4 *line, const float2 *__restrict__ tw) {
    constexpr int H1 = N1 / 2;
    cp2 o[H1];
    o[0] = e[0];
#pragma unroll
    for (int n1 = 1; n1 < H1; ++n1) o[n1] = pmulw(e[n1], __ldg(tw + n1 * N2), false);
    pdft<H1>(e, false);
    pdft<H1>(o, false);
#pragma unroll
    for (int u = 0; u < H1; ++u) {
        const int ka = 2 * u, kb = 2 * u + 1;
        line[sk(ka * N2 + n2)] = pstore((n2 && ka) ? pmulw(e[u], __ldg(tw + n2 * ka), false) : e[u]);
        line[sk(kb * N2 + n2)] = pstore(n2 ? pmulw(o[u], __ldg(tw + n2 * kb), false) : o[u]);
    }
}

template <int N1, int N2>
__device__ __forceinline__ void phalf_idft_load(cp2 (&e)[N1 / 2], int n2, const float4 *line,
                                                const float2 *__restrict__ tw) {
    constexpr int H1 = N1 / 2;
    cp2 o[H1];
#pragma unroll
    for (int u = 0; u < H1; ++u) {
        e[u] = pload(line[sk(2 * u * N2 + n2)]);
        o[u] = pload(line[sk((2 * u + 1) * N2 + n2)]);
    }
    pdft<H1>(e, true);
    pdft<H1>(o, true);
    e[0] = padd(e[0], o[0]);
#pragma unroll
    for (int n1 = 1; n1 < H1; ++n1) e[n1] = padd(e[n1], pmulw(o[n1], __ldg(tw + n1 * N2), true));
}

}  // namespace fm
