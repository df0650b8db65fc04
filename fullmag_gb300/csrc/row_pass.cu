// row_pass.cu -- the fused per-row pass: inverse x-transform of the demag
// spectrum, exchange + Zeeman + anisotropy + LLG torque, FP64 statistics,
// next-stage combination and forward x-transform.
//
// Reference behaviour restated here (paths in mzrptu/fullmag):
//   exchange stencil, Neumann clamp, mask      native/backends/fdm/src/exchange_fp32.cu:21-122
//                                              crates/fullmag-engine/src/fdm_fields.rs:445-527
//   zero-padded tensor convolution             native/backends/fdm/src/demag_fp32.cu:50-199,406-502
//                                              crates/fullmag-engine/src/fdm_fields.rs:528-609
//   Zeeman + uniaxial + cubic local terms      native/backends/fdm/src/demag_fp32.cu:201-318
//   LLG right-hand side                        native/backends/fdm/src/llg_fp32.cu:32-60
//                                              crates/fullmag-engine/src/fdm_fields.rs:2151-2162
//   stage combination with normalisation      native/backends/fdm/src/llg_fp32.cu:204-261,
//                                              llg_rk4_fp32.cu:37-80, llg_dp45_fp32.cu:37-106
//   energies and max norms (FP64 accumulate)   native/backends/fdm/src/reductions_fp64.cu:123-342,605-642
//   DP45 error norm                            native/backends/fdm/src/llg_dp45_fp32.cu:108-128,175-184
// The structure is new: the x-transforms live inside the per-row pass, the
// y/z transforms and the tensor multiply live in column passes, and no
// padded real-space array or cuFFT plan exists.
#include "engine.h"

#include <cfloat>

namespace fm {

namespace {

constexpr int kThreads = 256;
constexpr int kRowVec = 4;  // cells per thread on the unmasked path (2 measured slower)
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// a / (2i) = -i a / 2
__device__ __forceinline__ float2 div2i(float2 a) { return make_float2(0.5f * a.y, -0.5f * a.x); }
__device__ __forceinline__ float2 mul_i(float2 a) { return make_float2(-a.y, a.x); }

__device__ __forceinline__ bool cell_active(const uint8_t *mask, long long i) { return mask == nullptr || mask[i] != 0; }

// butterfly all-reduce of a float-float value; every lane ends with the same bits
// because each level combines the pair in lane order
__device__ __forceinline__ void warp_ff_sum(float &h, float &l) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, h, o);
        const float ol = __shfl_xor_sync(0xffffffffu, l, o);
        const bool low = (threadIdx.x & o) == 0;
        float ah = low ? h : oh, al = low ? l : ol;
        const float bh = low ? oh : h, bl = low ? ol : l;
        ff_add(ah, al, bh);
        h = ah;
        l = al + bl;
    }
}
__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// ---- x-transforms in the pruned two-level form (half = px/2 = N1 * N2, a power of two) ----
// The real x line of length px is carried as the half-length complex line
// z[j] = s[2j] + i s[2j+1]; its nonzero samples are j < nx/2 <= half/2 and only those
// are needed after the inverse, so both outer passes run on half lines
// (half_dft_store / half_idft_load).

__host__ __device__ __forceinline__ bool row_x_fused_ok(const Grid &g) {
    const int h = g.half;
    return (h == 16 || h == 32 || h == 64 || h == 128 || h == 256) && g.nx <= h;
}

// X rows (global, nkx = half + 1 values per line) -> H_d samples in
// hd[line*lsx + sk(x/2)] (.x for even x, .y for odd x), x < nx.  Phase A (line, k1):
// Z[k] = (a + b') + i (a - b') conj(e^{-2 pi i k/px}), a = X[k], b' = conj(X[half-k]),
// for k = k1 + N1 k2 from global loads, inverse N2-point DFT, conjugate twiddle;
// phase B (line, n2): half-output outer inverse.
template <int N1, int N2>
__device__ __forceinline__ void row_inverse_x(const RowPass &p, int rows, int row0, float2 *slots, float2 *hd) {
    constexpr int half = N1 * N2, H1 = N1 / 2;
    constexpr int lsx = skewed_len(half);
    const Grid &g = p.g;
    const int nkx = g.nkx, nrows = g.ny * g.nz, nl = rows * 3;
    const float2 *__restrict__ tw = p.xplan.tw;
    for (int it = threadIdx.x; it < nl * N1; it += blockDim.x) {
        const int line = it / N1, k1 = it & (N1 - 1);
        const int rr = line / 3, c = line - 3 * rr;
        const float2 *X = p.x_in + ((size_t)c * nrows + row0 + rr) * nkx;
        float2 v[N2];
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) {
            const int k = k1 + N1 * k2;
            const float2 a = X[k];
            const float2 b = cconj(X[half - k]);
            const float2 O = cmul(csub(a, b), cconj(__ldg(p.xpost + k)));
            v[k2] = cadd(cadd(a, b), mul_i(O));
        }
        dft_small<N2>(v, true);
        float2 *sl = slots + line * lsx;
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) sl[sk(k1 * N2 + n2)] = (n2 && k1) ? cmul(v[n2], cconj(__ldg(tw + n2 * k1))) : v[n2];
    }
    __syncthreads();
    for (int it = threadIdx.x; it < nl * N2; it += blockDim.x) {
        const int line = it / N2, n2 = it & (N2 - 1);
        float2 e[H1];
        half_idft_load<N1, N2>(e, n2, slots + line * lsx, tw);
        float2 *h = hd + line * lsx;
#pragma unroll
        for (int j1 = 0; j1 < H1; ++j1) h[sk(N2 * j1 + n2)] = e[j1];
    }
    __syncthreads();
}

// Next-stage samples s[x], x < nx, in pack[line*lsx + sk(x/2)] -> X rows (global).
// Phase 1 (line, n2): half-input outer DFT of z[j], j < half/2 (samples x >= nx read
// as zero); phase 2 (line, k1): inner N2-point DFTs into natural order; phase 3
// (line, k): the real-to-half-spectrum split
// X[k] = (Z[k] + Z'[k])/2 + e^{-2 pi i k/px} (Z[k] - Z'[k])/(2i), Z'[k] = conj(Z[half-k]).
template <int N1, int N2>
__device__ __forceinline__ void row_forward_x(const RowPass &p, int rows, int row0, float2 *pack, float2 *slots) {
    constexpr int half = N1 * N2, H1 = N1 / 2;
    constexpr int lsx = skewed_len(half);
    const Grid &g = p.g;
    const int nx = g.nx, nkx = g.nkx, nrows = g.ny * g.nz, nl = rows * 3;
    const float2 *__restrict__ tw = p.xplan.tw;
    for (int it = threadIdx.x; it < nl * N2; it += blockDim.x) {
        const int line = it / N2, n2 = it & (N2 - 1);
        const float2 *src = pack + line * lsx;
        float2 e[H1];
#pragma unroll
        for (int j1 = 0; j1 < H1; ++j1) {
            const int j = N2 * j1 + n2;
            float2 v = src[sk(j)];
            if (2 * j + 1 >= nx) {
                v.y = 0.f;
                if (2 * j >= nx) v.x = 0.f;
            }
            e[j1] = v;
        }
        half_dft_store<N1, N2>(e, n2, slots + line * lsx, tw);
    }
    __syncthreads();
    for (int it = threadIdx.x; it < nl * N1; it += blockDim.x) {
        const int line = it / N1, k1 = it & (N1 - 1);
        const float2 *sl = slots + line * lsx;
        float2 v[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) v[n2] = sl[sk(k1 * N2 + n2)];
        dft_small<N2>(v, false);
        float2 *z = pack + line * lsx;
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) z[sk(k1 + N1 * k2)] = v[k2];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < nl * nkx; idx += blockDim.x) {
        const int line = g.fd_nkx.div(idx);
        const int k = idx - line * nkx;
        const int rr = line / 3;
        const int c = line - rr * 3;
        const float2 *zl = pack + line * lsx;
        const float2 a = zl[sk(k == half ? 0 : k)];
        const float2 b = cconj(zl[sk(k == 0 ? 0 : half - k)]);
        const float2 E = cscale(cadd(a, b), 0.5f);
        const float2 O = div2i(csub(a, b));
        p.x_out[((size_t)c * nrows + row0 + rr) * nkx + k] = cadd(E, cmul(__ldg(p.xpost + k), O));
    }
}

__device__ __forceinline__ void row_inverse_x_fused(const RowPass &p, int rows, int row0, float2 *slots, float2 *hd) {
    switch (p.g.half) {
        case 16: row_inverse_x<4, 4>(p, rows, row0, slots, hd); break;
        case 32: row_inverse_x<8, 4>(p, rows, row0, slots, hd); break;
        case 64: row_inverse_x<8, 8>(p, rows, row0, slots, hd); break;
        case 128: row_inverse_x<16, 8>(p, rows, row0, slots, hd); break;
        default: row_inverse_x<16, 16>(p, rows, row0, slots, hd); break;
    }
}

__device__ __forceinline__ void row_forward_x_fused(const RowPass &p, int rows, int row0, float2 *pack, float2 *slots) {
    switch (p.g.half) {
        case 16: row_forward_x<4, 4>(p, rows, row0, pack, slots); break;
        case 32: row_forward_x<8, 4>(p, rows, row0, pack, slots); break;
        case 64: row_forward_x<8, 8>(p, rows, row0, pack, slots); break;
        case 128: row_forward_x<16, 8>(p, rows, row0, pack, slots); break;
        default: row_forward_x<16, 16>(p, rows, row0, pack, slots); break;
    }
}

// Adjoint helpers (the element-wise equations of adjoint.cu, inlined into the row pass)
struct A3 {
    float x, y, z;
};
__device__ __forceinline__ A3 a3_ld(const float *a, long long n, long long i) { return {a[i], a[n + i], a[2 * n + i]}; }
__device__ __forceinline__ void a3_st(float *a, long long n, long long i, A3 v) {
    a[i] = v.x;
    a[n + i] = v.y;
    a[2 * n + i] = v.z;
}
__device__ __forceinline__ A3 a3_cross(A3 a, A3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float a3_dot(A3 a, A3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ A3 a3_axpy(float s, A3 a, A3 b) { return {s * a.x + b.x, s * a.y + b.y, s * a.z + b.z}; }

// ---- per-cell work on V consecutive cells per thread ----
// Unmasked grids with nx a multiple of V and at least one group of V cells per thread
// (the 256x256x64 volume) take this path: every x-contiguous array (state, its y+-1 and
// z+-1 neighbour rows, stage derivatives, field map, outputs) moves as one V-wide vector
// per component, the x-neighbours come from the same registers (two scalar loads at the
// group's ends), and the row / column index arithmetic is done once per group.  Every
// buffer is a 256-byte aligned arena slice of 3n floats and n is a multiple of V, so the
// vector accesses are aligned.  The per-cell arithmetic is the scalar loop's; only the
// forward-pair exchange energy sums its terms per component first.
template <int V>
__device__ __forceinline__ void ldv(const float *p, float (&v)[V]) {
    if constexpr (V == 4) {
        const float4 a = *reinterpret_cast<const float4 *>(p);
        v[0] = a.x;
        v[1] = a.y;
        v[2] = a.z;
        v[3] = a.w;
    } else {
        const float2 a = *reinterpret_cast<const float2 *>(p);
        v[0] = a.x;
        v[1] = a.y;
    }
}
template <int V>
__device__ __forceinline__ void stv(float *p, const float (&v)[V]) {
    if constexpr (V == 4)
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    else
        *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]);
}

template <int V>
__device__ __forceinline__ void cells_vec(const RowPass &p, int rows, int row0, const float2 *hd, float2 *pack, int lsx,
                                           float (&sum_hi)[5], float (&sum_lo)[5], float (&mx2)[4], float dt_f,
                                           double err_dt) {
    const Grid &g = p.g;
    const Material &M = p.mat;
    const int nx = g.nx, nxv = nx / V, ny = g.ny, nz = g.nz;
    const long long n = g.n;
    const int plane = nx * ny;
    for (int gi = threadIdx.x; gi < rows * nxv; gi += blockDim.x) {
        const int rr = (V == 4 ? g.fd_nx4 : g.fd_nx2).div(gi);
        const int x0 = (gi - rr * nxv) * V;
        const int row = row0 + rr;
        const int z = g.fd_ny.div(row);
        const int y = row - z * ny;
        const long long i0 = (long long)row * nx + x0;
        float kv[3][V] = {};
        if (p.m_in) {
            // per component: exchange Laplacian, demag, external and map fields summed into
            // h in the scalar loop's order; m.h_d, |h_d|^2 and the forward-pair |dm|^2
            // accumulate across the components (clamped neighbours give zero differences,
            // so the last cell of a row / column / plane needs no mask)
            float m0v[3][V], hv[3][V], e_pair[V];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float *mc = p.m_in + c * n;
                float cc[V], ex[V], dv[V];
                ldv<V>(mc + i0, cc);
#pragma unroll
                for (int j = 0; j < V; ++j) m0v[c][j] = cc[j];
                if (M.ex_pref != 0.f) {
                    float ym[V], yp[V], zm[V], zp[V], xm[V], xp[V];
                    // open axes clamp (Neumann), periodic axes wrap around
                    const int per = g.per;
                    ldv<V>(mc + i0 + (y > 0 ? -nx : (per & 2) ? plane - nx : 0), ym);
                    ldv<V>(mc + i0 + (y < ny - 1 ? nx : (per & 2) ? nx - plane : 0), yp);
                    ldv<V>(mc + i0 + (z > 0 ? -(long long)plane : (per & 4) ? (long long)plane * (nz - 1) : 0), zm);
                    ldv<V>(mc + i0 + (z < nz - 1 ? (long long)plane : (per & 4) ? -(long long)plane * (nz - 1) : 0), zp);
                    xm[0] = x0 > 0 ? mc[i0 - 1] : (per & 1) ? mc[i0 + nx - 1] : cc[0];
                    xp[V - 1] = x0 + V < nx ? mc[i0 + V] : (per & 1) ? mc[i0 + V - nx] : cc[V - 1];
#pragma unroll
                    for (int j = 1; j < V; ++j) {
                        xm[j] = cc[j - 1];
                        xp[j - 1] = cc[j];
                    }
#pragma unroll
                    for (int j = 0; j < V; ++j) {
                        ex[j] = M.ex_pref * ((xp[j] - 2.f * cc[j] + xm[j]) * M.idx2 + (yp[j] - 2.f * cc[j] + ym[j]) * M.idy2 +
                                             (zp[j] - 2.f * cc[j] + zm[j]) * M.idz2);
                        if (p.partials) {
                            const float d0 = xp[j] - cc[j], d1 = yp[j] - cc[j], d2 = zp[j] - cc[j];
                            const float t = d0 * d0 * M.idx2 + d1 * d1 * M.idy2 + d2 * d2 * M.idz2;
                            e_pair[j] = c ? e_pair[j] + t : t;
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < V; ++j) {
                        ex[j] = 0.f;
                        e_pair[j] = 0.f;
                    }
                }
                if (hd) {
#pragma unroll
                    for (int j = 0; j < V; j += 2) {
                        const float2 h2 = hd[(rr * 3 + c) * lsx + sk((x0 + j) >> 1)];
                        dv[j] = h2.x;
                        dv[j + 1] = h2.y;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < V; ++j) dv[j] = 0.f;
                }
                float hm[V];
                if (p.hmap) ldv<V>(p.hmap + c * n + i0, hm);
#pragma unroll
                for (int j = 0; j < V; ++j) {
                    float h = ex[j] + dv[j];
                    if (M.has_ext) h += M.hext[c];
                    if (p.hmap) h += hm[j];
                    hv[c][j] = h;
                }
                if (p.h_ex_out) stv<V>(p.h_ex_out + c * n + i0, ex);
                if (p.h_d_out) stv<V>(p.h_d_out + c * n + i0, dv);
            }
#pragma unroll
            for (int j = 0; j < V; ++j) {
                const float m0x = m0v[0][j], m0y = m0v[1][j], m0z = m0v[2][j];
                float hx = hv[0][j], hy = hv[1][j], hz = hv[2][j];
                float e_uni = 0.f, e_cub = 0.f;
                if (M.has_uni) {
                    const float mu = m0x * M.u[0] + m0y * M.u[1] + m0z * M.u[2];
                    const float cf = M.ku1c * mu + M.ku2c * mu * mu * mu;
                    hx += cf * M.u[0];
                    hy += cf * M.u[1];
                    hz += cf * M.u[2];
                    const float s = mu * mu;
                    e_uni = M.ku1f * s + M.ku2f * s * s;
                }
                if (M.has_cub) {
                    const float a1 = m0x * M.c1[0] + m0y * M.c1[1] + m0z * M.c1[2];
                    const float a2 = m0x * M.c2[0] + m0y * M.c2[1] + m0z * M.c2[2];
                    const float a3 = m0x * M.c3[0] + m0y * M.c3[1] + m0z * M.c3[2];
                    const float s1 = a1 * a1, s2 = a2 * a2, s3 = a3 * a3;
                    const float sig = s1 * s2 + s2 * s3 + s1 * s3;
                    const float g1 = M.kc1c * a1 * (s2 + s3) + M.kc2c * a1 * s2 * s3 + M.kc3c * sig * a1 * (s2 + s3);
                    const float g2 = M.kc1c * a2 * (s1 + s3) + M.kc2c * a2 * s1 * s3 + M.kc3c * sig * a2 * (s1 + s3);
                    const float g3 = M.kc1c * a3 * (s1 + s2) + M.kc2c * a3 * s1 * s2 + M.kc3c * sig * a3 * (s1 + s2);
                    hx += g1 * M.c1[0] + g2 * M.c2[0] + g3 * M.c3[0];
                    hy += g1 * M.c1[1] + g2 * M.c2[1] + g3 * M.c3[1];
                    hz += g1 * M.c1[2] + g2 * M.c2[2] + g3 * M.c3[2];
                    e_cub = M.kc1f * sig + M.kc2f * s1 * s2 * s3 + M.kc3f * sig * sig;
                }
                const float px_ = m0y * hz - m0z * hy;
                const float py_ = m0z * hx - m0x * hz;
                const float pz_ = m0x * hy - m0y * hx;
                const float qx = m0y * pz_ - m0z * py_;
                const float qy = m0z * px_ - m0x * pz_;
                const float qz = m0x * py_ - m0y * px_;
                kv[0][j] = -M.gbar * (M.prec * px_ + M.alpha * qx);
                kv[1][j] = -M.gbar * (M.prec * py_ + M.alpha * qy);
                kv[2][j] = -M.gbar * (M.prec * pz_ + M.alpha * qz);
                if (p.partials) {
                    // H_d of this cell again from shared memory (no registers held across the loop)
                    float dx_ = 0.f, dy_ = 0.f, dz_ = 0.f;
                    if (hd) {
                        const int h = sk((x0 + j) >> 1);
                        const float2 a = hd[(rr * 3 + 0) * lsx + h], b = hd[(rr * 3 + 1) * lsx + h], d = hd[(rr * 3 + 2) * lsx + h];
                        dx_ = (j & 1) ? a.y : a.x;
                        dy_ = (j & 1) ? b.y : b.x;
                        dz_ = (j & 1) ? d.y : d.x;
                    }
                    ff_add(sum_hi[0], sum_lo[0], e_pair[j]);
                    ff_add(sum_hi[1], sum_lo[1], m0x * dx_ + m0y * dy_ + m0z * dz_);
                    if (M.has_ext) ff_add(sum_hi[2], sum_lo[2], m0x * M.hext[0] + m0y * M.hext[1] + m0z * M.hext[2]);
                    if (p.hmap) {
                        const long long i = i0 + j;
                        ff_add(sum_hi[2], sum_lo[2], m0x * p.hmap[i] + m0y * p.hmap[n + i] + m0z * p.hmap[2 * n + i]);
                    }
                    ff_add(sum_hi[3], sum_lo[3], e_uni);
                    ff_add(sum_hi[V], sum_lo[V], e_cub);
                    mx2[0] = fmaxf(mx2[0], hx * hx + hy * hy + hz * hz);
                    mx2[1] = fmaxf(mx2[1], dx_ * dx_ + dy_ * dy_ + dz_ * dz_);
                    mx2[2] = fmaxf(mx2[2], kv[0][j] * kv[0][j] + kv[1][j] * kv[1][j] + kv[2][j] * kv[2][j]);
                }
                if (p.h_eff_out) {
                    const long long i = i0 + j;
                    p.h_eff_out[i] = hx;
                    p.h_eff_out[n + i] = hy;
                    p.h_eff_out[2 * n + i] = hz;
                }
            }
            if (p.partials && p.n_err > 0) {
                // |dt sum_t e_t k_t|^2 per cell in FP64, one component at a time
                double esq[V];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    double e[V] = {};
                    for (int t = 0; t < p.n_err; ++t) {
                        const float *kk = p.err_k[t];
                        const double w = p.err_c[t];
                        float kc[V];
                        if (kk) ldv<V>(kk + c * n + i0, kc);
#pragma unroll
                        for (int j = 0; j < V; ++j) e[j] += w * (double)(kk ? kc[j] : kv[c][j]);
                    }
#pragma unroll
                    for (int j = 0; j < V; ++j) {
                        const double ej = e[j] * err_dt;
                        esq[j] = c ? esq[j] + ej * ej : ej * ej;
                    }
                }
#pragma unroll
                for (int j = 0; j < V; ++j) mx2[3] = fmaxf(mx2[3], (float)esq[j]);
            }
            if (p.k_out)
#pragma unroll
                for (int c = 0; c < 3; ++c) stv<V>(p.k_out + c * n + i0, kv[c]);
        }
        // ---- next stage input: m0 + dt sum_t c_t k_t, normalised ----
        float nv[3][V];
        if (p.m0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float sv[V] = {};
                for (int t = 0; t < p.n_comb; ++t) {
                    const float *kk = p.comb_k[t];
                    const float w = p.comb_c[t];
                    float kc[V];
                    if (kk) ldv<V>(kk + c * n + i0, kc);
#pragma unroll
                    for (int j = 0; j < V; ++j) sv[j] += w * (kk ? kc[j] : kv[c][j]);
                }
                float mb[V];
                ldv<V>(p.m0 + c * n + i0, mb);
#pragma unroll
                for (int j = 0; j < V; ++j) nv[c][j] = mb[j] + dt_f * sv[j];
            }
#pragma unroll
            for (int j = 0; j < V; ++j) {
                const float vx = nv[0][j], vy = nv[1][j], vz = nv[2][j];
                const float nn = sqrtf(vx * vx + vy * vy + vz * vz);
                const float inv = nn > 0.f ? 1.0f / nn : 0.f;
                nv[0][j] = vx * inv;
                nv[1][j] = vy * inv;
                nv[2][j] = vz * inv;
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) stv<V>(p.m_next + c * n + i0, nv[c]);
        } else if (p.m_fwd) {
#pragma unroll
            for (int c = 0; c < 3; ++c) ldv<V>(p.m_fwd + c * n + i0, nv[c]);
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int j = 0; j < V; ++j) nv[c][j] = 0.f;
        }
        if (p.x_out) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
#pragma unroll
                for (int j = 0; j < V; j += 2) pack[(rr * 3 + c) * lsx + sk((x0 + j) >> 1)] = make_float2(nv[c][j], nv[c][j + 1]);
            }
        }
    }
}

// Body of the row pass for CTA `bid` of `nblk`; shared by the single-problem kernel
// and the batched kernel that walks a (problem, block) work table.  ADJ compiles the
// adjoint modes (a separate kernel, so the forward kernel's registers are unaffected).
// XH = 512: the instance for x half-length 512 (px = 1024, e.g. 512-cell rows), whose
// two-level x-transforms (32 x 16) hold 16 complex values a thread; compiled as a kernel
// of its own so that its registers do not weigh on the other sizes.
template <bool ADJ, int XH = 0>
__device__ __forceinline__ void row_pass_body(const RowPass &p, const int bid, const int nblk) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int nx = g.nx, half = g.half, nkx = g.nkx;
    const long long n = g.n;
    const int nrows = g.ny * g.nz;
    const int row0 = bid * p.rows;
    const int rows = min(p.rows, nrows - row0);
    const bool use_fft = (p.x_in != nullptr) || (p.x_out != nullptr);
    const int lsx = skewed_len(half);  // line stride of the x-transform buffers
    const int flen = p.rows * 3 * lsx;
    float2 *fa = reinterpret_cast<float2 *>(smem);
    float2 *fb = fa + (use_fft ? flen : 0);
    float2 *red = fb + (use_fft ? flen : 0);  // per-warp statistics

    // ---- (1) inverse x-transform of the demag spectrum ----
    float2 *hd = nullptr;
    const bool fused_x = XH == 512 || row_x_fused_ok(g);
    if (p.x_in && fused_x) {
        if constexpr (XH == 512) row_inverse_x<32, 16>(p, rows, row0, fa, fb);
        else row_inverse_x_fused(p, rows, row0, fa, fb);
        hd = fb;
    } else if (p.x_in) {
        // stage the spectrum rows in smem (batched loads), then form the half-length input
        batched_copy<8>(
            rows * 3 * nkx,
            [&](int idx) {
                const int line = g.fd_nkx.div(idx), k = idx - line * nkx;
                const int rr = line / 3, c = line - 3 * rr;
                return p.x_in[((size_t)c * nrows + row0 + rr) * nkx + k];
            },
            [&](int idx, float2 v) {
                const int line = g.fd_nkx.div(idx), k = idx - line * nkx;
                fb[line * lsx + sk(k)] = v;  // lsx >= nkx + 1 holds the nkx values
            });
        __syncthreads();
        for (int idx = threadIdx.x; idx < rows * 3 * half; idx += blockDim.x) {
            const int line = g.fd_half.div(idx), k = idx - line * half;
            const float2 a = fb[line * lsx + sk(k)];
            const float2 b = cconj(fb[line * lsx + sk(half - k)]);
            const float2 E = cadd(a, b);
            const float2 O = cmul(csub(a, b), cconj(__ldg(p.xpost + k)));
            fa[line * lsx + sk(k)] = cadd(E, mul_i(O));
        }
        __syncthreads();
        hd = fft_lines(fa, fb, rows * 3, lsx, p.xplan, true);
    }
    float2 *pack = (fused_x || hd == fb) ? fa : fb;  // free buffer for the forward transform input

    // ---- (2)-(4) per-cell work ----
    // statistics: compensated float-float sums (TwoSum) for the energies, FP32 maxima
    // of squared norms; FP64 only for the per-cell DP45 error combination
    float sum_hi[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, sum_lo[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    float mx2[4] = {0.f, 0.f, 0.f, 0.f};
    const Material &M = p.mat;
    const double dt_d = p.dt_dev ? *p.dt_dev : (double)p.dt;  // step size of this pass
    const float dt_f = (float)dt_d;
    const double err_dt = p.dt_dev ? dt_d : p.err_dt;
    bool vec = false;
    if constexpr (!ADJ) vec = p.mask == nullptr && (nx & (kRowVec - 1)) == 0 && rows * (nx / kRowVec) >= (int)blockDim.x;
    if (vec) cells_vec<kRowVec>(p, rows, row0, hd, pack, lsx, sum_hi, sum_lo, mx2, dt_f, err_dt);
    for (int idx = vec ? rows * nx : threadIdx.x; idx < rows * nx; idx += blockDim.x) {
        const int rr = g.fd_nx.div(idx);
        const int x = idx - rr * nx;
        const int row = row0 + rr;
        const int z = g.fd_ny.div(row);
        const int y = row - z * g.ny;
        const long long i = (long long)row * nx + x;
        const bool act = cell_active(p.mask, i);
        float kx_ = 0.f, ky_ = 0.f, kz_ = 0.f;
        if (p.m_in) {
            const float *mi = p.m_in;
            const float m0x = mi[i], m0y = mi[n + i], m0z = mi[2 * n + i];
            float hx = 0.f, hy = 0.f, hz = 0.f;      // effective field
            float ex = 0.f, ey = 0.f, ez = 0.f;      // exchange
            float dx_ = 0.f, dy_ = 0.f, dz_ = 0.f;   // demag
            float e_pair = 0.f;
            if (act) {
                if (M.ex_pref != 0.f) {
                    // open axes clamp (Neumann), periodic axes wrap around (fdm_types.rs:126-132)
                    long long nb[6];
                    const long long pl = (long long)nx * g.ny;
                    nb[0] = x > 0 ? i - 1 : (g.per & 1) ? i + nx - 1 : i;
                    nb[1] = x < nx - 1 ? i + 1 : (g.per & 1) ? i - (nx - 1) : i;
                    nb[2] = y > 0 ? i - nx : (g.per & 2) ? i + pl - nx : i;
                    nb[3] = y < g.ny - 1 ? i + nx : (g.per & 2) ? i - pl + nx : i;
                    nb[4] = z > 0 ? i - pl : (g.per & 4) ? i + pl * (g.nz - 1) : i;
                    nb[5] = z < g.nz - 1 ? i + pl : (g.per & 4) ? i - pl * (g.nz - 1) : i;
                    if (p.mask) {
#pragma unroll
                        for (int q = 0; q < 6; ++q)
                            if (p.mask[nb[q]] == 0) nb[q] = i;
                    }
                    float v[6][3];
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        v[q][0] = mi[nb[q]];
                        v[q][1] = mi[n + nb[q]];
                        v[q][2] = mi[2 * n + nb[q]];
                    }
                    const float c0[3] = {m0x, m0y, m0z};
                    float e3[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        e3[c] = M.ex_pref * ((v[1][c] - 2.f * c0[c] + v[0][c]) * M.idx2 +
                                             (v[3][c] - 2.f * c0[c] + v[2][c]) * M.idy2 +
                                             (v[5][c] - 2.f * c0[c] + v[4][c]) * M.idz2);
                    ex = e3[0];
                    ey = e3[1];
                    ez = e3[2];
                    if (p.partials) {
                        // forward pairs only (x+1, y+1, z+1), each active pair once
                        const float w[3] = {M.idx2, M.idy2, M.idz2};
                        const bool has[3] = {x < nx - 1 || (g.per & 1), y < g.ny - 1 || (g.per & 2), z < g.nz - 1 || (g.per & 4)};
#pragma unroll
                        for (int a = 0; a < 3; ++a) {
                            const int q = 2 * a + 1;
                            if (has[a] && nb[q] != i) {
                                const float d0 = v[q][0] - m0x, d1 = v[q][1] - m0y, d2 = v[q][2] - m0z;
                                e_pair += (d0 * d0 + d1 * d1 + d2 * d2) * w[a];
                            }
                        }
                    }
                }
                if (hd) {
                    const float2 a = hd[(rr * 3 + 0) * lsx + sk(x >> 1)];
                    const float2 b = hd[(rr * 3 + 1) * lsx + sk(x >> 1)];
                    const float2 c = hd[(rr * 3 + 2) * lsx + sk(x >> 1)];
                    dx_ = (x & 1) ? a.y : a.x;
                    dy_ = (x & 1) ? b.y : b.x;
                    dz_ = (x & 1) ? c.y : c.x;
                }
                hx = ex + dx_;
                hy = ey + dy_;
                hz = ez + dz_;
                if (M.has_ext) {
                    hx += M.hext[0];
                    hy += M.hext[1];
                    hz += M.hext[2];
                }
                if (p.hmap) {
                    hx += p.hmap[i];
                    hy += p.hmap[n + i];
                    hz += p.hmap[2 * n + i];
                }
                float e_uni = 0.f, e_cub = 0.f;
                if (M.has_uni) {
                    const float mu = m0x * M.u[0] + m0y * M.u[1] + m0z * M.u[2];
                    const float cf = M.ku1c * mu + M.ku2c * mu * mu * mu;
                    hx += cf * M.u[0];
                    hy += cf * M.u[1];
                    hz += cf * M.u[2];
                    const float s = mu * mu;
                    e_uni = M.ku1f * s + M.ku2f * s * s;
                }
                if (M.has_cub) {
                    const float a1 = m0x * M.c1[0] + m0y * M.c1[1] + m0z * M.c1[2];
                    const float a2 = m0x * M.c2[0] + m0y * M.c2[1] + m0z * M.c2[2];
                    const float a3 = m0x * M.c3[0] + m0y * M.c3[1] + m0z * M.c3[2];
                    const float s1 = a1 * a1, s2 = a2 * a2, s3 = a3 * a3;
                    const float sig = s1 * s2 + s2 * s3 + s1 * s3;
                    const float g1 = M.kc1c * a1 * (s2 + s3) + M.kc2c * a1 * s2 * s3 + M.kc3c * sig * a1 * (s2 + s3);
                    const float g2 = M.kc1c * a2 * (s1 + s3) + M.kc2c * a2 * s1 * s3 + M.kc3c * sig * a2 * (s1 + s3);
                    const float g3 = M.kc1c * a3 * (s1 + s2) + M.kc2c * a3 * s1 * s2 + M.kc3c * sig * a3 * (s1 + s2);
                    hx += g1 * M.c1[0] + g2 * M.c2[0] + g3 * M.c3[0];
                    hy += g1 * M.c1[1] + g2 * M.c2[1] + g3 * M.c3[1];
                    hz += g1 * M.c1[2] + g2 * M.c2[2] + g3 * M.c3[2];
                    e_cub = M.kc1f * sig + M.kc2f * s1 * s2 * s3 + M.kc3f * sig * sig;
                }
                // LLG: k = -gbar (m x H + alpha m x (m x H))
                const float px_ = m0y * hz - m0z * hy;
                const float py_ = m0z * hx - m0x * hz;
                const float pz_ = m0x * hy - m0y * hx;
                const float qx = m0y * pz_ - m0z * py_;
                const float qy = m0z * px_ - m0x * pz_;
                const float qz = m0x * py_ - m0y * px_;
                kx_ = -M.gbar * (M.prec * px_ + M.alpha * qx);
                ky_ = -M.gbar * (M.prec * py_ + M.alpha * qy);
                kz_ = -M.gbar * (M.prec * pz_ + M.alpha * qz);
                if (p.partials) {
                    ff_add(sum_hi[0], sum_lo[0], e_pair);
                    ff_add(sum_hi[1], sum_lo[1], m0x * dx_ + m0y * dy_ + m0z * dz_);
                    if (M.has_ext) ff_add(sum_hi[2], sum_lo[2], m0x * M.hext[0] + m0y * M.hext[1] + m0z * M.hext[2]);
                    if (p.hmap) ff_add(sum_hi[2], sum_lo[2], m0x * p.hmap[i] + m0y * p.hmap[n + i] + m0z * p.hmap[2 * n + i]);
                    ff_add(sum_hi[3], sum_lo[3], e_uni);
                    ff_add(sum_hi[4], sum_lo[4], e_cub);
                    mx2[0] = fmaxf(mx2[0], hx * hx + hy * hy + hz * hz);
                    mx2[1] = fmaxf(mx2[1], dx_ * dx_ + dy_ * dy_ + dz_ * dz_);
                    mx2[2] = fmaxf(mx2[2], kx_ * kx_ + ky_ * ky_ + kz_ * kz_);
                }
            }
            if (p.partials && p.n_err > 0) {
                double e0 = 0.0, e1 = 0.0, e2 = 0.0;
                for (int t = 0; t < p.n_err; ++t) {
                    const float *kk = p.err_k[t];
                    const double w = p.err_c[t];
                    if (kk) {
                        e0 += w * (double)kk[i];
                        e1 += w * (double)kk[n + i];
                        e2 += w * (double)kk[2 * n + i];
                    } else {
                        e0 += w * (double)kx_;
                        e1 += w * (double)ky_;
                        e2 += w * (double)kz_;
                    }
                }
                e0 *= err_dt;
                e1 *= err_dt;
                e2 *= err_dt;
                mx2[3] = fmaxf(mx2[3], (float)(e0 * e0 + e1 * e1 + e2 * e2));
            }
            if (p.k_out) {
                p.k_out[i] = kx_;
                p.k_out[n + i] = ky_;
                p.k_out[2 * n + i] = kz_;
            }
            if (p.h_eff_out) {
                p.h_eff_out[i] = hx;
                p.h_eff_out[n + i] = hy;
                p.h_eff_out[2 * n + i] = hz;
            }
            if (p.h_ex_out) {
                p.h_ex_out[i] = ex;
                p.h_ex_out[n + i] = ey;
                p.h_ex_out[2 * n + i] = ez;
            }
            if (p.h_d_out) {
                p.h_d_out[i] = dx_;
                p.h_d_out[n + i] = dy_;
                p.h_d_out[2 * n + i] = dz_;
            }
            if constexpr (ADJ) {
                if (p.adj_mode & 2) {
                    // lambda_y = lambda_m + H_lin(lambda_H), then through the stage normalisation
                    const A3 ly = a3_axpy(1.f, a3_ld(p.adj_lam_m, n, i), A3{hx, hy, hz});
                    const A3 ly0 = a3_ld(p.adj_lam_y0, n, i);
                    if (p.adj_k) {
                        const A3 v = a3_axpy(p.adj_ch, a3_ld(p.adj_k, n, i), a3_ld(p.adj_y0, n, i));
                        const float nn = sqrtf(a3_dot(v, v));
                        A3 mu{0.f, 0.f, 0.f};
                        if (nn > 0.f) {
                            const float inv = 1.0f / nn;
                            const A3 u{v.x * inv, v.y * inv, v.z * inv};
                            const A3 t = a3_axpy(-a3_dot(u, ly), u, ly);
                            mu = {t.x * inv, t.y * inv, t.z * inv};
                        }
                        a3_st(p.adj_lam_y0, n, i, a3_axpy(1.f, mu, ly0));
                        a3_st(p.adj_lam_k, n, i, a3_axpy(p.adj_ch, mu, a3_ld(p.adj_lam_k, n, i)));
                    } else {
                        a3_st(p.adj_lam_y0, n, i, a3_axpy(1.f, ly, ly0));
                    }
                }
            }
        }
        // ---- (4) next stage input ----
        float nxv = 0.f, nyv = 0.f, nzv = 0.f;
        bool adj_local = false;
        if constexpr (ADJ) adj_local = (p.adj_mode & 1) != 0;
        if (adj_local) {
            if constexpr (ADJ) {
                // local VJP of k = -gbar [prec m x H + alpha m x (m x H)] with cotangent w
                const A3 m = a3_ld(p.adj_m, n, i), H = a3_ld(p.adj_H, n, i), w = a3_ld(p.adj_w, n, i);
                const A3 q = a3_axpy(M.alpha, a3_cross(w, m), A3{M.prec * w.x, M.prec * w.y, M.prec * w.z});
                const A3 pv = a3_cross(m, H);
                const A3 t = a3_axpy(M.alpha, a3_cross(pv, w), a3_cross(H, q));
                A3 lm{-M.gbar * t.x, -M.gbar * t.y, -M.gbar * t.z};
                const A3 qm = a3_cross(q, m);
                const A3 lh{-M.gbar * qm.x, -M.gbar * qm.y, -M.gbar * qm.z};
                if (p.adj_uni) {
                    const A3 u{M.u[0], M.u[1], M.u[2]};
                    const float mu = a3_dot(m, u);
                    lm = a3_axpy((M.ku1c + 3.0f * M.ku2c * mu * mu) * a3_dot(u, lh), u, lm);
                }
                a3_st(p.adj_lam_m, n, i, lm);
                a3_st(p.adj_lam_h, n, i, lh);
                const float lv[3] = {lh.x, lh.y, lh.z};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    float hi = p.adj_g_hi[c * n + i], lo = p.adj_g_lo[c * n + i];
                    ff_add(hi, lo, lv[c]);
                    p.adj_g_hi[c * n + i] = hi;
                    p.adj_g_lo[c * n + i] = lo;
                }
                nxv = lh.x;
                nyv = lh.y;
                nzv = lh.z;
            }
        } else if (p.m0) {
            float sx = 0.f, sy = 0.f, sz = 0.f;
            for (int t = 0; t < p.n_comb; ++t) {
                const float *kk = p.comb_k[t];
                const float w = p.comb_c[t];
                if (kk) {
                    sx += w * kk[i];
                    sy += w * kk[n + i];
                    sz += w * kk[2 * n + i];
                } else {
                    sx += w * kx_;
                    sy += w * ky_;
                    sz += w * kz_;
                }
            }
            const float vx = p.m0[i] + dt_f * sx;
            const float vy = p.m0[n + i] + dt_f * sy;
            const float vz = p.m0[2 * n + i] + dt_f * sz;
            const float nn = sqrtf(vx * vx + vy * vy + vz * vz);
            const float inv = nn > 0.f ? 1.0f / nn : 0.f;
            nxv = vx * inv;
            nyv = vy * inv;
            nzv = vz * inv;
            p.m_next[i] = nxv;
            p.m_next[n + i] = nyv;
            p.m_next[2 * n + i] = nzv;
        } else if (p.m_fwd) {
            nxv = p.m_fwd[i];
            nyv = p.m_fwd[n + i];
            nzv = p.m_fwd[2 * n + i];
        }
        if (p.x_out) {
            float *pk = reinterpret_cast<float *>(pack);
            // real sample x of line L lives at float index 2*(L*lsx + sk(x/2)) + (x&1)
            const int base = 2 * ((rr * 3) * lsx + sk(x >> 1)) + (x & 1);
            pk[base] = nxv;
            pk[base + 2 * lsx] = nyv;
            pk[base + 4 * lsx] = nzv;
        }
    }

    // ---- (3) block statistics ----
    if (p.partials) {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            float h = sum_hi[s], l = sum_lo[s];
            warp_ff_sum(h, l);
            if (lane == 0) red[wid * kNumStats + s] = make_float2(h, l);
        }
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const float v = warp_maxf(mx2[s]);
            if (lane == 0) red[wid * kNumStats + 5 + s] = make_float2(v, 0.f);
        }
        __syncthreads();
        if (threadIdx.x < kNumStats) {
            const int s = threadIdx.x;
            float h = 0.f, l = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                const float2 v = red[w * kNumStats + s];
                if (s < 5) {
                    ff_add(h, l, v.x);
                    l += v.y;
                } else {
                    h = fmaxf(h, v.x);
                }
            }
            p.partials[(size_t)s * nblk + bid] = make_float2(h, l);
        }
    }

    // ---- (5) forward x-transform of the next stage input ----
    if (p.x_out && fused_x) {
        __syncthreads();  // every sample packed, every H_d sample of fb read
        if constexpr (XH == 512) row_forward_x<32, 16>(p, rows, row0, pack, fb);
        else row_forward_x_fused(p, rows, row0, pack, fb);
    } else if (p.x_out) {
        // zero the padded half x in [nx, px) of every packed line
        float *pk = reinterpret_cast<float *>(pack);
        const int padw = 2 * half - nx;
        for (int idx = threadIdx.x; idx < rows * 3 * padw; idx += blockDim.x) {
            const int line = g.fd_padw.div(idx);
            const int x = nx + (idx - line * padw);
            pk[2 * (line * lsx + sk(x >> 1)) + (x & 1)] = 0.f;
        }
        __syncthreads();
        float2 *other = (pack == fa) ? fb : fa;
        float2 *Z = fft_lines(pack, other, rows * 3, lsx, p.xplan, false);
        for (int idx = threadIdx.x; idx < rows * 3 * nkx; idx += blockDim.x) {
            const int line = g.fd_nkx.div(idx);
            const int k = idx - line * nkx;
            const int rr = line / 3;
            const int c = line - rr * 3;
            const float2 *zl = Z + line * lsx;
            const float2 a = zl[sk(k == half ? 0 : k)];
            const float2 b = cconj(zl[sk(k == 0 ? 0 : half - k)]);
            const float2 E = cscale(cadd(a, b), 0.5f);
            const float2 O = div2i(csub(a, b));
            p.x_out[((size_t)c * nrows + row0 + rr) * nkx + k] = cadd(E, cmul(__ldg(p.xpost + k), O));
        }
    }
}

__global__ void __launch_bounds__(kThreads, 3) row_pass_kernel(const RowPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
    row_pass_body<false>(p, blockIdx.x, gridDim.x);
}
__global__ void __launch_bounds__(kThreads, 2) row_pass_x512_kernel(const RowPass p) {
    pdl_wait();
    if (p.early) pdl_trigger();
    row_pass_body<false, 512>(p, blockIdx.x, gridDim.x);
}
__global__ void __launch_bounds__(kThreads) row_pass_adj_kernel(const RowPass p) { row_pass_body<true>(p, blockIdx.x, gridDim.x); }

// One launch for many problems: work[blockIdx.x] = (problem, block within problem).
__global__ void __launch_bounds__(kThreads, 3) row_pass_batched_kernel(const RowPass *__restrict__ ps,
                                                                    const int2 *__restrict__ work) {
    // stage the problem's descriptor in shared memory once per CTA: the body reads its
    // fields in every loop, and global reads could not be hoisted past the stores
    __shared__ __align__(16) unsigned char desc[sizeof(RowPass)];
    const int2 w = work[blockIdx.x];
    // a finished problem (step size 0 in its control block) keeps its blocks in the table
    // until the round is rebuilt; the whole CTA leaves before its first barrier
    const double *dtp = ps[w.x].dt_dev;
    if (dtp && *dtp <= 0.0) return;
    const int *src = reinterpret_cast<const int *>(ps + w.x);
    for (int i = threadIdx.x; i < (int)(sizeof(RowPass) / sizeof(int)); i += blockDim.x)
        reinterpret_cast<int *>(desc)[i] = src[i];
    __syncthreads();
    const RowPass &p = *reinterpret_cast<const RowPass *>(desc);
    row_pass_body<false>(p, w.y, (p.g.ny * p.g.nz + p.rows - 1) / p.rows);
}

}  // namespace

cudaError_t launch_row_pass_batched(const RowPass *ps, const int2 *work, int nwork, size_t smem, cudaStream_t s) {
    cudaError_t e = smem > 48 * 1024 ? cudaFuncSetAttribute((const void *)row_pass_batched_kernel,
                                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                                     : cudaSuccess;
    if (e != cudaSuccess) return e;
    row_pass_batched_kernel<<<nwork, kThreads, smem, s>>>(ps, work);
    return cudaGetLastError();
}

// ---- host launchers ----

size_t row_pass_smem(const RowPass &p) {
    const bool use_fft = (p.x_in != nullptr) || (p.x_out != nullptr);
    size_t b = 0;
    if (use_fft) b += 2 * sizeof(float2) * (size_t)p.rows * 3 * skewed_len(p.g.half);
    b += sizeof(double) * kWarps * kNumStats;
    return b;
}

int row_pass_blocks(const RowPass &p) {
    const int nrows = p.g.ny * p.g.nz;
    return (nrows + p.rows - 1) / p.rows;
}

static cudaError_t ensure_smem(const void *fn, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t launch_row_pass(const RowPass &p, cudaStream_t s) {
    const size_t sm = row_pass_smem(p);
    const bool x512 = p.g.half == 512 && p.g.nx <= 512;
    const auto fn = x512 ? row_pass_x512_kernel : row_pass_kernel;
    cudaError_t e = ensure_smem((const void *)fn, sm);
    if (e != cudaSuccess) return e;
    return launch_pdl(fn, dim3(row_pass_blocks(p)), dim3(kThreads), sm, s, p);
}

cudaError_t launch_row_pass_adj(const RowPass &p, cudaStream_t s) {
    const size_t sm = row_pass_smem(p);
    cudaError_t e = ensure_smem((const void *)row_pass_adj_kernel, sm);
    if (e != cudaSuccess) return e;
    row_pass_adj_kernel<<<row_pass_blocks(p), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

}  // namespace fm
