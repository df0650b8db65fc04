// kernels.cu -- the demag FFT passes and the fused field/torque/stage pass.
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
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// a / (2i) = -i a / 2
__device__ __forceinline__ float2 div2i(float2 a) { return make_float2(0.5f * a.y, -0.5f * a.x); }
__device__ __forceinline__ float2 mul_i(float2 a) { return make_float2(-a.y, a.x); }

__device__ __forceinline__ bool cell_active(const uint8_t *mask, long long i) { return mask == nullptr || mask[i] != 0; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__global__ void __launch_bounds__(kThreads) row_pass_kernel(const RowPass p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int nx = g.nx, half = g.half, nkx = g.nkx;
    const long long n = g.n;
    const int nrows = g.ny * g.nz;
    const int row0 = blockIdx.x * p.rows;
    const int rows = min(p.rows, nrows - row0);
    const bool use_fft = (p.x_in != nullptr) || (p.x_out != nullptr);
    const int flen = p.rows * 3 * half;
    float2 *fa = reinterpret_cast<float2 *>(smem);
    float2 *fb = fa + (use_fft ? flen : 0);
    double *red = reinterpret_cast<double *>(fb + (use_fft ? flen : 0));

    // ---- (1) inverse x-transform of the demag spectrum ----
    float2 *hd = nullptr;
    if (p.x_in) {
        for (int idx = threadIdx.x; idx < rows * 3 * half; idx += blockDim.x) {
            const int rr = idx / (3 * half);
            const int rem = idx - rr * 3 * half;
            const int c = rem / half;
            const int k = rem - c * half;
            const float2 *X = p.x_in + ((size_t)c * nrows + row0 + rr) * nkx;
            const float2 a = X[k];
            const float2 b = cconj(X[half - k]);
            const float2 E = cadd(a, b);
            const float2 O = cmul(csub(a, b), cconj(__ldg(p.xpost + k)));
            fa[(rr * 3 + c) * half + k] = cadd(E, mul_i(O));
        }
        __syncthreads();
        hd = fft_lines(fa, fb, rows * 3, half, p.xplan, true);
    }
    float2 *pack = (hd == fb) ? fa : fb;  // free buffer for the forward transform input

    // ---- (2)-(4) per-cell work ----
    double acc[kNumStats];
#pragma unroll
    for (int s = 0; s < kNumStats; ++s) acc[s] = 0.0;
    const Material &M = p.mat;
    for (int idx = threadIdx.x; idx < rows * nx; idx += blockDim.x) {
        const int rr = idx / nx;
        const int x = idx - rr * nx;
        const int row = row0 + rr;
        const int y = row % g.ny;
        const int z = row / g.ny;
        const long long i = (long long)row * nx + x;
        const bool act = cell_active(p.mask, i);
        float kx_ = 0.f, ky_ = 0.f, kz_ = 0.f;
        if (p.m_in) {
            const float *mi = p.m_in;
            const float m0x = mi[i], m0y = mi[n + i], m0z = mi[2 * n + i];
            float hx = 0.f, hy = 0.f, hz = 0.f;      // effective field
            float ex = 0.f, ey = 0.f, ez = 0.f;      // exchange
            float dx_ = 0.f, dy_ = 0.f, dz_ = 0.f;   // demag
            double e_pair = 0.0;
            if (act) {
                if (M.ex_pref != 0.f) {
                    long long nb[6];
                    nb[0] = x > 0 ? i - 1 : i;
                    nb[1] = x < nx - 1 ? i + 1 : i;
                    nb[2] = y > 0 ? i - nx : i;
                    nb[3] = y < g.ny - 1 ? i + nx : i;
                    nb[4] = z > 0 ? i - (long long)nx * g.ny : i;
                    nb[5] = z < g.nz - 1 ? i + (long long)nx * g.ny : i;
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
                        const bool has[3] = {x < nx - 1, y < g.ny - 1, z < g.nz - 1};
#pragma unroll
                        for (int a = 0; a < 3; ++a) {
                            const int q = 2 * a + 1;
                            if (has[a] && nb[q] != i) {
                                const float d0 = v[q][0] - m0x, d1 = v[q][1] - m0y, d2 = v[q][2] - m0z;
                                e_pair += (double)(d0 * d0 + d1 * d1 + d2 * d2) * (double)w[a];
                            }
                        }
                    }
                }
                if (hd) {
                    const float2 a = hd[(rr * 3 + 0) * half + (x >> 1)];
                    const float2 b = hd[(rr * 3 + 1) * half + (x >> 1)];
                    const float2 c = hd[(rr * 3 + 2) * half + (x >> 1)];
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
                double e_uni = 0.0, e_cub = 0.0;
                if (M.has_uni) {
                    const float mu = m0x * M.u[0] + m0y * M.u[1] + m0z * M.u[2];
                    const float cf = M.ku1c * mu + M.ku2c * mu * mu * mu;
                    hx += cf * M.u[0];
                    hy += cf * M.u[1];
                    hz += cf * M.u[2];
                    const double s = (double)mu * (double)mu;
                    e_uni = M.ku1 * s + M.ku2 * s * s;
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
                    const double ds1 = (double)s1, ds2 = (double)s2, ds3 = (double)s3;
                    const double dsig = ds1 * ds2 + ds2 * ds3 + ds1 * ds3;
                    e_cub = M.kc1 * dsig + M.kc2 * ds1 * ds2 * ds3 + M.kc3 * dsig * dsig;
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
                    acc[0] += e_pair;
                    acc[1] += (double)m0x * dx_ + (double)m0y * dy_ + (double)m0z * dz_;
                    if (M.has_ext) acc[2] += (double)m0x * M.hext[0] + (double)m0y * M.hext[1] + (double)m0z * M.hext[2];
                    acc[3] += e_uni;
                    acc[4] += e_cub;
                    acc[5] = fmax(acc[5], (double)hx * hx + (double)hy * hy + (double)hz * hz);
                    acc[6] = fmax(acc[6], (double)dx_ * dx_ + (double)dy_ * dy_ + (double)dz_ * dz_);
                    acc[7] = fmax(acc[7], (double)kx_ * kx_ + (double)ky_ * ky_ + (double)kz_ * kz_);
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
                e0 *= p.err_dt;
                e1 *= p.err_dt;
                e2 *= p.err_dt;
                acc[8] = fmax(acc[8], e0 * e0 + e1 * e1 + e2 * e2);
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
        }
        // ---- (4) next stage input ----
        float nxv = 0.f, nyv = 0.f, nzv = 0.f;
        if (p.m0) {
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
            const float vx = p.m0[i] + p.dt * sx;
            const float vy = p.m0[n + i] + p.dt * sy;
            const float vz = p.m0[2 * n + i] + p.dt * sz;
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
            // real sample x of component c lives at float index 2*((rr*3+c)*half + x/2) + (x&1)
            const int base = (rr * 3) * half * 2 + x;
            pk[base] = nxv;
            pk[base + 2 * half] = nyv;
            pk[base + 4 * half] = nzv;
        }
    }

    // ---- (3) block statistics ----
    if (p.partials) {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
        for (int s = 0; s < kNumStats; ++s) {
            const double v = s < 5 ? warp_sum(acc[s]) : warp_max(acc[s]);
            if (lane == 0) red[wid * kNumStats + s] = v;
        }
        __syncthreads();
        if (threadIdx.x < kNumStats) {
            const int s = threadIdx.x;
            double v = s < 5 ? 0.0 : 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = s < 5 ? v + red[w * kNumStats + s] : fmax(v, red[w * kNumStats + s]);
            p.partials[(size_t)blockIdx.x * kNumStats + s] = v;
        }
    }

    // ---- (5) forward x-transform of the next stage input ----
    if (p.x_out) {
        // zero the padded half x in [nx, px) of every packed line
        float *pk = reinterpret_cast<float *>(pack);
        const int padw = 2 * half - nx;
        for (int idx = threadIdx.x; idx < rows * 3 * padw; idx += blockDim.x) {
            const int line = idx / padw;
            const int x = nx + (idx - line * padw);
            pk[line * half * 2 + x] = 0.f;
        }
        __syncthreads();
        float2 *other = (pack == fa) ? fb : fa;
        float2 *Z = fft_lines(pack, other, rows * 3, half, p.xplan, false);
        for (int idx = threadIdx.x; idx < rows * 3 * nkx; idx += blockDim.x) {
            const int line = idx / nkx;
            const int k = idx - line * nkx;
            const int rr = line / 3;
            const int c = line - rr * 3;
            const float2 *zl = Z + line * half;
            const float2 a = zl[k == half ? 0 : k];
            const float2 b = cconj(zl[k == 0 ? 0 : half - k]);
            const float2 E = cscale(cadd(a, b), 0.5f);
            const float2 O = div2i(csub(a, b));
            p.x_out[((size_t)c * nrows + row0 + rr) * nkx + k] = cadd(E, cmul(__ldg(p.xpost + k), O));
        }
    }
}

// ---- column passes ----

__device__ __forceinline__ void kernel_mirror(int k, int p, int &km, float &sg) {
    if (k > p / 2) {
        km = p - k;
        sg = -1.f;
    } else {
        km = k;
        sg = 1.f;
    }
}

__global__ void __launch_bounds__(kThreads) y_forward_kernel(const ColPass p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = blockIdx.x * tx, ncol = min(tx, g.nkx - kx0);
    const int z = blockIdx.y, c = blockIdx.z;
    const int ls = g.py + 1;
    float2 *a = reinterpret_cast<float2 *>(smem);
    float2 *b = a + tx * ls;
    const float2 *src = p.in + ((size_t)c * g.nz + z) * g.ny * g.nkx;
    for (int idx = threadIdx.x; idx < g.py * tx; idx += blockDim.x) {
        const int y = idx / tx, col = idx - y * tx;
        a[col * ls + y] = (y < g.ny && col < ncol) ? src[(size_t)y * g.nkx + kx0 + col] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *r = fft_lines(a, b, tx, ls, p.plan, false);
    float2 *dst = p.out + ((size_t)c * g.nz + z) * g.py * g.nkx;
    for (int idx = threadIdx.x; idx < g.py * tx; idx += blockDim.x) {
        const int y = idx / tx, col = idx - y * tx;
        if (col < ncol) dst[(size_t)y * g.nkx + kx0 + col] = r[col * ls + y];
    }
}

__global__ void __launch_bounds__(kThreads) y_inverse_kernel(const ColPass p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = blockIdx.x * tx, ncol = min(tx, g.nkx - kx0);
    const int z = blockIdx.y, c = blockIdx.z;
    const int ls = g.py + 1;
    float2 *a = reinterpret_cast<float2 *>(smem);
    float2 *b = a + tx * ls;
    const float2 *src = p.in + ((size_t)c * g.nz + z) * g.py * g.nkx;
    for (int idx = threadIdx.x; idx < g.py * tx; idx += blockDim.x) {
        const int y = idx / tx, col = idx - y * tx;
        a[col * ls + y] = col < ncol ? src[(size_t)y * g.nkx + kx0 + col] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *r = fft_lines(a, b, tx, ls, p.plan, true);
    float2 *dst = p.out + ((size_t)c * g.nz + z) * g.ny * g.nkx;
    for (int idx = threadIdx.x; idx < g.ny * tx; idx += blockDim.x) {
        const int y = idx / tx, col = idx - y * tx;
        if (col < ncol) dst[(size_t)y * g.nkx + kx0 + col] = r[col * ls + y];
    }
}

__global__ void __launch_bounds__(kThreads) z_convolve_kernel(const ColPass p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = blockIdx.x * tx, ncol = min(tx, g.nkx - kx0);
    const int ky = blockIdx.y;
    const int ls = g.pz + 1;
    const int nl = 3 * tx;
    float2 *a = reinterpret_cast<float2 *>(smem);
    float2 *b = a + nl * ls;
    const size_t cstride = (size_t)g.nz * g.py * g.nkx;  // component stride of Y
    const size_t zstride = (size_t)g.py * g.nkx;
    for (int idx = threadIdx.x; idx < 3 * g.pz * tx; idx += blockDim.x) {
        const int c = idx / (g.pz * tx);
        const int rem = idx - c * g.pz * tx;
        const int z = rem / tx, col = rem - z * tx;
        a[(c * tx + col) * ls + z] = (z < g.nz && col < ncol)
                                         ? p.in[c * cstride + z * zstride + (size_t)ky * g.nkx + kx0 + col]
                                         : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *r = fft_lines(a, b, nl, ls, p.plan, false);
    float2 *o = (r == a) ? b : a;
    int kym;
    float sy;
    kernel_mirror(ky, g.py, kym, sy);
    const size_t kc = (size_t)g.nkz * g.nky * g.nkx;
    for (int idx = threadIdx.x; idx < g.pz * tx; idx += blockDim.x) {
        const int kz = idx / tx, col = idx - kz * tx;
        const int kx = min(kx0 + col, g.nkx - 1);
        int kzm;
        float sz;
        kernel_mirror(kz, g.pz, kzm, sz);
        const float *K = p.kern + ((size_t)kzm * g.nky + kym) * g.nkx + kx;
        const float kxx = __ldg(K), kyy = __ldg(K + kc), kzz = __ldg(K + 2 * kc);
        const float kxy = sy * __ldg(K + 3 * kc), kxz = sz * __ldg(K + 4 * kc), kyz = sy * sz * __ldg(K + 5 * kc);
        const float2 mx = r[(0 * tx + col) * ls + kz];
        const float2 my = r[(1 * tx + col) * ls + kz];
        const float2 mz = r[(2 * tx + col) * ls + kz];
        r[(0 * tx + col) * ls + kz] = make_float2(-(kxx * mx.x + kxy * my.x + kxz * mz.x), -(kxx * mx.y + kxy * my.y + kxz * mz.y));
        r[(1 * tx + col) * ls + kz] = make_float2(-(kxy * mx.x + kyy * my.x + kyz * mz.x), -(kxy * mx.y + kyy * my.y + kyz * mz.y));
        r[(2 * tx + col) * ls + kz] = make_float2(-(kxz * mx.x + kyz * my.x + kzz * mz.x), -(kxz * mx.y + kyz * my.y + kzz * mz.y));
    }
    __syncthreads();
    float2 *q = fft_lines(r, o, nl, ls, p.plan, true);
    for (int idx = threadIdx.x; idx < 3 * g.nz * tx; idx += blockDim.x) {
        const int c = idx / (g.nz * tx);
        const int rem = idx - c * g.nz * tx;
        const int z = rem / tx, col = rem - z * tx;
        if (col < ncol) p.out[c * cstride + z * zstride + (size_t)ky * g.nkx + kx0 + col] = q[(c * tx + col) * ls + z];
    }
}

__global__ void __launch_bounds__(kThreads) y_convolve_2d_kernel(const ColPass p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grid &g = p.g;
    const int tx = p.tx, kx0 = blockIdx.x * tx, ncol = min(tx, g.nkx - kx0);
    const int ls = g.py + 1;
    const int nl = 3 * tx;
    float2 *a = reinterpret_cast<float2 *>(smem);
    float2 *b = a + nl * ls;
    const size_t cstride = (size_t)g.ny * g.nkx;
    for (int idx = threadIdx.x; idx < 3 * g.py * tx; idx += blockDim.x) {
        const int c = idx / (g.py * tx);
        const int rem = idx - c * g.py * tx;
        const int y = rem / tx, col = rem - y * tx;
        a[(c * tx + col) * ls + y] =
            (y < g.ny && col < ncol) ? p.in[c * cstride + (size_t)y * g.nkx + kx0 + col] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *r = fft_lines(a, b, nl, ls, p.plan, false);
    float2 *o = (r == a) ? b : a;
    const size_t kc = (size_t)g.nky * g.nkx;
    for (int idx = threadIdx.x; idx < g.py * tx; idx += blockDim.x) {
        const int ky = idx / tx, col = idx - ky * tx;
        const int kx = min(kx0 + col, g.nkx - 1);
        int kym;
        float sy;
        kernel_mirror(ky, g.py, kym, sy);
        const float *K = p.kern + (size_t)kym * g.nkx + kx;
        const float kxx = __ldg(K), kyy = __ldg(K + kc), kzz = __ldg(K + 2 * kc), kxy = sy * __ldg(K + 3 * kc);
        const float2 mx = r[(0 * tx + col) * ls + ky];
        const float2 my = r[(1 * tx + col) * ls + ky];
        const float2 mz = r[(2 * tx + col) * ls + ky];
        r[(0 * tx + col) * ls + ky] = make_float2(-(kxx * mx.x + kxy * my.x), -(kxx * mx.y + kxy * my.y));
        r[(1 * tx + col) * ls + ky] = make_float2(-(kxy * mx.x + kyy * my.x), -(kxy * mx.y + kyy * my.y));
        r[(2 * tx + col) * ls + ky] = make_float2(-(kzz * mz.x), -(kzz * mz.y));
    }
    __syncthreads();
    float2 *q = fft_lines(r, o, nl, ls, p.plan, true);
    for (int idx = threadIdx.x; idx < 3 * g.ny * tx; idx += blockDim.x) {
        const int c = idx / (g.ny * tx);
        const int rem = idx - c * g.ny * tx;
        const int y = rem / tx, col = rem - y * tx;
        if (col < ncol) p.out[c * cstride + (size_t)y * g.nkx + kx0 + col] = q[(c * tx + col) * ls + y];
    }
}

// Deterministic final reduction of the per-block partials: compensated
// (Neumaier) FP64 sums for the energies, plain max for the norms.
__global__ void __launch_bounds__(kThreads) finalize_stats_kernel(const double *__restrict__ partials, int nblocks,
                                                                  double *__restrict__ out) {
    __shared__ double sh_s[kThreads];
    __shared__ double sh_c[kThreads];
    for (int s = 0; s < kNumStats; ++s) {
        double sum = 0.0, comp = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
            const double v = partials[(size_t)b * kNumStats + s];
            if (s < 5) {
                const double t = sum + v;
                if (fabs(sum) >= fabs(v)) comp += (sum - t) + v;
                else comp += (v - t) + sum;
                sum = t;
            } else {
                sum = fmax(sum, v);
            }
        }
        sh_s[threadIdx.x] = sum;
        sh_c[threadIdx.x] = comp;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tot = 0.0, tc = 0.0;
            for (int t = 0; t < (int)blockDim.x; ++t) {
                if (s < 5) {
                    const double v = sh_s[t];
                    const double u = tot + v;
                    if (fabs(tot) >= fabs(v)) tc += (tot - u) + v;
                    else tc += (v - u) + tot;
                    tot = u;
                    tc += sh_c[t];
                } else {
                    tot = fmax(tot, sh_s[t]);
                }
            }
            out[s] = tot + tc;
        }
        __syncthreads();
    }
}

}  // namespace

// ---- host launchers ----

size_t row_pass_smem(const RowPass &p) {
    const bool use_fft = (p.x_in != nullptr) || (p.x_out != nullptr);
    size_t b = 0;
    if (use_fft) b += 2 * sizeof(float2) * (size_t)p.rows * 3 * p.g.half;
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
    cudaError_t e = ensure_smem((const void *)row_pass_kernel, sm);
    if (e != cudaSuccess) return e;
    row_pass_kernel<<<row_pass_blocks(p), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

int col_tile(const Grid &g, int lines_per_col, int len) {
    // largest tile (<= 8 columns) whose two ping-pong buffers fit in 200 KB
    int tx = 8;
    while (tx > 1 && (size_t)2 * lines_per_col * tx * (len + 1) * sizeof(float2) > 200u * 1024u) tx >>= 1;
    return tx;
}

static unsigned tiles(const ColPass &p) { return (unsigned)((p.g.nkx + p.tx - 1) / p.tx); }

cudaError_t launch_y_forward(const ColPass &p, cudaStream_t s) {
    const size_t sm = 2 * sizeof(float2) * (size_t)p.tx * (p.g.py + 1);
    cudaError_t e = ensure_smem((const void *)y_forward_kernel, sm);
    if (e != cudaSuccess) return e;
    y_forward_kernel<<<dim3(tiles(p), p.g.nz, 3), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_y_inverse(const ColPass &p, cudaStream_t s) {
    const size_t sm = 2 * sizeof(float2) * (size_t)p.tx * (p.g.py + 1);
    cudaError_t e = ensure_smem((const void *)y_inverse_kernel, sm);
    if (e != cudaSuccess) return e;
    y_inverse_kernel<<<dim3(tiles(p), p.g.nz, 3), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_z_convolve(const ColPass &p, cudaStream_t s) {
    const size_t sm = 2 * sizeof(float2) * (size_t)3 * p.tx * (p.g.pz + 1);
    cudaError_t e = ensure_smem((const void *)z_convolve_kernel, sm);
    if (e != cudaSuccess) return e;
    z_convolve_kernel<<<dim3(tiles(p), p.g.py), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_y_convolve_2d(const ColPass &p, cudaStream_t s) {
    const size_t sm = 2 * sizeof(float2) * (size_t)3 * p.tx * (p.g.py + 1);
    cudaError_t e = ensure_smem((const void *)y_convolve_2d_kernel, sm);
    if (e != cudaSuccess) return e;
    y_convolve_2d_kernel<<<tiles(p), kThreads, sm, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_finalize_stats(const double *partials, int nblocks, double *out, cudaStream_t s) {
    finalize_stats_kernel<<<1, kThreads, 0, s>>>(partials, nblocks, out);
    return cudaGetLastError();
}

}  // namespace fm
