// extra_field.cu -- field terms evaluated by a pass of their own before each
// right-hand-side row pass and added by the row pass as its field map: DMI and the
// magnetoelastic field of a prescribed strain.
//
// Reference behaviour restated (paths in mzrptu/fullmag):
//   interfacial / bulk DMI field, central differences with the Neumann clamp and the
//   active mask                                 native/backends/fdm/src/demag_fp32.cu:319-366
//   magnetoelastic field (B1, B2, prescribed strain; shear strains halved from Voigt)
//                                               native/backends/fdm/src/demag_fp32.cu:368-376,582-583
//   DMI energy (sums of the FP32 state)         native/backends/fdm/src/reductions_fp64.cu:647-720
//   Oersted field of a cylindrical conductor, scaled by I(t)
//                                               native/backends/fdm/src/context.cu:844-905,
//                                               demag_fp32.cu:585-616
//   Zhang-Li and Slonczewski spin-transfer torque, spin-orbit torque
//                                               native/backends/fdm/src/llg_fp32.cu:65-195
//                                               prefactors api.cpp:250-300, context.hpp:321-339
//   Brown thermal field: SplitMix64 counter keyed by (seed, step, cell, stream), Box-Muller
//                                               crates/fullmag-engine/src/fdm_fields.rs:818-896
//   exchange with region ids and a 256 x 256 stiffness table
//                                               native/backends/fdm/src/exchange_fp32.cu:48-104,
//                                               api.cpp:405-420, reductions_fp64.cu:123-215
// A torque T perpendicular to m is passed as the field H = a T + b (m x T), which the row
// pass's LLG right-hand side maps back to exactly T; m.H = 0, so it adds no energy.
// The reference reports the bulk DMI energy as +V D m.(curl m) while its field is
// +2D/(mu0 Ms) curl m; both are kept as they are, so the energy is summed from its own
// formula, not from m.H.  The row pass adds this pass's output as its field map, so its
// own Zeeman sum would include these terms: the Zeeman sum m.(H_ext + H_map) is taken
// here instead.  Every energy term is formed in FP32 and summed in float-float pairs
// (TwoSum); only the per-CTA reduction runs in FP64, whose throughput is a small fraction
// of FP32 on this part.
#include "engine.h"
#include "fft_smem.cuh"

#include <algorithm>
#include <atomic>

namespace fm {

namespace {

constexpr int kThreads = 256;

// SplitMix64 output function (Vigna's published finaliser)
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// b < 2^54 as FP32 from its two 32-bit halves (32-bit conversions and one FMA, which keep
// the 64-bit conversion off the slow pipe)
__device__ __forceinline__ float u54_to_float(unsigned long long b) {
    return fmaf((float)(unsigned)(b >> 32), 4294967296.0f, (float)(unsigned)b);
}

// u = ((bits >> 11) + 1) / (2^53 + 1) in (0, 1], as FP32
__device__ __forceinline__ float unit_of(unsigned long long bits) { return u54_to_float((bits >> 11) + 1ull) * 0x1p-53f; }

// -2 ln u: logf of u itself up to u = 1/2, log1pf(-(1 - u)) above, with 1 - u formed from
// the exact integer so that u near 1 keeps its relative accuracy
__device__ __forceinline__ float neg2log_of(unsigned long long bits) {
    const unsigned long long b = (bits >> 11) + 1ull;  // 1 .. 2^53
    if (b <= (1ull << 52)) return -2.f * logf(u54_to_float(b) * 0x1p-53f);
    return -2.f * log1pf(-u54_to_float((1ull << 53) + 1ull - b) * 0x1p-53f);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// fixed-order block sum of the five partial sums; thread 0 returns the CTA's total
__device__ __forceinline__ ExtraSums block_sum(ExtraSums v) {
    __shared__ ExtraSums red[kThreads / 32];
    v.zee = warp_sum(v.zee);
    v.dmi = warp_sum(v.dmi);
    v.uni = warp_sum(v.uni);
    v.cub = warp_sum(v.cub);
    v.exch = warp_sum(v.exch);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    ExtraSums t{0.0, 0.0, 0.0, 0.0, 0.0};
    if (threadIdx.x == 0)
        for (int w = 0; w < kThreads / 32; ++w) {
            t.zee += red[w].zee;
            t.dmi += red[w].dmi;
            t.uni += red[w].uni;
            t.cub += red[w].cub;
            t.exch += red[w].exch;
        }
    return t;
}

// three CTAs per SM (80 registers, no spills)
// kNb: neighbour stencils (DMI, Zhang-Li) compiled in; kRg: exchange with region ids;
// kTh: thermal field.  The instances without them keep fewer registers.
template <bool kNb, bool kRg, bool kTh>
__global__ void __launch_bounds__(kThreads, kRg ? 3 : 4) extra_field_kernel(const ExtraField p) {
    pdl_wait();
    if (p.early) pdl_trigger();
    const Grid &g = p.g;
    const long long n = g.n;
    const float *m = p.m;
    // energy sums: FP32 terms in float-float pairs (TwoSum); FP64 only in the CTA reduction,
    // since FP64 throughput is a small fraction of FP32 on this part
    enum { kZee, kDmi, kUni, kCub, kExch };
    float sh[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, sl[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    // one cell: its state (mx, my, mz) is loaded by the caller
    auto cell = [&](const long long i, const float mx, const float my, const float mz) {
        float hx = 0.f, hy = 0.f, hz = 0.f;
        float rx = 0.f, ry = 0.f, rz = 0.f;  // region exchange (the H_EX observable)
        if (p.mask == nullptr || p.mask[i] != 0) {
            float ax = 0.f, ay = 0.f, az = 0.f;  // DMI + magnetoelastic
            if ((kNb || kRg) && (p.has_int || p.has_bulk || (kRg && p.region))) {
                // neighbours with the Neumann clamp: a missing or inactive neighbour is the cell
                // itself; on a periodic axis the neighbour wraps around (fdm_types.rs:126-132)
                const int x = (int)(i % g.nx);
                const long long r = i / g.nx;
                const int y = (int)(r % g.ny), z = (int)(r / g.ny);
                const long long sxy = (long long)g.nx * g.ny;
                const int per = g.per;
                long long xm = x > 0 ? i - 1 : (per & 1) ? i + g.nx - 1 : i;
                long long xp = x < g.nx - 1 ? i + 1 : (per & 1) ? i - (g.nx - 1) : i;
                long long ym = y > 0 ? i - g.nx : (per & 2) ? i + sxy - g.nx : i;
                long long yp = y < g.ny - 1 ? i + g.nx : (per & 2) ? i - sxy + g.nx : i;
                long long zm = z > 0 ? i - sxy : (per & 4) ? i + sxy * (g.nz - 1) : i;
                long long zp = z < g.nz - 1 ? i + sxy : (per & 4) ? i - sxy * (g.nz - 1) : i;
                if (p.mask) {
                    if (!p.mask[xm]) xm = i;
                    if (!p.mask[xp]) xp = i;
                    if (!p.mask[ym]) ym = i;
                    if (!p.mask[yp]) yp = i;
                    if (!p.mask[zm]) zm = i;
                    if (!p.mask[zp]) zp = i;
                }
                if (kRg && p.region) {
                    // sum_q A[r_i][r_q] (m_q - m_i) / d_q^2 in the order x+, x-, y+, y-, z+, z-
                    const float *row = p.lut + (size_t)p.region[i] * 256;
                    const long long nb[6] = {xp, xm, yp, ym, zp, zm};
                    const float w[6] = {p.idx2, p.idx2, p.idy2, p.idy2, p.idz2, p.idz2};
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const long long j = nb[q];
                        const float a = row[p.region[j]] * w[q];
                        rx += a * (m[j] - mx);
                        ry += a * (m[n + j] - my);
                        rz += a * (m[2 * n + j] - mz);
                    }
                    rx *= p.ex_s;
                    ry *= p.ex_s;
                    rz *= p.ex_s;
                    ax += rx;
                    ay += ry;
                    az += rz;
                    if (p.partials) {
                        // forward pairs (x+1, y+1, z+1) with an active neighbour, each pair once
                        const float fwv[3] = {p.idx2, p.idy2, p.idz2};
                        const long long fw[3] = {xp, yp, zp};
#pragma unroll
                        for (int a = 0; a < 3; ++a) {
                            const long long j = fw[a];
                            if (j == i) continue;
                            const float d0 = m[j] - mx, d1 = m[n + j] - my, d2 = m[2 * n + j] - mz;
                            ff_add(sh[kExch], sl[kExch], row[p.region[j]] * (d0 * d0 + d1 * d1 + d2 * d2) * fwv[a]);
                        }
                    }
                }
                // differences of neighbour values: component c of cell j at m[c n + j]
                auto dif = [&](int c, long long a, long long b) { return m[c * n + a] - m[c * n + b]; };
                if (p.has_int || p.has_bulk) {
                    const float dmx_dx = dif(0, xp, xm) * p.inv2dx, dmy_dx = dif(1, xp, xm) * p.inv2dx;
                    const float dmz_dx = dif(2, xp, xm) * p.inv2dx;
                    const float dmx_dy = dif(0, yp, ym) * p.inv2dy, dmy_dy = dif(1, yp, ym) * p.inv2dy;
                    const float dmz_dy = dif(2, yp, ym) * p.inv2dy;
                    const float dmx_dz = dif(0, zp, zm) * p.inv2dz, dmy_dz = dif(1, zp, zm) * p.inv2dz;
                    if (p.has_int) {
                        ax += p.dmi_int * dmz_dx;
                        ay += p.dmi_int * dmz_dy;
                        az -= p.dmi_int * (dmx_dx + dmy_dy);
                    }
                    if (p.has_bulk) {
                        ax += p.dmi_bulk * (dmz_dy - dmy_dz);
                        ay += p.dmi_bulk * (dmx_dz - dmz_dx);
                        az += p.dmi_bulk * (dmy_dx - dmx_dy);
                    }
                    if (p.partials) {  // energy densities from the same central differences
                        if (p.has_int)
                            ff_add(sh[kDmi], sl[kDmi], p.d_int * (mz * (dmx_dx + dmy_dy) - mx * dmz_dx - my * dmz_dy));
                        if (p.has_bulk)
                            ff_add(sh[kDmi], sl[kDmi], p.d_bulk * (mx * (dmz_dy - dmy_dz) + my * (dmx_dz - dmz_dx) +
                                                                   mz * (dmy_dx - dmx_dy)));
                    }
                }
            }
            if (p.has_mel) {
                ax += p.mel_pref * (2.f * p.b1 * mx * p.e11 + p.b2 * (my * p.e12 + mz * p.e13));
                ay += p.mel_pref * (2.f * p.b1 * my * p.e22 + p.b2 * (mx * p.e12 + mz * p.e23));
                az += p.mel_pref * (2.f * p.b1 * mz * p.e33 + p.b2 * (mx * p.e13 + my * p.e23));
            }
            if (p.aniso) {
                // per-cell anisotropy, the row pass's formulas with constants from the maps
                // (native/backends/fdm/src/demag_fp32.cu:271-317)
                if (p.has_uni) {
                    const float k1 = p.ku1m ? p.ku1m[i] : p.ku1, k2 = p.ku2m ? p.ku2m[i] : p.ku2;
                    const float mu = mx * p.u[0] + my * p.u[1] + mz * p.u[2];
                    const float cf = 2.f * p.inv_mu0ms * (k1 * mu + 2.f * k2 * mu * mu * mu);
                    ax += cf * p.u[0];
                    ay += cf * p.u[1];
                    az += cf * p.u[2];
                    if (p.partials) {
                        const float s2 = mu * mu;
                        ff_add(sh[kUni], sl[kUni], k1 * s2 + k2 * s2 * s2);
                    }
                }
                if (p.has_cub) {
                    const float k1 = p.kc1m ? p.kc1m[i] : p.kc1, k2 = p.kc2m ? p.kc2m[i] : p.kc2;
                    const float k3 = p.kc3m ? p.kc3m[i] : p.kc3;
                    const float a1 = mx * p.c1[0] + my * p.c1[1] + mz * p.c1[2];
                    const float a2 = mx * p.c2[0] + my * p.c2[1] + mz * p.c2[2];
                    const float a3 = mx * p.c3[0] + my * p.c3[1] + mz * p.c3[2];
                    const float s1 = a1 * a1, s2 = a2 * a2, s3 = a3 * a3;
                    const float sig = s1 * s2 + s2 * s3 + s1 * s3;
                    const float f1 = -2.f * k1 * p.inv_mu0ms, f2 = -2.f * k2 * p.inv_mu0ms, f3 = -4.f * k3 * p.inv_mu0ms;
                    const float g1 = f1 * a1 * (s2 + s3) + f2 * a1 * s2 * s3 + f3 * sig * a1 * (s2 + s3);
                    const float g2 = f1 * a2 * (s1 + s3) + f2 * a2 * s1 * s3 + f3 * sig * a2 * (s1 + s3);
                    const float g3 = f1 * a3 * (s1 + s2) + f2 * a3 * s1 * s2 + f3 * sig * a3 * (s1 + s2);
                    ax += g1 * p.c1[0] + g2 * p.c2[0] + g3 * p.c3[0];
                    ay += g1 * p.c1[1] + g2 * p.c2[1] + g3 * p.c3[1];
                    az += g1 * p.c1[2] + g2 * p.c2[2] + g3 * p.c3[2];
                    if (p.partials) ff_add(sh[kCub], sl[kCub], k1 * sig + k2 * s1 * s2 * s3 + k3 * sig * sig);
                }
            }
            if (p.torques && (p.has_zl || p.has_slon || p.has_sot)) {
                float tx = 0.f, ty = 0.f, tz = 0.f;
                if (kNb && p.has_zl) {
                    // D = (u.grad) m by upwind differences: the upwind neighbour when it
                    // exists, read without the mask (native/backends/fdm/src/llg_fp32.cu:65-140)
                    const long long r = i / g.nx;
                    const int pos[3] = {(int)(i % g.nx), (int)(r % g.ny), (int)(r / g.ny)};
                    const int ext[3] = {g.nx, g.ny, g.nz};
                    const long long st[3] = {1, g.nx, (long long)g.nx * g.ny};
                    const float inv[3] = {p.inv_dx, p.inv_dy, p.inv_dz};
                    float Dx = 0.f, Dy = 0.f, Dz = 0.f;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const float u = p.zl_u[a];
                        // a periodic axis always has its upwind neighbour, wrapped around
                        // (fdm_fields.rs:1288-1320)
                        const bool wrap = (g.per >> a) & 1;
                        if (u > 0.f && (pos[a] > 0 || wrap)) {
                            const long long q = pos[a] > 0 ? i - st[a] : i + st[a] * (ext[a] - 1);
                            Dx += u * (mx - m[q]) * inv[a];
                            Dy += u * (my - m[n + q]) * inv[a];
                            Dz += u * (mz - m[2 * n + q]) * inv[a];
                        } else if (u < 0.f && (pos[a] < ext[a] - 1 || wrap)) {
                            const long long q = pos[a] < ext[a] - 1 ? i + st[a] : i - st[a] * (ext[a] - 1);
                            Dx += u * (m[q] - mx) * inv[a];
                            Dy += u * (m[n + q] - my) * inv[a];
                            Dz += u * (m[2 * n + q] - mz) * inv[a];
                        }
                    }
                    const float c1x = my * Dz - mz * Dy, c1y = mz * Dx - mx * Dz, c1z = mx * Dy - my * Dx;
                    const float c2x = my * c1z - mz * c1y, c2y = mz * c1x - mx * c1z, c2z = mx * c1y - my * c1x;
                    tx += -c2x - p.zl_beta * c1x;
                    ty += -c2y - p.zl_beta * c1y;
                    tz += -c2z - p.zl_beta * c1z;
                }
                if (p.has_slon) {  // llg_fp32.cu:142-170
                    const float px_ = p.slon_p[0], py_ = p.slon_p[1], pz_ = p.slon_p[2];
                    const float mp = mx * px_ + my * py_ + mz * pz_;
                    const float gs = p.slon_pf * (p.slon_P * p.slon_l2) / ((p.slon_l2 + 1.f) + (p.slon_l2 - 1.f) * mp);
                    const float c1x = my * pz_ - mz * py_, c1y = mz * px_ - mx * pz_, c1z = mx * py_ - my * px_;
                    const float c2x = my * c1z - mz * c1y, c2y = mz * c1x - mx * c1z, c2z = mx * c1y - my * c1x;
                    tx += gs * (c2x + p.slon_eps * c1x);
                    ty += gs * (c2y + p.slon_eps * c1y);
                    tz += gs * (c2z + p.slon_eps * c1z);
                }
                if (p.has_sot) {  // llg_fp32.cu:172-195
                    const float sx = p.sot_s[0], sy = p.sot_s[1], sz = p.sot_s[2];
                    const float ms_ = mx * sx + my * sy + mz * sz;
                    tx += p.sot_amp * (-p.sot_xi_dl * (ms_ * mx - sx) + p.sot_xi_fl * (my * sz - mz * sy));
                    ty += p.sot_amp * (-p.sot_xi_dl * (ms_ * my - sy) + p.sot_xi_fl * (mz * sx - mx * sz));
                    tz += p.sot_amp * (-p.sot_xi_dl * (ms_ * mz - sz) + p.sot_xi_fl * (mx * sy - my * sx));
                }
                // the field whose LLG right-hand side is T
                ax += p.tq_a * tx + p.tq_b * (my * tz - mz * ty);
                ay += p.tq_a * ty + p.tq_b * (mz * tx - mx * tz);
                az += p.tq_a * tz + p.tq_b * (mx * ty - my * tx);
            }
            if (p.h_oe) {  // counted in no energy, as the reference's energies leave it out
                const float I = *p.oe_scale;
                ax += I * p.h_oe[i];
                ay += I * p.h_oe[n + i];
                az += I * p.h_oe[2 * n + i];
            }
            if (kTh && p.th) {  // in no energy sum, as in the reference
                const float sg = p.th->sigma;
                if (sg > 0.f) {
                    constexpr unsigned long long kCell = 0x517CC1B727220A95ull, kStream = 0x6C62272E07BB0142ull;
                    const unsigned long long key = p.th->key + (unsigned long long)i * kCell;
                    const float r1 = sqrtf(neg2log_of(mix64(key)));
                    const float r2 = sqrtf(neg2log_of(mix64(key + 2ull * kStream)));
                    float s1, c1, s2, c2;
                    sincospif(2.f * unit_of(mix64(key + kStream)), &s1, &c1);
                    sincospif(2.f * unit_of(mix64(key + 3ull * kStream)), &s2, &c2);
                    ax += sg * r1 * c1;
                    ay += sg * r1 * s1;
                    az += sg * r2 * c2;
                }
            }
            hx = ax;
            hy = ay;
            hz = az;
            float zx = 0.f, zy = 0.f, zz = 0.f;  // applied field of the Zeeman sum
            if (p.has_ext) {
                zx = p.hext[0];
                zy = p.hext[1];
                zz = p.hext[2];
            }
            if (p.hmap) {
                const float ux = p.hmap[i], uy = p.hmap[n + i], uz = p.hmap[2 * n + i];
                hx += ux;
                hy += uy;
                hz += uz;
                zx += ux;
                zy += uy;
                zz += uz;
            }
            if (p.partials) ff_add(sh[kZee], sl[kZee], mx * zx + my * zy + mz * zz);
        }
        p.out[i] = hx;
        p.out[n + i] = hy;
        p.out[2 * n + i] = hz;
        if (p.h_ex_out) {
            p.h_ex_out[i] = rx;
            p.h_ex_out[n + i] = ry;
            p.h_ex_out[2 * n + i] = rz;
        }
    };
    const long long T = (long long)gridDim.x * blockDim.x;
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if constexpr (!kNb && !kRg && !kTh) {
        // local terms only: four cells a thread strided by the grid, their state loads
        // issued together ahead of the work (four times the bytes in flight of one cell per
        // iteration; each load instruction still reads 32 consecutive cells of a warp).
        // Measured on 256x256x64: magnetoelastic field 38.6 -> 31.7 us, spin-orbit torque
        // 39.4 -> 32.8 us; the stencil and thermal instances keep one cell per iteration,
        // where it measured slower (DMI +10 %, thermal +3 %).
        for (; i + 3 * T < n; i += 4 * T) {
            float v[4][3];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                v[j][0] = m[i + j * T];
                v[j][1] = m[n + i + j * T];
                v[j][2] = m[2 * n + i + j * T];
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) cell(i + j * T, v[j][0], v[j][1], v[j][2]);
        }
    }
    for (; i < n; i += T) cell(i, m[i], m[n + i], m[2 * n + i]);
    if (p.partials) {
        const ExtraSums t = block_sum(ExtraSums{(double)sh[kZee] + (double)sl[kZee], (double)sh[kDmi] + (double)sl[kDmi],
                                                (double)sh[kUni] + (double)sl[kUni], (double)sh[kCub] + (double)sl[kCub],
                                                (double)sh[kExch] + (double)sl[kExch]});
        if (threadIdx.x == 0) p.partials[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kThreads) extra_finalize_kernel(const ExtraSums *__restrict__ partials, int nblocks,
                                                                  double *__restrict__ out, int early) {
    pdl_wait();
    if (early) pdl_trigger();
    ExtraSums v{0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) {
        v.zee += partials[k].zee;
        v.dmi += partials[k].dmi;
        v.uni += partials[k].uni;
        v.cub += partials[k].cub;
        v.exch += partials[k].exch;
    }
    const ExtraSums t = block_sum(v);
    if (threadIdx.x == 0) {
        out[0] = t.zee;
        out[1] = t.dmi;
        out[2] = t.uni;
        out[3] = t.cub;
        out[4] = t.exch;
    }
}

}  // namespace

// 12 CTAs per SM (1824 on the 152 SMs of a GB300), threads striding over the cells: three
// full waves of the four-CTA-per-SM instances (no region exchange) and four of the
// three-CTA region instances.  The SM count is read once from the current device.
int extra_field_blocks(const Grid &g) {
    static std::atomic<int> sms{0};
    int k = sms.load(std::memory_order_relaxed);
    if (k == 0) {
        int dev = 0, v = 0;
        k = (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
             v > 0)
                ? v
                : 152;
        sms.store(k, std::memory_order_relaxed);
    }
    return (int)std::min<long long>((g.n + kThreads - 1) / kThreads, (long long)k * 3 * 4);
}

cudaError_t launch_extra_field(const ExtraField &p, cudaStream_t s) {
    const bool rg = p.region != nullptr, th = p.th != nullptr;
    const bool nb = p.has_int || p.has_bulk || (p.torques && p.has_zl);
    const dim3 grid(extra_field_blocks(p.g));
    const dim3 block(kThreads);
    if (rg)  // region exchange: the full instance (neighbours, with or without thermal)
        return th ? launch_pdl(extra_field_kernel<true, true, true>, grid, block, 0, s, p)
                  : launch_pdl(extra_field_kernel<true, true, false>, grid, block, 0, s, p);
    if (nb)
        return th ? launch_pdl(extra_field_kernel<true, false, true>, grid, block, 0, s, p)
                  : launch_pdl(extra_field_kernel<true, false, false>, grid, block, 0, s, p);
    return th ? launch_pdl(extra_field_kernel<false, false, true>, grid, block, 0, s, p)
              : launch_pdl(extra_field_kernel<false, false, false>, grid, block, 0, s, p);
}

cudaError_t launch_extra_finalize(const ExtraSums *partials, int nblocks, double *out, cudaStream_t s, int early) {
    return launch_pdl(extra_finalize_kernel, dim3(1), dim3(kThreads), 0, s, partials, nblocks, out, early);
}

}  // namespace fm
