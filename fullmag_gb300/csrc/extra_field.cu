// extra_field.cu -- field terms evaluated by a pass of their own before each
// right-hand-side row pass and added by the row pass as its field map: DMI and the
// magnetoelastic field of a prescribed strain.
//
// Reference behaviour restated (paths in mzrptu/fullmag):
//   interfacial / bulk DMI field, central differences with the Neumann clamp and the
//   active mask                                 native/backends/fdm/src/demag_fp32.cu:319-366
//   magnetoelastic field (B1, B2, prescribed strain; shear strains halved from Voigt)
//                                               native/backends/fdm/src/demag_fp32.cu:368-376,582-583
//   DMI energy (FP64 sums of the FP32 state)    native/backends/fdm/src/reductions_fp64.cu:647-720
// The reference reports the bulk DMI energy as +V D m.(curl m) while its field is
// +2D/(mu0 Ms) curl m; both are kept as they are, so the energy is summed from its own
// formula, not from m.H.  The row pass adds this pass's output as its field map, so its
// own Zeeman sum would include these terms: the Zeeman sum m.(H_ext + H_map) is taken
// here instead, in FP64.
#include "engine.h"

#include <algorithm>

namespace fm {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kThreads) extra_field_kernel(const ExtraField p) {
    __shared__ double2 red[kThreads / 32];
    const Grid &g = p.g;
    const long long n = g.n;
    const float *m = p.m;
    double s_zee = 0.0, s_dmi = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float hx = 0.f, hy = 0.f, hz = 0.f;
        if (p.mask == nullptr || p.mask[i] != 0) {
            const float mx = m[i], my = m[n + i], mz = m[2 * n + i];
            float ax = 0.f, ay = 0.f, az = 0.f;  // DMI + magnetoelastic
            if (p.has_int || p.has_bulk) {
                const int x = (int)(i % g.nx);
                const long long r = i / g.nx;
                const int y = (int)(r % g.ny), z = (int)(r / g.ny);
                const long long sxy = (long long)g.nx * g.ny;
                long long xm = x > 0 ? i - 1 : i, xp = x < g.nx - 1 ? i + 1 : i;
                long long ym = y > 0 ? i - g.nx : i, yp = y < g.ny - 1 ? i + g.nx : i;
                long long zm = z > 0 ? i - sxy : i, zp = z < g.nz - 1 ? i + sxy : i;
                if (p.mask) {
                    if (!p.mask[xm]) xm = i;
                    if (!p.mask[xp]) xp = i;
                    if (!p.mask[ym]) ym = i;
                    if (!p.mask[yp]) yp = i;
                    if (!p.mask[zm]) zm = i;
                    if (!p.mask[zp]) zp = i;
                }
                // differences of neighbour values: component c of cell j at m[c n + j]
                auto dif = [&](int c, long long a, long long b) { return m[c * n + a] - m[c * n + b]; };
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
                if (p.partials) {
                    // the energy sums take the differences in FP64 of the FP32 state
                    auto ddif = [&](int c, long long a, long long b) { return (double)m[c * n + a] - (double)m[c * n + b]; };
                    const double i2x = p.dinv2dx, i2y = p.dinv2dy, i2z = p.dinv2dz;
                    const double Mx = mx, My = my, Mz = mz;
                    if (p.has_int)
                        s_dmi += p.d_int * (Mz * (ddif(0, xp, xm) * i2x + ddif(1, yp, ym) * i2y) - Mx * ddif(2, xp, xm) * i2x -
                                            My * ddif(2, yp, ym) * i2y);
                    if (p.has_bulk) {
                        const double cx = ddif(2, yp, ym) * i2y - ddif(1, zp, zm) * i2z;
                        const double cy = ddif(0, zp, zm) * i2z - ddif(2, xp, xm) * i2x;
                        const double cz = ddif(1, xp, xm) * i2x - ddif(0, yp, ym) * i2y;
                        s_dmi += p.d_bulk * (Mx * cx + My * cy + Mz * cz);
                    }
                }
            }
            if (p.has_mel) {
                ax += p.mel_pref * (2.f * p.b1 * mx * p.e11 + p.b2 * (my * p.e12 + mz * p.e13));
                ay += p.mel_pref * (2.f * p.b1 * my * p.e22 + p.b2 * (mx * p.e12 + mz * p.e23));
                az += p.mel_pref * (2.f * p.b1 * mz * p.e33 + p.b2 * (mx * p.e13 + my * p.e23));
            }
            hx = ax;
            hy = ay;
            hz = az;
            double zx = 0.0, zy = 0.0, zz = 0.0;  // applied field of the Zeeman sum
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
            if (p.partials) s_zee += (double)mx * zx + (double)my * zy + (double)mz * zz;
        }
        p.out[i] = hx;
        p.out[n + i] = hy;
        p.out[2 * n + i] = hz;
    }
    if (p.partials) {
        const double a = warp_sum(s_zee), b = warp_sum(s_dmi);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(a, b);
        __syncthreads();
        if (threadIdx.x == 0) {
            double2 t = make_double2(0.0, 0.0);
            for (int w = 0; w < kThreads / 32; ++w) {
                t.x += red[w].x;
                t.y += red[w].y;
            }
            p.partials[blockIdx.x] = t;
        }
    }
}

__global__ void __launch_bounds__(kThreads) extra_finalize_kernel(const double2 *__restrict__ partials, int nblocks,
                                                                  double *__restrict__ out) {
    __shared__ double2 red[kThreads / 32];
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) {
        a += partials[k].x;
        b += partials[k].y;
    }
    a = warp_sum(a);
    b = warp_sum(b);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(a, b);
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = make_double2(0.0, 0.0);
        for (int w = 0; w < kThreads / 32; ++w) {
            t.x += red[w].x;
            t.y += red[w].y;
        }
        out[0] = t.x;
        out[1] = t.y;
    }
}

}  // namespace

int extra_field_blocks(const Grid &g) { return (int)std::min<long long>((g.n + kThreads - 1) / kThreads, 152 * 8); }

cudaError_t launch_extra_field(const ExtraField &p, cudaStream_t s) {
    extra_field_kernel<<<extra_field_blocks(p.g), kThreads, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_extra_finalize(const double2 *partials, int nblocks, double *out, cudaStream_t s) {
    extra_finalize_kernel<<<1, kThreads, 0, s>>>(partials, nblocks, out);
    return cudaGetLastError();
}

}  // namespace fm
