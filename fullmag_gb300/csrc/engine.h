// engine.h -- device-side data layout and pass descriptors of the GB300 FDM engine.
//
// Layout in HBM (one allocation per buffer class, all 256-byte aligned):
//   vector fields : SoA float, component c of cell i at base[c*n + i],
//                   cell i = x + nx*(y + ny*z)
//   X spectrum    : x-transformed half spectrum, float2 X[c][z][y][kx],
//                   kx in [0, px/2], rows only for y < ny, z < nz (zero rows pruned)
//   Y spectrum    : (3-D only) y-transformed, float2 Y[c][z][ky][kx], ky in [0, py)
//   demag kernel  : with a periodic axis complex and full, pre-scaled by Ms/P:
//                   float2 K[6][pz][py][kx] (2-D: K[4][py][kx]); otherwise
//                   real, octant-unique, pre-scaled by Ms/P:
//                   3-D K[6][pz/2+1][py/2+1][kx]   (xx yy zz xy xz yz)
//                   2-D K[4][py/2+1][kx]           (xx yy zz xy)
//                   engines on the fused y+z path (small 3-D grids, every batched
//                   3-D problem) hold K[6][pz/2+1][kx][py/2+1]: their CTAs take one
//                   or a few kx columns and spread the threads over ky, so ky-fastest
//                   loads coalesce
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "fft_smem.cuh"

namespace fm {

// Programmatic dependent launch (sm_90 and later).  Every kernel of a step starts with
// pdl_wait(): it returns once the grid it depends on has completed and its memory is
// visible, so nothing it reads or writes can race the previous kernel.  With the pass's
// `early` flag, pdl_trigger() right after lets the next kernel's CTAs be scheduled as
// soon as this grid's last CTAs have started, so that kernel is resident and waiting
// when this one ends instead of being launched after it.  The engine sets the flag for
// small fixed-step problems, whose steps are a chain of sub-wave launches (measured:
// 256x64x1 RK4 -12 %, 64x32x4 Heun -21 % per step); on the 256x256x64 volume (+2 %) and
// the adaptive 512x128x1 film (+21 %) the early-resident CTAs cost more than they save.
// Launched without the attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// <<<grid, block, smem, s>>>(args) with programmatic stream serialisation allowed
template <typename... Exp, typename... Act>
cudaError_t launch_pdl(void (*kernel)(Exp...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Act &&...args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Act &&>(args)...);
}

constexpr int kNumStats = 9;  // e_ex e_d e_ext e_uni e_cub | max|Heff|^2 max|Hd|^2 max|k|^2 max err^2
constexpr int kMaxTerms = 8;

struct Material {
    float ex_pref;              // 2A/(mu0 Ms)
    float idx2, idy2, idz2;     // 1/d^2
    int has_ext;
    float hext[3];
    int has_uni;
    float ku1c, ku2c;           // 2Ku1/(mu0 Ms), 4Ku2/(mu0 Ms)
    float u[3];
    int has_cub;
    float kc1c, kc2c, kc3c;     // -2Kc1/(mu0 Ms), -2Kc2/(mu0 Ms), -4Kc3/(mu0 Ms)
    float c1[3], c2[3], c3[3];
    float gbar;                 // gamma/(1+alpha^2)
    float alpha;
    float prec;                 // 1 precession on, 0 damping only
    // energy densities (raw Ku, Kc in J/m^3) for the float-float reductions
    float ku1f, ku2f, kc1f, kc2f, kc3f;
};

struct Grid {
    int nx, ny, nz;
    long long n;
    int px, py, pz;  // padded extents (pz == 1 on the thin-film path)
    int nkx;         // px/2 + 1
    int half;        // px/2
    int nky, nkz;    // py/2+1, pz/2+1 (kernel octant extents)
    int thin;        // 1: 2-D transform (nz == 1, pz == 1)
    int per;         // periodic axes (bit 0 x, 1 y, 2 z): wrap-around stencils, unpadded transforms
    // dividers for the index arithmetic of the passes
    FastDiv fd_nx, fd_ny, fd_nz, fd_half, fd_nkx, fd_py, fd_pz, fd_padw;
    FastDiv fd_nx2, fd_nx4;  // nx / 2, nx / 4 (1 when nx is not a multiple)
};

inline void grid_dividers(Grid &g) {
    g.fd_nx = FastDiv((uint32_t)g.nx);
    g.fd_ny = FastDiv((uint32_t)g.ny);
    g.fd_nz = FastDiv((uint32_t)g.nz);
    g.fd_half = FastDiv((uint32_t)g.half);
    g.fd_nkx = FastDiv((uint32_t)g.nkx);
    g.fd_py = FastDiv((uint32_t)g.py);
    g.fd_pz = FastDiv((uint32_t)g.pz);
    g.fd_padw = FastDiv((uint32_t)(2 * g.half - g.nx > 0 ? 2 * g.half - g.nx : 1));
    g.fd_nx2 = FastDiv((uint32_t)(g.nx % 2 == 0 && g.nx >= 2 ? g.nx / 2 : 1));
    g.fd_nx4 = FastDiv((uint32_t)(g.nx % 4 == 0 && g.nx >= 4 ? g.nx / 4 : 1));
}

// Fused row pass: one CTA owns `rows` consecutive x-rows.  Depending on the
// flags it (1) inverts the x-transform of the demag spectrum, (2) evaluates
// exchange + Zeeman + anisotropy + torque, (3) accumulates FP64 statistics,
// (4) forms the next stage input normalize(m0 + dt*sum c_j k_j), and
// (5) forward-transforms that input along x for the next evaluation.
struct RowPass {
    Grid g;
    Material mat;
    const uint8_t *mask;
    // (1)
    const float2 *x_in;      // NULL: no demag
    FftPlan xplan;           // length px/2
    const float2 *xpost;     // e^{-2 pi i k / px}, k in [0, px/2]
    // (2)
    const float *m_in;       // stage input (SoA); NULL: no right-hand side in this pass
    float *k_out;            // NULL: keep the right-hand side in registers only
    // (3)
    float2 *partials;        // NULL: no statistics; else [kNumStats][gridDim.x] (hi, lo) pairs
    int n_err;               // DP45 error terms (0: none); NULL pointer = current k
    const float *err_k[kMaxTerms];
    double err_c[kMaxTerms];
    double err_dt;
    // (4)
    const float *m0;         // NULL: no stage combination (forward pass of m_fwd)
    float *m_next;
    int n_comb;
    const float *comb_k[kMaxTerms];  // NULL entry = current k
    float comb_c[kMaxTerms];
    float dt;
    const double *dt_dev;    // non-NULL: dt (and err_dt) read from device memory (graph replays)
    // (5)
    float2 *x_out;           // NULL: no forward transform
    const float *m_fwd;      // forward-transform source when m0 == NULL
    // per-cell applied field map (SoA, A/m), added to H_eff at active cells; NULL: none
    const float *hmap;
    // observables
    float *h_ex_out, *h_d_out, *h_eff_out;  // NULL: not written
    int rows;                // rows per CTA
    int early;               // let the next kernel launch early (pdl_trigger)
    // adjoint passes (launch_row_pass_adj only; see adjoint.cu for the equations); adj_mode
    // is a bit set, bit 2 runs before bit 1 at each cell:
    //   bit 2, after H_lin(lambda_H) (m_in = lambda_H, local terms off): lambda_y = adj_lam_m
    //          + H_lin; through y_s = N(y0 + ch k) into adj_lam_y0 and adj_lam_k (adj_k NULL:
    //          stage 0, lambda_y added to adj_lam_y0)
    //   bit 1, local VJP of k = f(m, H) with cotangent w (adj_uni: uniaxial Jacobian term):
    //          lambda_H -> adj_lam_h and the forward x-transform, lambda_m -> adj_lam_m
    //          (in place after bit 2 read it), lambda_H added to (adj_g_hi, adj_g_lo)
    int adj_mode;
    int adj_uni;
    const float *adj_m, *adj_H, *adj_w;
    float *adj_lam_h, *adj_lam_m, *adj_g_hi, *adj_g_lo;
    const float *adj_y0, *adj_k;
    float adj_ch;
    float *adj_lam_y0, *adj_lam_k;
};

struct ColPass {
    Grid g;
    FftPlan plan;
    FftPlan plan2;           // z plan of the fused y+z pass
    int tx;                  // kx columns per CTA
    FastDiv fd_tx;
    FastDiv fd_last;         // live columns of the last kx tile: nkx % tx, or tx
    const float2 *in;
    float2 *out;
    const float *kern;       // demag kernel (multiply passes)
    int inverse;
    const double *skip_dt;   // batched rounds: the problem's step size; <= 0 skips its tiles
    int pipe;                // z pass: 1 = the packed ky-pair kernel (tile 8)
    int split;               // two-level passes: 0 the default radix split N1 x N2, 1 the alternative
    int early;               // let the next kernel launch early (pdl_trigger)
};

// Launchers (kernels.cu)
size_t row_pass_smem(const RowPass &p);
cudaError_t launch_row_pass(const RowPass &p, cudaStream_t s);
cudaError_t launch_row_pass_adj(const RowPass &p, cudaStream_t s);  // adjoint modes 1 and 2
cudaError_t launch_y_forward(const ColPass &p, cudaStream_t s);     // X -> Y  (3-D)
cudaError_t launch_z_convolve(const ColPass &p, cudaStream_t s);    // Y -> Y  (3-D, z FFT, multiply, inverse)
cudaError_t launch_y_inverse(const ColPass &p, cudaStream_t s);     // Y -> X  (3-D)
cudaError_t launch_y_convolve_2d(const ColPass &p, cudaStream_t s); // X -> X  (thin film)
cudaError_t launch_yz_convolve(const ColPass &p, cudaStream_t s);  // X -> X (small 3-D, uses plan2 for z)
size_t yz_convolve_smem(const Grid &g, int tx);
// The truncated-image periodic kernel (layout above) of a grid with g.per != 0, as FP32
// (kern) or FP64 (kern64) complex values; exactly one of the two is non-null
bool newell_periodic_spectrum_gpu(const Grid &g, double dx, double dy, double dz, double ms, const uint32_t images[3],
                                  float2 *kern, double2 *kern64, cudaStream_t s, std::string &err);
// K[c][kz][ky][kx] -> K[c][kz][kx][ky] (the fused y+z path's layout), out of place
cudaError_t launch_kern_ky_fast(const float *in, float *out, int ncomp, int nkz, int nky, int nkx, cudaStream_t s);
size_t z_convolve_smem(const Grid &g, int tx);
// the packed ky-pair z pass exists for this grid at tile tx
bool z_convolve_pair_ok(const Grid &g, int tx);
size_t y_pass_smem(const Grid &g, int tx);
size_t y_convolve_2d_smem(const Grid &g, int tx);

// Field terms computed by a pass of their own before each right-hand-side row pass
// (extra_field.cu): interfacial and bulk DMI (central differences, Neumann clamp, mask)
// and the magnetoelastic field of a prescribed strain, plus the applied field map.  The
// row pass adds `out` as its field map; H = 0 at inactive cells.
// per-CTA sums of the extra field pass (each thread accumulates float-float pairs, the CTA
// adds them in FP64): Zeeman m.(H_ext + H_map), DMI energy density,
// with per-cell anisotropy maps the uniaxial and cubic energy densities, and with region ids
// the exchange pair sum sum A_ij |m_j - m_i|^2 / d^2
struct ExtraSums {
    double zee, dmi, uni, cub, exch;
};
// Brown thermal field of one evaluation: key = seed + step counter * 0x9E3779B97F4A7C15
// (wrapping) and the amplitude sigma (A/m); sigma 0 adds nothing
struct ThermalSlot {
    unsigned long long key;
    float sigma;
    float pad;
};

struct ExtraField {
    Grid g;
    const uint8_t *mask;
    const float *m;            // stage input (SoA)
    const float *hmap;         // applied field map or NULL
    float *out;                // H_extra (SoA)
    ExtraSums *partials;       // NULL: no sums; else one entry per CTA
    int has_ext;               // uniform applied field hext (A/m) in the Zeeman sum
    float hext[3];
    int has_int, has_bulk, has_mel;
    float dmi_int, dmi_bulk;   // 2 D / (mu0 Ms), A/m per unit gradient
    float d_int, d_bulk;       // D (J/m^2) for the energy sums
    float inv2dx, inv2dy, inv2dz;     // 1/(2 d)
    float mel_pref;            // -1 / (mu0 Ms)
    float b1, b2, e11, e22, e33, e23, e13, e12;  // B1, B2 (J/m^3), strain tensor (e_ij, i != j halved Voigt)
    // spin torques T (added to dm/dt by the reference) enter as the field H = a T + b m x T,
    // which the LLG right-hand side maps back to T for T perpendicular to m:
    // a = alpha / (gbar (s + alpha^2)), b = s / (gbar (s + alpha^2)), s = 1 with precession
    int torques;               // 0: leave the torque terms out (observable passes)
    int has_zl, has_slon, has_sot;
    float zl_u[3], zl_beta;    // Zhang-Li drift velocity (m/s) and non-adiabaticity
    float inv_dx, inv_dy, inv_dz;
    float slon_pf, slon_P, slon_l2, slon_eps, slon_p[3];  // Slonczewski
    float sot_amp, sot_xi_dl, sot_xi_fl, sot_s[3];        // spin-orbit torque
    float tq_a, tq_b;
    // per-cell anisotropy (any of the maps present): the whole uniaxial and cubic terms move
    // here from the row pass, each constant taken from its map when there is one
    int aniso;
    int has_uni, has_cub;
    const float *ku1m, *ku2m, *kc1m, *kc2m, *kc3m;  // maps (J/m^3) or NULL
    float ku1, ku2, kc1, kc2, kc3;                  // uniform values (J/m^3)
    float inv_mu0ms;                                // 1 / (mu0 Ms)
    float u[3], c1[3], c2[3], c3[3];
    // Oersted field: oe_scale[0] * h_oe (I(t) times the field for 1 A, SoA) or NULL
    const float *h_oe;
    const float *oe_scale;
    // exchange with region ids (exchange_fp32.cu:48-104): 2/(mu0 Ms) sum_q A[r_i][r_q] (m_q - m_i)/d_q^2
    // with A from the 256 x 256 FP64 table, read as FP32 for the field; the row pass's
    // exchange is off, and this pass writes the H_EX observable (h_ex_out) when asked
    const uint8_t *region;     // region id per cell (validated < 256, one byte each) or NULL
    const float *lut;          // exchange stiffness table as FP32, row-major [r_i][r_j] (J/m)
    float ex_s;                // 2 / (mu0 Ms)
    float idx2, idy2, idz2;    // 1 / d^2
    float *h_ex_out;
    // thermal field (crates/fullmag-engine/src/fdm_fields.rs:818-896) or NULL
    const ThermalSlot *th;
    int early;                 // let the next kernel launch early (pdl_trigger)
};
int extra_field_blocks(const Grid &g);
cudaError_t launch_extra_field(const ExtraField &p, cudaStream_t s);
// sums the per-CTA partials into out[0..4] (fixed order)
cudaError_t launch_extra_finalize(const ExtraSums *partials, int nblocks, double *out, cudaStream_t s, int early = 0);

// Adjoint (reverse-mode RK4): the final-combination pass (adjoint.cu); all fields SoA.
// The local VJP and the stage update are the row pass's adjoint modes.
struct AdjFinal {
    long long n;
    const float *lam_next, *y0, *k1, *k2, *k3, *k4;
    float h;
    float *lam_y0, *lk1, *lk2, *lk3, *lk4;
};
cudaError_t launch_adj_final(const AdjFinal &a, cudaStream_t s);

// Batched launches: one grid covering many problems through a (problem, block) table.
struct FinDesc {
    const float2 *partials;
    int nblocks;
    int pad;
};
cudaError_t launch_row_pass_batched(const RowPass *ps, const int2 *work, int nwork, size_t smem, cudaStream_t s);
cudaError_t launch_col_batched(const ColPass *ps, const int2 *work, int nwork, int kind, size_t smem, cudaStream_t s);
cudaError_t launch_finalize_batched(const FinDesc *fd, int nproblems, double *out, cudaStream_t s);
cudaError_t launch_finalize_stats(const float2 *partials, int nblocks, double *out, cudaStream_t s, int early = 0);
int row_pass_blocks(const RowPass &p);
// Kernel of the batched column pass for a grid: 0 thin film pruned, 1 fused y+z pruned,
// 2 thin film general, 3 fused y+z general.
int col_batched_kind(const Grid &g);
int col_tile(const Grid &g, int lines_per_col, int len);

}  // namespace fm
