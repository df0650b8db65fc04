/*
 * fdm_oracle.h -- FP64 CPU restatement of the reference FDM LLG path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the parity checker for the CUDA
 * engine and the timed CPU baseline; the product library never links it.
 * It restates, in plain C with OpenMP, the algorithms of
 *   crates/fullmag-fdm-demag/src/newell.rs      (Newell f/g, 27-point stencil, octants)
 *   crates/fullmag-engine/src/fdm_fft.rs        (zero-padded FFT convolution)
 *   crates/fullmag-engine/src/fdm_fields.rs     (exchange, demag, local terms, RHS, energies)
 *   crates/fullmag-engine/src/fdm_integrators.rs (Heun, RK4, Dormand-Prince 5(4)),
 *   native/backends/fdm/src/llg_rk23_fp32.cu, llg_abm3_fp32.cu (RK23, ABM3 as the ABI runs them)
 * and the step/stat semantics of native/backends/fdm (the C ABI this engine replaces).
 * The reference's FFT comes from rustfft 6.4.1 (Cargo.lock:3647-3649), which is not
 * in the reference tree; fo_fft1d is an own mixed-radix FFT validated against numpy.fft.
 */
#ifndef FDM_ORACLE_H
#define FDM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Newell tensor ---- */
double fo_newell_f(double x, double y, double z);
double fo_newell_g(double x, double y, double z);

/* Real-space tensors on the (2nx,2ny,2nz) padded grid, out = 6 arrays
 * [xx, yy, zz, xy, xz, yz] of 8*nx*ny*nz doubles each. */
int fo_newell_kernels(int nx, int ny, int nz, double dx, double dy, double dz, double *out);

/* Spectra as handed to the C ABI: 6 arrays of 2*P interleaved complex values.
 * thin_film_2d != 0 (requires nz == 1) uses P = 2nx*2ny, else P = 2nx*2ny*2nz. */
int fo_newell_spectra(int nx, int ny, int nz, double dx, double dy, double dz,
                      int thin_film_2d, double *out);

/* ---- FFT (interleaved complex, unnormalised; inverse uses e^{+i}) ---- */
int fo_fft1d(double *data, int n, int inverse);
int fo_fft3d(double *data, int px, int py, int pz, int inverse);

/* ---- Problem ---- */
typedef struct {
    int32_t nx, ny, nz;
    int32_t integrator;          /* 1 Heun, 2 DP45, 3 ABM3, 4 RK4, 5 RK23 (ABI values) */
    double dx, dy, dz;
    double ms, a_ex, alpha, gamma;
    int32_t enable_exchange, enable_demag, has_external_field, disable_precession;
    double h_ext[3];
    int32_t has_uniaxial;
    int32_t has_cubic;
    double ku1, ku2, u_axis[3];
    double kc1, kc2, kc3, c1[3], c2[3];
    /* adaptive control */
    double max_error, dt_min, dt_max, headroom;
    double rtol, growth_limit, shrink_limit;
    int32_t dp45_norm;           /* 0: ABI absolute max-norm, 1: CPU mixed atol/rtol norm */
    int32_t pad0;
    const uint8_t *active_mask;  /* optional, copied at create */
    /* optional region ids (< FO_MAX_REGIONS) and the inter-region exchange table
     * A[r_i * FO_MAX_REGIONS + r_j] in J/m (NULL with regions: A on the diagonal, 0 off
     * it), copied at create; native/backends/fdm/src/exchange_fp32.cu:48-104, api.cpp:405-420 */
    const uint32_t *region_mask;
    const double *exchange_lut;
    /* DMI (J/m^2) and magnetoelastic coupling (B1, B2 in J/m^3, Voigt strain e11 e22 e33
     * 2e23 2e13 2e12): native/backends/fdm/src/demag_fp32.cu:319-376,582-583 */
    int32_t has_interfacial_dmi, has_bulk_dmi;
    double dmi_d_interfacial, dmi_d_bulk;
    int32_t has_magnetoelastic, pad1;
    double mel_b1, mel_b2;
    double mel_strain[6];
    /* spin-transfer and spin-orbit torques (native/backends/fdm/src/llg_fp32.cu:65-195;
     * prefactors api.cpp:250-300, context.hpp:321-339) */
    double current_density[3];   /* A/m^2: Zhang-Li drift (with stt_degree > 0) and Slonczewski |j| */
    double stt_degree, stt_beta;
    double stt_p[3];             /* Slonczewski polarisation (not normalised, as the reference) */
    double stt_lambda, stt_epsilon_prime;
    int32_t has_sot, pad2;
    double sot_je, sot_xi_dl, sot_xi_fl;
    double sot_sigma[3];
    double sot_thickness;
    /* optional per-cell Ku1 Ku2 Kc1 Kc2 Kc3 (J/m^3, one per cell), copied at create
     * (native/backends/fdm/src/demag_fp32.cu:275-292) */
    const double *ku1_field, *ku2_field, *kc1_field, *kc2_field, *kc3_field;
    /* Oersted field of a cylindrical conductor along z through (cx, cy), radius R, current
     * I(t): kind 0 constant, 1 I (sin(2 pi f t + phase) + offset), 2 I on [t_on, t_off)
     * (native/backends/fdm/src/context.cu:826-905, demag_fp32.cu:585-616) */
    int32_t has_oersted, oersted_kind;
    double oersted_current, oersted_radius, oersted_center[3];
    double oersted_freq, oersted_phase, oersted_offset, oersted_t_on, oersted_t_off;
    /* Brown thermal field at temperature T (K, 0 = none): counter-based Gaussian noise keyed
     * by (seed, step counter, cell) with sigma^2 = 2 alpha kB T / (gamma (1 + alpha^2) mu0 Ms V dt)
     * (crates/fullmag-engine/src/fdm_fields.rs:818-896, fdm_problem.rs:24-35,244-273) */
    double temperature;
    uint64_t thermal_seed;
    /* boundary correction of the double-precision path (all copied at create):
     * tier 0 none, 1 T0 face-link exchange (native/backends/fdm/src/exchange_t0_fp64.cu:27-164),
     * 2 T1 boundary stencil (exchange_t1_fp64.cu:38-204); with a tier the demag input is
     * phi Ms m (demag_fp64.cu:55-90) and the energies weight each cell by phi
     * (reductions_fp64.cu:123-260); face and delta are +x -x +y -y +z -z */
    int32_t boundary_tier, pad3;
    double phi_floor, delta_min;
    const double *volume_fraction;
    const double *face[6];
    const double *delta[6];
    /* sparse demag correction H_d(t) -= sum_s dN(t, s) phi_s Ms m_s, tensor rows xx xy xz yy
     * yz zz (demag_boundary_fp64.cu:23-76); phi_s = 1 without volume fractions */
    const int32_t *corr_target_idx;
    const int32_t *corr_source_idx;
    const double *corr_tensor;
    uint32_t corr_targets, corr_stencil;
    /* periodic boundaries of the reference CPU engine (crates/fullmag-engine/src/fdm_types.rs:84-132,
     * fdm_problem.rs:19-23): per axis 0 open, 1 periodic, and the demag images on each side
     * of a periodic axis (the reference default is 10) */
    int32_t periodic[3];
    uint32_t image_counts[3];
} fo_params;

#define FO_MAX_REGIONS 256

typedef struct {
    double step, time, dt_used, suggested_next_dt;
    double e_exchange;           /* pair sum A V |dm|^2 / d^2 (equals -1/2 mu0 Ms V m.H_ex) */
    double e_exchange_field;     /* -1/2 mu0 Ms V sum m.H_ex (CPU reference form) */
    double e_demag;              /* -1/2 mu0 Ms V sum m.H_d */
    double e_external;           /* -mu0 Ms V sum m.H_ext */
    double e_uniaxial;           /* -V sum (Ku1 (m.u)^2 + Ku2 (m.u)^4)  (C ABI convention) */
    double e_cubic;              /* V sum (Kc1 s + Kc2 p + Kc3 s^2)    (C ABI convention) */
    double e_anis_cpu;           /* -1/2 mu0 Ms V sum m.H_anis          (CPU reference convention) */
    double e_total;              /* e_exchange + e_demag + e_external + e_uniaxial + e_cubic + e_dmi */
    double max_h_eff, max_h_demag, max_rhs;
    double rejected_attempts;
    double e_dmi;                /* V sum of the DMI energy densities (reductions_fp64.cu:647-720 forms) */
} fo_stats;

typedef struct fo_problem fo_problem;

fo_problem *fo_create(const fo_params *p, const double *m0_aos);
void fo_destroy(fo_problem *pr);
int fo_set_m(fo_problem *pr, const double *m_aos);
int fo_get_m(const fo_problem *pr, double *m_aos);
/* Per-cell applied field (AoS, A/m) added to H_eff at active cells; NULL removes it. */
int fo_set_field_map(fo_problem *pr, const double *h_aos);
/* Fields at an arbitrary state (AoS in/out, any pointer may be NULL). */
int fo_fields(fo_problem *pr, const double *m_aos, double *h_ex, double *h_demag,
              double *h_ext, double *h_eff, double *rhs);
/* Stats of the current state (fields recomputed). */
int fo_observe(fo_problem *pr, fo_stats *st);
/* One accepted step with the ABI semantics of the configured integrator. */
int fo_step(fo_problem *pr, double dt, fo_stats *st);
/* FP64 tangent-linear model of n_steps fixed RK4 steps from the current state (which
 * it advances): dm_out = d m_final [dm0, dh] for an initial-state perturbation dm0 and
 * a field-map perturbation dh (A/m), either may be NULL.  Returns -1 with cubic
 * anisotropy (not differentiated). */
int fo_tangent_rk4(fo_problem *pr, double dt, uint64_t n_steps, const double *dh_aos, const double *dm0_aos,
                   double *dm_out);
/* Spatial truncated-image tensor of a grid with periodic axes (fdm_fft.rs:614-717): six
 * real arrays over (px, py, pz), px = nx on a periodic axis and 2 nx on an open one, entry
 * (i, j, k) = sum over |m_a| <= images_a on periodic axes of the open tensor at offset
 * (i + m_x nx, ...), open axes at their one signed offset; images summed z, y, x (outer
 * to inner).  Components xx yy zz xy xz yz, each px*py*pz values. */
int fo_periodic_newell_kernels(int nx, int ny, int nz, double dx, double dy, double dz, const int32_t periodic[3],
                               const uint32_t images[3], double *out);
/* Demag field by direct O(N^2) real-space Newell sum (FFT-independent check); with
 * periodic axes the offset along each is taken modulo n and summed over the images. */
int fo_demag_direct(fo_problem *pr, const double *m_aos, double *h_demag);

int fo_num_threads(void);
void fo_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
