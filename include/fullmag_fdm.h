/*
 * fullmag_fdm.h -- C ABI of the GB300 finite-difference LLG engine.
 *
 * Drop-in for the FDM backend interface of mzrptu/fullmag
 * (native/include/fullmag_fdm.h, bound by crates/fullmag-fdm-sys/src/lib.rs:281-401).
 * Every type below keeps the field order, field types, enum values and
 * constants of that interface so that a library built from this repository
 * can be linked in its place (FULLMAG_FDM_LIB_DIR, crates/fullmag-fdm-sys/build.rs:2-8).
 * The implementation behind it is new: sm_103a kernels, FP32 field state,
 * FP64 Newell setup and FP64 reductions.
 *
 * Entry points after the 22 of the reference interface are additive
 * (batched sweeps, adjoint gradients, device-resident stepping); they have
 * no counterpart in the reference and callers of the reference interface
 * never see them.
 */

#ifndef FULLMAG_FDM_H
#define FULLMAG_FDM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Return codes (reference fullmag_fdm.h:37-41). */
#define FULLMAG_FDM_OK               0
#define FULLMAG_FDM_ERR_INVALID     -1
#define FULLMAG_FDM_ERR_CUDA        -2
#define FULLMAG_FDM_ERR_INTERNAL    -3
#define FULLMAG_FDM_ERR_INTERRUPTED -4

/* Size of one side of the inter-region exchange table (reference fullmag_fdm.h:44). */
#define FULLMAG_FDM_MAX_EXCHANGE_REGIONS 256

/* Enumerations (reference fullmag_fdm.h:48-80). C enums are int-sized. */
typedef enum {
    FULLMAG_FDM_PRECISION_SINGLE = 1,
    FULLMAG_FDM_PRECISION_DOUBLE = 2
} fullmag_fdm_precision;

typedef enum {
    FULLMAG_FDM_INTEGRATOR_HEUN = 1,
    FULLMAG_FDM_INTEGRATOR_DP45 = 2,
    FULLMAG_FDM_INTEGRATOR_ABM3 = 3,
    FULLMAG_FDM_INTEGRATOR_RK4  = 4,
    FULLMAG_FDM_INTEGRATOR_RK23 = 5
} fullmag_fdm_integrator;

typedef enum {
    FULLMAG_FDM_OBSERVABLE_M       = 1,
    FULLMAG_FDM_OBSERVABLE_H_EX    = 2,
    FULLMAG_FDM_OBSERVABLE_H_DEMAG = 3,
    FULLMAG_FDM_OBSERVABLE_H_EXT   = 4,
    FULLMAG_FDM_OBSERVABLE_H_EFF   = 5
} fullmag_fdm_observable;

typedef enum {
    FULLMAG_FDM_SNAPSHOT_SCALAR_F32 = 1,
    FULLMAG_FDM_SNAPSHOT_SCALAR_F64 = 2
} fullmag_fdm_snapshot_scalar_type;

typedef enum {
    FULLMAG_FDM_BOUNDARY_NONE   = 0,
    FULLMAG_FDM_BOUNDARY_VOLUME = 1,
    FULLMAG_FDM_BOUNDARY_FULL   = 2
} fullmag_fdm_boundary_correction;

/* Host callback polled between device passes; non-zero requests an interrupt. */
typedef int (*fullmag_fdm_interrupt_poll_fn)(void *user_data);

/* Grid: nx*ny*nz cells of dx*dy*dz metres, cell index i = x + nx*(y + ny*z). */
typedef struct {
    uint32_t nx;
    uint32_t ny;
    uint32_t nz;
    double   dx;
    double   dy;
    double   dz;
} fullmag_fdm_grid_desc;

typedef struct {
    double saturation_magnetisation; /* Ms, A/m */
    double exchange_stiffness;       /* A, J/m */
    double damping;                  /* alpha */
    double gyromagnetic_ratio;       /* gamma, m/(A s), Gilbert form */
} fullmag_fdm_material_desc;

/*
 * Executable plan (reference fullmag_fdm.h:100-269). All pointers are borrowed
 * for the duration of fullmag_fdm_backend_create only; the backend copies what
 * it keeps.
 */
typedef struct {
    fullmag_fdm_grid_desc     grid;
    fullmag_fdm_material_desc material;
    fullmag_fdm_precision     precision;
    fullmag_fdm_integrator    integrator;
    int    disable_precession;          /* 1: damping-only right-hand side */
    int    enable_exchange;
    int    enable_demag;
    int    has_external_field;
    double external_field_am[3];        /* H_ext, A/m */

    int    has_uniaxial_anisotropy;
    double uniaxial_anisotropy_constant; /* Ku1, J/m^3 */
    double uniaxial_anisotropy_k2;       /* Ku2, J/m^3 */
    double anisotropy_axis[3];
    const double *ku1_field;             /* optional per-cell Ku1 */
    const double *ku2_field;             /* optional per-cell Ku2 */

    int    has_cubic_anisotropy;
    double cubic_Kc1;
    double cubic_Kc2;
    double cubic_Kc3;
    double cubic_axis1[3];
    double cubic_axis2[3];               /* c3 = c1 x c2 */
    const double *kc1_field;
    const double *kc2_field;
    const double *kc3_field;

    int    has_interfacial_dmi;
    double dmi_D_interfacial;
    int    has_bulk_dmi;
    double dmi_D_bulk;

    int    has_magnetoelastic;
    double mel_b1;
    double mel_b2;
    double mel_strain[6];                /* Voigt e11 e22 e33 2e23 2e13 2e12 */

    double temperature;                  /* K; 0 disables thermal noise */

    double current_density_x;            /* Zhang-Li spin-transfer torque */
    double current_density_y;
    double current_density_z;
    double stt_degree;
    double stt_beta;

    double stt_p_x;                      /* Slonczewski spin-transfer torque */
    double stt_p_y;
    double stt_p_z;
    double stt_lambda;
    double stt_epsilon_prime;

    int    has_sot;                      /* spin-orbit torque */
    double sot_je;
    double sot_xi_dl;
    double sot_xi_fl;
    double sot_sigma[3];
    double sot_thickness;

    int      has_oersted_cylinder;       /* Oersted field of a cylindrical conductor */
    double   oersted_current;
    double   oersted_radius;
    double   oersted_center[3];
    double   oersted_axis[3];
    uint32_t oersted_time_dep_kind;
    double   oersted_time_dep_freq;
    double   oersted_time_dep_phase;
    double   oersted_time_dep_offset;
    double   oersted_time_dep_t_on;
    double   oersted_time_dep_t_off;

    /*
     * Newell tensor spectra on the zero-padded grid, interleaved complex f64
     * [re0, im0, re1, im1, ...] per component. Length = 2*(2nx*2ny*2nz), or for
     * nz == 1 optionally 2*(2nx*2ny) (thin-film 2-D transform). When the length
     * is 0 and demag is enabled, this engine builds the tensor itself on the GPU
     * in FP64.
     */
    const double *demag_kernel_xx_spectrum;
    const double *demag_kernel_yy_spectrum;
    const double *demag_kernel_zz_spectrum;
    const double *demag_kernel_xy_spectrum;
    const double *demag_kernel_xz_spectrum;
    const double *demag_kernel_yz_spectrum;
    uint64_t      demag_kernel_spectrum_len;

    const uint8_t *active_mask;          /* optional, 1 = active */
    uint64_t       active_mask_len;

    const uint32_t *region_mask;         /* optional region ids */
    uint64_t        region_mask_len;

    const double *exchange_lut;          /* optional MAX_EXCHANGE_REGIONS^2 A_ij table */
    uint64_t      exchange_lut_len;

    fullmag_fdm_boundary_correction boundary_correction;
    double boundary_phi_floor;
    double boundary_delta_min;

    const double *volume_fraction;
    uint64_t      volume_fraction_len;

    const double *face_link_xp;
    const double *face_link_xm;
    const double *face_link_yp;
    const double *face_link_ym;
    const double *face_link_zp;
    const double *face_link_zm;

    const double *delta_xp;
    const double *delta_xm;
    const double *delta_yp;
    const double *delta_ym;
    const double *delta_zp;
    const double *delta_zm;

    int            has_demag_boundary_corr;
    const int32_t *demag_corr_target_idx;
    const int32_t *demag_corr_source_idx;
    const double  *demag_corr_tensor;
    uint32_t       demag_corr_target_count;
    uint32_t       demag_corr_stencil_size;

    const double *initial_magnetization_xyz; /* AoS [m0x m0y m0z m1x ...] */
    uint64_t      initial_magnetization_len; /* 3 * cell_count */

    double adaptive_max_error;           /* 0 -> 1e-5 */
    double adaptive_dt_min;              /* 0 -> 1e-18 */
    double adaptive_dt_max;              /* 0 -> 1e-10 */
    double adaptive_headroom;            /* 0 -> 0.8 */
} fullmag_fdm_plan_desc;

/* Per-step diagnostics (reference fullmag_fdm.h:273-289). */
typedef struct {
    uint64_t step;
    double   time_seconds;
    double   dt_seconds;
    double   exchange_energy_joules;
    double   demag_energy_joules;
    double   external_energy_joules;
    double   anisotropy_energy_joules;
    double   cubic_energy_joules;
    double   dmi_energy_joules;
    double   total_energy_joules;
    double   max_effective_field_amplitude;
    double   max_demag_field_amplitude;
    double   max_rhs_amplitude;
    double   suggested_next_dt;
    uint64_t wall_time_ns;
} fullmag_fdm_step_stats;

typedef struct {
    char name[128];
    int  compute_capability_major;
    int  compute_capability_minor;
    int  driver_version;
    int  runtime_version;
} fullmag_fdm_device_info;

typedef struct {
    uint64_t cell_count;
    uint32_t component_count;
    uint32_t scalar_bytes;
    fullmag_fdm_snapshot_scalar_type scalar_type;
} fullmag_fdm_snapshot_desc;

typedef struct fullmag_fdm_backend fullmag_fdm_backend;
typedef struct fullmag_fdm_field_snapshot fullmag_fdm_field_snapshot;
typedef struct fullmag_fdm_preview_snapshot fullmag_fdm_preview_snapshot;

/* ---- The 22 entry points of the reference interface ---- */

/* 1 when a CUDA device is usable (reference fullmag_fdm.h:320, api.cpp:151-166). */
int fullmag_fdm_is_available(void);

/* Copies the plan, allocates device state, uploads m0 and evaluates the fields.
 * Returns a handle even when validation fails; the caller must check
 * fullmag_fdm_backend_last_error (reference fullmag_fdm.h:327, api.cpp:170-519). */
fullmag_fdm_backend *fullmag_fdm_backend_create(const fullmag_fdm_plan_desc *plan);

/* One accepted step; for DP45 dt is the first trial step
 * (reference fullmag_fdm.h:335, api.cpp:523-594). */
int fullmag_fdm_backend_step(fullmag_fdm_backend *handle, double dt_seconds,
                             fullmag_fdm_step_stats *out_stats);

/* reference fullmag_fdm.h:340, api.cpp:596-611 */
int fullmag_fdm_backend_set_interrupt_poll(fullmag_fdm_backend *handle,
                                           fullmag_fdm_interrupt_poll_fn poll_fn,
                                           void *user_data);

/* AoS copies of one observable (reference fullmag_fdm.h:349-365, api.cpp:615-665). */
int fullmag_fdm_backend_copy_field_f64(fullmag_fdm_backend *handle,
                                       fullmag_fdm_observable observable,
                                       double *out_xyz, uint64_t out_len);
int fullmag_fdm_backend_copy_field_f32(fullmag_fdm_backend *handle,
                                       fullmag_fdm_observable observable,
                                       float *out_xyz, uint64_t out_len);

/* Bin-averaged previews (reference fullmag_fdm.h:373-397, api.cpp:667-770). */
int fullmag_fdm_backend_copy_field_preview_f64(fullmag_fdm_backend *handle,
                                               fullmag_fdm_observable observable,
                                               uint32_t preview_nx, uint32_t preview_ny,
                                               uint32_t preview_nz, uint32_t z_origin,
                                               uint32_t z_stride, double *out_xyz,
                                               uint64_t out_len);
int fullmag_fdm_backend_copy_field_preview_f32(fullmag_fdm_backend *handle,
                                               fullmag_fdm_observable observable,
                                               uint32_t preview_nx, uint32_t preview_ny,
                                               uint32_t preview_nz, uint32_t z_origin,
                                               uint32_t z_stride, float *out_xyz,
                                               uint64_t out_len);

/* Asynchronous snapshots (reference fullmag_fdm.h:413-473, api.cpp:772-918). */
fullmag_fdm_field_snapshot *fullmag_fdm_backend_begin_field_snapshot(
    fullmag_fdm_backend *handle, fullmag_fdm_observable observable);
fullmag_fdm_preview_snapshot *fullmag_fdm_backend_begin_preview_snapshot(
    fullmag_fdm_backend *handle, fullmag_fdm_observable observable,
    uint32_t preview_nx, uint32_t preview_ny, uint32_t preview_nz,
    uint32_t z_origin, uint32_t z_stride);
int fullmag_fdm_field_snapshot_wait(fullmag_fdm_field_snapshot *snapshot,
                                    const void **out_data, uint64_t *out_len_bytes,
                                    fullmag_fdm_snapshot_desc *out_desc);
int fullmag_fdm_preview_snapshot_wait(fullmag_fdm_preview_snapshot *snapshot,
                                      const void **out_data, uint64_t *out_len_bytes,
                                      fullmag_fdm_snapshot_desc *out_desc);
void fullmag_fdm_field_snapshot_destroy(fullmag_fdm_field_snapshot *snapshot);
void fullmag_fdm_preview_snapshot_destroy(fullmag_fdm_preview_snapshot *snapshot);

/* State replacement; follow with refresh_observables (reference fullmag_fdm.h:480-497,
 * api.cpp:920-968). */
int fullmag_fdm_backend_upload_magnetization_f64(fullmag_fdm_backend *handle,
                                                 const double *m_xyz, uint64_t len);
int fullmag_fdm_backend_upload_magnetization_f32(fullmag_fdm_backend *handle,
                                                 const float *m_xyz, uint64_t len);

/* reference fullmag_fdm.h:503-507, api.cpp:970-1004 */
int fullmag_fdm_backend_refresh_observables(fullmag_fdm_backend *handle);
int fullmag_fdm_backend_refresh_demag_observable(fullmag_fdm_backend *handle);

/* reference fullmag_fdm.h:516, api.cpp:1006-1022 */
int fullmag_fdm_backend_snapshot_stats(fullmag_fdm_backend *handle,
                                       fullmag_fdm_step_stats *out_stats);

/* reference fullmag_fdm.h:522, api.cpp:1026-1045 */
int fullmag_fdm_backend_get_device_info(fullmag_fdm_backend *handle,
                                        fullmag_fdm_device_info *out_info);

/* NULL when no error; valid until the next call on the handle
 * (reference fullmag_fdm.h:531, api.cpp:1049-1057). */
const char *fullmag_fdm_backend_last_error(fullmag_fdm_backend *handle);

/* NULL-safe (reference fullmag_fdm.h:537, api.cpp:1061-1069). */
void fullmag_fdm_backend_destroy(fullmag_fdm_backend *handle);

/* ---- Additive entry points (no counterpart in the reference interface) ---- */

/*
 * Runs n_steps accepted steps back to back without host round trips between
 * them (fixed-step integrators only; DP45 returns ERR_INVALID). Stats describe
 * the state after the last step. Used by throughput measurements and by
 * callers that only sample output every n steps.
 */
int fullmag_fdm_backend_step_many(fullmag_fdm_backend *handle, double dt_seconds,
                                  uint64_t n_steps, fullmag_fdm_step_stats *out_stats);

/* Device-resident SoA view of m (FP32, three arrays of cell_count floats). */
int fullmag_fdm_backend_device_magnetization(fullmag_fdm_backend *handle,
                                             void **out_mx, void **out_my, void **out_mz);

/* The CUDA stream every kernel of this handle is launched on. */
int fullmag_fdm_backend_stream(fullmag_fdm_backend *handle, void **out_stream);

/* Launch shapes the autotuner chose at create: rows per CTA of the fused row pass,
 * then the kx tile widths of the y-forward, z-convolution, y-inverse and thin-film
 * passes (out9[0..4]), 1 in out9[5] when the z convolution runs on y-frequency pairs
 * in packed FP32x2 arithmetic, and the radix split (0 default, 1 alternative) of the
 * y-forward, z and y-inverse passes (out9[6..8]). */
int fullmag_fdm_backend_tuning(fullmag_fdm_backend *handle, uint32_t *out9);

/* Number of kernels this handle has launched so far (instrumentation). */
int fullmag_fdm_backend_launch_count(fullmag_fdm_backend *handle, uint64_t *out_count);

/* Padded FFT extents the engine chose (px, py, pz; pz == 1 for the thin-film path). */
int fullmag_fdm_backend_fft_shape(fullmag_fdm_backend *handle, uint32_t *out_px,
                                  uint32_t *out_py, uint32_t *out_pz);

/* ---- Per-kernel timing (additive; no counterpart in the reference interface) ----
 * With timing enabled, fixed steps run launch by launch (no CUDA graph) and every
 * kernel launch is bracketed by CUDA events on the handle's stream.  Enabling or
 * disabling resets the totals.  kernel_times fills n_kinds entries in the order
 * row pass, y forward, z convolve, y inverse, fused y+z, thin-film y, statistics
 * finalize, extra-field pass: total milliseconds and launch counts since timing was
 * enabled. */
int fullmag_fdm_backend_set_kernel_timing(fullmag_fdm_backend *handle, int enable);
int fullmag_fdm_backend_kernel_times(fullmag_fdm_backend *handle, double *total_ms, uint64_t *counts, uint32_t n_kinds);

/* ---- Adjoint gradients (additive; no counterpart in the reference interface) ----
 * A per-cell applied field map (A/m, AoS, 3*cell_count) is added to H_eff at active
 * cells; NULL removes it.  The adjoint of a fixed-step RK4 run is split in two calls:
 * adjoint_forward integrates n_steps from the current state keeping a checkpoint every
 * checkpoint_every steps (0: ceil(sqrt(n_steps))); the caller then reads the final
 * state, evaluates its loss and passes d loss / d m_final to adjoint_backward, which
 * returns d loss / d field map (per A/m, AoS) and, optionally, d loss / d m_initial.
 * The backward pass recomputes each segment from its checkpoint, so device memory is
 * O(n/C + 12 C) states.  RK4 only; uniaxial anisotropy supported, cubic not. */
int fullmag_fdm_backend_set_field_map(fullmag_fdm_backend *handle, const double *h_xyz, uint64_t len);
int fullmag_fdm_adjoint_forward(fullmag_fdm_backend *handle, double dt_seconds, uint64_t n_steps,
                                uint32_t checkpoint_every);
int fullmag_fdm_adjoint_backward(fullmag_fdm_backend *handle, const double *lambda_xyz, uint64_t len,
                                 double *grad_field_map_xyz, double *lambda0_xyz);

/* ---- Batched sweeps (additive; no counterpart in the reference interface) ----
 * Many independent problems of uneven grid size advanced together: every problem
 * owns its device state and CUDA stream, each step is a replayed CUDA graph, and one
 * attempt is issued for every unfinished problem before any of them is waited on,
 * so small problems fill the GPU concurrently instead of one after another. */
typedef struct fullmag_fdm_batch fullmag_fdm_batch;

/* One problem per plan; plans follow fullmag_fdm_backend_create.  Check
 * fullmag_fdm_batch_last_error on a non-NULL result. */
fullmag_fdm_batch *fullmag_fdm_batch_create(const fullmag_fdm_plan_desc *plans, uint32_t count);
const char *fullmag_fdm_batch_last_error(fullmag_fdm_batch *batch);
uint32_t fullmag_fdm_batch_size(fullmag_fdm_batch *batch);

/* Advances every problem to simulated time t_end.  DP45 problems start from dt0 and
 * carry their suggested step; fixed-step problems use dt0.  out_steps (optional,
 * size entries) receives the accepted steps per problem, out_wall_ns (optional) the
 * wall time from the call's start at which each problem reached t_end. */
int fullmag_fdm_batch_step_until(fullmag_fdm_batch *batch, double t_end, double dt0, uint64_t *out_steps,
                                 uint64_t *out_wall_ns);
int fullmag_fdm_batch_get_stats(fullmag_fdm_batch *batch, uint32_t index, fullmag_fdm_step_stats *out_stats);
int fullmag_fdm_batch_copy_field_f64(fullmag_fdm_batch *batch, uint32_t index, fullmag_fdm_observable observable,
                                     double *out_xyz, uint64_t out_len);
void fullmag_fdm_batch_destroy(fullmag_fdm_batch *batch);

/* ---- Allocation-free upload (additive; no counterpart in the reference interface) ----
 * Same result as fullmag_fdm_backend_upload_magnetization_f64, but it calls no
 * allocating routine: the host doubles are staged in a fixed 6 MiB device array
 * compiled into the library instead of a buffer the handle allocates on first use.
 * For callers that must not allocate mid-run, e.g. a loop editing the state while
 * other streams work (cudaMalloc/cudaFree can synchronise the whole device) or a
 * process whose device memory is reserved up front.  Limits: grids of at most
 * 262,144 cells (larger ones get FULLMAG_FDM_ERR_INVALID); the first call for a
 * device resolves the array's address with cudaGetSymbolAddress and, under lazy
 * module loading, loads the array itself, which may synchronise the device once, so
 * make one call before any stream capture and before the latency-critical part of a
 * run; the address stays valid until the device's primary context is destroyed
 * (cudaDeviceReset); all handles on a device share the array, so calls that
 * overlap in time (several host threads) race and must be serialised by the caller. */
int fullmag_fdm_backend_upload_magnetization_f64_noalloc(fullmag_fdm_backend *handle, const double *m_xyz,
                                                         uint64_t len);

/* ---- Periodic boundaries (additive) ----
 * The reference carries periodicity only into its Rust CPU engine: per-axis open /
 * periodic policy (crates/fullmag-engine/src/fdm_types.rs:84-117, FdmBoundaryPolicy,
 * fed from FdmPeriodicityIR by crates/fullmag-runner/src/cpu_reference.rs:272-285) and
 * the demag image counts (fdm_problem.rs:19-23, default 10 per axis).  On a periodic
 * axis the exchange, DMI and Zhang-Li stencils wrap around (fdm_types.rs:126-132,
 * fdm_fields.rs:109-160,356-445,1253-1340), the FFT extent is the cell count (no zero padding)
 * and the demag tensor is the truncated image sum N(i) = sum_{|m| <= I} N_open(i + m n)
 * for i in [0, n) (fdm_fft.rs:140-233,614-717), whose spectrum is complex.  This entry
 * point is fullmag_fdm_backend_create with that policy added, for single- and
 * double-precision state.  The backend builds the tensor itself, so the plan must carry
 * no demag spectra; with single-precision state a periodic x extent must be even; the
 * boundary-correction tiers are not combined with periodic axes. */
typedef struct fullmag_fdm_periodicity_desc {
    uint32_t periodic[3];       /* x, y, z: 0 open, 1 periodic */
    uint32_t has_image_counts;  /* 0: 10 images on every periodic axis */
    uint32_t image_counts[3];   /* images on each side along a periodic axis */
} fullmag_fdm_periodicity_desc;

fullmag_fdm_backend *fullmag_fdm_backend_create_periodic(const fullmag_fdm_plan_desc *plan,
                                                         const fullmag_fdm_periodicity_desc *periodicity);

#ifdef __cplusplus
}
#endif

#endif /* FULLMAG_FDM_H */
