// fp64.h -- the double-precision state path of the C ABI (plan precision
// FULLMAG_FDM_PRECISION_DOUBLE).  A handle created with that precision owns one
// Fp64Engine and every C ABI call of the handle is served by it.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/fullmag_fdm.h"

namespace fm {

struct Grid;
struct Fp64Engine;

// Validates the plan, builds the engine on the current device and evaluates the initial
// state.  nullptr and a message in err when the plan is rejected or a CUDA call fails.
// periodic: axes with periodic boundaries (bit 0 x, 1 y, 2 z), images: demag images per
// periodic axis.
Fp64Engine *fp64_create(const fullmag_fdm_plan_desc *plan, std::string &err, int periodic = 0,
                        const uint32_t *images = nullptr);
void fp64_destroy(Fp64Engine *e);
// One accepted step (the adaptive integrators retry internally, as the FP32 path does).
// Returns a FULLMAG_FDM_* code; interrupted steps leave the state untouched.
int fp64_step(Fp64Engine *e, double dt, fullmag_fdm_step_stats *out, fullmag_fdm_interrupt_poll_fn poll, void *user,
              std::string &err);
// Observable as AoS doubles (3 n values).
bool fp64_download(Fp64Engine *e, int observable, double *out, std::string &err);
bool fp64_upload(Fp64Engine *e, const double *m_xyz, std::string &err);
bool fp64_refresh(Fp64Engine *e, std::string &err);
void fp64_stats(const Fp64Engine *e, fullmag_fdm_step_stats *out);
void fp64_grid(const Fp64Engine *e, int &nx, int &ny, int &nz);
int fp64_device(const Fp64Engine *e);
void fp64_fft_shape(const Fp64Engine *e, uint32_t &px, uint32_t &py, uint32_t &pz);

// Forward FP64 FFT along one axis of layout [outer][p][inner] (real input in_re, or
// complex c_in), the first nout outputs into out[outer][nout][inner]; synchronises s.
bool fft64_axis(const double *in_re, const double2 *c_in, double2 *out, long long outer, int p, int nout, int inner,
                cudaStream_t s, std::string &err);

// GPU Newell builder with FP64 output (newell.cu)
bool newell_spectrum_gpu64(const Grid &g, double dx, double dy, double dz, double ms, double *kern, cudaStream_t s,
                           std::string &err);

}  // namespace fm
