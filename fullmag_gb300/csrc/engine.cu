// engine.cu -- host side of the GB300 FDM engine and the C ABI of include/fullmag_fdm.h.
//
// One handle = one problem on one GPU, one CUDA stream, one device arena.
// Semantics follow the reference C ABI (native/backends/fdm/src/api.cpp:151-1070,
// context.cu:934-1060, llg_fp32.cu:267-389, llg_rk4_fp32.cu, llg_dp45_fp32.cu:188-342):
// create returns a handle even on validation failure with last_error set, step
// advances one accepted step and reports post-step statistics, observables are
// AoS on the host.  Internally the step is a chain of fused passes (see
// kernels.cu); the field evaluation at the new state that every step reports
// statistics for doubles as the first stage of the next step.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/fullmag_fdm.h"
#include "engine.h"
#include "fp64.h"
#include "noalloc.h"

namespace fm {

static constexpr double kMu0 = 4.0 * M_PI * 1e-7;
// device statistics slots: the kNumStats row-pass statistics, the step size of graph
// replays, and the extra field pass's five sums (ExtraSums: Zeeman m.(H_ext + H_map), DMI,
// uniaxial and cubic energy densities, region exchange pair sum)
static constexpr int kStatSlots = kNumStats + 6;

bool newell_spectrum_gpu(const Grid &g, double dx, double dy, double dz, double ms, float *kern, cudaStream_t s,
                         std::string &err);

// Device conversions between the ABI's AoS host layout and SoA device state.
__global__ void aos_to_soa_kernel(const double *__restrict__ in_d, const float *__restrict__ in_f, float *__restrict__ out,
                                  const uint8_t *__restrict__ mask, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const bool act = mask == nullptr || mask[i] != 0;
        for (int c = 0; c < 3; ++c) {
            const float v = in_d ? (float)in_d[3 * i + c] : in_f[3 * i + c];
            out[c * n + i] = act ? v : 0.f;
        }
    }
}
// Box-average preview of a SoA float field: preview cell o = px + pnx (py + pny pz) averages
// x in [px nx/pnx, (px+1) nx/pnx), the same for y, and z in [z0 + pz zst, z0 + (pz+1) zst)
// (each range at least one cell, clamped to the grid).  FP64 sums in z, y, x order: the
// operations of a host loop over the field converted to double, so the output does not
// depend on where it is computed.  Output AoS.
template <typename T>
__global__ void preview_kernel(const float *__restrict__ f, long long n, unsigned fx, unsigned fy, unsigned fz,
                               unsigned pnx, unsigned pny, unsigned pnz, unsigned z0, unsigned zst, T *__restrict__ out) {
    const long long np = (long long)pnx * pny * pnz;
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < np; o += (long long)gridDim.x * blockDim.x) {
        const unsigned px = (unsigned)(o % pnx);
        const unsigned py = (unsigned)((o / pnx) % pny);
        const unsigned pz = (unsigned)(o / ((long long)pnx * pny));
        unsigned zs0 = z0 + pz * zst;
        if (zs0 >= fz) zs0 = fz - 1;
        unsigned ze = z0 + (pz + 1) * zst;
        if (ze <= zs0) ze = zs0 + 1;
        if (ze > fz) ze = fz;
        unsigned ys = (unsigned)(((unsigned long long)py * fy) / pny), ye = (unsigned)(((unsigned long long)(py + 1) * fy) / pny);
        if (ye <= ys) ye = ys + 1;
        if (ye > fy) ye = fy;
        unsigned xs = (unsigned)(((unsigned long long)px * fx) / pnx), xe = (unsigned)(((unsigned long long)(px + 1) * fx) / pnx);
        if (xe <= xs) xe = xs + 1;
        if (xe > fx) xe = fx;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, cnt = 0.0;
        for (unsigned z = zs0; z < ze; ++z)
            for (unsigned y = ys; y < ye; ++y)
                for (unsigned x = xs; x < xe; ++x) {
                    const long long i = ((long long)z * fy + y) * fx + x;
                    a0 += (double)f[i];
                    a1 += (double)f[n + i];
                    a2 += (double)f[2 * n + i];
                    cnt += 1.0;
                }
        out[3 * o] = (T)(a0 / cnt);
        out[3 * o + 1] = (T)(a1 / cnt);
        out[3 * o + 2] = (T)(a2 / cnt);
    }
}

// Control block of a batched DP45 attempt (host-pinned, copied to the device by the
// first node of the attempt graph).
struct BatchCtl {
    double dt;        // step size of this attempt
    int accept_prev;  // 1: the previous attempt was accepted and still has to be committed
    int pad;
};

// Commit of an accepted batched attempt, run at the start of the next one:
// S0 <- S1 (proposal becomes the state) and K0 <- K6 (first-same-as-last).
__global__ void batch_commit_kernel(const BatchCtl *__restrict__ ctl, float *__restrict__ s0, const float *__restrict__ s1,
                                    float *__restrict__ k0, const float *__restrict__ k6, long long n3) {
    if (ctl->accept_prev == 0) return;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3; i += (long long)gridDim.x * blockDim.x) {
        s0[i] = s1[i];
        k0[i] = k6[i];
    }
}

struct CommitDesc {
    float *s0;
    const float *s1;
    float *k0;
    const float *k6;
    long long n3;
};

// Batched commit: blockIdx.y selects the problem.
__global__ void batch_commit_all_kernel(const CommitDesc *__restrict__ cd, const BatchCtl *__restrict__ ctl) {
    if (ctl[blockIdx.y].accept_prev == 0) return;
    const CommitDesc d = cd[blockIdx.y];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.n3; i += (long long)gridDim.x * blockDim.x) {
        d.s0[i] = d.s1[i];
        d.k0[i] = d.k6[i];
    }
}

// Step control of one batched problem, kept on the device: after every round the control
// kernel applies the C ABI's accept/reject rule (native/backends/fdm/src/llg_dp45_fp32.cu:
// 286-341, as finish_dp45_attempt does on the host for single problems), advances the
// problem's time and picks the next attempt's size, so a graph can chain many rounds
// without the host in between.
struct BatchState {
    double time, t_end, next_dt;
    double max_error, dt_min, dt_max, headroom, ctrl_exp;
    double acc_stats[kNumStats];  // statistics of the last accepted step
    double dt_used, suggested;
    unsigned long long steps;     // steps accepted since the host last read the state
    int done, pad;
};

__global__ void batch_control_kernel(BatchCtl *__restrict__ ctl, BatchState *__restrict__ st,
                                     const double *__restrict__ stats, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    BatchState &s = st[k];
    BatchCtl &c = ctl[k];
    if (s.done) {  // any commit it still had ran at the start of this round
        c.accept_prev = 0;
        c.dt = 0.0;
        return;
    }
    const double dt = c.dt;
    const double err = sqrt(stats[(size_t)k * kNumStats + 8]);
    double nd;
    if (err <= s.max_error || dt <= s.dt_min) {
        nd = err > 0.0 ? fmin(fmax(s.headroom * dt * pow(s.max_error / err, s.ctrl_exp), s.dt_min), s.dt_max) : s.dt_max;
        s.time += dt;
        s.steps += 1;
        for (int q = 0; q < kNumStats; ++q) s.acc_stats[q] = stats[(size_t)k * kNumStats + q];
        s.dt_used = dt;
        s.suggested = nd;
        c.accept_prev = 1;
    } else {
        nd = fmin(fmax(s.headroom * dt * pow(s.max_error / err, s.ctrl_exp), s.dt_min), s.dt_max);
        c.accept_prev = 0;
    }
    s.next_dt = nd;
    if (s.time >= s.t_end * (1.0 - 1e-12)) {
        s.done = 1;
        c.dt = 0.0;
    } else {
        c.dt = fmin(nd, s.t_end - s.time);
    }
}

__global__ void soa_to_aos_kernel(const float *__restrict__ in, double *__restrict__ out_d, float *__restrict__ out_f,
                                  long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        for (int c = 0; c < 3; ++c) {
            const float v = in[c * n + i];
            if (out_d) out_d[3 * i + c] = (double)v;
            else out_f[3 * i + c] = v;
        }
    }
}

// Pinned host buffers for snapshot payloads.  Page-locking tens of MB takes
// milliseconds, so buffers are reused: a snapshot takes one at begin and returns it
// at destroy.  Shared between a backend and its snapshots, since a snapshot may
// outlive the backend.
struct PinnedPool {
    std::mutex mu;
    std::vector<std::pair<void *, size_t>> free_bufs;
    void *take(size_t bytes, size_t &cap) {
        std::lock_guard<std::mutex> lk(mu);
        size_t best = free_bufs.size();
        for (size_t k = 0; k < free_bufs.size(); ++k)
            if (free_bufs[k].second >= bytes && (best == free_bufs.size() || free_bufs[k].second < free_bufs[best].second))
                best = k;
        if (best < free_bufs.size()) {
            void *p = free_bufs[best].first;
            cap = free_bufs[best].second;
            free_bufs.erase(free_bufs.begin() + (long)best);
            return p;
        }
        void *p = nullptr;
        if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
        cap = bytes;
        return p;
    }
    void give(void *p, size_t cap) {
        std::lock_guard<std::mutex> lk(mu);
        free_bufs.emplace_back(p, cap);
    }
    ~PinnedPool() {
        for (auto &b : free_bufs) cudaFreeHost(b.first);
    }
};

// Snapshot payload: host-synthesised bytes, or a pinned buffer that a device-to-host
// copy on the backend's snapshot stream fills; `done` marks the end of that copy.
// Box average of a full AoS field (3 values per cell) onto a pnx x pny x pnz preview grid:
// x and y bins split the grid evenly, z bins start at z0 and are zs planes thick; FP64
// sums in z, y, x order.
template <typename T>
static void host_preview(const double *full, uint32_t fx, uint32_t fy, uint32_t fz, uint32_t pnx, uint32_t pny,
                         uint32_t pnz, uint32_t z0, uint32_t zs, T *out) {
    for (uint32_t pz = 0; pz < pnz; ++pz) {
        uint32_t zs0 = z0 + pz * zs;
        if (zs0 >= fz) zs0 = fz - 1;
        uint32_t ze = z0 + (pz + 1) * zs;
        if (ze <= zs0) ze = zs0 + 1;
        if (ze > fz) ze = fz;
        for (uint32_t py = 0; py < pny; ++py) {
            uint32_t ys = (uint32_t)(((uint64_t)py * fy) / pny), ye = (uint32_t)(((uint64_t)(py + 1) * fy) / pny);
            if (ye <= ys) ye = ys + 1;
            if (ye > fy) ye = fy;
            for (uint32_t px = 0; px < pnx; ++px) {
                uint32_t xs = (uint32_t)(((uint64_t)px * fx) / pnx), xe = (uint32_t)(((uint64_t)(px + 1) * fx) / pnx);
                if (xe <= xs) xe = xs + 1;
                if (xe > fx) xe = fx;
                double a[3] = {0, 0, 0}, cnt = 0;
                for (uint32_t z = zs0; z < ze; ++z)
                    for (uint32_t y = ys; y < ye; ++y)
                        for (uint32_t x = xs; x < xe; ++x) {
                            const size_t i = ((size_t)z * fy + y) * fx + x;
                            for (int c = 0; c < 3; ++c) a[c] += full[3 * i + c];
                            cnt += 1.0;
                        }
                const size_t o = ((size_t)pz * pny + py) * pnx + px;
                for (int c = 0; c < 3; ++c) out[3 * o + c] = (T)(a[c] / cnt);
            }
        }
    }
}

struct SnapshotPayload {
    std::vector<unsigned char> bytes;
    std::shared_ptr<PinnedPool> pool;
    void *pinned = nullptr;
    size_t cap = 0, len = 0;
    cudaEvent_t done = nullptr;
    fullmag_fdm_snapshot_desc desc{};
    bool ok = false;
    ~SnapshotPayload() {
        if (done) {
            cudaEventSynchronize(done);  // the copy must finish before the buffer is reused
            cudaEventDestroy(done);
        }
        if (pinned && pool) pool->give(pinned, cap);
    }
};

struct Engine {
    // ---- configuration ----
    Grid g{};
    Material mat{};
    int integrator = FULLMAG_FDM_INTEGRATOR_HEUN;
    bool demag = false;
    double dx = 0, dy = 0, dz = 0, ms = 0, a_ex = 0, alpha = 0, gamma = 0;
    bool has_ext = false, has_uni = false, has_cub = false, exchange = false;
    double hext[3] = {0, 0, 0};
    double max_error = 1e-5, dt_min = 1e-18, dt_max = 1e-10, headroom = 0.8;
    std::vector<uint8_t> mask_host;
    bool has_mask = false;

    // ---- device state ----
    int device = 0;
    cudaStream_t stream = nullptr;
    char *arena = nullptr;
    size_t arena_bytes = 0;
    float *S[2] = {nullptr, nullptr};
    float *A[2] = {nullptr, nullptr};
    float *K[7] = {};
    int nk = 0;
    float *h_ex = nullptr, *h_d = nullptr, *h_eff = nullptr;
    float *hmap = nullptr;  // per-cell applied field map (SoA, A/m), allocated on first use
    // DMI / magnetoelastic terms: their pass writes hextra (with the field map added), which
    // the right-hand-side row passes take as their field map; xpart holds its per-CTA sums
    bool has_extra = false;
    bool has_torque = false;   // spin torques among the extra terms
    bool torques_off = false;  // set while an observable pass runs
    ExtraField xf{};
    float *hextra = nullptr;
    ExtraSums *xpart = nullptr;
    float *kmaps[5] = {};  // per-cell Ku1 Ku2 Kc1 Kc2 Kc3 (device, FP32) or NULL
    // exchange with region ids (api.cpp:405-420): ids and the stiffness table (FP32) on the
    // device; the whole exchange term then runs in the extra pass
    uint8_t *regions = nullptr;  // ids below 256, one byte per cell
    float *lut = nullptr;
    // Brown thermal field (crates/fullmag-engine/src/fdm_fields.rs:818-896): sigma^2 =
    // th_pref / dt with the step's dt (1e-13 s for adaptive integrators); a step counter that
    // advances once per completed step; th_dev[0] for the evaluations inside a step,
    // th_dev[1] for its final evaluation (the next step's k1)
    bool has_thermal = false;
    double th_pref = 0.0, th_dt = 1e-13;
    unsigned long long th_seed = 42, th_step = 0;
    ThermalSlot *th_dev = nullptr;
    // Oersted field (context.cu:844-905, demag_fp32.cu:585-616): the field for 1 A and the
    // device scales I(t): [0] for the stages of a step, [1] for its final evaluation
    bool has_oersted = false;
    float *h_oe = nullptr, *oe_dev = nullptr;
    int oe_kind = 0;
    double oe_current = 0.0, oe_freq = 0.0, oe_phase = 0.0, oe_offset = 0.0, oe_t_on = 0.0, oe_t_off = 0.0;

    double oersted_current_at(double t) const {
        double I = oe_current;
        if (oe_kind == 1) I *= sin(2.0 * M_PI * oe_freq * t + oe_phase) + oe_offset;
        else if (oe_kind == 2) I *= (t >= oe_t_on && t < oe_t_off) ? 1.0 : 0.0;
        return I;
    }
    // I(t_stage) for the stages, I(t_final) for the final evaluation, enqueued on the stream
    // ahead of the launches (or graph) that read them
    // the thermal keys and amplitude of a step's evaluations (counter c_stage) and of its
    // final evaluation (c_final), written in stream order before the step's launches
    bool set_thermal(unsigned long long c_stage, unsigned long long c_final) {
        if (!has_thermal) return true;
        const float sg = (float)sqrt(th_pref / th_dt);
        const ThermalSlot v[2] = {{th_seed + c_stage * 0x9E3779B97F4A7C15ull, sg, 0.f},
                                  {th_seed + c_final * 0x9E3779B97F4A7C15ull, sg, 0.f}};
        return !cuda_fail("thermal keys", cudaMemcpyAsync(th_dev, v, sizeof(v), cudaMemcpyHostToDevice, stream));
    }
    // the amplitude's dt for a step of size dt; a change makes the stored k1 stale
    void thermal_dt_for(double dt) {
        if (!has_thermal) return;
        const double d = adaptive() ? 1e-13 : dt;
        if (d != th_dt) {
            th_dt = d;
            k1_valid = false;
            stats_valid = false;
            fields_valid = false;
        }
    }
    bool set_oersted(double t_stage, double t_final) {
        if (!has_oersted) return true;
        const float v[2] = {(float)oersted_current_at(t_stage), (float)oersted_current_at(t_final)};
        return !cuda_fail("Oersted current", cudaMemcpyAsync(oe_dev, v, sizeof(v), cudaMemcpyHostToDevice, stream));
    }
    float2 *X = nullptr, *Y = nullptr;
    float *kern = nullptr;
    uint8_t *mask = nullptr;
    float2 *partials = nullptr;  // [kNumStats][row blocks] float-float partial sums
    double *dstats = nullptr;
    double *hstats = nullptr;  // pinned
    float2 *twid = nullptr;
    float2 *xpost = nullptr;
    FftPlan plan_x{}, plan_y{}, plan_z{};
    void *staging = nullptr;  // lazily allocated 3n doubles for host transfers
    int row_rows = 1;
    int max_row_blocks = 1;

    // ---- dynamic state ----
    int cur = 0;
    bool k1_valid = false, fields_valid = false, stats_valid = false;
    uint64_t step_count = 0;
    double time = 0.0;
    double stat_raw[kStatSlots] = {};
    fullmag_fdm_step_stats cur_stats{};

    fullmag_fdm_interrupt_poll_fn poll = nullptr;
    void *poll_user = nullptr;
    bool interrupted = false;
    uint64_t launches = 0;  // kernels this handle has launched
    fullmag_fdm_device_info info{};
    bool info_valid = false;
    std::string last_error;

    ~Engine() { release(); }

    // a handle created with FULLMAG_FDM_PRECISION_DOUBLE is served by the FP64 path (fp64.cu)
    Fp64Engine *f64 = nullptr;

    void release() {
        if (f64) {
            fp64_destroy(f64);
            f64 = nullptr;
        }
        if (stream) cudaStreamSynchronize(stream);
        if (snap_stream) {
            cudaStreamSynchronize(snap_stream);
            cudaStreamDestroy(snap_stream);
            snap_stream = nullptr;
        }
        drop_graphs();
        kt_free();
        adj_free();
        if (hmap) cudaFree(hmap);
        hmap = nullptr;
        if (hextra) cudaFree(hextra);
        if (xpart) cudaFree(xpart);
        hextra = nullptr;
        xpart = nullptr;
        for (float *&km : kmaps) {
            if (km) cudaFree(km);
            km = nullptr;
        }
        if (regions) cudaFree(regions);
        if (lut) cudaFree(lut);
        regions = nullptr;
        lut = nullptr;
        if (th_dev) cudaFree(th_dev);
        th_dev = nullptr;
        if (h_oe) cudaFree(h_oe);
        if (oe_dev) cudaFree(oe_dev);
        h_oe = nullptr;
        oe_dev = nullptr;
        if (arena) cudaFree(arena);
        arena = nullptr;
        if (staging) cudaFree(staging);
        staging = nullptr;
        if (hstats) cudaFreeHost(hstats);
        hstats = nullptr;
        if (dt_host) cudaFreeHost(dt_host);
        dt_host = nullptr;
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }

    bool cuda_fail(const char *what, cudaError_t e) {
        if (e == cudaSuccess) return false;
        last_error = std::string(what) + ": " + cudaGetErrorString(e);
        return true;
    }

    bool poll_hit() {
        if (poll && poll(poll_user) != 0) {
            interrupted = true;
            return true;
        }
        return false;
    }

    // ---------------- setup ----------------
    static void factorize(int n, std::vector<int> &r) {
        int m = n;
        while (m % 8 == 0) { r.push_back(8); m /= 8; }
        while (m % 4 == 0) { r.push_back(4); m /= 4; }
        while (m % 2 == 0) { r.push_back(2); m /= 2; }
        for (int q = 3; q * q <= m; q += 2)
            while (m % q == 0) { r.push_back(q); m /= q; }
        if (m > 1) r.push_back(m);
    }

    bool make_plan(FftPlan &p, int n, std::vector<float2> &host_tw, std::vector<size_t> &offs) {
        std::vector<int> r;
        factorize(n, r);
        if ((int)r.size() > kMaxStages) {
            last_error = "FFT length " + std::to_string(n) + " has too many factors";
            return false;
        }
        for (int x : r)
            if (x > 8 && x > kMaxGenericRadix) {
                last_error = "FFT length " + std::to_string(n) + " has a prime factor above 64 (" + std::to_string(x) + ")";
                return false;
            }
        p.n = n;
        p.nstages = (int)r.size();
        p.log2n = -1;
        if (n >= 2 && (n & (n - 1)) == 0) {
            int l = 0;
            while ((1 << l) < n) ++l;
            p.log2n = l;
        }
        for (int i = 0; i < p.nstages; ++i) p.radix[i] = r[i];
        offs.push_back(host_tw.size());
        for (int e = 0; e < n; ++e) {
            const double ang = 2.0 * M_PI * (double)e / (double)n;
            host_tw.push_back(make_float2((float)cos(ang), (float)-sin(ang)));
        }
        return true;
    }

    bool use_gpu_newell = false;
    // small fixed-step problems: each kernel lets the next one launch as soon as its own
    // last CTAs have started (programmatic dependent launch, engine.h)
    bool early_launch = false;
    // periodic boundary policy requested at create (bit 0 x, 1 y, 2 z) and the demag
    // image counts per axis (fdm_problem.rs:19-23,89-90)
    int per_req = 0;
    uint32_t images[3] = {10, 10, 10};

    // largest prime factor <= 7 for the fast radix kernels; up to 64 still works
    static bool smooth_enough(int n) {
        int m = n;
        for (int q : {2, 3, 5, 7}) while (m % q == 0) m /= q;
        return m == 1;
    }
    static int next_smooth(int n, bool even) {
        for (int m = std::max(n, 1);; ++m) {
            if (even && (m & 1)) continue;
            if (smooth_enough(m)) return m;
        }
    }
    // Padded extent >= n when the engine builds the tensor: the next power of two.
    // It is at most 2x the 2,3,5,7-smooth extent, and the compile-time radix-16/8/4
    // path it selects runs several times faster per point than the generic radices.
    static int pad_extent(int n, bool even) {
        int p2 = 1;
        while (p2 < std::max(n, even ? 2 : 1)) p2 <<= 1;
        return p2;
    }

    bool setup(const fullmag_fdm_plan_desc *plan);
    bool upload_spectra(const fullmag_fdm_plan_desc *plan, bool thin_from_len);

    // ---------------- passes ----------------
    RowPass row_base() const {
        RowPass p{};
        p.g = g;
        p.mat = mat;
        p.mask = mask;
        p.xplan = plan_x;
        p.xpost = xpost;
        p.rows = row_rows;
        p.hmap = hmap;
        p.early = early_launch ? 1 : 0;
        return p;
    }

    // Recording mode (batched execution): passes are appended as descriptors instead
    // of being launched; column passes record their batched kind (col_batched_kind).
    std::vector<RowPass> *rec_rows = nullptr;
    std::vector<int> *rec_cols = nullptr;

    // ---- per-kernel timing (off by default) ----
    // With timing on, fixed steps run eagerly (no graph) and every launch is bracketed
    // by a pair of events on the engine's stream; the elapsed times are summed per
    // kernel kind whenever the stream has been synchronised.
    enum { KT_ROW, KT_YF, KT_Z, KT_YI, KT_YZ, KT_Y2D, KT_FIN, KT_EXTRA, KT_N };
    bool ktime = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> kt_ev;
    std::vector<int> kt_kind;
    size_t kt_used = 0;
    double kt_ms[KT_N] = {};
    uint64_t kt_cnt[KT_N] = {};

    bool kt_armed = false;
    void kt_begin(int kind) {
        kt_armed = false;
        if (!ktime || rec_rows) return;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
        if (kt_used == kt_ev.size()) {
            cudaEvent_t a = nullptr, b = nullptr;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            kt_ev.push_back({a, b});
            kt_kind.push_back(0);
        }
        kt_kind[kt_used] = kind;
        kt_armed = cudaEventRecord(kt_ev[kt_used].first, stream) == cudaSuccess;
    }
    void kt_end() {
        if (!kt_armed) return;
        kt_armed = false;
        if (cudaEventRecord(kt_ev[kt_used].second, stream) == cudaSuccess) ++kt_used;
    }
    // call only after the stream has been synchronised
    void kt_collect() {
        bool failed = false;
        for (size_t i = 0; i < kt_used; ++i) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, kt_ev[i].first, kt_ev[i].second) == cudaSuccess) {
                kt_ms[kt_kind[i]] += ms;
                kt_cnt[kt_kind[i]] += 1;
            } else {
                failed = true;
            }
        }
        if (failed) cudaGetLastError();  // a pair that did not complete: skipped, not an engine error
        kt_used = 0;
    }
    void kt_free() {
        for (auto &e : kt_ev) {
            cudaEventDestroy(e.first);
            cudaEventDestroy(e.second);
        }
        kt_ev.clear();
        kt_kind.clear();
        kt_used = 0;
    }

    bool run_row_adj(RowPass &p) {
        if (!demag) {
            p.x_in = nullptr;
            p.x_out = nullptr;
        }
        launches += 1;
        kt_begin(KT_ROW);
        const cudaError_t rc = launch_row_pass_adj(p, stream);
        kt_end();
        return !cuda_fail("adjoint row pass", rc);
    }

    // The extra field pass for a right-hand side at p.m_in, enqueued before its row pass
    // (with the energy sums when that pass collects statistics); p then takes its output
    // as the field map.
    bool run_extra(RowPass &p) {
        if (!has_extra || !p.m_in) return true;
        if (rec_rows) {
            last_error = "DMI and magnetoelastic problems run outside batched rounds";
            return false;
        }
        ExtraField q = xf;
        q.g = g;
        q.mask = mask;
        q.m = p.m_in;
        q.hmap = hmap;
        q.out = hextra;
        q.partials = p.partials ? xpart : nullptr;
        q.torques = torques_off ? 0 : 1;
        q.h_oe = h_oe;
        q.oe_scale = oe_dev ? oe_dev + (p.partials ? 1 : 0) : nullptr;
        q.th = th_dev ? th_dev + (p.partials ? 1 : 0) : nullptr;
        if (xf.region) {  // the row pass's exchange is off: this pass writes H_EX
            q.h_ex_out = p.h_ex_out;
            p.h_ex_out = nullptr;
        }
        launches += 1;
        kt_begin(KT_EXTRA);
        const cudaError_t rc = launch_extra_field(q, stream);
        kt_end();
        if (cuda_fail("extra field", rc)) return false;
        p.hmap = hextra;
        return true;
    }

    bool run_row(RowPass &p) {
        if (p.x_out) prep_ready = false;  // X no longer holds a prepared first stage
        if (!run_extra(p)) return false;
        if (!demag) {
            p.x_in = nullptr;
            p.x_out = nullptr;
        }
        if (rec_rows) {
            rec_rows->push_back(p);
            return true;
        }
        launches += 1;
        kt_begin(KT_ROW);
        const cudaError_t rc = launch_row_pass(p, stream);
        kt_end();
        return !cuda_fail("row pass", rc);
    }

    // kx tile widths of the column passes (autotuned at create, see autotune());
    // tx_z doubles as the tile of the fused y+z pass when the (y, z) plane of a kx
    // column fits in shared memory (use_yz)
    int tx_yf = 1, tx_z = 1, tx_yi = 1, tx_2d = 1;
    int z_pair = 0;  // 1: the z pass runs the packed ky-pair kernel (tile 8)
    int split_yf = 0, split_z = 0, split_yi = 0;  // radix split of each two-level column pass
    bool use_yz = false;
    int row_blocks = 1;  // CTAs of the row pass at the current rows-per-CTA

    ColPass col_pass(const FftPlan &plan, int tx, const float2 *in, float2 *out) const {
        ColPass c{};
        c.g = g;
        c.kern = kern;
        c.plan = plan;
        c.tx = tx;
        c.fd_tx = FastDiv((uint32_t)tx);
        c.fd_last = FastDiv((uint32_t)(g.nkx % tx ? g.nkx % tx : tx));
        c.in = in;
        c.out = out;
        c.plan2 = plan_z;
        c.early = early_launch ? 1 : 0;
        return c;
    }

    bool run_columns() {
        if (!demag) return true;
        if (rec_cols) {
            if (!g.thin && !use_yz) {
                last_error = "grid too large for the batched passes";
                return false;
            }
            rec_cols->push_back(col_batched_kind(g));
            return true;
        }
        cudaError_t rc;
        if (g.thin) {
            launches += 1;
            kt_begin(KT_Y2D);
            rc = launch_y_convolve_2d(col_pass(plan_y, tx_2d, X, X), stream);
            kt_end();
            return !cuda_fail("y convolve", rc);
        }
        if (use_yz) {
            launches += 1;
            kt_begin(KT_YZ);
            rc = launch_yz_convolve(col_pass(plan_y, tx_z, X, X), stream);
            kt_end();
            return !cuda_fail("yz convolve", rc);
        }
        kt_begin(KT_YF);
        ColPass yf = col_pass(plan_y, tx_yf, X, Y);
        yf.split = split_yf;
        rc = launch_y_forward(yf, stream);
        kt_end();
        if (cuda_fail("y forward", rc)) return false;
        kt_begin(KT_Z);
        ColPass zp = col_pass(plan_z, tx_z, Y, Y);
        zp.pipe = z_pair;
        zp.split = split_z;
        rc = launch_z_convolve(zp, stream);
        kt_end();
        if (cuda_fail("z convolve", rc)) return false;
        launches += 3;
        kt_begin(KT_YI);
        ColPass yi = col_pass(plan_y, tx_yi, Y, X);
        yi.split = split_yi;
        rc = launch_y_inverse(yi, stream);
        kt_end();
        return !cuda_fail("y inverse", rc);
    }

    // ---- autotuner: tile widths of the column passes and rows per CTA of the row
    // pass, timed on the live buffers at create time and cached per grid shape ----
    float time_ms(const std::function<bool()> &fn) {
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        bool ok = fn();  // warm-up (also sets shared-memory attributes)
        cudaEventRecord(e0, stream);
        for (int r = 0; r < 3 && ok; ++r) ok = fn();
        cudaEventRecord(e1, stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (!ok) {
            cudaGetLastError();
            last_error.clear();
            return 1e30f;
        }
        return ms;
    }

    bool autotune();

    // forward x-transform of a state (no combination)
    bool pass_forward(const float *m) {
        if (!demag) return true;
        RowPass p = row_base();
        p.m_fwd = m;
        p.x_out = X;
        return run_row(p) && run_columns();
    }

    bool enqueue_stats() {
        if (rec_rows) return true;  // the batched round finalizes all problems at once
        launches += 1;
        kt_begin(KT_FIN);
        const cudaError_t rc = launch_finalize_stats(partials, row_blocks, dstats, stream, early_launch ? 1 : 0);
        kt_end();
        if (cuda_fail("finalize", rc)) return false;
        if (has_extra) {  // the extra pass before this evaluation left its per-CTA sums
            launches += 1;
            if (cuda_fail("extra finalize",
                          launch_extra_finalize(xpart, extra_field_blocks(g), dstats + kNumStats + 1, stream, early_launch ? 1 : 0)))
                return false;
        }
        return !cuda_fail("stats copy",
                          cudaMemcpyAsync(hstats, dstats, sizeof(double) * kStatSlots, cudaMemcpyDeviceToHost, stream));
    }

    bool read_stats() {
        if (!enqueue_stats() || cuda_fail("stream sync", cudaStreamSynchronize(stream))) return false;
        kt_collect();
        return true;
    }

    void fill_stats(const double *d, fullmag_fdm_step_stats &st) const {
        const double V = dx * dy * dz;
        // with region ids the exchange pair sum is the extra pass's (slot kNumStats + 5, A inside)
        st.exchange_energy_joules = exchange ? (xf.region ? V * d[kNumStats + 5] : a_ex * V * d[0]) : 0.0;
        st.demag_energy_joules = demag ? -0.5 * kMu0 * ms * V * d[1] : 0.0;
        // with an extra pass, the row pass's field-map sum includes its terms; the Zeeman
        // sum m.(H_ext + H_map) then comes from the extra pass (slot kNumStats + 1)
        const double zeeman = has_extra ? d[kNumStats + 1] : d[2];
        st.external_energy_joules = (has_ext || hmap) ? -kMu0 * ms * V * zeeman : 0.0;
        // with per-cell anisotropy maps both terms are the extra pass's (slots kNumStats + 3, + 4)
        st.anisotropy_energy_joules = has_uni ? -V * (xf.aniso ? d[kNumStats + 3] : d[3]) : 0.0;
        st.cubic_energy_joules = has_cub ? V * (xf.aniso ? d[kNumStats + 4] : d[4]) : 0.0;
        st.dmi_energy_joules = has_extra ? V * d[kNumStats + 2] : 0.0;
        st.total_energy_joules = st.exchange_energy_joules + st.demag_energy_joules + st.external_energy_joules +
                                 st.anisotropy_energy_joules + st.cubic_energy_joules + st.dmi_energy_joules;
        st.max_effective_field_amplitude = sqrt(d[5]);
        st.max_demag_field_amplitude = demag ? sqrt(d[6]) : 0.0;
        st.max_rhs_amplitude = sqrt(d[7]);
    }

    // RHS at the committed state -> K[0], statistics, optionally observables.
    bool eval_state(bool write_fields) {
        if (!set_oersted(time, time) || !set_thermal(th_step, th_step)) return false;
        if (!pass_forward(S[cur])) return false;
        bool fields_written = false;
        if (write_fields && has_torque) {
            // the observables leave the spin torques out (they are not fields in the
            // reference): one pass writes them without the torque terms, the next computes
            // k1 and the statistics with them
            RowPass q = row_base();
            q.x_in = X;
            q.m_in = S[cur];
            q.h_ex_out = h_ex;
            q.h_d_out = h_d;
            q.h_eff_out = h_eff;
            torques_off = true;
            const bool ok = run_row(q);
            torques_off = false;
            if (!ok) return false;
            write_fields = false;
            fields_written = true;
        }
        RowPass p = row_base();
        p.x_in = X;
        p.m_in = S[cur];
        // a valid k1 stays: after DP45 / RK23 it is the first-same-as-last derivative, taken
        // inside the step (with that step's Oersted current and thermal counter)
        p.k_out = k1_valid ? nullptr : K[0];
        p.partials = partials;
        if (write_fields) {
            p.h_ex_out = h_ex;
            p.h_d_out = h_d;
            p.h_eff_out = h_eff;
        }
        if (!run_row(p)) return false;
        if (!read_stats()) return false;
        memcpy(stat_raw, hstats, sizeof(stat_raw));
        k1_valid = true;
        stats_valid = true;
        if (write_fields || fields_written) fields_valid = true;
        fill_stats(stat_raw, cur_stats);
        cur_stats.step = step_count;
        cur_stats.time_seconds = time;
        return true;
    }

    // One pass: RHS at m_in (stored to k_out when non-null), combination into m_next.
    bool stage(const float *m_in, float *k_out, int ncomb, const int *kidx, const double *coef, double dt, float *m_next) {
        RowPass p = row_base();
        p.x_in = m_in ? X : nullptr;
        p.m_in = m_in;
        p.k_out = k_out;
        p.m0 = S[cur];
        p.m_next = m_next;
        p.n_comb = ncomb;
        for (int t = 0; t < ncomb; ++t) {
            p.comb_k[t] = kidx[t] < 0 ? nullptr : K[kidx[t]];
            p.comb_c[t] = (float)coef[t];
        }
        p.dt = (float)dt;
        p.dt_dev = pass_dt_dev;
        p.x_out = X;
        return run_row(p) && run_columns();
    }

    // Final RHS of an attempt (at the proposed state) with statistics and optional error terms.
    bool final_eval(const float *m_in, float *k_out, int nerr, const int *kidx, const double *coef, double dt,
                    bool sync = true) {
        RowPass p = row_base();
        p.x_in = X;
        p.m_in = m_in;
        p.k_out = k_out;
        p.partials = partials;
        p.n_err = nerr;
        for (int t = 0; t < nerr; ++t) {
            p.err_k[t] = kidx[t] < 0 ? nullptr : K[kidx[t]];
            p.err_c[t] = coef[t];
        }
        p.err_dt = dt;
        p.dt_dev = pass_dt_dev;
        return run_row(p) && (sync ? read_stats() : enqueue_stats());
    }

    // ---- fixed-step integrators: the whole step as one CUDA graph ----
    // One executable per state parity (the committed state alternates between
    // S[0] and S[1]); re-captured when dt changes.  With an interrupt poll
    // installed the step runs pass by pass instead, polling in between.
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    double gdt[2] = {0.0, 0.0};
    uint64_t gkernels[2] = {0, 0};
    bool use_graphs = true;

    void drop_graphs() {
        for (int c = 0; c < 2; ++c) {
            if (gexec[c]) cudaGraphExecDestroy(gexec[c]);
            gexec[c] = nullptr;
            if (dexec[c]) cudaGraphExecDestroy(dexec[c]);
            dexec[c] = nullptr;
        }
    }

    // The final evaluation of a fixed step can also form the next step's first stage input
    // A[0] = N(m' + c dt k1') for the same dt (c = 1/2 for RK4, 1 for Heun), transform it
    // along x and run the column passes on it: that is all the next step's first pass does,
    // and k1' is at hand in that evaluation's registers.  The next step at the same dt then
    // starts with its second pass (RK4: four row passes per step instead of five; Heun: two
    // instead of three).  prep_ready says that X and A[0] hold that stage for state
    // parity prep_cur and step prep_dt; any other pass that writes X clears it (run_row).
    bool prep_ready = false;
    int prep_cur = -1;
    double prep_dt = 0.0;

    double first_coef() const { return integrator == FULLMAG_FDM_INTEGRATOR_RK4 ? 0.5 : 1.0; }
    bool first_ready(double dt) const { return prep_ready && prep_cur == cur && prep_dt == dt; }
    void mark_next(double dt) {
        prep_ready = true;
        prep_cur = cur;
        prep_dt = dt;
    }

    // first pass of a fixed step: A[0] = N(m0 + c dt k1), forward x-transform, column passes
    bool first_stage(double dt) {
        const int k0[1] = {0};
        const double c[1] = {first_coef()};
        return stage(nullptr, nullptr, 1, k0, c, dt, A[0]);
    }

    // Final evaluation at m (k1' -> K[0], statistics) fused with the next step's first stage.
    bool final_prepare(float *m, double dt, bool sync) {
        RowPass p = row_base();
        p.x_in = X;
        p.m_in = m;
        p.k_out = K[0];
        p.partials = partials;
        p.m0 = m;
        p.m_next = A[0];
        p.n_comb = 1;
        p.comb_k[0] = nullptr;
        p.comb_c[0] = (float)first_coef();
        p.dt = (float)dt;
        p.x_out = X;
        return run_row(p) && run_columns() && (sync ? read_stats() : enqueue_stats());
    }

    // Enqueues a Heun or RK4 step from S[cur] into S[1-cur]; `poll_between` checks the
    // interrupt callback between passes (eager mode only).  with_first: run the first
    // pass (else X and A[0] already hold it); prepare: end with final_prepare.
    int enqueue_fixed_step(double dt, bool poll_between, bool with_first = true, bool prepare = false) {
        const int nxt = 1 - cur;
        if (integrator == FULLMAG_FDM_INTEGRATOR_RK4) {
            const int self[1] = {-1};
            const double h[1] = {0.5}, one[1] = {1.0};
            if (with_first && !first_stage(dt)) return -1;
            if (poll_between && poll_hit()) return 1;
            if (!stage(A[0], K[1], 1, self, h, dt, A[1])) return -1;
            if (poll_between && poll_hit()) return 1;
            if (!stage(A[1], K[2], 1, self, one, dt, A[0])) return -1;
            if (poll_between && poll_hit()) return 1;
            const int k[4] = {0, 1, 2, -1};
            const double c[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
            if (!stage(A[0], nullptr, 4, k, c, dt, S[nxt])) return -1;
        } else {
            if (with_first && !first_stage(dt)) return -1;
            if (poll_between && poll_hit()) return 1;
            const int k[2] = {0, -1};
            const double c[2] = {0.5, 0.5};
            if (!stage(A[0], nullptr, 2, k, c, dt, S[nxt])) return -1;
        }
        if (prepare) return final_prepare(S[nxt], dt, poll_between) ? 0 : -1;
        return final_eval(S[nxt], K[0], 0, nullptr, nullptr, dt, poll_between) ? 0 : -1;
    }

    bool capture_step(double dt) {
        if (gexec[cur]) {
            cudaGraphExecDestroy(gexec[cur]);
            gexec[cur] = nullptr;
        }
        const uint64_t l0 = launches;
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
        // the graph starts at the second pass: the first runs before it unless prepared
        const int rc = enqueue_fixed_step(dt, false, false, true);
        const cudaError_t e = cudaStreamEndCapture(stream, &graph);
        launches = l0;
        if (rc != 0 || e != cudaSuccess || graph == nullptr) {
            if (graph) cudaGraphDestroy(graph);
            return false;
        }
        size_t nnodes = 0;
        cudaGraphGetNodes(graph, nullptr, &nnodes);
        const cudaError_t ie = cudaGraphInstantiate(&gexec[cur], graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            gexec[cur] = nullptr;
            return false;
        }
        gkernels[cur] = nnodes > 0 ? nnodes - 1 : 0;  // every node but the stats copy is a kernel
        gdt[cur] = dt;
        return true;
    }

    int step_fixed(double dt) {
        thermal_dt_for(dt);
        if (!ensure_k1()) return -1;
        if (poll_hit()) return 1;
        // the stages see I(t) and the step's thermal counter; the final evaluation gives the
        // next step's k1, at I(t + dt) and the next counter
        if (!set_oersted(time, time + dt) || !set_thermal(th_step, th_step + 1)) return -1;
        const bool ready = first_ready(dt);
        if (poll == nullptr && use_graphs && !ktime) {
            if ((!gexec[cur] || gdt[cur] != dt) && !capture_step(dt)) {
                // capture unavailable: clear the sticky state and fall back to eager launches
                cudaGetLastError();
                use_graphs = false;
                last_error.clear();
            }
            if (use_graphs) {
                if (!ready && !first_stage(dt)) return -1;
                if (cuda_fail("graph launch", cudaGraphLaunch(gexec[cur], stream))) return -1;
                launches += gkernels[cur];
                if (cuda_fail("stream sync", cudaStreamSynchronize(stream))) return -1;
                commit(dt, hstats);
                mark_next(dt);
                return 0;
            }
        }
        const int rc = enqueue_fixed_step(dt, true, !ready, true);
        if (rc != 0) return rc;
        commit(dt, hstats);
        mark_next(dt);
        return 0;
    }

    bool ensure_k1() { return k1_valid || eval_state(false); }

    void commit(double dt, const double *raw) {
        kt_collect();
        cur = 1 - cur;
        memcpy(stat_raw, raw, sizeof(stat_raw));
        step_count += 1;
        th_step += 1;
        time += dt;
        k1_valid = true;
        stats_valid = true;
        fields_valid = false;
        fill_stats(stat_raw, cur_stats);
        cur_stats.step = step_count;
        cur_stats.time_seconds = time;
        cur_stats.dt_seconds = dt;
        cur_stats.suggested_next_dt = 0.0;
    }

    // ---- Dormand-Prince 5(4) with first-same-as-last ----
    // An attempt is seven passes from S[cur] into S[1-cur] ending with the error norm
    // and statistics at the proposed state.  With no interrupt poll it runs as one
    // CUDA graph per state parity: dt comes from a device scalar (an H2D node copies
    // the host value each replay) and the FSAL hand-over is a device copy K6 -> K0,
    // so the captured pointers never change.
    cudaGraphExec_t dexec[2] = {nullptr, nullptr};
    uint64_t dkernels[2] = {0, 0};
    double *dt_dev = nullptr;   // device scalar (arena)
    double *dt_host = nullptr;  // pinned
    const double *pass_dt_dev = nullptr;  // set while capturing: passes read dt from dt_dev
    bool dp45_pending = false;
    double dp45_dt = 0.0;

    // Adaptive integrators share the attempt machinery below: DP45 and RK23 differ in
    // their passes, the stored derivative handed to the next attempt (first-same-as-last)
    // and the exponent of the step-size rule.
    bool adaptive() const {
        return integrator == FULLMAG_FDM_INTEGRATOR_DP45 || integrator == FULLMAG_FDM_INTEGRATOR_RK23;
    }
    int fsal_index() const { return integrator == FULLMAG_FDM_INTEGRATOR_RK23 ? 3 : 6; }
    double ctrl_exp() const { return integrator == FULLMAG_FDM_INTEGRATOR_RK23 ? 1.0 / 3.0 : 0.2; }

    // Bogacki-Shampine 3(2) with FSAL (native/backends/fdm/src/llg_rk23_fp32.cu:150-265):
    // N(m0 + dt/2 k1), N(m0 + 3dt/4 k2), the proposal N(m0 + dt (2/9 k1 + 1/3 k2 + 4/9 k3))
    // into S[1-cur], then k4 at the proposal with the error dt (-5/72 k1 + 1/12 k2 + 1/9 k3
    // - 1/8 k4) and the statistics.
    int enqueue_rk23(double dt, bool poll_between) {
        static const double a2[1] = {0.5}, a3[1] = {0.75};
        static const double b[3] = {2.0 / 9.0, 1.0 / 3.0, 4.0 / 9.0};
        static const double e[4] = {-5.0 / 72.0, 1.0 / 12.0, 1.0 / 9.0, -1.0 / 8.0};
        const int nxt = 1 - cur;
        const int k1[1] = {0}, self[1] = {-1}, kb[3] = {0, 1, -1}, ke[4] = {0, 1, 2, -1};
        if (!stage(nullptr, nullptr, 1, k1, a2, dt, A[0])) return -1;
        if (poll_between && poll_hit()) return 1;
        if (!stage(A[0], K[1], 1, self, a3, dt, A[1])) return -1;
        if (poll_between && poll_hit()) return 1;
        if (!stage(A[1], K[2], 3, kb, b, dt, S[nxt])) return -1;
        if (poll_between && poll_hit()) return 1;
        return final_eval(S[nxt], K[3], 4, ke, e, dt, false) ? 0 : -1;
    }

    int enqueue_dp45(double dt, bool poll_between) {
        if (integrator == FULLMAG_FDM_INTEGRATOR_RK23) return enqueue_rk23(dt, poll_between);
        static const double a21[1] = {1.0 / 5.0};
        static const double a3[2] = {3.0 / 40.0, 9.0 / 40.0};
        static const double a4[3] = {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0};
        static const double a5[4] = {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0};
        static const double a6[5] = {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0};
        static const double b[5] = {35.0 / 384.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0};
        static const double e[6] = {71.0 / 57600.0, -71.0 / 16695.0, 71.0 / 1920.0, -17253.0 / 339200.0, 22.0 / 525.0,
                                    -1.0 / 40.0};
        const int nxt = 1 - cur;
        const int k1[1] = {0}, k2[2] = {0, -1}, k3[3] = {0, 1, -1}, k4[4] = {0, 1, 2, -1}, k5[5] = {0, 1, 2, 3, -1};
        const int kb[5] = {0, 2, 3, 4, -1}, ke[6] = {0, 2, 3, 4, 5, -1};
        if (!stage(nullptr, nullptr, 1, k1, a21, dt, A[0])) return -1;
        if (poll_between && poll_hit()) return 1;
        if (!stage(A[0], K[1], 2, k2, a3, dt, A[1])) return -1;
        if (poll_between && poll_hit()) return 1;
        if (!stage(A[1], K[2], 3, k3, a4, dt, A[0])) return -1;
        if (poll_between && poll_hit()) return 1;
        if (!stage(A[0], K[3], 4, k4, a5, dt, A[1])) return -1;
        if (poll_between && poll_hit()) return 1;
        if (!stage(A[1], K[4], 5, k5, a6, dt, A[0])) return -1;
        if (poll_between && poll_hit()) return 1;
        if (!stage(A[0], K[5], 5, kb, b, dt, S[nxt])) return -1;
        if (poll_between && poll_hit()) return 1;
        return final_eval(S[nxt], K[6], 6, ke, e, dt, false) ? 0 : -1;
    }

    bool capture_dp45() {
        if (dexec[cur]) {
            cudaGraphExecDestroy(dexec[cur]);
            dexec[cur] = nullptr;
        }
        const uint64_t l0 = launches;
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
        bool ok = cudaMemcpyAsync(dt_dev, dt_host, sizeof(double), cudaMemcpyHostToDevice, stream) == cudaSuccess;
        pass_dt_dev = dt_dev;
        if (ok) ok = enqueue_dp45(0.0, false) == 0;
        pass_dt_dev = nullptr;
        const cudaError_t e = cudaStreamEndCapture(stream, &graph);
        launches = l0;
        if (!ok || e != cudaSuccess || graph == nullptr) {
            if (graph) cudaGraphDestroy(graph);
            return false;
        }
        size_t nnodes = 0;
        cudaGraphGetNodes(graph, nullptr, &nnodes);
        const cudaError_t ie = cudaGraphInstantiate(&dexec[cur], graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            dexec[cur] = nullptr;
            return false;
        }
        dkernels[cur] = nnodes > 2 ? nnodes - 2 : 0;  // all but the dt and stats copies
        return true;
    }

    // Starts one attempt of size dt without waiting for it (graph path) or runs it
    // pass by pass with interrupt polls.  Returns 0 queued, 1 interrupted, -1 error.
    int begin_dp45_attempt(double dt) {
        if (!ensure_k1()) return -1;
        if (poll_hit()) return 1;
        // every stage and the first-same-as-last derivative see I(t), as the reference's do,
        // and the step's thermal counter
        if (!set_oersted(time, time) || !set_thermal(th_step, th_step)) return -1;
        dp45_dt = dt;
        if (poll == nullptr && use_graphs && !ktime) {
            if (!dexec[cur] && !capture_dp45()) {
                cudaGetLastError();
                use_graphs = false;
                last_error.clear();
            }
            if (use_graphs) {
                *dt_host = dt;
                if (cuda_fail("graph launch", cudaGraphLaunch(dexec[cur], stream))) return -1;
                launches += dkernels[cur];
                dp45_pending = true;
                return 0;
            }
        }
        const int rc = enqueue_dp45(dt, true);
        if (rc != 0) return rc;
        dp45_pending = true;
        return 0;
    }

    // Waits for the pending attempt and applies the accept/reject rule of the C ABI
    // (native/backends/fdm/src/llg_dp45_fp32.cu:286-341).  Returns 1 accepted,
    // 0 rejected (next_dt holds the retry size), -1 error.
    int finish_dp45_attempt(double &next_dt) {
        if (!dp45_pending) return -1;
        dp45_pending = false;
        if (cuda_fail("stream sync", cudaStreamSynchronize(stream))) return -1;
        kt_collect();
        const double dt = dp45_dt;
        const double err = sqrt(hstats[8]);
        if (err <= max_error || dt <= dt_min) {
            double dt_next = dt_max;
            if (err > 0.0) dt_next = std::min(std::max(headroom * dt * pow(max_error / err, ctrl_exp()), dt_min), dt_max);
            // first-same-as-last: the last derivative (at the accepted state) is the next step's k1
            if (cuda_fail("fsal copy", cudaMemcpyAsync(K[0], K[fsal_index()], sizeof(float) * 3 * (size_t)g.n,
                                                       cudaMemcpyDeviceToDevice, stream)))
                return -1;
            commit(dt, hstats);
            cur_stats.suggested_next_dt = dt_next;
            next_dt = dt_next;
            return 1;
        }
        next_dt = std::min(std::max(headroom * dt * pow(max_error / err, ctrl_exp()), dt_min), dt_max);
        // a retry starts from k1 at the step's own thermal counter and Oersted current: the
        // first-same-as-last derivative came from the previous step's evaluations
        if (has_thermal || (has_oersted && oe_kind != 0)) k1_valid = false;
        return 0;
    }

    // Asynchronous fixed-step step for the batch driver (no interrupt polling).
    bool fixed_pending = false;
    double fixed_dt = 0.0;
    int begin_fixed_step(double dt) {
        thermal_dt_for(dt);
        if (!ensure_k1()) return -1;
        if (!set_oersted(time, time + dt) || !set_thermal(th_step, th_step + 1)) return -1;
        if (use_graphs && (!gexec[cur] || gdt[cur] != dt) && !capture_step(dt)) {
            cudaGetLastError();
            use_graphs = false;
            last_error.clear();
        }
        const bool ready = first_ready(dt);
        if (use_graphs) {
            if (!ready && !first_stage(dt)) return -1;
            if (cuda_fail("graph launch", cudaGraphLaunch(gexec[cur], stream))) return -1;
            launches += gkernels[cur];
        } else if (enqueue_fixed_step(dt, false, !ready, true) != 0) {
            return -1;
        }
        fixed_pending = true;
        fixed_dt = dt;
        return 0;
    }
    int finish_fixed_step() {
        if (!fixed_pending) return -1;
        fixed_pending = false;
        if (cuda_fail("stream sync", cudaStreamSynchronize(stream))) return -1;
        commit(fixed_dt, hstats);
        mark_next(fixed_dt);
        return 1;
    }

    // ---- adjoint: reverse-mode RK4 with checkpointing ----
    // adjoint_forward integrates n steps from the current state, keeping the state
    // every C steps (C ~ sqrt(n)).  adjoint_backward walks the segments backwards:
    // it recomputes a segment from its checkpoint while storing every stage input
    // y0..y3, effective field H0..H3 and k1..k4, then applies the transposed step in
    // reverse (equations in adjoint.cu): per stage one row pass computes the local VJP
    // and forward-transforms lambda_H, the column passes convolve it, and a second row
    // pass adds H_lin(lambda_H) and pushes the result through the stage normalisation.
    // d loss / d field map accumulates in float-float.
    float *adj_ckpt = nullptr;  // [n_ckpt][3n]
    float *adj_seg = nullptr;   // [C][12][3n]: y0 y1 y2 y3 H0 H1 H2 H3 k1 k2 k3 k4
    float *adj_work = nullptr;  // [12][3n]: lam_next lam_y0 lk1 lk2 lk3 lk4 lam_h[0] lam_m lam_h[1] g_hi g_lo spare
    uint64_t adj_nsteps = 0;
    uint32_t adj_C = 0;
    size_t adj_nck = 0;
    double adj_h = 0.0;

    void adj_free() {
        if (adj_ckpt) cudaFree(adj_ckpt);
        if (adj_seg) cudaFree(adj_seg);
        if (adj_work) cudaFree(adj_work);
        adj_ckpt = adj_seg = adj_work = nullptr;
    }

    size_t vec3() const { return 3 * (size_t)g.n; }

    // One RK4 step from y0 into y_next.  out[1..3] receive y1..y3, out[4..7] H0..H3
    // (NULL: not stored), out[8..11] k1..k4 (k1..k3 required).  X must hold the
    // convolved transform of y0 on entry; on return it holds that of y_next.
    bool adj_step(const float *y0, float *const *out, float *y_next, double h) {
        const double cs[3] = {0.5, 0.5, 1.0};
        const float *ys[4] = {y0, out[1], out[2], out[3]};
        for (int s = 0; s < 4; ++s) {
            RowPass p = row_base();
            p.x_in = X;
            p.m_in = ys[s];
            p.k_out = out[8 + s];
            p.h_eff_out = out[4 + s];
            p.m0 = y0;
            p.dt = (float)h;
            p.x_out = X;
            if (s < 3) {
                p.m_next = out[1 + s];
                p.n_comb = 1;
                p.comb_k[0] = nullptr;
                p.comb_c[0] = (float)cs[s];
            } else {
                p.m_next = y_next;
                p.n_comb = 4;
                p.comb_k[0] = out[8];
                p.comb_k[1] = out[9];
                p.comb_k[2] = out[10];
                p.comb_k[3] = nullptr;
                p.comb_c[0] = (float)(1.0 / 6.0);
                p.comb_c[1] = (float)(1.0 / 3.0);
                p.comb_c[2] = (float)(1.0 / 3.0);
                p.comb_c[3] = (float)(1.0 / 6.0);
            }
            if (!run_row(p) || !run_columns()) return false;
        }
        return true;
    }

    int adjoint_forward(double h, uint64_t nsteps, uint32_t C) {
        if (integrator != FULLMAG_FDM_INTEGRATOR_RK4) {
            last_error = "the adjoint requires the RK4 integrator";
            return FULLMAG_FDM_ERR_INVALID;
        }
        if (nsteps == 0 || !(h > 0.0)) {
            last_error = "adjoint_forward needs n_steps > 0 and dt > 0";
            return FULLMAG_FDM_ERR_INVALID;
        }
        if (has_extra) {
            last_error = "the adjoint does not support DMI or magnetoelastic terms";
            return FULLMAG_FDM_ERR_INVALID;
        }
        if (C == 0) C = (uint32_t)std::max<uint64_t>(1, (uint64_t)std::ceil(std::sqrt((double)nsteps)));
        adj_free();
        adj_nsteps = nsteps;
        adj_C = C;
        adj_h = h;
        adj_nck = (size_t)((nsteps + C - 1) / C);
        const size_t v3 = vec3();
        if (cuda_fail("cudaMalloc(adjoint checkpoints)", cudaMalloc((void **)&adj_ckpt, sizeof(float) * v3 * adj_nck)))
            return FULLMAG_FDM_ERR_CUDA;
        // scratch stage buffers: y1 y2 y3 k1 k2 k3 (k4 stays in registers)
        float *scr = nullptr;
        if (cuda_fail("cudaMalloc(adjoint scratch)", cudaMalloc((void **)&scr, sizeof(float) * v3 * 6))) return FULLMAG_FDM_ERR_CUDA;
        float *out[12] = {nullptr, scr, scr + v3, scr + 2 * v3, nullptr, nullptr, nullptr, nullptr,
                          scr + 3 * v3, scr + 4 * v3, scr + 5 * v3, nullptr};
        bool ok = pass_forward(S[cur]);
        for (uint64_t st = 0; st < nsteps && ok; ++st) {
            if (st % C == 0)
                ok = !cuda_fail("checkpoint copy", cudaMemcpyAsync(adj_ckpt + (st / C) * v3, S[cur], sizeof(float) * v3,
                                                                   cudaMemcpyDeviceToDevice, stream));
            if (ok) ok = adj_step(S[cur], out, S[1 - cur], h);
            cur = 1 - cur;
        }
        if (ok) ok = !cuda_fail("adjoint sync", cudaStreamSynchronize(stream));
        cudaFree(scr);
        if (!ok) return FULLMAG_FDM_ERR_CUDA;
        step_count += nsteps;
        time += h * (double)nsteps;
        k1_valid = fields_valid = stats_valid = false;
        abm_restart();
        return eval_state(false) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
    }

    int adjoint_backward(const double *lam_T, double *grad_out, double *lam0_out) {
        if (!adj_ckpt) {
            last_error = "adjoint_backward needs a preceding adjoint_forward";
            return FULLMAG_FDM_ERR_INVALID;
        }
        if (has_cub) {
            last_error = "the adjoint does not support cubic anisotropy";
            return FULLMAG_FDM_ERR_INVALID;
        }
        if (has_extra) {
            last_error = "the adjoint does not support DMI or magnetoelastic terms";
            return FULLMAG_FDM_ERR_INVALID;
        }
        const size_t v3 = vec3();
        const long long n = g.n;
        if (!adj_seg && cuda_fail("cudaMalloc(adjoint segment)", cudaMalloc((void **)&adj_seg, sizeof(float) * v3 * 12 * adj_C)))
            return FULLMAG_FDM_ERR_CUDA;
        if (!adj_work && cuda_fail("cudaMalloc(adjoint work)", cudaMalloc((void **)&adj_work, sizeof(float) * v3 * 12)))
            return FULLMAG_FDM_ERR_CUDA;
        float *W[12];
        for (int i = 0; i < 12; ++i) W[i] = adj_work + i * v3;
        float *lam_next = W[0], *lam_y0 = W[1], *lk[5] = {nullptr, W[2], W[3], W[4], W[5]};
        float *lam_hb[2] = {W[6], W[8]}, *lam_m = W[7], *g_hi = W[9], *g_lo = W[10], *spare = W[11];
        if (!ensure_staging()) return FULLMAG_FDM_ERR_CUDA;
        if (cuda_fail("cudaMemcpy(lambda)", cudaMemcpyAsync(staging, lam_T, sizeof(double) * v3, cudaMemcpyHostToDevice, stream)))
            return FULLMAG_FDM_ERR_CUDA;
        aos_to_soa_kernel<<<std::min<long long>((n + 255) / 256, 4096), 256, 0, stream>>>((const double *)staging, nullptr,
                                                                                          lam_next, mask, n);
        if (cuda_fail("zero", cudaMemsetAsync(g_hi, 0, sizeof(float) * v3 * 2, stream))) return FULLMAG_FDM_ERR_CUDA;
        const double h = adj_h;
        const float hf = (float)h;
        const float cs[4] = {0.f, 0.5f, 0.5f, 1.0f};
        bool ok = true;
        for (long long seg = (long long)adj_nck - 1; seg >= 0 && ok; --seg) {
            const uint64_t s0 = (uint64_t)seg * adj_C;
            const uint64_t len = std::min<uint64_t>(adj_C, adj_nsteps - s0);
            auto slot = [&](uint64_t t, int f) { return adj_seg + (t * 12 + f) * v3; };
            ok = !cuda_fail("segment copy", cudaMemcpyAsync(slot(0, 0), adj_ckpt + seg * v3, sizeof(float) * v3,
                                                            cudaMemcpyDeviceToDevice, stream)) &&
                 pass_forward(slot(0, 0));
            for (uint64_t t = 0; t < len && ok; ++t) {
                float *out[12];
                for (int f = 0; f < 12; ++f) out[f] = slot(t, f);
                ok = adj_step(slot(t, 0), out, t + 1 < len ? slot(t + 1, 0) : spare, h);
            }
            for (long long t = (long long)len - 1; t >= 0 && ok; --t) {
                AdjFinal af{n, lam_next, slot(t, 0), slot(t, 8), slot(t, 9), slot(t, 10), slot(t, 11), hf,
                            lam_y0, lk[1], lk[2], lk[3], lk[4]};
                ok = !cuda_fail("adjoint final", launch_adj_final(af, stream));
                // Five row passes per step, like a forward step: the local VJP of stage s - 1
                // (bit 1) shares a pass with the stage-s update after H_lin (bit 2), because the
                // cotangent of k_s it needs is complete at each cell once bit 2 has run there.
                // lambda_H alternates between two buffers (the stencil reads its neighbours).
                int lh = 0;
                for (int s = 4; s >= 0 && ok; --s) {
                    RowPass b = row_base();
                    b.mat.has_ext = 0;
                    b.mat.has_uni = 0;
                    b.mat.has_cub = 0;
                    b.hmap = nullptr;
                    b.adj_uni = mat.has_uni;
                    b.adj_mode = 0;
                    if (s <= 3) {  // bit 2: update of stage s from H_lin(lambda_H of stage s)
                        b.adj_mode |= 2;
                        b.x_in = X;
                        b.m_in = lam_hb[lh];
                        b.adj_lam_m = lam_m;
                        b.adj_y0 = slot(t, 0);
                        b.adj_k = s >= 1 ? slot(t, 8 + s - 1) : nullptr;
                        b.adj_ch = cs[s] * hf;
                        b.adj_lam_y0 = lam_y0;
                        b.adj_lam_k = s >= 1 ? lk[s] : nullptr;
                    }
                    if (s >= 1) {  // bit 1: local VJP of stage s - 1, forward x-transform of its lambda_H
                        b.adj_mode |= 1;
                        b.adj_m = slot(t, s - 1);
                        b.adj_H = slot(t, 4 + s - 1);
                        b.adj_w = lk[s];
                        b.adj_lam_h = lam_hb[1 - lh];
                        b.adj_lam_m = lam_m;
                        b.adj_g_hi = g_hi;
                        b.adj_g_lo = g_lo;
                        b.x_out = X;
                    }
                    ok = run_row_adj(b) && (s == 0 || run_columns());
                    lh = 1 - lh;
                }
                std::swap(lam_next, lam_y0);
            }
        }
        if (!ok) return FULLMAG_FDM_ERR_CUDA;
        // gradient: g_hi + g_lo (per A/m of the map), lambda_0 = lam_next
        std::vector<float> hi(v3), lo(v3), l0(v3);
        if (cuda_fail("cudaMemcpy(grad)", cudaMemcpyAsync(hi.data(), g_hi, sizeof(float) * v3, cudaMemcpyDeviceToHost, stream)) ||
            cuda_fail("cudaMemcpy(grad)", cudaMemcpyAsync(lo.data(), g_lo, sizeof(float) * v3, cudaMemcpyDeviceToHost, stream)) ||
            cuda_fail("cudaMemcpy(lambda0)",
                      cudaMemcpyAsync(l0.data(), lam_next, sizeof(float) * v3, cudaMemcpyDeviceToHost, stream)) ||
            cuda_fail("adjoint sync", cudaStreamSynchronize(stream)))
            return FULLMAG_FDM_ERR_CUDA;
        for (long long i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) {
                if (grad_out) grad_out[3 * i + c] = (double)hi[c * n + i] + (double)lo[c * n + i];
                if (lam0_out) lam0_out[3 * i + c] = (double)l0[c * n + i];
            }
        return FULLMAG_FDM_OK;
    }

    bool set_field_map(const double *h_xyz) {
        if (!h_xyz) {
            drop_graphs();  // captured passes hold the map pointer freed here
            if (hmap) cudaFree(hmap);
            hmap = nullptr;
            k1_valid = fields_valid = stats_valid = false;
            abm_restart();
            return true;
        }
        if (!hmap && cuda_fail("cudaMalloc(field map)", cudaMalloc((void **)&hmap, sizeof(float) * vec3()))) return false;
        if (!ensure_staging()) return false;
        if (cuda_fail("cudaMemcpy(field map)",
                      cudaMemcpyAsync(staging, h_xyz, sizeof(double) * vec3(), cudaMemcpyHostToDevice, stream)))
            return false;
        aos_to_soa_kernel<<<std::min<long long>((g.n + 255) / 256, 4096), 256, 0, stream>>>((const double *)staging, nullptr,
                                                                                            hmap, mask, g.n);
        if (cuda_fail("field map convert", cudaGetLastError())) return false;
        drop_graphs();  // captured passes hold the previous map pointer
        k1_valid = fields_valid = stats_valid = false;
        abm_restart();
        return !cuda_fail("field map sync", cudaStreamSynchronize(stream));
    }

    // ---- batched DP45 (fullmag_fdm_batch_*) ----
    // A batched attempt always reads the committed state S[0] and writes its proposal
    // to S[1]; an accepted proposal is committed on the device at the start of the
    // next round (S0 <- S1, K0 <- K6), so the recorded pass descriptors never change
    // and every round of the batch replays one CUDA graph.
    // Tiles for batched rounds.  The autotuner picks tiles that make one small grid fill
    // the GPU (many thin CTAs); in a batched round the problems fill the GPU together, so
    // each CTA takes more work instead: row passes of at least ~512 cells, and the widest
    // kx tile of the fused column pass within 64 KB of shared memory.
    void batch_tiling() {
        const int nrows = g.ny * g.nz;
        int r = 1;
        while (r < 16 && r * g.nx < 512 && 2 * r <= nrows) {
            RowPass t = row_base();
            t.rows = 2 * r;
            t.x_in = demag ? X : nullptr;
            t.x_out = demag ? X : nullptr;
            if (row_pass_smem(t) > 64u * 1024u) break;
            r *= 2;
        }
        if (r > row_rows) {
            row_rows = r;
            row_blocks = (nrows + row_rows - 1) / row_rows;
        }
        if (!demag) return;
        int tx = 1;
        auto smem = [&](int t) { return g.thin ? y_convolve_2d_smem(g, t) : yz_convolve_smem(g, t); };
        while (tx < 16 && 2 * tx <= g.nkx && smem(2 * tx) <= 64u * 1024u) tx *= 2;
        if (g.thin) tx_2d = std::max(tx_2d, tx);
        else if (use_yz) tx_z = std::max(tx_z, tx);
    }

    bool batch_prepare() {
        if (cur != 0) {  // bring the committed state to S[0]
            if (cuda_fail("state copy", cudaMemcpyAsync(S[0], S[1], sizeof(float) * 3 * (size_t)g.n,
                                                        cudaMemcpyDeviceToDevice, stream)))
                return false;
            cur = 0;
            k1_valid = false;
        }
        if (!ensure_k1()) return false;
        return !cuda_fail("stream sync", cudaStreamSynchronize(stream));
    }

    // Records the seven row passes and six column passes of one attempt, with dt read
    // from dt_ptr.  False when a pass cannot run batched (large 3-D grids).
    bool record_attempt(const double *dt_ptr, std::vector<RowPass> &rows, std::vector<int> &cols) {
        rows.clear();
        cols.clear();
        if (has_extra) return false;  // the extra field pass is not part of the batched rounds
        rec_rows = &rows;
        rec_cols = &cols;
        pass_dt_dev = dt_ptr;
        const int rc = enqueue_dp45(0.0, false);
        rec_rows = nullptr;
        rec_cols = nullptr;
        pass_dt_dev = nullptr;
        return rc == 0 && rows.size() == 7 && (cols.size() == 6 || (!demag && cols.empty()));
    }

    // Takes over the device step control of the batched rounds: the accepted steps since the
    // last hand-over, the time they reached and the statistics of the last one.
    void batch_apply(const BatchState &st) {
        time = st.time;
        if (st.steps == 0) return;
        step_count += st.steps;
        memcpy(stat_raw, st.acc_stats, sizeof(double) * kNumStats);  // batched rounds carry no extra-field sums
        stats_valid = true;
        fields_valid = false;
        fill_stats(stat_raw, cur_stats);
        cur_stats.step = step_count;
        cur_stats.time_seconds = time;
        cur_stats.dt_seconds = st.dt_used;
        cur_stats.suggested_next_dt = st.suggested;
    }

    int step_dp45(double dt) {
        for (;;) {
            const int rc = begin_dp45_attempt(dt);
            if (rc != 0) return rc;
            double next = dt;
            const int ok = finish_dp45_attempt(next);
            if (ok < 0) return -1;
            if (ok == 1) return cuda_fail("stream sync", cudaStreamSynchronize(stream)) ? -1 : 0;
            dt = next;
        }
    }

    // ---- Adams-Bashforth-Moulton 3 (native/backends/fdm/src/llg_abm3_fp32.cu:115-266) ----
    // History f_n, f_{n-1}, f_{n-2} in K[abm_hist[0..2]], K[abm_kf] receives f at the
    // prediction; the indices rotate instead of the buffers.  While fewer than three steps
    // built the history, or when dt moved by more than 10 % since the last step, a step is
    // a Heun step and f at its accepted state (K[0] after the final evaluation) becomes
    // f_n.  Otherwise: predictor N(m + dt (23 f_n - 16 f_{n-1} + 5 f_{n-2})/12), f_s at the
    // prediction, corrector N(m + dt (5 f_s + 8 f_n - f_{n-1})/12), and f_s becomes f_n.
    // A new state or field map restarts the history (the reference keeps it).
    int abm_startup = 0;
    double abm_last_dt = 0.0;
    int abm_hist[3] = {1, 2, 3}, abm_kf = 4;

    void abm_restart() {
        abm_startup = 0;
        abm_last_dt = 0.0;
    }

    int step_abm3(double dt) {
        if (abm_last_dt > 0.0 && std::fabs(dt - abm_last_dt) / abm_last_dt > 0.1) abm_startup = 0;
        thermal_dt_for(dt);
        if (!ensure_k1()) return -1;
        if (poll_hit()) return 1;
        if (!set_oersted(time, time + dt) || !set_thermal(th_step, th_step + 1)) return -1;
        const int nxt = 1 - cur;
        if (abm_startup < 3) {
            const int rc = enqueue_fixed_step(dt, true);  // the Heun sequence (ends with K[0] = f at S[nxt])
            if (rc != 0) return rc;
            const int slot = abm_hist[2];
            abm_hist[2] = abm_hist[1];
            abm_hist[1] = abm_hist[0];
            abm_hist[0] = slot;
            if (cuda_fail("history copy",
                          cudaMemcpyAsync(K[slot], K[0], sizeof(float) * 3 * (size_t)g.n, cudaMemcpyDeviceToDevice, stream)))
                return -1;
            abm_startup += 1;
        } else {
            const int kp[3] = {abm_hist[0], abm_hist[1], abm_hist[2]};
            const double cp[3] = {23.0 / 12.0, -16.0 / 12.0, 5.0 / 12.0};
            if (!stage(nullptr, nullptr, 3, kp, cp, dt, A[0])) return -1;
            if (poll_hit()) return 1;
            const int kc[3] = {-1, abm_hist[0], abm_hist[1]};
            const double cc[3] = {5.0 / 12.0, 8.0 / 12.0, -1.0 / 12.0};
            if (!stage(A[0], K[abm_kf], 3, kc, cc, dt, S[nxt])) return -1;
            if (poll_hit()) return 1;
            if (!final_eval(S[nxt], K[0], 0, nullptr, nullptr, dt, true)) return -1;
            const int freed = abm_hist[2];
            abm_hist[2] = abm_hist[1];
            abm_hist[1] = abm_hist[0];
            abm_hist[0] = abm_kf;
            abm_kf = freed;
        }
        abm_last_dt = dt;
        commit(dt, hstats);
        return 0;
    }

    int step(double dt) {
        interrupted = false;
        switch (integrator) {
            case FULLMAG_FDM_INTEGRATOR_RK4: return step_fixed(dt);
            case FULLMAG_FDM_INTEGRATOR_DP45:
            case FULLMAG_FDM_INTEGRATOR_RK23: return step_dp45(dt);
            case FULLMAG_FDM_INTEGRATOR_ABM3: return step_abm3(dt);
            default: return step_fixed(dt);
        }
    }

    // ---------------- transfers ----------------
    bool ensure_staging() {
        if (staging) return true;
        return !cuda_fail("cudaMalloc(staging)", cudaMalloc(&staging, sizeof(double) * 3 * (size_t)g.n));
    }

    template <typename T>
    bool upload(const T *m_xyz) {
        if (!ensure_staging()) return false;
        const size_t bytes = sizeof(T) * 3 * (size_t)g.n;
        if (cuda_fail("cudaMemcpy(m)", cudaMemcpyAsync(staging, m_xyz, bytes, cudaMemcpyHostToDevice, stream))) return false;
        const bool isd = sizeof(T) == 8;
        aos_to_soa_kernel<<<std::min<long long>((g.n + 255) / 256, 4096), 256, 0, stream>>>(
            isd ? (const double *)staging : nullptr, isd ? nullptr : (const float *)staging, S[cur], mask, g.n);
        if (cuda_fail("upload convert", cudaGetLastError())) return false;
        if (cuda_fail("upload sync", cudaStreamSynchronize(stream))) return false;
        k1_valid = false;
        abm_restart();
        fields_valid = false;
        stats_valid = false;
        return true;
    }

    // Same result as upload<double>, staged through the static scratch of noalloc.cu
    // instead of the handle's lazily allocated staging buffer.
    bool upload_noalloc(const double *m_xyz) {
        if (cuda_fail("upload (no allocation)", noalloc_upload_f64(device, m_xyz, g.n, S[cur], mask, stream))) return false;
        k1_valid = false;
        abm_restart();
        fields_valid = false;
        stats_valid = false;
        return true;
    }

    const float *field_ptr(int obs) {
        switch (obs) {
            case FULLMAG_FDM_OBSERVABLE_M: return S[cur];
            case FULLMAG_FDM_OBSERVABLE_H_EX: return h_ex;
            case FULLMAG_FDM_OBSERVABLE_H_DEMAG: return h_d;
            case FULLMAG_FDM_OBSERVABLE_H_EFF: return h_eff;
            default: return nullptr;
        }
    }

    template <typename T>
    bool download(int obs, T *out) {
        const long long n = g.n;
        if (obs == FULLMAG_FDM_OBSERVABLE_H_EXT) {
            for (long long i = 0; i < n; ++i) {
                const bool act = !has_mask || mask_host[i] != 0;
                for (int c = 0; c < 3; ++c) out[3 * i + c] = (T)((has_ext && act) ? hext[c] : 0.0);
            }
            return true;
        }
        if (obs < FULLMAG_FDM_OBSERVABLE_M || obs > FULLMAG_FDM_OBSERVABLE_H_EFF) {
            last_error = "unknown observable " + std::to_string(obs);
            return false;
        }
        if (obs != FULLMAG_FDM_OBSERVABLE_M && !fields_valid) {
            if (!eval_state(true)) return false;
        }
        const float *src = field_ptr(obs);
        if (!ensure_staging()) return false;
        const bool isd = sizeof(T) == 8;
        soa_to_aos_kernel<<<std::min<long long>((n + 255) / 256, 4096), 256, 0, stream>>>(
            src, isd ? (double *)staging : nullptr, isd ? nullptr : (float *)staging, n);
        if (cuda_fail("download convert", cudaGetLastError())) return false;
        if (cuda_fail("cudaMemcpy(field)",
                      cudaMemcpyAsync(out, staging, sizeof(T) * 3 * (size_t)n, cudaMemcpyDeviceToHost, stream)))
            return false;
        return !cuda_fail("download sync", cudaStreamSynchronize(stream));
    }

    // ---- asynchronous snapshots ----
    cudaStream_t snap_stream = nullptr;  // device-to-host copies of snapshot payloads
    std::shared_ptr<PinnedPool> pinned_pool = std::make_shared<PinnedPool>();

    // `produce(dev)` enqueues a payload of `bytes` into a stream-ordered device buffer on
    // the engine stream; a copy on the snapshot stream then fills a pinned buffer of s,
    // and s->done marks its end.  Later steps run on the engine stream meanwhile.
    template <typename F>
    bool begin_snapshot(size_t bytes, F &&produce, SnapshotPayload *s) {
        if (!snap_stream &&
            cuda_fail("cudaStreamCreate(snapshot)", cudaStreamCreateWithFlags(&snap_stream, cudaStreamNonBlocking)))
            return false;
        s->pool = pinned_pool;
        s->pinned = pinned_pool->take(bytes, s->cap);
        if (!s->pinned) {
            last_error = "cudaMallocHost(snapshot) failed";
            return false;
        }
        s->len = bytes;
        cudaEvent_t ready = nullptr;
        if (cuda_fail("cudaEventCreate(snapshot)", cudaEventCreateWithFlags(&ready, cudaEventDisableTiming))) return false;
        if (cuda_fail("cudaEventCreate(snapshot)", cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming))) {
            cudaEventDestroy(ready);
            return false;
        }
        void *dev = nullptr;
        bool ok = !cuda_fail("cudaMallocAsync(snapshot)", cudaMallocAsync(&dev, bytes, stream));
        if (ok) {
            ok = produce(dev) && !cuda_fail("snapshot event", cudaEventRecord(ready, stream)) &&
                 !cuda_fail("snapshot stream wait", cudaStreamWaitEvent(snap_stream, ready, 0)) &&
                 !cuda_fail("cudaMemcpy(snapshot)", cudaMemcpyAsync(s->pinned, dev, bytes, cudaMemcpyDeviceToHost, snap_stream));
            cudaFreeAsync(dev, ok ? snap_stream : stream);
            if (ok) ok = !cuda_fail("snapshot event", cudaEventRecord(s->done, snap_stream));
        }
        cudaEventDestroy(ready);
        return ok;
    }

    // Device-resident observable `obs` made current (fields evaluated if stale); NULL for
    // H_EXT (synthesised on the host) and unknown observables (last_error set).
    const float *current_field(int obs) {
        if (obs < FULLMAG_FDM_OBSERVABLE_M || obs > FULLMAG_FDM_OBSERVABLE_H_EFF || obs == FULLMAG_FDM_OBSERVABLE_H_EXT) {
            if (obs != FULLMAG_FDM_OBSERVABLE_H_EXT) last_error = "unknown observable " + std::to_string(obs);
            return nullptr;
        }
        if (obs != FULLMAG_FDM_OBSERVABLE_M && !fields_valid && !eval_state(true)) return nullptr;
        return field_ptr(obs);
    }

    // Box-average preview of a device field into dev_out (AoS T) on stream s.
    template <typename T>
    bool enqueue_preview(const float *field, uint32_t pnx, uint32_t pny, uint32_t pnz, uint32_t z0, uint32_t zs, T *dev_out,
                         cudaStream_t s) {
        const long long np = (long long)pnx * pny * pnz;
        preview_kernel<T><<<(unsigned)std::min<long long>((np + 255) / 256, 4096), 256, 0, s>>>(
            field, g.n, (unsigned)g.nx, (unsigned)g.ny, (unsigned)g.nz, pnx, pny, pnz, z0, zs, dev_out);
        return !cuda_fail("preview", cudaGetLastError());
    }

    template <typename T>
    bool preview(int obs, uint32_t pnx, uint32_t pny, uint32_t pnz, uint32_t z0, uint32_t zs, T *out) {
        if (z0 >= (uint32_t)g.nz) {
            last_error = "preview z_origin out of range";
            return false;
        }
        if (obs != FULLMAG_FDM_OBSERVABLE_H_EXT) {
            const float *field = current_field(obs);
            if (!field) return false;
            const size_t bytes = sizeof(T) * 3 * (size_t)pnx * pny * pnz;
            void *dev = nullptr;
            if (cuda_fail("cudaMallocAsync(preview)", cudaMallocAsync(&dev, bytes, stream))) return false;
            const bool ok = enqueue_preview<T>(field, pnx, pny, pnz, z0, zs, (T *)dev, stream) &&
                            !cuda_fail("cudaMemcpy(preview)", cudaMemcpyAsync(out, dev, bytes, cudaMemcpyDeviceToHost, stream));
            cudaFreeAsync(dev, stream);
            return !cuda_fail("preview sync", cudaStreamSynchronize(stream)) && ok;
        }
        // H_EXT lives on the host: the same box average over the synthesised field
        std::vector<double> full(3 * (size_t)g.n);
        if (!download<double>(obs, full.data())) return false;
        host_preview<T>(full.data(), g.nx, g.ny, g.nz, pnx, pny, pnz, z0, zs, out);
        return true;
    }
};

// ---------------- setup ----------------

static bool unsupported(Engine &e, bool cond, const char *what) {
    if (cond) e.last_error = std::string("not supported by the GB300 engine: ") + what;
    return cond;
}

bool Engine::setup(const fullmag_fdm_plan_desc *plan) {
    g.nx = (int)plan->grid.nx;
    g.ny = (int)plan->grid.ny;
    g.nz = (int)plan->grid.nz;
    g.n = (long long)g.nx * g.ny * g.nz;
    dx = plan->grid.dx;
    dy = plan->grid.dy;
    dz = plan->grid.dz;
    ms = plan->material.saturation_magnetisation;
    a_ex = plan->material.exchange_stiffness;
    alpha = plan->material.damping;
    gamma = plan->material.gyromagnetic_ratio;
    integrator = plan->integrator;
    exchange = plan->enable_exchange != 0;
    demag = plan->enable_demag != 0;
    has_ext = plan->has_external_field != 0;
    has_uni = plan->has_uniaxial_anisotropy != 0;
    has_cub = plan->has_cubic_anisotropy != 0;
    for (int c = 0; c < 3; ++c) hext[c] = has_ext ? plan->external_field_am[c] : 0.0;
    max_error = plan->adaptive_max_error > 0 ? plan->adaptive_max_error : 1e-5;
    dt_min = plan->adaptive_dt_min > 0 ? plan->adaptive_dt_min : 1e-18;
    dt_max = plan->adaptive_dt_max > 0 ? plan->adaptive_dt_max : 1e-10;
    headroom = plan->adaptive_headroom > 0 ? plan->adaptive_headroom : 0.8;

    // ---- validation (reference api.cpp:324-395) ----
    if (g.n == 0) {
        last_error = "grid has zero cells";
        return false;
    }
    if (plan->initial_magnetization_xyz == nullptr || plan->initial_magnetization_len != 3 * (uint64_t)g.n) {
        last_error = "initial_magnetization_len mismatch: expected " + std::to_string(3 * (uint64_t)g.n) + ", got " +
                     std::to_string(plan->initial_magnetization_len);
        return false;
    }
    if (plan->region_mask && plan->region_mask_len != (uint64_t)g.n) {
        last_error = "region_mask_len mismatch: expected " + std::to_string(g.n) + ", got " +
                     std::to_string(plan->region_mask_len);
        return false;
    }
    if (plan->region_mask) {  // ids index a 256-row table; larger ids have no row
        for (long long i = 0; i < g.n; ++i)
            if (plan->region_mask[i] >= FULLMAG_FDM_MAX_EXCHANGE_REGIONS) {
                last_error = "region_mask ids must be below " + std::to_string(FULLMAG_FDM_MAX_EXCHANGE_REGIONS);
                return false;
            }
    }
    if (plan->active_mask && plan->active_mask_len != (uint64_t)g.n) {
        last_error = "active_mask_len mismatch: expected " + std::to_string(g.n) + ", got " +
                     std::to_string(plan->active_mask_len);
        return false;
    }
    if (!(dx > 0 && dy > 0 && dz > 0)) {
        last_error = "cell sizes must be positive";
        return false;
    }
    if (!(ms > 0)) {
        last_error = "saturation_magnetisation must be positive";
        return false;
    }
    if (unsupported(*this, plan->precision == FULLMAG_FDM_PRECISION_DOUBLE, "double precision state (use SINGLE)") ||
        unsupported(*this, integrator != FULLMAG_FDM_INTEGRATOR_HEUN && integrator != FULLMAG_FDM_INTEGRATOR_RK4 &&
                               integrator != FULLMAG_FDM_INTEGRATOR_DP45 && integrator != FULLMAG_FDM_INTEGRATOR_RK23 &&
                               integrator != FULLMAG_FDM_INTEGRATOR_ABM3,
                    "integrators other than HEUN, RK4, DP45, RK23, ABM3") ||
        unsupported(*this, plan->boundary_correction != FULLMAG_FDM_BOUNDARY_NONE, "boundary correction tiers"))
        return false;

    if (plan->active_mask) {
        has_mask = true;
        mask_host.assign(plan->active_mask, plan->active_mask + g.n);
    }

    // ---- padded geometry ----
    // With caller spectra the padded grid is the reference's (2nx, 2ny, 2nz) or, for
    // nz == 1 and 2-D spectra, (2nx, 2ny).  When the engine builds the tensor itself
    // any extent p >= 2n - 1 keeps the circular convolution exact on the physical
    // cells, so awkward sizes are rounded up to 2,3,5,7-smooth FFT lengths.
    bool thin = false;
    use_gpu_newell = false;
    g.px = 2 * g.nx;
    g.py = 2 * g.ny;
    g.per = per_req;
    if (g.per) {
        // periodic axes (fdm_fft.rs:140-160): the extent is the cell count, unpadded; open
        // axes keep a padded extent >= 2n - 1; the tensor is always built here
        if ((g.per & 1) && (g.nx & 1)) {
            last_error = "a periodic x axis needs an even number of cells";
            return false;
        }
        if (demag && plan->demag_kernel_spectrum_len != 0) {
            last_error = "periodic boundaries: the backend builds the image-sum demag tensor, the plan must carry no spectra";
            return false;
        }
        thin = g.nz == 1;
        use_gpu_newell = demag;
        g.px = (g.per & 1) ? g.nx : pad_extent(2 * g.nx - 1, true);
        g.py = (g.per & 2) ? g.ny : pad_extent(2 * g.ny - 1, false);
    } else if (demag) {
        const uint64_t len3 = 2ull * (uint64_t)(2 * g.nx) * (2 * g.ny) * (2 * g.nz);
        const uint64_t len2 = 2ull * (uint64_t)(2 * g.nx) * (2 * g.ny);
        if (plan->demag_kernel_spectrum_len == 0) {
            use_gpu_newell = true;
            thin = g.nz == 1;
        } else {
            if (!plan->demag_kernel_xx_spectrum || !plan->demag_kernel_yy_spectrum || !plan->demag_kernel_zz_spectrum ||
                !plan->demag_kernel_xy_spectrum || !plan->demag_kernel_xz_spectrum || !plan->demag_kernel_yz_spectrum) {
                last_error = "demag kernel spectra pointers must all be present when demag_kernel_spectrum_len is set";
                return false;
            }
            if (g.nz == 1 && plan->demag_kernel_spectrum_len == len2) thin = true;
            else if (plan->demag_kernel_spectrum_len != len3) {
                last_error = "demag_kernel_spectrum_len mismatch: expected " + std::to_string(len3) + " (3D)" +
                             (g.nz == 1 ? " or " + std::to_string(len2) + " (thin-film 2D)" : std::string()) + ", got " +
                             std::to_string(plan->demag_kernel_spectrum_len);
                return false;
            }
            // the given spectra fix P = 2n; lengths with a prime factor the shared-memory
            // FFT does not handle are rebuilt on the GPU at smooth extents instead
            if (!smooth_enough(2 * g.nx) || !smooth_enough(2 * g.ny) || (!thin && !smooth_enough(2 * g.nz)))
                use_gpu_newell = true;
        }
        if (use_gpu_newell) {
            g.px = pad_extent(2 * g.nx - 1, true);
            g.py = pad_extent(2 * g.ny - 1, false);
        }
    }
    g.thin = thin ? 1 : 0;
    g.pz = thin ? 1 : (g.per & 4) ? g.nz : (use_gpu_newell ? pad_extent(2 * g.nz - 1, false) : 2 * g.nz);
    if (g.px < 2) g.px = 2;
    g.half = g.px / 2;
    g.nkx = g.half + 1;
    g.nky = g.py / 2 + 1;
    g.nkz = g.pz / 2 + 1;
    grid_dividers(g);
    early_launch = (integrator == FULLMAG_FDM_INTEGRATOR_HEUN || integrator == FULLMAG_FDM_INTEGRATOR_RK4) && g.n <= 65536;

    // ---- material constants ----
    const double mu0ms = kMu0 * ms;
    mat.ex_pref = exchange ? (float)(2.0 * a_ex / mu0ms) : 0.f;
    mat.idx2 = (float)(1.0 / (dx * dx));
    mat.idy2 = (float)(1.0 / (dy * dy));
    mat.idz2 = (float)(1.0 / (dz * dz));
    mat.has_ext = has_ext;
    for (int c = 0; c < 3; ++c) mat.hext[c] = (float)hext[c];
    auto unit = [](const double *v, double *o) {
        double nn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (nn < 1e-30) nn = 1e-30;
        for (int c = 0; c < 3; ++c) o[c] = v[c] / nn;
    };
    mat.has_uni = has_uni;
    if (has_uni) {
        double u[3];
        unit(plan->anisotropy_axis, u);
        for (int c = 0; c < 3; ++c) mat.u[c] = (float)u[c];
        mat.ku1c = (float)(2.0 * plan->uniaxial_anisotropy_constant / mu0ms);
        mat.ku2c = (float)(4.0 * plan->uniaxial_anisotropy_k2 / mu0ms);
        mat.ku1f = (float)plan->uniaxial_anisotropy_constant;
        mat.ku2f = (float)plan->uniaxial_anisotropy_k2;
    }
    mat.has_cub = has_cub;
    if (has_cub) {
        double c1[3], c2[3];
        unit(plan->cubic_axis1, c1);
        unit(plan->cubic_axis2, c2);
        const double c3[3] = {c1[1] * c2[2] - c1[2] * c2[1], c1[2] * c2[0] - c1[0] * c2[2], c1[0] * c2[1] - c1[1] * c2[0]};
        for (int c = 0; c < 3; ++c) {
            mat.c1[c] = (float)c1[c];
            mat.c2[c] = (float)c2[c];
            mat.c3[c] = (float)c3[c];
        }
        mat.kc1c = (float)(-2.0 * plan->cubic_Kc1 / mu0ms);
        mat.kc2c = (float)(-2.0 * plan->cubic_Kc2 / mu0ms);
        mat.kc3c = (float)(-4.0 * plan->cubic_Kc3 / mu0ms);
        mat.kc1f = (float)plan->cubic_Kc1;
        mat.kc2f = (float)plan->cubic_Kc2;
        mat.kc3f = (float)plan->cubic_Kc3;
    }
    mat.gbar = (float)(gamma / (1.0 + alpha * alpha));
    mat.alpha = (float)alpha;
    mat.prec = plan->disable_precession ? 0.f : 1.f;

    // DMI and magnetoelastic terms (api.cpp plan mapping; demag_fp32.cu:319-376,582-583)
    xf = ExtraField{};
    xf.early = early_launch ? 1 : 0;
    xf.has_int = plan->has_interfacial_dmi ? 1 : 0;
    xf.has_bulk = plan->has_bulk_dmi ? 1 : 0;
    xf.has_mel = plan->has_magnetoelastic ? 1 : 0;
    xf.has_ext = has_ext ? 1 : 0;
    for (int c = 0; c < 3; ++c) xf.hext[c] = (float)hext[c];
    xf.d_int = plan->dmi_D_interfacial;
    xf.d_bulk = plan->dmi_D_bulk;
    xf.dmi_int = (float)(2.0 * plan->dmi_D_interfacial / mu0ms);
    xf.dmi_bulk = (float)(2.0 * plan->dmi_D_bulk / mu0ms);
    xf.inv2dx = (float)(0.5 / dx);
    xf.inv2dy = (float)(0.5 / dy);
    xf.inv2dz = (float)(0.5 / dz);
    xf.mel_pref = (float)(-1.0 / mu0ms);
    xf.b1 = (float)plan->mel_b1;
    xf.b2 = (float)plan->mel_b2;
    xf.e11 = (float)plan->mel_strain[0];
    xf.e22 = (float)plan->mel_strain[1];
    xf.e33 = (float)plan->mel_strain[2];
    xf.e23 = (float)(0.5 * plan->mel_strain[3]);  // Voigt 2 e23 -> e23
    xf.e13 = (float)(0.5 * plan->mel_strain[4]);
    xf.e12 = (float)(0.5 * plan->mel_strain[5]);
    // spin torques (prefactors as api.cpp:250-300 and context.hpp:321-339 compute them)
    {
        const double MU_B = 9.274009994e-24, E_CH = 1.60217662e-19, HBAR = 1.054571817e-34;
        const double j[3] = {plan->current_density_x, plan->current_density_y, plan->current_density_z};
        const bool has_j = j[0] != 0.0 || j[1] != 0.0 || j[2] != 0.0;
        xf.has_zl = has_j && plan->stt_degree > 0.0 && ms > 0.0;
        if (xf.has_zl) {
            const double b = plan->stt_degree * MU_B / (E_CH * ms * (1.0 + plan->stt_beta * plan->stt_beta));
            for (int c = 0; c < 3; ++c) xf.zl_u[c] = (float)(b * j[c]);
            xf.zl_beta = (float)plan->stt_beta;
        }
        xf.inv_dx = (float)(1.0 / dx);
        xf.inv_dy = (float)(1.0 / dy);
        xf.inv_dz = (float)(1.0 / dz);
        const double p2 = plan->stt_p_x * plan->stt_p_x + plan->stt_p_y * plan->stt_p_y + plan->stt_p_z * plan->stt_p_z;
        xf.has_slon = p2 > 0.0 && plan->stt_lambda > 0.0 && has_j && ms > 0.0 && dz > 0.0;
        if (xf.has_slon) {
            const double js = sqrt(j[0] * j[0] + j[1] * j[1] + j[2] * j[2]);
            xf.slon_pf = (float)(js * HBAR / (2.0 * E_CH * kMu0 * ms * dz));
            xf.slon_P = (float)(plan->stt_degree > 0.0 ? plan->stt_degree : 1.0);
            xf.slon_l2 = (float)(plan->stt_lambda * plan->stt_lambda);
            xf.slon_eps = (float)plan->stt_epsilon_prime;
            xf.slon_p[0] = (float)plan->stt_p_x;
            xf.slon_p[1] = (float)plan->stt_p_y;
            xf.slon_p[2] = (float)plan->stt_p_z;
        }
        xf.has_sot = plan->has_sot != 0 && ms > 0.0;
        if (xf.has_sot) {
            const double t = plan->sot_thickness > 0.0 ? plan->sot_thickness : 1.0e-9;
            const double *sg = plan->sot_sigma;
            const double len = sqrt(sg[0] * sg[0] + sg[1] * sg[1] + sg[2] * sg[2]);
            const double inv = len > 1e-30 ? 1.0 / len : 0.0;
            for (int c = 0; c < 3; ++c) xf.sot_s[c] = (float)(sg[c] * inv);
            xf.sot_amp = (float)(std::fabs(plan->sot_je) * HBAR / (2.0 * E_CH * kMu0 * ms * t));
            xf.sot_xi_dl = (float)plan->sot_xi_dl;
            xf.sot_xi_fl = (float)plan->sot_xi_fl;
        }
        has_torque = xf.has_zl || xf.has_slon || xf.has_sot;
        const double s = plan->disable_precession ? 0.0 : 1.0, gb = gamma / (1.0 + alpha * alpha);
        if (has_torque && s + alpha * alpha <= 0.0) {
            last_error = "spin torques need precession or damping (disable_precession with alpha = 0)";
            return false;
        }
        if (has_torque) {
            xf.tq_a = (float)(alpha / (gb * (s + alpha * alpha)));
            xf.tq_b = (float)(s / (gb * (s + alpha * alpha)));
        }
    }
    // per-cell anisotropy maps: the uniaxial and cubic terms move to the extra pass
    {
        const bool uni_map = has_uni && (plan->ku1_field || plan->ku2_field);
        const bool cub_map = has_cub && (plan->kc1_field || plan->kc2_field || plan->kc3_field);
        xf.aniso = (uni_map || cub_map) && ms > 0.0;
        if (xf.aniso) {
            xf.has_uni = has_uni;
            xf.has_cub = has_cub;
            xf.ku1 = mat.ku1f;
            xf.ku2 = mat.ku2f;
            xf.kc1 = mat.kc1f;
            xf.kc2 = mat.kc2f;
            xf.kc3 = mat.kc3f;
            xf.inv_mu0ms = (float)(1.0 / mu0ms);
            for (int c = 0; c < 3; ++c) {
                xf.u[c] = mat.u[c];
                xf.c1[c] = mat.c1[c];
                xf.c2[c] = mat.c2[c];
                xf.c3[c] = mat.c3[c];
            }
            mat.has_uni = 0;  // the row pass leaves them to the extra pass
            mat.has_cub = 0;
        }
    }
    has_oersted = plan->has_oersted_cylinder != 0;
    if (has_oersted) {
        if (!(plan->oersted_radius > 0.0)) {
            last_error = "oersted_radius must be positive";
            return false;
        }
        oe_kind = (int)plan->oersted_time_dep_kind;
        oe_current = plan->oersted_current;
        oe_freq = plan->oersted_time_dep_freq;
        oe_phase = plan->oersted_time_dep_phase;
        oe_offset = plan->oersted_time_dep_offset;
        oe_t_on = plan->oersted_time_dep_t_on;
        oe_t_off = plan->oersted_time_dep_t_off;
    }
    // exchange with region ids (exchange_fp32.cu:48-104) moves whole to the extra pass
    const bool region_exchange = plan->region_mask && exchange && ms > 0.0;
    if (region_exchange) {
        xf.ex_s = (float)(2.0 / mu0ms);
        xf.idx2 = mat.idx2;
        xf.idy2 = mat.idy2;
        xf.idz2 = mat.idz2;
        mat.ex_pref = 0.f;
    }
    // thermal field: sigma^2 = 2 alpha kB T / (gamma (1 + alpha^2) mu0 Ms V dt)
    // (crates/fullmag-engine/src/fdm_fields.rs:836-842; no noise without damping)
    has_thermal = plan->temperature > 0.0 && ms > 0.0 && alpha > 0.0;
    if (has_thermal)
        th_pref = 2.0 * alpha * 1.380649e-23 * plan->temperature /
                  (gamma * (1.0 + alpha * alpha) * 1.2566370614359173e-6 * ms * dx * dy * dz);
    has_extra = (ms > 0.0 && (xf.has_int || xf.has_bulk || xf.has_mel || has_torque || xf.aniso)) || has_oersted ||
                region_exchange || has_thermal;

    // ---- device and stream ----
    if (cuda_fail("cudaGetDevice", cudaGetDevice(&device))) return false;
    if (cuda_fail("cudaStreamCreate", cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking))) return false;

    // ---- FFT plans ----
    std::vector<float2> tw;
    std::vector<size_t> offs;
    if (demag) {
        if (!make_plan(plan_x, g.half, tw, offs) || !make_plan(plan_y, g.py, tw, offs) || !make_plan(plan_z, g.pz, tw, offs))
            return false;
    }
    const size_t xpost_off = tw.size();
    for (int k = 0; k <= g.half; ++k) {
        const double ang = 2.0 * M_PI * (double)k / (double)g.px;
        tw.push_back(make_float2((float)cos(ang), (float)-sin(ang)));
    }

    // ---- arena ----
    // stage derivatives: DP45 k1..k7, RK23 k1..k4, RK4 k1..k3 (k4 stays in registers),
    // ABM3 k1 + three history entries + f at the prediction, Heun k1
    switch (integrator) {
        case FULLMAG_FDM_INTEGRATOR_DP45: nk = 7; break;
        case FULLMAG_FDM_INTEGRATOR_ABM3: nk = 5; break;
        case FULLMAG_FDM_INTEGRATOR_RK23: nk = 4; break;
        case FULLMAG_FDM_INTEGRATOR_RK4: nk = 3; break;
        default: nk = 1; break;
    }
    const char *rr_env = std::getenv("FULLMAG_FDM_ROWS_PER_CTA");
    row_rows = rr_env ? std::max(1, std::atoi(rr_env)) : std::max(1, std::min(16, 512 / std::max(1, g.nx)));
    max_row_blocks = g.ny * g.nz;  // statistics partials sized for one row per CTA
    row_blocks = (g.ny * g.nz + row_rows - 1) / row_rows;
    tx_yf = tx_yi = col_tile(g, 1, g.py);
    tx_z = col_tile(g, 6, g.pz);
    tx_2d = col_tile(g, 3, g.py);
    {
        const char *no_yz = std::getenv("FULLMAG_FDM_NO_FUSED_YZ");
        use_yz = demag && !thin && !g.per && !(no_yz && *no_yz && *no_yz != '0') && yz_convolve_smem(g, 1) <= 200u * 1024u;
        if (use_yz) {
            tx_z = 1;
            while (tx_z < 8 && yz_convolve_smem(g, 2 * tx_z) <= 200u * 1024u) tx_z *= 2;
        }
    }
    const size_t vec = sizeof(float) * 3 * (size_t)g.n;
    const size_t xlen = demag ? sizeof(float2) * 3 * (size_t)g.nz * g.ny * g.nkx : 0;
    const size_t ylen = (demag && !thin && !use_yz) ? sizeof(float2) * 3 * (size_t)g.nz * g.py * g.nkx : 0;
    const size_t klen = !demag ? 0
                        : g.per ? sizeof(float2) * (thin ? 4 : 6) * (size_t)g.pz * g.py * g.nkx
                                : sizeof(float) * (thin ? 4 : 6) * (size_t)g.nkz * g.nky * g.nkx;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t off = 0;
    std::vector<size_t> o;
    auto take = [&](size_t b) {
        o.push_back(off);
        off += al(b);
    };
    take(vec); take(vec); take(vec); take(vec);            // S0 S1 A0 A1
    for (int i = 0; i < nk; ++i) take(vec);                 // K
    take(vec); take(vec); take(vec);                        // observables
    take(xlen); take(ylen); take(klen);                     // spectra + kernel
    take(has_mask ? (size_t)g.n : 0);                       // mask
    take(sizeof(float2) * kNumStats * (size_t)max_row_blocks);
    take(sizeof(double) * kStatSlots);
    take(sizeof(float2) * tw.size());
    arena_bytes = off;
    if (cuda_fail("cudaMalloc(arena)", cudaMalloc((void **)&arena, arena_bytes))) return false;
    if (cuda_fail("cudaMemset(arena)", cudaMemsetAsync(arena, 0, arena_bytes, stream))) return false;
    int q = 0;
    S[0] = (float *)(arena + o[q++]);
    S[1] = (float *)(arena + o[q++]);
    A[0] = (float *)(arena + o[q++]);
    A[1] = (float *)(arena + o[q++]);
    for (int i = 0; i < nk; ++i) K[i] = (float *)(arena + o[q++]);
    h_ex = (float *)(arena + o[q++]);
    h_d = (float *)(arena + o[q++]);
    h_eff = (float *)(arena + o[q++]);
    X = demag ? (float2 *)(arena + o[q]) : nullptr;
    q++;
    Y = ylen ? (float2 *)(arena + o[q]) : nullptr;
    q++;
    kern = demag ? (float *)(arena + o[q]) : nullptr;
    q++;
    mask = has_mask ? (uint8_t *)(arena + o[q]) : nullptr;
    q++;
    partials = (float2 *)(arena + o[q++]);
    dstats = (double *)(arena + o[q++]);
    twid = (float2 *)(arena + o[q++]);
    if (cuda_fail("cudaMallocHost(stats)", cudaMallocHost((void **)&hstats, sizeof(double) * kStatSlots))) return false;
    if (has_extra &&
        (cuda_fail("cudaMalloc(extra field)", cudaMalloc((void **)&hextra, sizeof(float) * 3 * (size_t)g.n)) ||
         cuda_fail("cudaMalloc(extra sums)", cudaMalloc((void **)&xpart, sizeof(ExtraSums) * (size_t)extra_field_blocks(g)))))
        return false;
    if (xf.aniso) {  // per-cell anisotropy constants, FP32 on the device
        const double *src[5] = {plan->ku1_field, plan->ku2_field, plan->kc1_field, plan->kc2_field, plan->kc3_field};
        std::vector<float> tmp((size_t)g.n);
        for (int k = 0; k < 5; ++k) {
            if (!src[k]) continue;
            for (long long i = 0; i < g.n; ++i) tmp[i] = (float)src[k][i];
            if (cuda_fail("cudaMalloc(anisotropy map)", cudaMalloc((void **)&kmaps[k], sizeof(float) * (size_t)g.n)) ||
                cuda_fail("anisotropy map upload",
                          cudaMemcpy(kmaps[k], tmp.data(), sizeof(float) * (size_t)g.n, cudaMemcpyHostToDevice)))
                return false;
        }
        xf.ku1m = kmaps[0];
        xf.ku2m = kmaps[1];
        xf.kc1m = kmaps[2];
        xf.kc2m = kmaps[3];
        xf.kc3m = kmaps[4];
    }
    if (has_thermal && cuda_fail("cudaMalloc(thermal keys)", cudaMalloc((void **)&th_dev, 2 * sizeof(ThermalSlot))))
        return false;
    if (region_exchange) {
        // the caller's table when it has 256 x 256 entries, else A on the diagonal
        // (api.cpp:405-420)
        // (api.cpp:405-420), held as FP32 as the reference's field kernel reads it
        constexpr size_t R = FULLMAG_FDM_MAX_EXCHANGE_REGIONS;
        std::vector<float> table(R * R, 0.f);
        if (plan->exchange_lut && plan->exchange_lut_len == R * R)
            for (size_t k = 0; k < R * R; ++k) table[k] = (float)plan->exchange_lut[k];
        else
            for (size_t r = 0; r < R; ++r) table[r * R + r] = (float)a_ex;
        std::vector<uint8_t> ids((size_t)g.n);  // validated below 256 at the top of setup
        for (long long i = 0; i < g.n; ++i) ids[i] = (uint8_t)plan->region_mask[i];
        if (cuda_fail("cudaMalloc(region ids)", cudaMalloc((void **)&regions, (size_t)g.n)) ||
            cuda_fail("cudaMalloc(exchange table)", cudaMalloc((void **)&lut, sizeof(float) * R * R)) ||
            cuda_fail("region ids upload",
                      cudaMemcpy(regions, ids.data(), (size_t)g.n, cudaMemcpyHostToDevice)) ||
            cuda_fail("exchange table upload", cudaMemcpy(lut, table.data(), sizeof(float) * R * R, cudaMemcpyHostToDevice)))
            return false;
        xf.region = regions;
        xf.lut = lut;
    }
    if (has_oersted) {
        // field of a z-directed cylinder through (cx, cy) for I = 1 A at the cell centres:
        // H_phi = r / (2 pi R^2) inside, 1 / (2 pi r) outside, zero on the axis
        const double R = plan->oersted_radius, cx = plan->oersted_center[0], cy = plan->oersted_center[1];
        std::vector<float> f(3 * (size_t)g.n, 0.f);
        for (long long i = 0; i < g.n; ++i) {
            const long long ix = i % g.nx, iy = (i / g.nx) % g.ny;
            const double ddx = (ix + 0.5) * dx - cx, ddy = (iy + 0.5) * dy - cy;
            const double r = sqrt(ddx * ddx + ddy * ddy);
            if (r < 1e-30) continue;
            const double hphi = r < R ? r / (2.0 * M_PI * R * R) : 1.0 / (2.0 * M_PI * r);
            f[i] = (float)(-hphi * ddy / r);
            f[g.n + i] = (float)(hphi * ddx / r);
        }
        if (cuda_fail("cudaMalloc(Oersted field)", cudaMalloc((void **)&h_oe, sizeof(float) * f.size())) ||
            cuda_fail("cudaMalloc(Oersted current)", cudaMalloc((void **)&oe_dev, 2 * sizeof(float))) ||
            cuda_fail("Oersted field upload", cudaMemcpy(h_oe, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice)))
            return false;
    }
    if (cuda_fail("cudaMallocHost(dt)", cudaMallocHost((void **)&dt_host, sizeof(double)))) return false;
    dt_dev = dstats + kNumStats;  // slot kNumStats holds dt (kStatSlots)

    if (cuda_fail("cudaMemcpy(twiddles)", cudaMemcpyAsync(twid, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice, stream)))
        return false;
    if (demag) {
        plan_x.tw = twid + offs[0];
        plan_y.tw = twid + offs[1];
        plan_z.tw = twid + offs[2];
    }
    xpost = twid + xpost_off;
    if (has_mask && cuda_fail("cudaMemcpy(mask)", cudaMemcpyAsync(mask, mask_host.data(), (size_t)g.n, cudaMemcpyHostToDevice, stream)))
        return false;
    if (demag) {
        if (g.per) {
            std::string err;
            if (!newell_periodic_spectrum_gpu(g, dx, dy, dz, ms, images, reinterpret_cast<float2 *>(kern), nullptr, stream, err)) {
                last_error = err;
                return false;
            }
        } else if (use_gpu_newell) {
            std::string err;
            if (!newell_spectrum_gpu(g, dx, dy, dz, ms, kern, stream, err)) {
                last_error = err;
                return false;
            }
        } else if (!upload_spectra(plan, thin)) {
            return false;
        }
        if (use_yz) {  // the fused y+z passes read the kernel ky-fastest
            float *tmp = nullptr;
            if (cuda_fail("cudaMalloc(kernel transpose)", cudaMalloc((void **)&tmp, klen))) return false;
            const bool ok = !cuda_fail("kernel transpose", launch_kern_ky_fast(kern, tmp, 6, g.nkz, g.nky, g.nkx, stream)) &&
                            !cuda_fail("kernel transpose copy", cudaMemcpyAsync(kern, tmp, klen, cudaMemcpyDeviceToDevice, stream)) &&
                            !cuda_fail("kernel transpose sync", cudaStreamSynchronize(stream));
            cudaFree(tmp);
            if (!ok) return false;
        }
    }
    if (cuda_fail("setup sync", cudaStreamSynchronize(stream))) return false;
    const char *no_tune = std::getenv("FULLMAG_FDM_NO_TUNE");
    if (!(no_tune && *no_tune && *no_tune != '0') && !autotune()) return false;
    return true;
}

namespace {
struct TuneKey {
    int nx, ny, nz, px, py, pz, thin, masked, per;
    bool operator<(const TuneKey &o) const {
        return std::tie(nx, ny, nz, px, py, pz, thin, masked, per) <
               std::tie(o.nx, o.ny, o.nz, o.px, o.py, o.pz, o.thin, o.masked, o.per);
    }
};
struct TuneChoice {
    int tx_yf, tx_z, tx_yi, tx_2d, rows, z_pair, split_yf, split_z, split_yi;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneChoice> g_tune_cache;
}  // namespace

// Picks the kx tile width of each column pass and the rows per CTA of the row pass
// by timing the candidates (3 launches each, CUDA events on the engine stream) on
// the live, still-unused buffers.  Results are cached per grid shape in the process,
// so batched problems of the same shape pay for the search once.
bool Engine::autotune() {
    const TuneKey key{g.nx, g.ny, g.nz, g.px, g.py, g.pz, g.thin, has_mask ? 1 : 0, g.per};
    // FULLMAG_FDM_TUNE="rows,tx_yf,tx_z,tx_yi,tx_2d,z_pair,split_yf,split_z,split_yi" fixes every
    // choice (the values fullmag_fdm_backend_tuning reports), e.g. so that a profiler run uses
    // the launch shapes of an unprofiled one
    if (const char *fix = std::getenv("FULLMAG_FDM_TUNE")) {
        int v[9];
        if (std::sscanf(fix, "%d,%d,%d,%d,%d,%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6], &v[7], &v[8]) == 9) {
            row_rows = std::max(1, v[0]);
            tx_yf = std::max(1, v[1]);
            tx_z = std::max(1, v[2]);
            tx_yi = std::max(1, v[3]);
            tx_2d = std::max(1, v[4]);
            z_pair = v[5] && z_convolve_pair_ok(g, tx_z) ? 1 : 0;
            split_yf = v[6] != 0;
            split_z = v[7] != 0;
            split_yi = v[8] != 0;
            row_blocks = (g.ny * g.nz + row_rows - 1) / row_rows;
            return true;
        }
    }
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            tx_yf = it->second.tx_yf;
            tx_z = it->second.tx_z;
            tx_yi = it->second.tx_yi;
            tx_2d = it->second.tx_2d;
            z_pair = it->second.z_pair;
            split_yf = it->second.split_yf;
            split_z = it->second.split_z;
            split_yi = it->second.split_yi;
            if (!std::getenv("FULLMAG_FDM_ROWS_PER_CTA")) row_rows = it->second.rows;
            row_blocks = (g.ny * g.nz + row_rows - 1) / row_rows;
            return true;
        }
    }
    // The fastest tile of one pass timed alone; with early launch (small fixed-step
    // problems) the widest tile within 5 % of it: fewer CTAs of the next kernel are then
    // resident and waiting beside the current one (measured on 256x64x1 RK4: 0.0645 ms/step
    // with 65 thin-film CTAs against 0.0755 with 129, which timed alike on their own).
    auto pick_tile = [&](const std::vector<std::pair<int, float>> &cand, int cur) {
        if (cand.empty()) return cur;
        float bt = 1e30f;
        int best = cur;
        for (const auto &c : cand)
            if (c.second < bt) {
                bt = c.second;
                best = c.first;
            }
        if (early_launch)
            for (const auto &c : cand)
                if (c.second <= 1.05f * bt && c.first > best) best = c.first;
        return best;
    };
    if (demag) {
        if (g.thin) {
            std::vector<std::pair<int, float>> cand;
            for (int tx : {1, 2, 4, 8, 16}) {
                if (tx > std::max(1, g.nkx) || y_convolve_2d_smem(g, tx) > 200u * 1024u) continue;
                cand.emplace_back(tx, time_ms([&] { return launch_y_convolve_2d(col_pass(plan_y, tx, X, X), stream) == cudaSuccess; }));
            }
            tx_2d = pick_tile(cand, tx_2d);
        } else if (use_yz) {
            std::vector<std::pair<int, float>> cand;
            for (int tx : {1, 2, 4, 8}) {
                if (tx > std::max(1, g.nkx) || yz_convolve_smem(g, tx) > 200u * 1024u) continue;
                cand.emplace_back(tx, time_ms([&] { return launch_yz_convolve(col_pass(plan_y, tx, X, X), stream) == cudaSuccess; }));
            }
            tx_z = pick_tile(cand, tx_z);
        } else {
            // tile widths and radix splits of the three column passes, each timed on its own
            // (power-of-two lengths 16..256 have a second split N1 x N2)
            auto two_splits = [](int len) { return len >= 16 && len <= 256 && (len & (len - 1)) == 0; };
            auto tune = [&](int cur_tx, int &split, bool alt, const std::function<size_t(int)> &smem,
                            const std::function<bool(int, int)> &run) {
                int best = cur_tx, best_split = 0;
                float bt = 1e30f;
                for (int sp = 0; sp < (alt ? 2 : 1); ++sp)
                    for (int tx : {1, 2, 4, 8, 16}) {
                        if (tx > std::max(1, g.nkx) || smem(tx) > 200u * 1024u) continue;
                        const float t = time_ms([&] { return run(tx, sp); });
                        if (t < bt) {
                            bt = t;
                            best = tx;
                            best_split = sp;
                        }
                    }
                split = best_split;
                return best;
            };
            auto ysm = [&](int tx) { return y_pass_smem(g, tx); };
            auto cp = [&](const FftPlan &pl, int tx, int sp, const float2 *in, float2 *out) {
                ColPass c = col_pass(pl, tx, in, out);
                c.split = sp;
                return c;
            };
            tx_yf = tune(tx_yf, split_yf, two_splits(g.py), ysm,
                         [&](int tx, int sp) { return launch_y_forward(cp(plan_y, tx, sp, X, Y), stream) == cudaSuccess; });
            tx_z = tune(tx_z, split_z, two_splits(g.pz), [&](int tx) { return z_convolve_smem(g, tx); },
                        [&](int tx, int sp) { return launch_z_convolve(cp(plan_z, tx, sp, Y, Y), stream) == cudaSuccess; });
            // the packed ky-pair z pass (tile 8) against the best unpaired launch;
            // FULLMAG_FDM_Z_PAIR=0 or 1 forces the choice
            z_pair = 0;
            const char *zp_env = std::getenv("FULLMAG_FDM_Z_PAIR");
            if (z_convolve_pair_ok(g, 8) && zp_env && zp_env[0] == '1') {
                tx_z = 8;
                z_pair = 1;
                split_z = 0;
            } else if (z_convolve_pair_ok(g, 8) && !(zp_env && zp_env[0] == '0')) {
                ColPass best = cp(plan_z, tx_z, split_z, Y, Y), paired = col_pass(plan_z, 8, Y, Y);
                paired.pipe = 1;
                const float t_best = time_ms([&] { return launch_z_convolve(best, stream) == cudaSuccess; });
                const float t_pair = time_ms([&] { return launch_z_convolve(paired, stream) == cudaSuccess; });
                if (t_pair < t_best) {
                    tx_z = 8;
                    z_pair = 1;
                    split_z = 0;
                }
            }
            tx_yi = tune(tx_yi, split_yi, two_splits(g.py), ysm,
                         [&](int tx, int sp) { return launch_y_inverse(cp(plan_y, tx, sp, Y, X), stream) == cudaSuccess; });
        }
    }
    if (!std::getenv("FULLMAG_FDM_ROWS_PER_CTA")) {
        // a full stage pass: inverse x, fields, statistics, combination, forward x
        int best = row_rows;
        float bt = 1e30f;
        const int nrows = g.ny * g.nz;
        for (int rows : {1, 2, 4, 8, 16}) {
            if (rows > nrows || rows * g.nx > 8192) continue;
            RowPass p = row_base();
            p.rows = rows;
            p.x_in = demag ? X : nullptr;
            p.m_in = S[0];
            p.k_out = K[0];
            p.partials = partials;
            p.m0 = S[1];
            p.m_next = A[0];
            p.n_comb = 1;
            p.comb_k[0] = nullptr;
            p.comb_c[0] = 0.f;
            p.x_out = demag ? X : nullptr;
            if (row_pass_smem(p) > 200u * 1024u) continue;
            const float t = time_ms([&] { return launch_row_pass(p, stream) == cudaSuccess; });
            if (t < bt) {
                bt = t;
                best = rows;
            }
        }
        row_rows = best;
    }
    row_blocks = (g.ny * g.nz + row_rows - 1) / row_rows;
    // the timed launches only wrote scratch (X, Y, A[0], K[0], partials); every one of
    // those is rewritten before it is read again
    if (cuda_fail("autotune sync", cudaStreamSynchronize(stream))) return false;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = TuneChoice{tx_yf, tx_z, tx_yi, tx_2d, row_rows, z_pair, split_yf, split_z, split_yi};
    return true;
}

// Real, octant-unique part of the given FP64 spectra, scaled by Ms/P (the
// FFT normalisation and M = Ms m folded into the kernel), converted to FP32.
bool Engine::upload_spectra(const fullmag_fdm_plan_desc *plan, bool thin) {
    const double *src[6] = {plan->demag_kernel_xx_spectrum, plan->demag_kernel_yy_spectrum, plan->demag_kernel_zz_spectrum,
                            plan->demag_kernel_xy_spectrum, plan->demag_kernel_xz_spectrum, plan->demag_kernel_yz_spectrum};
    const int ncomp = thin ? 4 : 6;
    const double P = (double)g.px * g.py * (thin ? 1 : g.pz);
    const double scale = ms / P;
    const size_t per = (size_t)g.nkz * g.nky * g.nkx;
    std::vector<float> h((size_t)ncomp * per);
    for (int c = 0; c < ncomp; ++c)
        for (int kz = 0; kz < g.nkz; ++kz)
            for (int ky = 0; ky < g.nky; ++ky)
                for (int kx = 0; kx < g.nkx; ++kx) {
                    const size_t s = (size_t)kx + (size_t)g.px * (ky + (size_t)g.py * kz);
                    h[(size_t)c * per + ((size_t)kz * g.nky + ky) * g.nkx + kx] = (float)(src[c][2 * s] * scale);
                }
    if (cuda_fail("cudaMemcpy(kernel)", cudaMemcpyAsync(kern, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice, stream)))
        return false;
    return !cuda_fail("kernel sync", cudaStreamSynchronize(stream));
}

}  // namespace fm

// =====================================================================
// C ABI
// =====================================================================

using namespace fm;

static Engine *eng(fullmag_fdm_backend *h) { return reinterpret_cast<Engine *>(h); }

// copy of an observable of a double-precision handle (AoS doubles, or floats converted on the host)
template <typename T>
static int f64_copy(Engine *e, int observable, T *out, uint64_t out_len) {
    int nx, ny, nz;
    fp64_grid(e->f64, nx, ny, nz);
    const uint64_t n = (uint64_t)nx * ny * nz;
    if (out_len != 3 * n) {
        e->last_error = "out_len mismatch";
        return FULLMAG_FDM_ERR_INVALID;
    }
    if (observable < FULLMAG_FDM_OBSERVABLE_M || observable > FULLMAG_FDM_OBSERVABLE_H_EFF) {
        e->last_error = "unknown observable";
        return FULLMAG_FDM_ERR_INVALID;
    }
    std::vector<double> tmp;
    double *dst = reinterpret_cast<double *>(out);
    if (sizeof(T) != sizeof(double)) {
        tmp.resize(3 * n);
        dst = tmp.data();
    }
    std::string err;
    if (!fp64_download(e->f64, observable, dst, err)) {
        e->last_error = err;
        return FULLMAG_FDM_ERR_CUDA;
    }
    if (sizeof(T) != sizeof(double))
        for (uint64_t i = 0; i < 3 * n; ++i) out[i] = (T)tmp[i];
    return FULLMAG_FDM_OK;
}


static int device_from_env() {
    const char *a = std::getenv("FULLMAG_FDM_GPU_INDEX");
    const char *b = std::getenv("FULLMAG_CUDA_DEVICE_INDEX");
    const char *raw = a ? a : b;
    if (!raw || !*raw) return -1;
    char *end = nullptr;
    long v = std::strtol(raw, &end, 10);
    if (end == raw || *end != '\0' || v < 0) return -1;
    return (int)v;
}

template <typename T>
static int preview_impl(fullmag_fdm_backend *handle, fullmag_fdm_observable obs, uint32_t pnx, uint32_t pny, uint32_t pnz,
                        uint32_t z0, uint32_t zs, T *out, uint64_t out_len) {
    Engine *e = eng(handle);
    if (!e || !out || pnx == 0 || pny == 0 || pnz == 0 || zs == 0 || (!e->arena && !e->f64)) return FULLMAG_FDM_ERR_INVALID;
    if (out_len != (uint64_t)pnx * pny * pnz * 3) {
        e->last_error = "preview out_len mismatch";
        return FULLMAG_FDM_ERR_INVALID;
    }
    if (e->f64) {  // the box average of the FP64 field, on the host
        int nx, ny, nz;
        fp64_grid(e->f64, nx, ny, nz);
        if (z0 >= (uint32_t)nz) {
            e->last_error = "preview z_origin out of range";
            return FULLMAG_FDM_ERR_INVALID;
        }
        std::vector<double> full(3 * (size_t)nx * ny * nz);
        const int rc = f64_copy<double>(e, obs, full.data(), full.size());
        if (rc != FULLMAG_FDM_OK) return rc;
        host_preview<T>(full.data(), nx, ny, nz, pnx, pny, pnz, z0, zs, out);
        return FULLMAG_FDM_OK;
    }
    return e->preview<T>(obs, pnx, pny, pnz, z0, zs, out) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
}

// Snapshots (context.cu:1073-1745 semantics): begin captures the observable as it is at
// that moment (component-major SoA for field snapshots, AoS for previews) into memory
// owned by the snapshot, without waiting for the device-to-host copy; wait blocks on the
// copy only, never touches the backend and may run on another thread.
static int snap_wait(SnapshotPayload *s, const void **out_data, uint64_t *out_len, fullmag_fdm_snapshot_desc *out_desc) {
    if (!s || !out_data || !out_len || !out_desc) return FULLMAG_FDM_ERR_INVALID;
    if (!s->ok) return FULLMAG_FDM_ERR_CUDA;
    if (s->done && cudaEventSynchronize(s->done) != cudaSuccess) return FULLMAG_FDM_ERR_CUDA;
    *out_data = s->pinned ? s->pinned : (const void *)s->bytes.data();
    *out_len = s->pinned ? s->len : s->bytes.size();
    *out_desc = s->desc;
    return FULLMAG_FDM_OK;
}

extern "C" {

int fullmag_fdm_is_available(void) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) return 0;
    const int sel = device_from_env();
    if (sel >= 0 && sel >= count) return 0;
    return 1;
}

fullmag_fdm_backend *fullmag_fdm_backend_create(const fullmag_fdm_plan_desc *plan) {
    if (!plan) return nullptr;
    Engine *e = new (std::nothrow) Engine();
    if (!e) return nullptr;
    const int sel = device_from_env();
    if (sel >= 0) {
        cudaError_t err = cudaSetDevice(sel);
        if (err != cudaSuccess) {
            e->last_error = std::string("cudaSetDevice: ") + cudaGetErrorString(err);
            return reinterpret_cast<fullmag_fdm_backend *>(e);
        }
    }
    if (plan->precision == FULLMAG_FDM_PRECISION_DOUBLE) {
        std::string err;
        e->f64 = fp64_create(plan, err);
        if (!e->f64) e->last_error = err;
        return reinterpret_cast<fullmag_fdm_backend *>(e);
    }
    if (!e->setup(plan)) return reinterpret_cast<fullmag_fdm_backend *>(e);
    if (!e->upload<double>(plan->initial_magnetization_xyz)) return reinterpret_cast<fullmag_fdm_backend *>(e);
    if (!e->eval_state(true)) return reinterpret_cast<fullmag_fdm_backend *>(e);
    return reinterpret_cast<fullmag_fdm_backend *>(e);
}

fullmag_fdm_backend *fullmag_fdm_backend_create_periodic(const fullmag_fdm_plan_desc *plan,
                                                         const fullmag_fdm_periodicity_desc *periodicity) {
    if (!plan || !periodicity) return nullptr;
    Engine *e = new (std::nothrow) Engine();
    if (!e) return nullptr;
    const int sel = device_from_env();
    if (sel >= 0) {
        cudaError_t err = cudaSetDevice(sel);
        if (err != cudaSuccess) {
            e->last_error = std::string("cudaSetDevice: ") + cudaGetErrorString(err);
            return reinterpret_cast<fullmag_fdm_backend *>(e);
        }
    }
    for (int a = 0; a < 3; ++a) {
        if (periodicity->periodic[a] > 1) {
            e->last_error = "periodic[] entries must be 0 (open) or 1 (periodic)";
            return reinterpret_cast<fullmag_fdm_backend *>(e);
        }
        if (periodicity->periodic[a]) e->per_req |= 1 << a;
        if (periodicity->has_image_counts) {
            if (periodicity->image_counts[a] > 4096) {
                e->last_error = "image_counts above 4096";
                return reinterpret_cast<fullmag_fdm_backend *>(e);
            }
            e->images[a] = periodicity->image_counts[a];
        }
    }
    if (plan->precision == FULLMAG_FDM_PRECISION_DOUBLE) {
        std::string err;
        e->f64 = fp64_create(plan, err, e->per_req, e->images);
        if (!e->f64) e->last_error = err;
        return reinterpret_cast<fullmag_fdm_backend *>(e);
    }
    if (!e->setup(plan)) return reinterpret_cast<fullmag_fdm_backend *>(e);
    if (!e->upload<double>(plan->initial_magnetization_xyz)) return reinterpret_cast<fullmag_fdm_backend *>(e);
    if (!e->eval_state(true)) return reinterpret_cast<fullmag_fdm_backend *>(e);
    return reinterpret_cast<fullmag_fdm_backend *>(e);
}

int fullmag_fdm_backend_step(fullmag_fdm_backend *handle, double dt_seconds, fullmag_fdm_step_stats *out_stats) {
    Engine *e = eng(handle);
    if (!e || !out_stats) return FULLMAG_FDM_ERR_INVALID;
    if (!e->arena && !e->f64) return FULLMAG_FDM_ERR_INVALID;
    e->last_error.clear();
    if (!(dt_seconds > 0.0) || !std::isfinite(dt_seconds)) {
        e->last_error = "dt_seconds must be positive and finite";
        return FULLMAG_FDM_ERR_INVALID;
    }
    if (e->f64) {
        std::string err;
        const int rc = fp64_step(e->f64, dt_seconds, out_stats, e->poll, e->poll_user, err);
        if (rc != FULLMAG_FDM_OK) e->last_error = err;
        return rc;
    }
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = e->step(dt_seconds);
    if (rc < 0) return FULLMAG_FDM_ERR_CUDA;
    if (rc == 1) {
        if (!e->stats_valid && !e->eval_state(false)) return FULLMAG_FDM_ERR_CUDA;
        *out_stats = e->cur_stats;
        out_stats->dt_seconds = 0.0;
        return FULLMAG_FDM_ERR_INTERRUPTED;
    }
    const auto t1 = std::chrono::steady_clock::now();
    *out_stats = e->cur_stats;
    out_stats->wall_time_ns = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0).count();
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_step_many(fullmag_fdm_backend *handle, double dt_seconds, uint64_t n_steps,
                                  fullmag_fdm_step_stats *out_stats) {
    Engine *e = eng(handle);
    if (!e || !out_stats || (!e->arena && !e->f64)) return FULLMAG_FDM_ERR_INVALID;
    e->last_error.clear();
    if (!e->f64 && e->adaptive()) {
        e->last_error = "step_many supports fixed-step integrators only";
        return FULLMAG_FDM_ERR_INVALID;
    }
    for (uint64_t s = 0; s < n_steps; ++s) {
        const int rc = fullmag_fdm_backend_step(handle, dt_seconds, out_stats);
        if (rc != FULLMAG_FDM_OK) return rc;
    }
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_set_interrupt_poll(fullmag_fdm_backend *handle, fullmag_fdm_interrupt_poll_fn poll_fn, void *user_data) {
    Engine *e = eng(handle);
    if (!e) return FULLMAG_FDM_ERR_INVALID;
    e->poll = poll_fn;
    e->poll_user = user_data;
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_copy_field_f64(fullmag_fdm_backend *handle, fullmag_fdm_observable observable, double *out_xyz,
                                       uint64_t out_len) {
    Engine *e = eng(handle);
    if (e && out_xyz && e->f64) return f64_copy<double>(e, observable, out_xyz, out_len);
    if (!e || !out_xyz || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    if (out_len != 3 * (uint64_t)e->g.n) {
        e->last_error = "out_len mismatch";
        return FULLMAG_FDM_ERR_INVALID;
    }
    if (observable < FULLMAG_FDM_OBSERVABLE_M || observable > FULLMAG_FDM_OBSERVABLE_H_EFF) {
        e->last_error = "unknown observable";
        return FULLMAG_FDM_ERR_INVALID;
    }
    return e->download<double>(observable, out_xyz) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
}

int fullmag_fdm_backend_copy_field_f32(fullmag_fdm_backend *handle, fullmag_fdm_observable observable, float *out_xyz,
                                       uint64_t out_len) {
    Engine *e = eng(handle);
    if (e && out_xyz && e->f64) return f64_copy<float>(e, observable, out_xyz, out_len);
    if (!e || !out_xyz || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    if (out_len != 3 * (uint64_t)e->g.n) {
        e->last_error = "out_len mismatch";
        return FULLMAG_FDM_ERR_INVALID;
    }
    if (observable < FULLMAG_FDM_OBSERVABLE_M || observable > FULLMAG_FDM_OBSERVABLE_H_EFF) {
        e->last_error = "unknown observable";
        return FULLMAG_FDM_ERR_INVALID;
    }
    return e->download<float>(observable, out_xyz) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
}

int fullmag_fdm_backend_copy_field_preview_f64(fullmag_fdm_backend *handle, fullmag_fdm_observable observable,
                                               uint32_t preview_nx, uint32_t preview_ny, uint32_t preview_nz,
                                               uint32_t z_origin, uint32_t z_stride, double *out_xyz, uint64_t out_len) {
    return preview_impl<double>(handle, observable, preview_nx, preview_ny, preview_nz, z_origin, z_stride, out_xyz, out_len);
}

int fullmag_fdm_backend_copy_field_preview_f32(fullmag_fdm_backend *handle, fullmag_fdm_observable observable,
                                               uint32_t preview_nx, uint32_t preview_ny, uint32_t preview_nz,
                                               uint32_t z_origin, uint32_t z_stride, float *out_xyz, uint64_t out_len) {
    return preview_impl<float>(handle, observable, preview_nx, preview_ny, preview_nz, z_origin, z_stride, out_xyz, out_len);
}

fullmag_fdm_field_snapshot *fullmag_fdm_backend_begin_field_snapshot(fullmag_fdm_backend *handle,
                                                                     fullmag_fdm_observable observable) {
    Engine *e = eng(handle);
    if (!e || (!e->arena && !e->f64)) return nullptr;
    auto *s = new (std::nothrow) SnapshotPayload();
    if (!s) return nullptr;
    if (e->f64) {  // double precision: captured synchronously, component-major FP64
        int nx, ny, nz;
        fp64_grid(e->f64, nx, ny, nz);
        const size_t n = (size_t)nx * ny * nz;
        std::vector<double> aos(3 * n);
        if (f64_copy<double>(e, observable, aos.data(), aos.size()) != FULLMAG_FDM_OK) {
            delete s;
            return nullptr;
        }
        s->bytes.resize(sizeof(double) * 3 * n);
        double *soa = reinterpret_cast<double *>(s->bytes.data());
        for (size_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) soa[c * n + i] = aos[3 * i + c];
        s->desc.cell_count = n;
        s->desc.component_count = 3;
        s->desc.scalar_bytes = 8;
        s->desc.scalar_type = FULLMAG_FDM_SNAPSHOT_SCALAR_F64;
        s->ok = true;
        return reinterpret_cast<fullmag_fdm_field_snapshot *>(s);
    }
    const size_t n = (size_t)e->g.n;
    if (observable == FULLMAG_FDM_OBSERVABLE_H_EXT) {  // synthesised on the host
        std::vector<float> aos(3 * n);
        if (!e->download<float>(observable, aos.data())) {
            delete s;
            return nullptr;
        }
        s->bytes.resize(sizeof(float) * 3 * n);
        float *soa = reinterpret_cast<float *>(s->bytes.data());
        for (size_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) soa[c * n + i] = aos[3 * i + c];
    } else {
        // the device field is SoA already: one device copy on the engine stream pins the
        // state of this moment, the copy to the host runs on the snapshot stream
        const float *field = e->current_field(observable);
        const size_t bytes = sizeof(float) * 3 * n;
        if (!field || !e->begin_snapshot(
                          bytes,
                          [&](void *dev) {
                              return !e->cuda_fail("cudaMemcpy(snapshot field)",
                                                   cudaMemcpyAsync(dev, field, bytes, cudaMemcpyDeviceToDevice, e->stream));
                          },
                          s)) {
            delete s;
            return nullptr;
        }
    }
    s->desc.cell_count = n;
    s->desc.component_count = 3;
    s->desc.scalar_bytes = 4;
    s->desc.scalar_type = FULLMAG_FDM_SNAPSHOT_SCALAR_F32;
    s->ok = true;
    return reinterpret_cast<fullmag_fdm_field_snapshot *>(s);
}

fullmag_fdm_preview_snapshot *fullmag_fdm_backend_begin_preview_snapshot(fullmag_fdm_backend *handle,
                                                                         fullmag_fdm_observable observable,
                                                                         uint32_t preview_nx, uint32_t preview_ny,
                                                                         uint32_t preview_nz, uint32_t z_origin,
                                                                         uint32_t z_stride) {
    Engine *e = eng(handle);
    if (!e || (!e->arena && !e->f64) || preview_nx == 0 || preview_ny == 0 || preview_nz == 0 || z_stride == 0)
        return nullptr;
    auto *s = new (std::nothrow) SnapshotPayload();
    if (!s) return nullptr;
    const size_t n = (size_t)preview_nx * preview_ny * preview_nz;
    if (e->f64) {  // double precision: the FP64 box average, captured synchronously
        s->bytes.resize(sizeof(double) * 3 * n);
        if (preview_impl<double>(handle, observable, preview_nx, preview_ny, preview_nz, z_origin, z_stride,
                                 reinterpret_cast<double *>(s->bytes.data()), 3 * n) != FULLMAG_FDM_OK) {
            delete s;
            return nullptr;
        }
        s->desc.cell_count = n;
        s->desc.component_count = 3;
        s->desc.scalar_bytes = 8;
        s->desc.scalar_type = FULLMAG_FDM_SNAPSHOT_SCALAR_F64;
        s->ok = true;
        return reinterpret_cast<fullmag_fdm_preview_snapshot *>(s);
    }
    if (z_origin >= (uint32_t)e->g.nz) {
        e->last_error = "preview z_origin out of range";
        delete s;
        return nullptr;
    }
    if (observable == FULLMAG_FDM_OBSERVABLE_H_EXT) {  // synthesised on the host
        s->bytes.resize(sizeof(float) * 3 * n);
        if (!e->preview<float>(observable, preview_nx, preview_ny, preview_nz, z_origin, z_stride,
                               reinterpret_cast<float *>(s->bytes.data()))) {
            delete s;
            return nullptr;
        }
    } else {
        // downsampled on the device into the snapshot's buffer, copied out on the snapshot stream
        const float *field = e->current_field(observable);
        if (!field || !e->begin_snapshot(
                          sizeof(float) * 3 * n,
                          [&](void *dev) {
                              return e->enqueue_preview<float>(field, preview_nx, preview_ny, preview_nz, z_origin,
                                                               z_stride, (float *)dev, e->stream);
                          },
                          s)) {
            delete s;
            return nullptr;
        }
    }
    s->desc.cell_count = n;
    s->desc.component_count = 3;
    s->desc.scalar_bytes = 4;
    s->desc.scalar_type = FULLMAG_FDM_SNAPSHOT_SCALAR_F32;
    s->ok = true;
    return reinterpret_cast<fullmag_fdm_preview_snapshot *>(s);
}

int fullmag_fdm_field_snapshot_wait(fullmag_fdm_field_snapshot *snapshot, const void **out_data, uint64_t *out_len_bytes,
                                    fullmag_fdm_snapshot_desc *out_desc) {
    return snap_wait(reinterpret_cast<SnapshotPayload *>(snapshot), out_data, out_len_bytes, out_desc);
}

int fullmag_fdm_preview_snapshot_wait(fullmag_fdm_preview_snapshot *snapshot, const void **out_data, uint64_t *out_len_bytes,
                                      fullmag_fdm_snapshot_desc *out_desc) {
    return snap_wait(reinterpret_cast<SnapshotPayload *>(snapshot), out_data, out_len_bytes, out_desc);
}

void fullmag_fdm_field_snapshot_destroy(fullmag_fdm_field_snapshot *snapshot) {
    delete reinterpret_cast<SnapshotPayload *>(snapshot);
}

void fullmag_fdm_preview_snapshot_destroy(fullmag_fdm_preview_snapshot *snapshot) {
    delete reinterpret_cast<SnapshotPayload *>(snapshot);
}

// upload to a double-precision handle
static int f64_upload(Engine *e, const double *m_xyz, uint64_t len) {
    int nx, ny, nz;
    fp64_grid(e->f64, nx, ny, nz);
    if (len != 3 * (uint64_t)nx * ny * nz) {
        e->last_error = "magnetization length mismatch";
        return FULLMAG_FDM_ERR_INVALID;
    }
    std::string err;
    if (!fp64_upload(e->f64, m_xyz, err)) {
        e->last_error = err;
        return FULLMAG_FDM_ERR_CUDA;
    }
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_upload_magnetization_f64(fullmag_fdm_backend *handle, const double *m_xyz, uint64_t len) {
    Engine *e = eng(handle);
    if (e && m_xyz && e->f64) return f64_upload(e, m_xyz, len);
    if (!e || !m_xyz || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    if (len != 3 * (uint64_t)e->g.n) {
        e->last_error = "magnetization length mismatch";
        return FULLMAG_FDM_ERR_INVALID;
    }
    return e->upload<double>(m_xyz) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
}

int fullmag_fdm_backend_upload_magnetization_f64_noalloc(fullmag_fdm_backend *handle, const double *m_xyz,
                                                         uint64_t len) {
    Engine *e = eng(handle);
    if (!e || !m_xyz || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    if (len != 3 * (uint64_t)e->g.n) {
        e->last_error = "magnetization length mismatch";
        return FULLMAG_FDM_ERR_INVALID;
    }
    if (e->g.n > kNoAllocMaxCells) {
        e->last_error = "grid of " + std::to_string(e->g.n) + " cells exceeds the " + std::to_string(kNoAllocMaxCells) +
                        "-cell limit of the allocation-free upload; use fullmag_fdm_backend_upload_magnetization_f64";
        return FULLMAG_FDM_ERR_INVALID;
    }
    return e->upload_noalloc(m_xyz) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
}

int fullmag_fdm_backend_upload_magnetization_f32(fullmag_fdm_backend *handle, const float *m_xyz, uint64_t len) {
    Engine *e = eng(handle);
    if (e && m_xyz && e->f64) {
        std::vector<double> d(m_xyz, m_xyz + len);
        return f64_upload(e, d.data(), len);
    }
    if (!e || !m_xyz || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    if (len != 3 * (uint64_t)e->g.n) {
        e->last_error = "magnetization length mismatch";
        return FULLMAG_FDM_ERR_INVALID;
    }
    return e->upload<float>(m_xyz) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
}

int fullmag_fdm_backend_refresh_observables(fullmag_fdm_backend *handle) {
    Engine *e = eng(handle);
    if (e && e->f64) {
        std::string err;
        if (fp64_refresh(e->f64, err)) return FULLMAG_FDM_OK;
        e->last_error = err;
        return FULLMAG_FDM_ERR_CUDA;
    }
    if (!e || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    return e->eval_state(true) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
}

int fullmag_fdm_backend_refresh_demag_observable(fullmag_fdm_backend *handle) {
    Engine *e = eng(handle);
    if (e && e->f64) {
        std::string err;
        if (fp64_refresh(e->f64, err)) return FULLMAG_FDM_OK;
        e->last_error = err;
        return FULLMAG_FDM_ERR_CUDA;
    }
    if (!e || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    return e->eval_state(true) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
}

int fullmag_fdm_backend_snapshot_stats(fullmag_fdm_backend *handle, fullmag_fdm_step_stats *out_stats) {
    Engine *e = eng(handle);
    if (e && out_stats && e->f64) {
        fp64_stats(e->f64, out_stats);
        out_stats->dt_seconds = 0.0;
        out_stats->suggested_next_dt = 0.0;
        out_stats->wall_time_ns = 0;
        return FULLMAG_FDM_OK;
    }
    if (!e || !out_stats || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    if (!e->stats_valid && !e->eval_state(false)) return FULLMAG_FDM_ERR_CUDA;
    *out_stats = e->cur_stats;
    out_stats->step = e->step_count;
    out_stats->time_seconds = e->time;
    out_stats->dt_seconds = 0.0;
    out_stats->suggested_next_dt = 0.0;
    out_stats->wall_time_ns = 0;
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_get_device_info(fullmag_fdm_backend *handle, fullmag_fdm_device_info *out_info) {
    Engine *e = eng(handle);
    if (!e || !out_info) return FULLMAG_FDM_ERR_INVALID;
    if (!e->info_valid) {
        cudaDeviceProp prop;
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
            e->last_error = "cudaGetDeviceProperties failed";
            return FULLMAG_FDM_ERR_CUDA;
        }
        std::memset(&e->info, 0, sizeof(e->info));
        std::strncpy(e->info.name, prop.name, sizeof(e->info.name) - 1);
        e->info.compute_capability_major = prop.major;
        e->info.compute_capability_minor = prop.minor;
        cudaDriverGetVersion(&e->info.driver_version);
        cudaRuntimeGetVersion(&e->info.runtime_version);
        e->info_valid = true;
    }
    *out_info = e->info;
    return FULLMAG_FDM_OK;
}

const char *fullmag_fdm_backend_last_error(fullmag_fdm_backend *handle) {
    if (!handle) return "null handle";
    Engine *e = eng(handle);
    return e->last_error.empty() ? nullptr : e->last_error.c_str();
}

void fullmag_fdm_backend_destroy(fullmag_fdm_backend *handle) { delete eng(handle); }

int fullmag_fdm_backend_device_magnetization(fullmag_fdm_backend *handle, void **out_mx, void **out_my, void **out_mz) {
    Engine *e = eng(handle);
    if (!e || !e->arena || !out_mx || !out_my || !out_mz) return FULLMAG_FDM_ERR_INVALID;
    float *m = e->S[e->cur];
    *out_mx = m;
    *out_my = m + e->g.n;
    *out_mz = m + 2 * e->g.n;
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_stream(fullmag_fdm_backend *handle, void **out_stream) {
    Engine *e = eng(handle);
    if (!e || !out_stream) return FULLMAG_FDM_ERR_INVALID;
    *out_stream = (void *)e->stream;
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_set_field_map(fullmag_fdm_backend *handle, const double *h_xyz, uint64_t len) {
    Engine *e = eng(handle);
    if (!e || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    if (h_xyz && len != 3 * (uint64_t)e->g.n) {
        e->last_error = "field map length mismatch";
        return FULLMAG_FDM_ERR_INVALID;
    }
    return e->set_field_map(h_xyz) ? FULLMAG_FDM_OK : FULLMAG_FDM_ERR_CUDA;
}

int fullmag_fdm_adjoint_forward(fullmag_fdm_backend *handle, double dt_seconds, uint64_t n_steps,
                                uint32_t checkpoint_every) {
    Engine *e = eng(handle);
    if (!e || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    e->last_error.clear();
    if (e->g.per && e->demag) {
        // the backward pass applies the demag convolution as its own transpose, which
        // the truncated image sum (not symmetric under i -> -i) is not
        e->last_error = "adjoint gradients are not available with periodic demag";
        return FULLMAG_FDM_ERR_INVALID;
    }
    return e->adjoint_forward(dt_seconds, n_steps, checkpoint_every);
}

int fullmag_fdm_adjoint_backward(fullmag_fdm_backend *handle, const double *lambda_xyz, uint64_t len,
                                 double *grad_field_map_xyz, double *lambda0_xyz) {
    Engine *e = eng(handle);
    if (!e || !e->arena || !lambda_xyz) return FULLMAG_FDM_ERR_INVALID;
    if (len != 3 * (uint64_t)e->g.n) {
        e->last_error = "lambda length mismatch";
        return FULLMAG_FDM_ERR_INVALID;
    }
    e->last_error.clear();
    return e->adjoint_backward(lambda_xyz, grad_field_map_xyz, lambda0_xyz);
}

int fullmag_fdm_backend_set_kernel_timing(fullmag_fdm_backend *handle, int enable) {
    Engine *e = eng(handle);
    if (!e || !e->arena) return FULLMAG_FDM_ERR_INVALID;
    if (cudaStreamSynchronize(e->stream) != cudaSuccess) return FULLMAG_FDM_ERR_CUDA;
    e->kt_collect();
    e->ktime = enable != 0;
    for (int k = 0; k < Engine::KT_N; ++k) {
        e->kt_ms[k] = 0.0;
        e->kt_cnt[k] = 0;
    }
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_kernel_times(fullmag_fdm_backend *handle, double *total_ms, uint64_t *counts, uint32_t n_kinds) {
    Engine *e = eng(handle);
    if (!e || !e->arena || !total_ms || !counts) return FULLMAG_FDM_ERR_INVALID;
    if (cudaStreamSynchronize(e->stream) != cudaSuccess) return FULLMAG_FDM_ERR_CUDA;
    e->kt_collect();
    for (uint32_t k = 0; k < n_kinds; ++k) {
        total_ms[k] = k < (uint32_t)Engine::KT_N ? e->kt_ms[k] : 0.0;
        counts[k] = k < (uint32_t)Engine::KT_N ? e->kt_cnt[k] : 0;
    }
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_tuning(fullmag_fdm_backend *handle, uint32_t *out9) {
    Engine *e = eng(handle);
    if (!e || !out9) return FULLMAG_FDM_ERR_INVALID;
    out9[0] = (uint32_t)e->row_rows;
    out9[1] = (uint32_t)e->tx_yf;
    out9[2] = (uint32_t)e->tx_z;
    out9[3] = (uint32_t)e->tx_yi;
    out9[4] = (uint32_t)e->tx_2d;
    out9[5] = (uint32_t)e->z_pair;
    out9[6] = (uint32_t)e->split_yf;
    out9[7] = (uint32_t)e->split_z;
    out9[8] = (uint32_t)e->split_yi;
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_launch_count(fullmag_fdm_backend *handle, uint64_t *out_count) {
    Engine *e = eng(handle);
    if (!e || !out_count) return FULLMAG_FDM_ERR_INVALID;
    *out_count = e->launches;
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_backend_fft_shape(fullmag_fdm_backend *handle, uint32_t *out_px, uint32_t *out_py, uint32_t *out_pz) {
    Engine *e = eng(handle);
    if (!e || !out_px || !out_py || !out_pz) return FULLMAG_FDM_ERR_INVALID;
    if (e->f64) {
        fp64_fft_shape(e->f64, *out_px, *out_py, *out_pz);
        return FULLMAG_FDM_OK;
    }
    *out_px = e->g.px;
    *out_py = e->g.py;
    *out_pz = e->g.pz;
    return FULLMAG_FDM_OK;
}

}  // extern "C"

// =====================================================================
// Batched sweeps: many independent problems of uneven size
// =====================================================================

// One round of a batched sweep: the attempt of every member problem, executed as
// 7 batched row passes + 6 batched column passes (one launch per pass and column
// kind for all problems, through (problem, block) work tables) + one batched
// finalize, captured once as a CUDA graph and replayed every round.
struct BatchRound {
    std::vector<size_t> members;
    BatchCtl *h_ctl = nullptr;  // pinned [n]
    BatchCtl *d_ctl = nullptr;
    double *h_stats = nullptr;  // pinned [n * kNumStats]
    double *d_stats = nullptr;
    BatchState *h_state = nullptr;  // pinned [n]
    BatchState *d_state = nullptr;
    const CommitDesc *d_com = nullptr;  // inside d_blob
    long long max_n3 = 0;
    void *d_blob = nullptr;     // descriptors and work tables
    cudaGraphExec_t exec = nullptr;
    static constexpr int kRounds = 16;  // rounds per graph launch

    void release() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        if (h_ctl) cudaFreeHost(h_ctl);
        h_ctl = nullptr;
        if (h_stats) cudaFreeHost(h_stats);
        h_stats = nullptr;
        if (d_ctl) cudaFree(d_ctl);
        d_ctl = nullptr;
        if (d_stats) cudaFree(d_stats);
        d_stats = nullptr;
        if (d_blob) cudaFree(d_blob);
        d_blob = nullptr;
        if (h_state) cudaFreeHost(h_state);
        h_state = nullptr;
        if (d_state) cudaFree(d_state);
        d_state = nullptr;
    }
};

struct FdmBatch {
    std::vector<Engine *> items;
    std::vector<double> next_dt;  // per problem: suggested step (DP45) or 0 before the first step
    std::string last_error;
    cudaStream_t bstream = nullptr;
    // Branches of a captured round: the buckets of one pass (row buckets, column groups)
    // are independent launches, captured as parallel graph branches so that a bucket of
    // a few dozen CTAs runs beside the large ones instead of after them.
    static constexpr int kSide = 8;
    cudaStream_t side[kSide] = {};
    cudaEvent_t fork_ev = nullptr, join_ev[kSide] = {};
    BatchRound round;
    ~FdmBatch() {
        if (bstream) cudaStreamSynchronize(bstream);
        round.release();
        for (int j = 0; j < kSide; ++j) {
            if (side[j]) cudaStreamDestroy(side[j]);
            if (join_ev[j]) cudaEventDestroy(join_ev[j]);
        }
        if (fork_ev) cudaEventDestroy(fork_ev);
        if (bstream) cudaStreamDestroy(bstream);
        for (Engine *e : items) delete e;
    }

    bool ensure_branches() {
        if (fork_ev) return true;
        for (int j = 0; j < kSide; ++j)
            if (cudaStreamCreateWithFlags(&side[j], cudaStreamNonBlocking) != cudaSuccess ||
                cudaEventCreateWithFlags(&join_ev[j], cudaEventDisableTiming) != cudaSuccess)
                return false;
        return cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming) == cudaSuccess;
    }

    // Enqueues launch(id, stream) for every id as parallel branches that fork from and
    // join back into bstream (inside a capture: graph nodes with no edges between them).
    template <typename F>
    bool fan_out(const std::vector<int> &ids, F &&launch) {
        if (ids.empty()) return true;
        if (ids.size() == 1) return launch(ids[0], bstream) == cudaSuccess;
        const int ns = std::min<int>((int)ids.size(), kSide);
        if (cudaEventRecord(fork_ev, bstream) != cudaSuccess) return false;
        for (int j = 0; j < ns; ++j)
            if (cudaStreamWaitEvent(side[j], fork_ev, 0) != cudaSuccess) return false;
        for (size_t j = 0; j < ids.size(); ++j)
            if (launch(ids[j], side[j % ns]) != cudaSuccess) return false;
        for (int j = 0; j < ns; ++j)
            if (cudaEventRecord(join_ev[j], side[j]) != cudaSuccess || cudaStreamWaitEvent(bstream, join_ev[j], 0) != cudaSuccess)
                return false;
        return true;
    }

    // Builds (and captures) the round for `act`; false when a member cannot run batched.
    // Runs the commits still pending in the round's control blocks (device side) and
    // hands every member's device step control back to its engine: time, accepted steps,
    // statistics of the last accepted step, next step size.
    bool sync_states(std::string &err) {
        if (!round.exec) return true;
        const int n = (int)round.members.size();
        const unsigned gx = (unsigned)std::min<long long>((round.max_n3 + 255) / 256, 64);
        batch_commit_all_kernel<<<dim3(gx, n), 256, 0, bstream>>>(round.d_com, round.d_ctl);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(round.h_state, round.d_state, sizeof(BatchState) * n, cudaMemcpyDeviceToHost, bstream) != cudaSuccess ||
            cudaMemsetAsync(round.d_ctl, 0, sizeof(BatchCtl) * n, bstream) != cudaSuccess ||
            cudaStreamSynchronize(bstream) != cudaSuccess) {
            err = "batch commit failed";
            return false;
        }
        for (int k = 0; k < n; ++k) {
            const size_t i = round.members[k];
            BatchState &st = round.h_state[k];
            items[i]->batch_apply(st);
            next_dt[i] = st.next_dt;
            st.steps = 0;
        }
        return cudaMemcpyAsync(round.d_state, round.h_state, sizeof(BatchState) * n, cudaMemcpyHostToDevice, bstream) ==
                   cudaSuccess &&
               cudaStreamSynchronize(bstream) == cudaSuccess;
    }

    bool build_round(const std::vector<size_t> &act, double t_end, std::string &err) {
        // the old round's pending commits and step control go back to the engines first
        if (!sync_states(err)) return false;
        if (bstream) cudaStreamSynchronize(bstream);
        round.release();
        const int n = (int)act.size();
        round.members = act;
        if (cudaMallocHost((void **)&round.h_ctl, sizeof(BatchCtl) * n) != cudaSuccess ||
            cudaMallocHost((void **)&round.h_stats, sizeof(double) * kNumStats * n) != cudaSuccess ||
            cudaMallocHost((void **)&round.h_state, sizeof(BatchState) * n) != cudaSuccess ||
            cudaMalloc((void **)&round.d_ctl, sizeof(BatchCtl) * n) != cudaSuccess ||
            cudaMalloc((void **)&round.d_stats, sizeof(double) * kNumStats * n) != cudaSuccess ||
            cudaMalloc((void **)&round.d_state, sizeof(BatchState) * n) != cudaSuccess) {
            err = "batch round allocation failed";
            return false;
        }
        // Work is bucketed by shared-memory class so one large member does not set the
        // occupancy of every CTA: row buckets rb, column groups (kind, class).
        constexpr int NC = 5;
        auto smem_class = [](size_t b) {
            return b <= 24u * 1024u ? 0 : b <= 48u * 1024u ? 1 : b <= 96u * 1024u ? 2 : b <= 150u * 1024u ? 3 : 4;
        };
        std::vector<RowPass> rows[7];
        constexpr int NK = 4;  // column kernel kinds (col_batched_kind)
        std::vector<ColPass> cols[NK * NC];
        std::vector<int2> row_work[NC], col_work[NK * NC];
        std::vector<FinDesc> fin(n);
        std::vector<CommitDesc> com(n);
        size_t row_smem[NC] = {0, 0, 0, 0, 0}, col_smem[NK * NC] = {};
        std::vector<RowPass> rec;
        std::vector<int> kinds;
        for (int k = 0; k < n; ++k) {
            Engine *e = items[act[k]];
            BatchState &st = round.h_state[k];
            memset(&st, 0, sizeof(st));
            st.time = e->time;
            st.t_end = t_end;
            st.next_dt = next_dt[act[k]];
            st.max_error = e->max_error;
            st.dt_min = e->dt_min;
            st.dt_max = e->dt_max;
            st.headroom = e->headroom;
            st.ctrl_exp = e->ctrl_exp();
            st.done = e->time >= t_end * (1.0 - 1e-12);
            round.h_ctl[k] = BatchCtl{st.done ? 0.0 : std::min(st.next_dt, t_end - e->time), 0, 0};
            if (!e->record_attempt(&round.d_ctl[k].dt, rec, kinds)) {
                err = "problem " + std::to_string(act[k]) + ": " + (e->last_error.empty() ? "not batchable" : e->last_error);
                return false;
            }
            size_t rs = 0;
            for (int s = 0; s < 7; ++s) {
                rows[s].push_back(rec[s]);
                rs = std::max(rs, row_pass_smem(rec[s]));
            }
            const int rb = smem_class(rs);
            row_smem[rb] = std::max(row_smem[rb], rs);
            const int nb = row_pass_blocks(rec[0]);
            for (int b = 0; b < nb; ++b) row_work[rb].push_back(make_int2(k, b));
            if (e->demag) {
                const int kind = kinds[0];
                const bool thin = e->g.thin != 0;
                const int tx = thin ? e->tx_2d : e->tx_z;
                const size_t cs = thin ? y_convolve_2d_smem(e->g, tx) : yz_convolve_smem(e->g, tx);
                const int cg = kind * NC + smem_class(cs);
                ColPass c = e->col_pass(e->plan_y, tx, e->X, e->X);
                c.skip_dt = &round.d_ctl[k].dt;
                const int idx = (int)cols[cg].size();
                cols[cg].push_back(c);
                const int ntiles = (e->g.nkx + tx - 1) / tx;
                for (int t = 0; t < ntiles; ++t) col_work[cg].push_back(make_int2(idx, t));
                col_smem[cg] = std::max(col_smem[cg], cs);
            }
            fin[k] = FinDesc{e->partials, nb, 0};
            com[k] = CommitDesc{e->S[0], e->S[1], e->K[0], e->K[6], 3 * e->g.n};
        }
        // one device blob for every descriptor array
        size_t off = 0;
        auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
        size_t o_rows[7], o_cols[NK * NC], o_rw[NC], o_cw[NK * NC], o_fin, o_com;
        for (int s = 0; s < 7; ++s) { o_rows[s] = off; off += al(sizeof(RowPass) * rows[s].size()); }
        for (int k = 0; k < NK * NC; ++k) { o_cols[k] = off; off += al(sizeof(ColPass) * cols[k].size()); }
        for (int k = 0; k < NC; ++k) { o_rw[k] = off; off += al(sizeof(int2) * row_work[k].size()); }
        for (int k = 0; k < NK * NC; ++k) { o_cw[k] = off; off += al(sizeof(int2) * col_work[k].size()); }
        o_fin = off; off += al(sizeof(FinDesc) * n);
        o_com = off; off += al(sizeof(CommitDesc) * n);
        if (cudaMalloc(&round.d_blob, off) != cudaSuccess) {
            err = "batch descriptor allocation failed";
            return false;
        }
        char *blob = (char *)round.d_blob;
        std::vector<char> hb(off);
        for (int s = 0; s < 7; ++s) memcpy(hb.data() + o_rows[s], rows[s].data(), sizeof(RowPass) * rows[s].size());
        for (int k = 0; k < NK * NC; ++k) memcpy(hb.data() + o_cols[k], cols[k].data(), sizeof(ColPass) * cols[k].size());
        for (int k = 0; k < NC; ++k) memcpy(hb.data() + o_rw[k], row_work[k].data(), sizeof(int2) * row_work[k].size());
        for (int k = 0; k < NK * NC; ++k) memcpy(hb.data() + o_cw[k], col_work[k].data(), sizeof(int2) * col_work[k].size());
        memcpy(hb.data() + o_fin, fin.data(), sizeof(FinDesc) * n);
        memcpy(hb.data() + o_com, com.data(), sizeof(CommitDesc) * n);
        if (cudaMemcpy(blob, hb.data(), off, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(round.d_ctl, round.h_ctl, sizeof(BatchCtl) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(round.d_state, round.h_state, sizeof(BatchState) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
            err = "batch descriptor upload failed";
            return false;
        }
        round.d_com = (const CommitDesc *)(blob + o_com);
        // capture the round
        long long max_n3 = 0;
        for (auto &c : com) max_n3 = std::max(max_n3, c.n3);
        // set the shared-memory limits outside the capture
        size_t max_row = 0, max_col = 0;
        for (int k = 0; k < NC; ++k) max_row = std::max(max_row, row_smem[k]);
        for (int k = 0; k < NK * NC; ++k) max_col = std::max(max_col, col_smem[k]);
        launch_row_pass_batched((const RowPass *)(blob + o_rows[0]), (const int2 *)(blob + o_rw[0]), 0, max_row, bstream);
        for (int kd = 0; kd < NK; ++kd)
            launch_col_batched((const ColPass *)(blob + o_cols[0]), (const int2 *)(blob + o_cw[0]), 0, kd, max_col, bstream);
        cudaGetLastError();
        if (!ensure_branches()) {
            err = "batch stream or event creation failed";
            return false;
        }
        std::vector<int> row_ids, col_ids;
        for (int rb = 0; rb < NC; ++rb)
            if (!row_work[rb].empty()) row_ids.push_back(rb);
        for (int cg = 0; cg < NK * NC; ++cg)
            if (!col_work[cg].empty()) col_ids.push_back(cg);
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(bstream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            err = "batch capture failed";
            return false;
        }
        // kRounds rounds, each: the previous round's commits, the seven passes of an attempt
        // for every member, the statistics, and the device step control; then the control
        // state goes to the host once
        bool ok = true;
        round.max_n3 = max_n3;
        for (int r = 0; r < BatchRound::kRounds && ok; ++r) {
            const unsigned gx = (unsigned)std::min<long long>((max_n3 + 255) / 256, 64);
            batch_commit_all_kernel<<<dim3(gx, n), 256, 0, bstream>>>((const CommitDesc *)(blob + o_com), round.d_ctl);
            ok = cudaGetLastError() == cudaSuccess;
            for (int s = 0; s < 7 && ok; ++s) {
                ok = fan_out(row_ids, [&](int rb, cudaStream_t st) {
                    return launch_row_pass_batched((const RowPass *)(blob + o_rows[s]), (const int2 *)(blob + o_rw[rb]),
                                                   (int)row_work[rb].size(), row_smem[rb], st);
                });
                if (ok && s < 6)
                    ok = fan_out(col_ids, [&](int cg, cudaStream_t st) {
                        return launch_col_batched((const ColPass *)(blob + o_cols[cg]), (const int2 *)(blob + o_cw[cg]),
                                                  (int)col_work[cg].size(), cg / NC, col_smem[cg], st);
                    });
            }
            if (ok) ok = launch_finalize_batched((const FinDesc *)(blob + o_fin), n, round.d_stats, bstream) == cudaSuccess;
            if (ok) {
                batch_control_kernel<<<(n + 127) / 128, 128, 0, bstream>>>(round.d_ctl, round.d_state, round.d_stats, n);
                ok = cudaGetLastError() == cudaSuccess;
            }
        }
        if (ok)
            ok = cudaMemcpyAsync(round.h_state, round.d_state, sizeof(BatchState) * n, cudaMemcpyDeviceToHost, bstream) ==
                 cudaSuccess;
        const cudaError_t ce = cudaStreamEndCapture(bstream, &graph);
        if (!ok || ce != cudaSuccess || !graph) {
            if (graph) cudaGraphDestroy(graph);
            err = "batch round capture failed";
            return false;
        }
        const cudaError_t ie = cudaGraphInstantiate(&round.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            round.exec = nullptr;
            err = "batch round instantiation failed";
            return false;
        }
        return true;
    }
};

extern "C" {

fullmag_fdm_batch *fullmag_fdm_batch_create(const fullmag_fdm_plan_desc *plans, uint32_t count) {
    if (!plans || count == 0) return nullptr;
    auto *b = new (std::nothrow) FdmBatch();
    if (!b) return nullptr;
    b->items.reserve(count);
    for (uint32_t i = 0; i < count; ++i) {
        Engine *e = new (std::nothrow) Engine();
        if (!e) {
            b->last_error = "out of host memory";
            break;
        }
        b->items.push_back(e);
        if (!e->setup(&plans[i]) || !e->upload<double>(plans[i].initial_magnetization_xyz) || !e->eval_state(false)) {
            b->last_error = "problem " + std::to_string(i) + ": " + e->last_error;
            break;
        }
        e->batch_tiling();
    }
    b->next_dt.assign(b->items.size(), 0.0);
    return reinterpret_cast<fullmag_fdm_batch *>(b);
}

const char *fullmag_fdm_batch_last_error(fullmag_fdm_batch *batch) {
    if (!batch) return "null batch";
    auto *b = reinterpret_cast<FdmBatch *>(batch);
    return b->last_error.empty() ? nullptr : b->last_error.c_str();
}

uint32_t fullmag_fdm_batch_size(fullmag_fdm_batch *batch) {
    return batch ? (uint32_t)reinterpret_cast<FdmBatch *>(batch)->items.size() : 0u;
}

// Batched-kernel path (all problems DP45 and small enough for the fused column
// passes).  Each round replays one graph for all unfinished problems, waits once,
// then applies the accept/reject rule per problem on the host.  Problems that reached
// t_end stay in the round's work tables with step size 0, which makes their row and
// column CTAs return at once, until the round is rebuilt without them (when a tenth
// of its members have finished).  Returns 1 when not batchable.
// Batched DP45 rounds: each graph launch runs BatchRound::kRounds rounds with the step
// control on the device (batch_control_kernel); the host reads the control state once per
// launch to see which problems reached t_end, and rebuilds the round for the remaining
// ones when fewer than 90 % of its members are still running.  Time to solution is taken
// at the end of the launch in which a problem finished.
static int batch_step_until_batched(FdmBatch *b, double t_end, double dt0, uint64_t *out_steps, uint64_t *out_wall_ns) {
    const size_t n = b->items.size();
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<uint64_t> steps0(n);
    std::vector<char> done(n, 0);
    std::vector<size_t> active;
    if (!b->bstream && cudaStreamCreateWithFlags(&b->bstream, cudaStreamNonBlocking) != cudaSuccess) {
        b->last_error = "cudaStreamCreate failed";
        return FULLMAG_FDM_ERR_CUDA;
    }
    // a round left by an earlier call hands its state back before anything is read
    std::string err0;
    if (!b->sync_states(err0)) {
        b->last_error = err0;
        return FULLMAG_FDM_ERR_CUDA;
    }
    b->round.release();
    for (size_t i = 0; i < n; ++i) {
        Engine *e = b->items[i];
        steps0[i] = e->step_count;
        if (!e->batch_prepare()) {
            b->last_error = "problem " + std::to_string(i) + ": " + e->last_error;
            return FULLMAG_FDM_ERR_CUDA;
        }
        if (b->next_dt[i] <= 0.0) b->next_dt[i] = dt0;
        if (e->time < t_end * (1.0 - 1e-12)) active.push_back(i);
        else {
            done[i] = 1;
            if (out_wall_ns) out_wall_ns[i] = 0;
        }
    }
    bool built = false;
    while (!active.empty()) {
        if (!built || active.size() * 10 < b->round.members.size() * 9) {
            std::string err;
            if (!b->build_round(active, t_end, err)) {
                if (!built) return 1;  // not batchable: caller falls back
                b->last_error = err;
                return FULLMAG_FDM_ERR_CUDA;
            }
            built = true;
        }
        if (cudaGraphLaunch(b->round.exec, b->bstream) != cudaSuccess || cudaStreamSynchronize(b->bstream) != cudaSuccess) {
            b->last_error = "batch round launch failed";
            return FULLMAG_FDM_ERR_CUDA;
        }
        const auto now = std::chrono::steady_clock::now();
        const std::vector<size_t> &mem = b->round.members;
        std::vector<size_t> still;
        for (size_t k = 0; k < mem.size(); ++k) {
            const size_t i = mem[k];
            if (done[i]) continue;
            b->items[i]->launches += (uint64_t)BatchRound::kRounds * (7 + (b->items[i]->demag ? 6 : 0) + 1);
            if (b->round.h_state[k].done) {
                done[i] = 1;
                if (out_wall_ns) out_wall_ns[i] = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(now - t0).count();
            } else {
                still.push_back(i);
            }
        }
        active.swap(still);
    }
    std::string err;
    if (!b->sync_states(err)) {
        b->last_error = err;
        return FULLMAG_FDM_ERR_CUDA;
    }
    for (size_t i = 0; i < n; ++i) {
        b->items[i]->k1_valid = true;
        if (out_steps) out_steps[i] = b->items[i]->step_count - steps0[i];
    }
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_batch_step_until(fullmag_fdm_batch *batch, double t_end, double dt0, uint64_t *out_steps,
                                 uint64_t *out_wall_ns) {
    auto *b = reinterpret_cast<FdmBatch *>(batch);
    if (!b || !b->last_error.empty()) return FULLMAG_FDM_ERR_INVALID;
    if (!(dt0 > 0.0) || !std::isfinite(t_end)) {
        b->last_error = "dt0 must be positive and t_end finite";
        return FULLMAG_FDM_ERR_INVALID;
    }
    bool all_dp45 = true;
    for (Engine *e : b->items) all_dp45 = all_dp45 && e->integrator == FULLMAG_FDM_INTEGRATOR_DP45 && e->use_graphs;
    const char *nog = std::getenv("FULLMAG_FDM_BATCH_NO_GRAPH");
    if (all_dp45 && !(nog && *nog && *nog != '0')) {
        const int rc = batch_step_until_batched(b, t_end, dt0, out_steps, out_wall_ns);
        if (rc != 1) return rc;
    }
    const size_t n = b->items.size();
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<uint64_t> steps0(n);
    std::vector<size_t> active;
    for (size_t i = 0; i < n; ++i) {
        steps0[i] = b->items[i]->step_count;
        if (b->items[i]->time < t_end * (1.0 - 1e-12)) active.push_back(i);
        else if (out_wall_ns) out_wall_ns[i] = 0;
        if (b->next_dt[i] <= 0.0) b->next_dt[i] = dt0;
    }
    std::vector<size_t> still;
    while (!active.empty()) {
        // issue one attempt for every unfinished problem, then collect
        for (size_t i : active) {
            Engine *e = b->items[i];
            const bool adaptive = e->adaptive();
            const double want = adaptive ? b->next_dt[i] : dt0;
            const double d = std::min(want, t_end - e->time);
            // ABM3 steps synchronously (its history rotates on the host after each step)
            const int rc = adaptive ? e->begin_dp45_attempt(d)
                                    : e->integrator == FULLMAG_FDM_INTEGRATOR_ABM3 ? e->step(d) : e->begin_fixed_step(d);
            if (rc != 0) {
                b->last_error = "problem " + std::to_string(i) + ": " + e->last_error;
                return FULLMAG_FDM_ERR_CUDA;
            }
        }
        still.clear();
        for (size_t i : active) {
            Engine *e = b->items[i];
            const bool adaptive = e->adaptive();
            double nd = b->next_dt[i];
            const int rc = adaptive ? e->finish_dp45_attempt(nd)
                                    : e->integrator == FULLMAG_FDM_INTEGRATOR_ABM3 ? 0 : e->finish_fixed_step();
            if (rc < 0) {
                b->last_error = "problem " + std::to_string(i) + ": " + e->last_error;
                return FULLMAG_FDM_ERR_CUDA;
            }
            if (adaptive) b->next_dt[i] = nd;
            if (e->time >= t_end * (1.0 - 1e-12)) {
                if (out_wall_ns)
                    out_wall_ns[i] = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
                                         std::chrono::steady_clock::now() - t0)
                                         .count();
            } else {
                still.push_back(i);
            }
        }
        active.swap(still);
    }
    for (size_t i = 0; i < n; ++i) {
        Engine *e = b->items[i];
        if (cudaStreamSynchronize(e->stream) != cudaSuccess) {
            b->last_error = "problem " + std::to_string(i) + ": stream sync failed";
            return FULLMAG_FDM_ERR_CUDA;
        }
        if (out_steps) out_steps[i] = e->step_count - steps0[i];
    }
    return FULLMAG_FDM_OK;
}

int fullmag_fdm_batch_get_stats(fullmag_fdm_batch *batch, uint32_t index, fullmag_fdm_step_stats *out_stats) {
    auto *b = reinterpret_cast<FdmBatch *>(batch);
    if (!b || !out_stats || index >= b->items.size()) return FULLMAG_FDM_ERR_INVALID;
    return fullmag_fdm_backend_snapshot_stats(reinterpret_cast<fullmag_fdm_backend *>(b->items[index]), out_stats);
}

int fullmag_fdm_batch_copy_field_f64(fullmag_fdm_batch *batch, uint32_t index, fullmag_fdm_observable observable,
                                     double *out_xyz, uint64_t out_len) {
    auto *b = reinterpret_cast<FdmBatch *>(batch);
    if (!b || index >= b->items.size()) return FULLMAG_FDM_ERR_INVALID;
    return fullmag_fdm_backend_copy_field_f64(reinterpret_cast<fullmag_fdm_backend *>(b->items[index]), observable,
                                              out_xyz, out_len);
}

void fullmag_fdm_batch_destroy(fullmag_fdm_batch *batch) { delete reinterpret_cast<FdmBatch *>(batch); }

}  // extern "C"
