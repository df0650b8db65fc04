"""Throughput of the FDM LLG step on one GB300 (cell-steps/s), one JSON line.

Default workload: the large 3-D roofline volume -- 256x256x64 cells of 2 nm cubes,
Ms = 1.4e6 A/m, A = 2.1e-11 J/m, cubic K1 = -4.8e4 J/m^3 along (100)/(010)/(001),
alpha = 0.01, open boundaries, m0 = seeded random unit vectors smoothed by three
6-neighbour box-filter passes and renormalised, RK4 with dt = 2e-14 s.  Inputs are
synthetic (seeded) with exactly these shapes and parameters; the state plus the
spectra (~0.9 GB) exceed the 129 MB L2, so no extra flush is needed between steps.

value : device time (CUDA events on the engine's stream) of K steps through
        fullmag_fdm_backend_step with the state resident in HBM.
e2e   : the same metric, wall clock, through the C ABI with host buffers:
        upload_magnetization_f64 (AoS host array) + K x step (stats to the host
        every step) + copy_field_f64(M) back to the host.
--impl reference : the FP64 C restatement of the reference CPU engine (oracle/),
        OpenMP over all host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

MU0 = 4e-7 * np.pi
METRIC = "cell-steps/s per GB300 (fused FP32 engine, FP64 Newell/reductions)"

# Algorithmic bytes per cell-step, compulsory-traffic model v1 (fused 3-pass design):
# T(a) = 12(1+a) + 12 + 4S + K + 12 + 12 per evaluation with a earlier stages,
# S = 24 (nx+1)/nx, K = kernel bytes per cell; RK4 = T(0) + 3T(1) + 72.
def model_bytes_per_cell_step(nx, ny, nz, integrator="rk4"):
    S = 24.0 * (nx + 1) / nx
    n = nx * ny * nz
    if nz == 1:
        K = 4 * 4.0 * (nx + 1) * (ny + 1) / n
    else:
        K = 6 * 4.0 * (nx + 1) * (ny + 1) * (nz + 1) / n

    def T(a):
        return 12 * (1 + a) + 12 + 4 * S + K + 12 + 12

    if integrator == "rk4":
        return T(0) + 3 * T(1) + 72
    if integrator == "heun":
        return T(0) + T(1) + 48
    return sum(T(a) for a in (1, 2, 3, 4, 5, 5)) + 72


def kernel_bytes_per_launch(kind, nx, ny, nz, padded):
    """Algorithmic HBM bytes of one launch of a column pass: every spectrum element it
    owns read and written once, every kernel value read once (FP32 complex = 8 B,
    real kernel = 4 B).  Units: the X spectrum has 3 x nz x ny x nkx elements, the Y
    spectrum 3 x nz x py x nkx, the octant kernel ncomp x nkz x nky x nkx values."""
    px, py, pz = padded
    nkx, nky, nkz = px // 2 + 1, py // 2 + 1, pz // 2 + 1
    xs = 3 * nz * ny * nkx * 8
    ys = 3 * nz * py * nkx * 8
    if kind == "z_convolve":
        return 2 * ys + 6 * nkz * nky * nkx * 4
    if kind in ("y_forward", "y_inverse"):
        return xs + ys
    if kind == "yz_convolve":
        return 2 * xs + 6 * nkz * nky * nkx * 4
    if kind == "y_convolve_2d":
        return 2 * xs + 4 * nky * nkx * 4
    return None


def row_pass_bytes_per_launch(integrator, nx, ny, nz, demag=True):
    """Average algorithmic bytes of one row-pass launch over a fixed step at a repeated
    dt.  Per cell: state / stage vectors 12 B each, the X half spectrum S = 24 (nx + 1) / nx
    B (read before and written after each evaluation).  RK4 passes: (2), (3) inverse x,
    y_s, m0 -> k_s, y_{s+1}, forward x: 48 + 2S; (4) inverse x, y3, m0, k1..k3 -> m',
    forward x: 72 + 2S; (5) inverse x, m' -> k1' (+ statistics), the next step's first
    stage input N(m' + dt/2 k1'), forward x: 36 + 2S (the first pass of the next step is
    folded into it).  Heun: 60 + 2S, 36 + 2S."""
    n = nx * ny * nz
    S = 24.0 * (nx + 1) / nx if demag else 0.0
    if integrator == "rk4":
        per_cell = [48 + 2 * S, 48 + 2 * S, 72 + 2 * S, 36 + 2 * S]
    elif integrator == "dp45":
        # first pass m0 + k1 -> y2; stages s = 1..5 read y_s, m0 and s earlier k's, write
        # k_s and y_{s+1}; the last pass writes k7 and reads the 7 k's of the error norm
        per_cell = [36 + S] + [48 + 12 * s + 2 * S for s in range(1, 6)] + [108 + S]
    else:
        per_cell = [60 + 2 * S, 36 + 2 * S]
    return sum(per_cell) / len(per_cell) * n


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu capture of
# the timed steps of each workload
NCU_TRAFFIC = {("volume_256x256x64_rk4", "z_convolve"): 453.0e6, ("volume_256x256x64_rk4", "y_inverse"): 270.3e6,
               ("volume_256x256x64_rk4", "y_forward"): 241.1e6, ("volume_256x256x64_rk4", "row_pass"): 377.8e6,
               # the extra-field pass's stage launch
               ("volume_256x256x64_rk4_allterms", "extra_field"): 189.1e6}
# the column passes of the all-terms volume are the same launches on the same grid as the
# plain volume's (the extra terms enter only through the row pass's field map)
for _k in ("z_convolve", "y_forward", "y_inverse"):
    NCU_TRAFFIC[("volume_256x256x64_rk4_allterms", _k)] = NCU_TRAFFIC[("volume_256x256x64_rk4", _k)]


WORKLOADS = {
    "volume_256x256x64_rk4": dict(nx=256, ny=256, nz=64, d=2e-9, ms=1.4e6, a_ex=2.1e-11, alpha=0.01,
                                  kc1=-4.8e4, dt=2e-14, integrator="rk4", seed=3),
    "box_64x32x4_heun": dict(nx=64, ny=32, nz=4, d=4e-9, ms=8e5, a_ex=1.3e-11, alpha=0.5,
                             b_mt=(10.0, 5.0, 0.0), dt=5e-14, integrator="heun", seed=0),
    # the volume with every term of the extra-field pass: interfacial DMI, magnetoelastic
    # field, spin-orbit torque, a constant Oersted current, exchange with two regions and a
    # table, a per-cell Ku1 map and the thermal field at 300 K
    "volume_256x256x64_rk4_allterms": dict(nx=256, ny=256, nz=64, d=2e-9, ms=1.4e6, a_ex=2.1e-11, alpha=0.01,
                                           kc1=-4.8e4, ku1=4e3, dt=2e-14, integrator="rk4", seed=3, terms="all"),
    "film_256x64x1_rk4": dict(nx=256, ny=64, nz=1, d=4e-9, ms=8e5, a_ex=1.3e-11, alpha=0.05,
                              b_mt=(5.0, 0.0, 0.0), dt=5e-14, integrator="rk4", seed=2),
    # thin film, adaptive Dormand-Prince (max error 1e-5), Ku = 5e3 J/m^3 along x, driven at
    # (-24.6, 4.3, 0) mT from m0 = +x with a seeded uniform +-5 degree tilt per cell; every
    # step is offered dt = 2e-13 s and the controller may shrink it
    "film_512x128x1_dp45": dict(nx=512, ny=128, nz=1, d=(3.90625e-9, 3.90625e-9, 3e-9), ms=8e5, a_ex=1.3e-11,
                                alpha=0.02, ku1=5e3, b_mt=(-24.6, 4.3, 0.0), dt=2e-13, integrator="dp45",
                                max_error=1e-5, m0="tilt5", seed=4),
    # thin film periodic in x and y (the reference CPU engine's periodic boundaries: unpadded
    # transforms, the truncated image-sum demag kernel with 10 images per periodic axis)
    "film_256x256x1_periodic_rk4": dict(nx=256, ny=256, nz=1, d=(4e-9, 4e-9, 2e-9), ms=8e5, a_ex=1.3e-11,
                                        alpha=0.02, b_mt=(0.0, 0.0, 20.0), dt=5e-14, integrator="rk4", seed=6,
                                        periodic=(1, 1, 0), images=(10, 10, 0)),
}
DEFAULT_WORKLOAD = "volume_256x256x64_rk4"
SWEEP_WORKLOAD = "sweep_384_films_dp45"


def sweep_plans(count=384, seed=1):
    """Batched-sweep workload: independent films, grid and material drawn from `seed`:
    nx in {16..256}, ny in {16..128}, nz in {1,2,4}, 4 nm cells, Ms ~ U[4e5,1.2e6] A/m,
    A ~ U[5e-12,2e-11] J/m, alpha ~ U[0.005,0.1], |B| ~ U[0,100] mT at a uniform in-plane
    angle, random unit m0; Dormand-Prince with max error 1e-5."""
    from fullmag_gb300 import _abi
    rng = np.random.default_rng(seed)
    plans = []
    for _ in range(count):
        nx = int(rng.integers(16, 257))
        ny = int(rng.integers(16, 129))
        nz = int(rng.choice([1, 2, 4]))
        ms = float(rng.uniform(4e5, 1.2e6))
        a_ex = float(rng.uniform(5e-12, 2e-11))
        alpha = float(rng.uniform(0.005, 0.1))
        bmag = float(rng.uniform(0.0, 100.0)) * 1e-3
        ang = float(rng.uniform(0.0, 2 * np.pi))
        m0 = rng.standard_normal((nx * ny * nz, 3))
        m0 /= np.linalg.norm(m0, axis=1, keepdims=True)
        plans.append(dict(nx=nx, ny=ny, nz=nz, dx=4e-9, dy=4e-9, dz=4e-9, ms=ms, a_ex=a_ex, alpha=alpha,
                          gamma=2.211e5, m0=m0, h_ext=(bmag * np.cos(ang) / MU0, bmag * np.sin(ang) / MU0, 0.0),
                          integrator=_abi.INTEGRATOR_DP45, adaptive_max_error=1e-5))
    return plans


def shard_by_cost(costs, world):
    """Cost-balanced assignment of independent problems to ranks (longest processing
    time first): each problem goes to the rank with the least assigned cost.  Returns
    one sorted index list per rank."""
    loads = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: -costs[k]):
        r = min(range(world), key=lambda q: loads[q])
        parts[r].append(i)
        loads[r] += costs[i]
    return [sorted(p) for p in parts]


def run_sweep(args, rank=0, world=1, dist=None):
    """problems/s of the batched sweep vs one problem at a time (a subsample solved
    sequentially through fullmag_fdm_backend_step), with p50/p99 time-to-solution.
    With N ranks the set holds N x count films (weak scaling: count per GPU), sharded by
    estimated cost n log2 n with no collective on the data path; the time is the
    slowest rank's."""
    from fullmag_gb300 import FdmBackend, FdmBatch
    from fullmag_gb300.build import build
    build()
    count = args.sweep_count
    t_end, dt0 = args.sweep_t_end, 1e-13
    all_plans = sweep_plans(count * world)
    cells = [p["nx"] * p["ny"] * p["nz"] for p in all_plans]
    mine = shard_by_cost([c * np.log2(c) for c in cells], world)[rank]
    plans = [all_plans[i] for i in mine]
    t0 = time.perf_counter()
    batch = FdmBatch(plans)
    t_setup = time.perf_counter() - t0
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    steps, wall = batch.step_until(t_end, dt0)
    t_batch = time.perf_counter() - t0
    batch.close()
    if dist:
        t_batch = max_over_ranks(t_batch, dist, "cuda")
    if rank != 0:
        return
    seq_n = min(args.sweep_sequential, len(plans))
    seq_times = []
    stride = max(1, len(plans) // seq_n)  # evenly strided sample: unbiased estimate of the mean solve time
    for kw in plans[::stride][:seq_n]:
        be = FdmBackend(**kw)
        ts = time.perf_counter()
        t, dt = 0.0, dt0
        while t < t_end * (1 - 1e-12):
            st = be.step(min(dt, t_end - t))
            t, dt = st["time_seconds"], st["suggested_next_dt"]
        seq_times.append(time.perf_counter() - ts)
        be.close()
    seq_rate = seq_n / sum(seq_times)
    total = len(all_plans)
    value = whole_job_rate(1, total, t_batch)
    out = {"metric": "problems/s (batched sweep, DP45 to %.2g s)" % t_end, "value": value,
           "unit": "problems/s", "n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": SWEEP_WORKLOAD, "problems": total, "problems_per_gpu": count, "t_end": t_end,
                      "dt0": dt0, "cells_total": int(sum(cells)), "rank0_accepted_steps": int(steps.sum()),
                      "sharding": "cost-balanced (n log2 n), no collective" if world > 1 else "single"},
           "batch_wall_s": t_batch, "setup_s": t_setup,
           "time_to_solution_s": {"p50": float(np.percentile(wall, 50)), "p99": float(np.percentile(wall, 99))},
           "sequential": {"problems": seq_n, "sample": f"every {stride}th problem", "problems_per_s": seq_rate,
                          "time_to_solution_s": {"p50": float(np.percentile(seq_times, 50)),
                                                 "p99": float(np.percentile(seq_times, 99))}},
           "speedup_vs_sequential": (value / world) / seq_rate}
    print(json.dumps(out), flush=True)


def run_sweep_reference(args, world=1):
    """The reference's way to run a sweep: one problem after another on the CPU engine
    (the FP64 oracle, all host threads), each to t_end with its own DP45 controller
    (dt0 = 1e-13 s, max error 1e-5).  Bounded: evenly strided problems until about 150 s
    of CPU time; problems/s over the problems solved."""
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    plans = sweep_plans(args.sweep_count)
    t_end, budget = args.sweep_t_end, 150.0
    stride = max(1, len(plans) // 16)
    solved, spent = 0, 0.0
    for kw in plans[::stride]:
        p = dict(kw)
        p.pop("integrator")
        me = p.pop("adaptive_max_error")
        pr = O.Problem(**p, integrator=O.DP45, max_error=me)
        t0 = time.perf_counter()
        t, dt = 0.0, 1e-13
        while t < t_end * (1 - 1e-12):
            st = pr.step(min(dt, t_end - t))
            t, dt = st["time"], st["suggested_next_dt"]
            if time.perf_counter() - t0 > budget:
                break
        el = time.perf_counter() - t0
        pr.close()
        if t < t_end * (1 - 1e-12):
            break  # this problem alone exceeds the budget: not counted
        solved += 1
        spent += el
        if spent > budget:
            break
    v = solved / spent if spent > 0 else 0.0
    print(json.dumps({"metric": "problems/s (batched sweep, DP45 to %.2g s)" % t_end, "value": v,
                      "unit": "problems/s", "n_gpus": world, "higher_is_better": True, "dtype": "f64",
                      "data": "synthetic (seeded)", "impl": "reference",
                      "config": {"workload": SWEEP_WORKLOAD, "problems_solved": solved, "stride": stride,
                                 "threads": threads},
                      "cpu_baseline": {"value": v, "unit": "problems/s", "cores": threads, "kind": "port",
                                       "sample": f"{solved} problems, every {stride}th, solved one at a time"},
                      "e2e": {"value": v, "unit": "problems/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


ADJOINT_WORKLOAD = "adjoint_256x64x1_rk4_4000"


def adjoint_problem(nx=256, ny=64, seed=2):
    """Inverse-design workload: a 256x64x1 film of 4 nm cells, Ms 8e5 A/m, A 1.3e-11 J/m,
    alpha 0.05, uniform (5, 0, 0) mT plus a trainable in-plane field map B(x, y)
    initialised N(0, 2 mT) (FP32, seeded), m0 = +x, and a smooth target: +x plus eight
    seeded 2-D Gaussian bumps in m_y, renormalised."""
    from fullmag_gb300 import _abi
    rng = np.random.default_rng(seed)
    n = nx * ny
    bmap = rng.normal(0.0, 2e-3, size=(n, 2)).astype(np.float32)
    yy, xx = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    bump = np.zeros((ny, nx))
    for _ in range(8):
        cx, cy = rng.uniform(0, nx), rng.uniform(0, ny)
        sig = rng.uniform(4.0, 16.0)
        amp = rng.uniform(0.5, 1.5) * rng.choice([-1.0, 1.0])
        bump += amp * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (2 * sig ** 2))
    target = np.zeros((n, 3))
    target[:, 0] = 1.0
    target[:, 1] = bump.reshape(-1)
    target /= np.linalg.norm(target, axis=1, keepdims=True)
    m0 = np.tile([1.0, 0.0, 0.0], (n, 1))
    kw = dict(nx=nx, ny=ny, nz=1, dx=4e-9, dy=4e-9, dz=4e-9, ms=8e5, a_ex=1.3e-11, alpha=0.05, gamma=2.211e5,
              m0=m0, h_ext=(5e-3 / MU0, 0.0, 0.0), integrator=_abi.INTEGRATOR_RK4)
    return kw, bmap, target


def run_adjoint(args):
    """Gradients/s of mean |m_T - m*|^2 with respect to the field map through the
    torch.autograd.Function (4000 RK4 steps, sqrt(N) checkpoints), wall clock with host
    tensors in and out, plus the forward-only time of the same 4000 steps."""
    import torch
    from fullmag_gb300 import FdmBackend
    from fullmag_gb300.adjoint import rk4_final_state
    from fullmag_gb300.build import build
    build()
    kw, bmap, target = adjoint_problem()
    n = kw["nx"] * kw["ny"]
    dt, nsteps = 5e-14, args.adjoint_steps
    be = FdmBackend(**kw)
    m0 = torch.tensor(kw["m0"], dtype=torch.float64)
    tgt = torch.tensor(target, dtype=torch.float64)
    b = torch.tensor(bmap, requires_grad=True)
    free0 = torch.cuda.mem_get_info()[0]

    split = [0.0, 0.0]  # seconds in the checkpointed forward, in the backward sweep

    def gradient():
        b.grad = None
        ta = time.perf_counter()
        m_t = rk4_final_state(m0, b, be, dt, nsteps)
        loss = ((m_t - tgt) ** 2).mean()
        tb = time.perf_counter()
        loss.backward()
        tc = time.perf_counter()
        split[0] += tb - ta
        split[1] += tc - tb
        return float(loss.detach())

    for _ in range(max(1, args.warmup)):
        loss = gradient()
    free1 = torch.cuda.mem_get_info()[0]
    split[0] = split[1] = 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        loss = gradient()
    t_grad = (time.perf_counter() - t0) / args.steps
    t_fwd_ck, t_bwd = split[0] / args.steps, split[1] / args.steps
    g = b.grad.numpy().copy()
    # forward-only cost of the same run (CUDA-graph fixed steps), for the cost ratio
    be.upload(kw["m0"])
    be.step_many(dt, nsteps)
    t0 = time.perf_counter()
    be.upload(kw["m0"])
    be.step_many(dt, nsteps)
    t_fwd = time.perf_counter() - t0
    launches = be.launch_count()
    be.close()
    C = int(np.ceil(np.sqrt(nsteps)))
    state = 12 * n  # bytes of one FP32 SoA state
    out = {"metric": "adjoint gradients/s (d loss / d field map, %d RK4 steps)" % nsteps, "value": 1.0 / t_grad,
           "unit": "gradients/s", "n_gpus": 1, "steps": args.steps, "warmup": max(1, args.warmup),
           "ms_per_step": 1e3 * t_grad, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": ADJOINT_WORKLOAD, "grid": [kw["nx"], kw["ny"], 1], "dt": dt, "rk4_steps": nsteps,
                      "checkpoint_every": C},
           "e2e": {"value": 1.0 / t_grad, "unit": "gradients/s", "h2d_bytes_per_step": 24 * n + 8 * 2 * n + 24 * n,
                   "d2h_bytes_per_step": 24 * n + 24 * n + 24 * n},
           "forward_only_s": t_fwd, "gradient_s": t_grad, "gradient_over_forward": t_grad / t_fwd,
           "checkpointed_forward_s": t_fwd_ck, "backward_s": t_bwd, "backward_over_forward": t_bwd / t_fwd,
           "memory": {"checkpoints_bytes": state * ((nsteps + C - 1) // C), "segment_bytes": state * 12 * C,
                      "work_bytes": state * 12, "device_bytes_observed": int(free0 - free1),
                      "store_everything_bytes": state * 12 * nsteps},
           "loss": loss, "grad_abs_max": float(np.abs(g).max()), "engine_launches_total": launches}
    print(json.dumps(out), flush=True)


def smoothed_random_unit(nx, ny, nz, seed, passes=3):
    rng = np.random.default_rng(seed)
    m = rng.standard_normal((nz, ny, nx, 3))
    m /= np.linalg.norm(m, axis=-1, keepdims=True)
    for _ in range(passes):
        acc = m.copy()
        cnt = np.ones((nz, ny, nx, 1))
        for ax in (0, 1, 2):
            for sh in (1, -1):
                r = np.roll(m, sh, axis=ax)
                valid = np.ones((nz, ny, nx, 1))
                idx = [slice(None)] * 4
                idx[ax] = 0 if sh == 1 else -1
                r[tuple(idx)] = 0.0
                valid[tuple(idx)] = 0.0
                acc += r
                cnt += valid
        m = acc / cnt
        m /= np.linalg.norm(m, axis=-1, keepdims=True)
    return m.reshape(-1, 3)


def tilted_x(n, seed, deg=5.0):
    """+x with a seeded uniform tilt of up to `deg` degrees per cell (uniform azimuth)."""
    rng = np.random.default_rng(seed)
    th = np.deg2rad(deg) * rng.uniform(0.0, 1.0, n)
    ph = rng.uniform(0.0, 2 * np.pi, n)
    return np.stack([np.cos(th), np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph)], axis=1)


def plan_kwargs(w):
    from fullmag_gb300 import _abi
    d = w["d"] if isinstance(w["d"], tuple) else (w["d"],) * 3
    n = w["nx"] * w["ny"] * w["nz"]
    m0 = tilted_x(n, w["seed"]) if w.get("m0") == "tilt5" else smoothed_random_unit(w["nx"], w["ny"], w["nz"], w["seed"])
    kw = dict(nx=w["nx"], ny=w["ny"], nz=w["nz"], dx=d[0], dy=d[1], dz=d[2], ms=w["ms"],
              a_ex=w["a_ex"], alpha=w["alpha"], gamma=2.211e5, m0=m0)
    if "b_mt" in w:
        kw["h_ext"] = tuple(b * 1e-3 / MU0 for b in w["b_mt"])
    if "kc1" in w:
        kw.update(kc1=w["kc1"], c1=(1.0, 0.0, 0.0), c2=(0.0, 1.0, 0.0))
    if "ku1" in w:
        kw.update(ku1=w["ku1"], u_axis=(1.0, 0.0, 0.0))
    if w.get("terms") == "all":
        kw.update(extra_terms(w["nx"], w["ny"], w["nz"], d, w["seed"]))
    if "periodic" in w:
        kw.update(periodic=w["periodic"], image_counts=w.get("images"))
    integ = {"rk4": _abi.INTEGRATOR_RK4, "heun": _abi.INTEGRATOR_HEUN, "dp45": _abi.INTEGRATOR_DP45}[w["integrator"]]
    return kw, integ


def extra_terms(nx, ny, nz, d, seed):
    """Plan keywords of every extra-field term, sized for an (nx, ny, nz) grid of cells d."""
    n = nx * ny * nz
    rng = np.random.default_rng(seed + 100)
    x = np.tile(np.arange(nx, dtype=np.int64), ny * nz)
    reg = np.where(x < nx // 2, 1, 2).astype(np.uint32)
    lut = np.zeros((256, 256))
    lut[1, 1], lut[2, 2], lut[1, 2], lut[2, 1] = 2.1e-11, 1.5e-11, 0.5e-11, 0.5e-11
    return dict(dmi_d_interfacial=1.5e-3, mel_b1=-3e6, mel_b2=2e6, mel_strain=(1e-3, -5e-4, 2e-4, 1e-4, 0.0, 3e-4),
                sot_je=1e11, sot_xi_dl=0.2, sot_xi_fl=0.05, sot_sigma=(0.0, 1.0, 0.0), sot_thickness=2e-9,
                oersted_current=1e-3, oersted_radius=0.25 * nx * d[0],
                oersted_center=(0.5 * nx * d[0], 0.5 * ny * d[1], 0.0),
                region_mask=reg, exchange_lut=lut, ku1_field=rng.uniform(2e3, 6e3, n), temperature=300.0)


def extra_bytes_per_cell(w):
    """Algorithmic bytes per cell of one extra-field launch: m read and H_extra written
    (12 + 12), plus the region id (1, one byte per cell on the device), the Ku1 map (4)
    and the Oersted field (12) when present; the neighbour reads of DMI and exchange come
    from the same m rows."""
    if w.get("terms") != "all":
        return None
    return 12 + 12 + 1 + 4 + 12


def gpu_plan(w):
    """Plan keywords of the GPU engine (adds the DP45 error bound)."""
    kw, integ = plan_kwargs(w)
    if w["integrator"] == "dp45":
        kw["adaptive_max_error"] = w["max_error"]
    return kw, integ


def oracle_problem(O, w, sx, sy, sz):
    """The oracle on a (sx, sy, sz) sample of the workload."""
    kw, _ = plan_kwargs(dict(w, nx=sx, ny=sy, nz=sz))
    integ = {"rk4": O.RK4, "heun": O.HEUN, "dp45": O.DP45}[w["integrator"]]
    extra = {"max_error": w["max_error"]} if w["integrator"] == "dp45" else {}
    return O.Problem(**kw, integrator=integ, **extra)


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x, dist, device):
    """The largest value of x over all ranks (the slowest replica's time); x itself
    without a process group.  `device` is "cuda" under NCCL, "cpu" under gloo."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, units_per_rank, seconds):
    """Aggregate throughput of `world` replicas that each processed `units_per_rank`
    units, timed by the slowest one (the path does not shard: N independent replicas)."""
    return world * units_per_rank / seconds


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def oracle_sample_grid(O, w, steps, budget):
    """Largest sample of the workload's grid whose probe step says that `steps` steps
    fit `budget` seconds of CPU time: the full grid first, then halved per axis (cell-
    steps/s is per cell, so the sample size sets only the run time).  Returns the
    oracle problem (one probe step taken) and its grid."""
    sx, sy, sz = w["nx"], w["ny"], w["nz"]
    while True:
        pr = oracle_problem(O, w, sx, sy, sz)
        t0 = time.perf_counter()
        pr.step(w["dt"])  # probe step, not counted
        t_probe = time.perf_counter() - t0
        if steps * t_probe <= budget or sx * sy * sz <= 4096:
            return pr, (sx, sy, sz)
        pr.close()
        sx, sy, sz = max(sx // 2, 8), max(sy // 2, 8), max(sz // 2, 1)


def cpu_baseline(w, threads, h_eff_gpu=None):
    """FP64 oracle (C restatement of the reference CPU engine) on a bounded sample of
    the workload: the full grid when 3 steps fit about 30 s of CPU time, else the grid
    halved per axis until they do; up to 3 timed steps (10 s at most) after the probe
    step.  With the GPU's H_eff of the initial state (h_eff_gpu) and a full-grid sample
    it also returns the relative L2 error of that H_eff against the oracle's FP64 one;
    that comparison runs before the timed steps and is not timed."""
    from oracle import oracle as O
    O.build()
    O.set_threads(threads)
    heff_err = None
    full = (w["nx"], w["ny"], w["nz"])
    if h_eff_gpu is not None:
        pr = oracle_problem(O, w, *full)
        h_ref = pr.fields()["h_eff"]
        heff_err = float(np.linalg.norm(h_eff_gpu.reshape(-1) - h_ref.reshape(-1)) / np.linalg.norm(h_ref))
        del h_ref
        t0 = time.perf_counter()
        pr.step(w["dt"])  # probe step
        if 3 * (time.perf_counter() - t0) > 30.0:
            pr.close()
            pr, grid = oracle_sample_grid(O, w, 3, 30.0)
        else:
            grid = full
    else:
        pr, grid = oracle_sample_grid(O, w, 3, 30.0)
    t0 = time.perf_counter()
    steps = 0
    while True:
        pr.step(w["dt"])
        steps += 1
        if time.perf_counter() - t0 > 10.0 or steps >= 3:
            break
    el = time.perf_counter() - t0
    pr.close()
    sx, sy, sz = grid
    out = {"value": sx * sy * sz * steps / el, "unit": "cell-steps/s", "cores": threads, "kind": "port",
           "sample": f"{steps} {w['integrator'].upper()} step(s) of {sx}x{sy}x{sz} (same physics, FP64, "
                     f"after 1 untimed step), wall clock",
           "same_grid": tuple(grid) == full}
    return out, heff_err


def extra_roofline(w, n, ktimes, peak, workload):
    """HBM roofline of the extra-field pass (None when the workload has no extra terms)."""
    bpc = extra_bytes_per_cell(w)
    ms, cnt = ktimes.get("extra_field", (0.0, 0))
    if bpc is None or not cnt:
        return None
    avg_s = ms / cnt * 1e-3
    ach = bpc * n / avg_s / 1e9
    return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak if peak else None,
            "traffic": NCU_TRAFFIC.get((workload, "extra_field")), "kernel": "extra_field",
            "bytes_per_launch": bpc * n, "avg_launch_ms": avg_s * 1e3,
            "launches_timed": cnt, "note": f"{bpc} B/cell algorithmic; CUDA events per launch"}


def run_reference(args, w, name, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    from oracle import oracle as O
    O.build()
    O.set_threads(threads)
    # bounded sample: the full grid when warm-up + timed steps fit ~150 s of CPU time,
    # else the grid halved per axis until they do
    pr, (sx, sy, sz) = oracle_sample_grid(O, w, args.steps + args.warmup, 150.0)
    for _ in range(args.warmup):
        pr.step(w["dt"])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pr.step(w["dt"])
    el = time.perf_counter() - t0
    cells = sx * sy * sz
    v = cells * args.steps / el
    out = {"metric": METRIC, "value": v, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
           "impl": "reference",
           "config": {"workload": name, "grid": [w["nx"], w["ny"], w["nz"]], "sample_grid": [sx, sy, sz],
                      "same_grid": (sx, sy, sz) == (w["nx"], w["ny"], w["nz"]), "threads": threads},
           "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                            "sample": f"{args.steps} step(s) of {sx}x{sy}x{sz} per timed step set"},
           "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def relaunch_ranks(n):
    """`bench.py --gpus N` started as one process: run the same command as N ranks (one
    per GPU, LOCAL_RANK selects the device) under torch.distributed.run on 127.0.0.1 and
    return its exit status.  Every rank prints nothing but rank 0's single line."""
    import socket
    with socket.socket() as sock:
        sock.bind(("127.0.0.1", 0))
        port = sock.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={port}", str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.run(cmd).returncode


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default 300; 5 gradients for the adjoint)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS) + [SWEEP_WORKLOAD, ADJOINT_WORKLOAD])
    ap.add_argument("--adjoint-steps", type=int, default=4000)
    ap.add_argument("--sweep-count", type=int, default=384)
    ap.add_argument("--sweep-t-end", type=float, default=0.5e-9)
    ap.add_argument("--sweep-sequential", type=int, default=32, help="problems solved one at a time for the baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the cuFFT + unfused baseline leg")
    ap.add_argument("--profile", action="store_true", help="timed steps only: no e2e leg, no CPU baseline")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 5 if args.workload == ADJOINT_WORKLOAD else 300
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup

    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_ranks(args.gpus))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == SWEEP_WORKLOAD:
        if args.impl == "reference":
            if rank == 0:
                run_sweep_reference(args, world)
            return
        dist = None
        if world > 1:
            import torch
            import torch.distributed as dist
            torch.cuda.set_device(local)
            os.environ["FULLMAG_FDM_GPU_INDEX"] = str(local)
            dist.init_process_group("nccl")
        run_sweep(args, rank, world, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload == ADJOINT_WORKLOAD:
        if rank == 0:
            if args.impl == "reference":
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no adjoint (gradients "
                                  "of an LLG run are a capability only this engine provides)"}), flush=True)
            else:
                run_adjoint(args)
        return
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, w, args.workload, rank, world)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    os.environ["FULLMAG_FDM_GPU_INDEX"] = str(local if world > 1 else int(os.environ.get("FULLMAG_FDM_GPU_INDEX", "0")))
    torch.cuda.set_device(int(os.environ["FULLMAG_FDM_GPU_INDEX"]))

    from fullmag_gb300 import FdmBackend, _abi
    from fullmag_gb300.build import build
    build()
    kw, integ = gpu_plan(w)
    n = w["nx"] * w["ny"] * w["nz"]
    dt = w["dt"]

    be = FdmBackend(**kw, integrator=integ)
    # H_eff of the initial state (create ends with the observables refreshed), kept for the
    # comparison with the FP64 oracle in the CPU-baseline leg, after the timed region
    want_heff = rank == 0 and not args.no_cpu_baseline and world == 1 and not args.profile
    h_eff0 = be.copy_field(_abi.OBSERVABLE_H_EFF) if want_heff else None
    stream = torch.cuda.ExternalStream(be.stream())
    # the sampler starts before the warm-up so that nvidia-smi's own start-up does not
    # overlap the timed steps; its samples cover the warm-up and the timed region
    clocks = ClockSampler(int(os.environ["FULLMAG_FDM_GPU_INDEX"]))
    clocks.start()
    time.sleep(0.5)
    for _ in range(args.warmup):
        be.step(dt)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = be.launch_count()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        st = be.step(dt)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    launches = be.launch_count() - l0
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    if dist:
        ms = max_over_ranks(ms, dist, "cuda")
        dist.barrier()
    ms_per_step = ms / args.steps
    value = whole_job_rate(world, n * args.steps, ms * 1e-3)

    # ---- e2e through the C ABI with host buffers ----
    if args.profile:
        tun = be.tuning()
        be.close()
        print(json.dumps({"workload": args.workload, "profile_ms_per_step": ms_per_step, "gpu_launches": launches,
                          "tuning": tun}), flush=True)
        return
    m_host = np.ascontiguousarray(kw["m0"], dtype=np.float64)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    be.upload(m_host)
    for _ in range(args.steps):
        be.step(dt)
    m_out = be.copy_field(_abi.OBSERVABLE_M)
    t_e2e = time.perf_counter() - t0
    if dist:
        t_e2e = max_over_ranks(t_e2e, dist, "cuda")
    e2e = whole_job_rate(world, n * args.steps, t_e2e)
    h2d = 24.0 * n / args.steps
    d2h = 24.0 * n / args.steps + 120.0

    # ---- per-kernel CUDA-event timing of the same step (launch by launch, no graph) ----
    kt_steps = min(args.steps, 50)
    be.set_kernel_timing(True)
    for _ in range(kt_steps):
        be.step(dt)
    ktimes = be.kernel_times()
    be.set_kernel_timing(False)
    kt_total = sum(v[0] for v in ktimes.values())
    dominant = max(ktimes, key=lambda k: ktimes[k][0])
    dom_ms, dom_n = ktimes[dominant]
    dom_avg_s = dom_ms / max(dom_n, 1) * 1e-3
    padded = be.fft_shape()
    if dominant == "row_pass":
        dom_bytes = row_pass_bytes_per_launch(w["integrator"], w["nx"], w["ny"], w["nz"])
    else:
        dom_bytes = kernel_bytes_per_launch(dominant, w["nx"], w["ny"], w["nz"], padded)
    if not dom_avg_s > 0:
        dom_bytes = None  # no timed launches
    traffic = NCU_TRAFFIC.get((args.workload, dominant))

    peak, peak_kind = load_peaks()
    bpc = model_bytes_per_cell_step(w["nx"], w["ny"], w["nz"], w["integrator"])
    achieved = bpc * n / (ms_per_step * 1e-3) / 1e9
    dom_achieved = dom_bytes / dom_avg_s / 1e9 if dom_bytes else None
    out = {
        "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "grid": [w["nx"], w["ny"], w["nz"]], "integrator": w["integrator"],
                   "dt": dt, "padded": list(be.fft_shape()), "tuning": be.tuning(), "parallelism": "replicas" if world > 1 else "single",
                   "l2_flush": "none needed: working set > 129 MB L2"},
        "roofline": {"bound": "hbm", "achieved": dom_achieved, "peak": peak, "unit": "GB/s",
                     "frac": dom_achieved / peak if (peak and dom_achieved) else None, "traffic": traffic,
                     "kernel": dominant, "bytes_per_launch": dom_bytes, "avg_launch_ms": dom_avg_s * 1e3,
                     "launches_timed": dom_n, "share_of_step": dom_ms / kt_total if kt_total else None,
                     "note": f"dominant kernel, CUDA events per launch over {kt_steps} eager steps; "
                             f"peak {peak_kind} (copy bandwidth)"},
        "roofline_step": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak if peak else None,
                          "note": f"whole step, compulsory-traffic model v1 {bpc:.1f} B/cell-step"},
        "kernel_times_ms_per_launch": {k: (v[0] / v[1] if v[1] else None) for k, v in ktimes.items()},
        "roofline_extra": extra_roofline(w, n, ktimes, peak, args.workload),
        "e2e": {"value": e2e, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk,
        "final_total_energy_J": st["total_energy_joules"],
        "m_norm_max_dev": float(np.abs(np.linalg.norm(m_out, axis=1) - 1).max()),
    }
    be.close()
    # the plain path has Heun and RK4, open boundaries and none of the extra-field terms
    if not args.no_plain and w["integrator"] != "dp45" and w.get("terms") is None and "periodic" not in w:
        # the cuFFT + unfused path (reference per-step kernel structure), same workload;
        # each of its steps ends in blocking copies, so wall clock is its device time
        from fullmag_gb300.plain import PlainBaseline
        pb = PlainBaseline(**kw, integrator=integ)
        for _ in range(2):
            pb.step(dt)
        kp = min(args.steps, 30)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(kp):
            pb.step(dt)
        tp = time.perf_counter() - t0
        m_plain = pb.magnetization()
        pb.close()
        out["plain"] = {"value": n * kp / tp, "unit": "cell-steps/s", "ms_per_step": 1e3 * tp / kp, "steps": kp,
                        "kind": "repo-written cuFFT C2C + one kernel per operation (reference kernel sequence)"}
        out["fused_over_plain"] = value / out["plain"]["value"]
        del m_plain
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        out["cpu_baseline"], err = cpu_baseline(w, os.cpu_count() or 1, h_eff0)
        out["heff_rel_l2_vs_fp64"] = {"value": err, "step": 0, "grid": [w["nx"], w["ny"], w["nz"]],
                                      "bound": 1e-5, "oracle": "FP64 C restatement of the reference CPU engine"}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
