"""Python mirror of the reference's safe FDM wrapper.

Mirrors ``NativeFdmBackend`` (crates/fullmag-runner/src/native_fdm.rs:50-970): build a
``fullmag_fdm_plan_desc`` from plan parameters, create the backend, check
``last_error`` on a non-NULL handle (native_fdm.rs:477-492), step with interrupt
support (native_fdm.rs:516-569), copy fields as AoS (n, 3) arrays, upload and
refresh (native_fdm.rs:829-857) and destroy.  Everything runs through the C ABI of
``libfullmag_fdm.so``; there is no CPU path.  ``FdmBatch`` wraps the additive batched
sweep entry points.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from . import _abi
from ._abi import PlanDesc, StepStats

MU0 = 4.0e-7 * np.pi
DEFAULT_GAMMA = 2.211e5

_LIB = None


class FdmError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{message} (code {code})")
        self.code = code


class FdmInterrupted(FdmError):
    pass


def library_path() -> Path:
    env = os.environ.get("FULLMAG_FDM_LIB")
    if env:
        return Path(env)
    return Path(__file__).resolve().parent / "_build" / "libfullmag_fdm.so"


def load_library(build_if_missing: bool = True) -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = library_path()
        if not path.exists() and build_if_missing:
            from .build import build
            build()
        if not path.exists():
            raise FdmError(_abi.ERR_INTERNAL, f"libfullmag_fdm.so not found at {path}; run fullmag_gb300.build")
        _LIB = _abi.bind(C.CDLL(str(path)))
    return _LIB


library = load_library


def _dptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def make_plan(*, nx: int, ny: int, nz: int, dx: float, dy: float, dz: float,
              ms: float, a_ex: float, alpha: float, gamma: float = DEFAULT_GAMMA,
              m0: np.ndarray, integrator: int = _abi.INTEGRATOR_HEUN,
              enable_exchange: bool = True, enable_demag: bool = True,
              h_ext: Optional[Sequence[float]] = None, disable_precession: bool = False,
              ku1: Optional[float] = None, ku2: float = 0.0, u_axis=(0.0, 0.0, 1.0),
              kc1: Optional[float] = None, kc2: float = 0.0, kc3: float = 0.0,
              c1=(1.0, 0.0, 0.0), c2=(0.0, 1.0, 0.0),
              dmi_d_interfacial: Optional[float] = None, dmi_d_bulk: Optional[float] = None,
              mel_b1: Optional[float] = None, mel_b2: float = 0.0, mel_strain=(0.0,) * 6,
              current_density=(0.0, 0.0, 0.0), stt_degree: float = 0.0, stt_beta: float = 0.0,
              stt_p=(0.0, 0.0, 0.0), stt_lambda: float = 0.0, stt_epsilon_prime: float = 0.0,
              sot_je: Optional[float] = None, sot_xi_dl: float = 0.0, sot_xi_fl: float = 0.0,
              sot_sigma=(0.0, 0.0, 1.0), sot_thickness: float = 0.0,
              ku1_field: Optional[np.ndarray] = None, ku2_field: Optional[np.ndarray] = None,
              kc1_field: Optional[np.ndarray] = None, kc2_field: Optional[np.ndarray] = None,
              kc3_field: Optional[np.ndarray] = None,
              oersted_current: Optional[float] = None, oersted_radius: float = 0.0,
              oersted_center=(0.0, 0.0, 0.0), oersted_axis=(0.0, 0.0, 1.0), oersted_kind: int = 0,
              oersted_freq: float = 0.0, oersted_phase: float = 0.0, oersted_offset: float = 0.0,
              oersted_t_on: float = 0.0, oersted_t_off: float = 0.0,
              active_mask: Optional[np.ndarray] = None,
              region_mask: Optional[np.ndarray] = None, exchange_lut: Optional[np.ndarray] = None,
              temperature: float = 0.0,
              spectra: Optional[np.ndarray] = None,
              adaptive_max_error: float = 0.0, adaptive_dt_min: float = 0.0,
              adaptive_dt_max: float = 0.0, adaptive_headroom: float = 0.0,
              precision: int = _abi.PRECISION_SINGLE, boundary: Optional[dict] = None):
    """Fill a fullmag_fdm_plan_desc the way native_fdm.rs:132-499 does.

    ``boundary`` (double precision only) holds the boundary-correction geometry the
    runner computes (native_fdm.rs:379-468): ``tier`` (``_abi.BOUNDARY_VOLUME`` for T0
    face links, ``_abi.BOUNDARY_FULL`` for T1 distances), ``volume_fraction``, ``face``
    (six arrays +x -x +y -y +z -z) or ``delta`` (six arrays), ``phi_floor``,
    ``delta_min``, and optionally ``corr = (target_idx, source_idx, tensor)`` for the
    sparse demag correction.
    ``spectra`` is an optional (6, 2P) array of interleaved FP64 Newell spectra
    (xx yy zz xy xz yz) as the reference computes them on the host; when omitted the
    engine builds the tensor on the GPU.  Returns (plan, keepalive): the arrays in
    keepalive back the plan's pointers and must outlive the create call."""
    p = PlanDesc()
    keep = []
    p.grid.nx, p.grid.ny, p.grid.nz = nx, ny, nz
    p.grid.dx, p.grid.dy, p.grid.dz = dx, dy, dz
    p.material.saturation_magnetisation = ms
    p.material.exchange_stiffness = a_ex
    p.material.damping = alpha
    p.material.gyromagnetic_ratio = gamma
    p.precision = precision
    p.integrator = integrator
    p.disable_precession = int(disable_precession)
    p.temperature = temperature
    p.enable_exchange = int(enable_exchange)
    p.enable_demag = int(enable_demag)
    p.has_external_field = int(h_ext is not None)
    p.external_field_am[:] = list(h_ext) if h_ext is not None else [0.0, 0.0, 0.0]
    p.has_uniaxial_anisotropy = int(ku1 is not None)
    p.uniaxial_anisotropy_constant = ku1 or 0.0
    p.uniaxial_anisotropy_k2 = ku2
    p.anisotropy_axis[:] = list(u_axis)
    p.has_cubic_anisotropy = int(kc1 is not None)
    p.cubic_Kc1, p.cubic_Kc2, p.cubic_Kc3 = (kc1 or 0.0), kc2, kc3
    p.cubic_axis1[:] = list(c1)
    p.cubic_axis2[:] = list(c2)
    p.has_interfacial_dmi = int(dmi_d_interfacial is not None)
    p.dmi_D_interfacial = dmi_d_interfacial or 0.0
    p.has_bulk_dmi = int(dmi_d_bulk is not None)
    p.dmi_D_bulk = dmi_d_bulk or 0.0
    p.has_magnetoelastic = int(mel_b1 is not None)
    p.mel_b1, p.mel_b2 = (mel_b1 or 0.0), mel_b2
    p.mel_strain[:] = list(mel_strain)
    p.current_density_x, p.current_density_y, p.current_density_z = current_density
    p.stt_degree, p.stt_beta = stt_degree, stt_beta
    p.stt_p_x, p.stt_p_y, p.stt_p_z = stt_p
    p.stt_lambda, p.stt_epsilon_prime = stt_lambda, stt_epsilon_prime
    p.has_sot = int(sot_je is not None)
    p.sot_je, p.sot_xi_dl, p.sot_xi_fl = (sot_je or 0.0), sot_xi_dl, sot_xi_fl
    p.sot_sigma[:] = list(sot_sigma)
    p.sot_thickness = sot_thickness
    for name, arr in (("ku1_field", ku1_field), ("ku2_field", ku2_field), ("kc1_field", kc1_field),
                      ("kc2_field", kc2_field), ("kc3_field", kc3_field)):
        if arr is not None:  # one value per cell, borrowed for the create call like every plan array
            a = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
            keep.append(a)
            setattr(p, name, _dptr(a))
    p.has_oersted_cylinder = int(oersted_current is not None)
    p.oersted_current, p.oersted_radius = (oersted_current or 0.0), oersted_radius
    p.oersted_center[:] = list(oersted_center)
    p.oersted_axis[:] = list(oersted_axis)
    p.oersted_time_dep_kind = oersted_kind
    p.oersted_time_dep_freq, p.oersted_time_dep_phase = oersted_freq, oersted_phase
    p.oersted_time_dep_offset = oersted_offset
    p.oersted_time_dep_t_on, p.oersted_time_dep_t_off = oersted_t_on, oersted_t_off
    if spectra is not None and enable_demag:
        sp = np.ascontiguousarray(spectra, dtype=np.float64)
        keep.append(sp)
        (p.demag_kernel_xx_spectrum, p.demag_kernel_yy_spectrum, p.demag_kernel_zz_spectrum,
         p.demag_kernel_xy_spectrum, p.demag_kernel_xz_spectrum,
         p.demag_kernel_yz_spectrum) = [_dptr(sp[i]) for i in range(6)]
        p.demag_kernel_spectrum_len = sp.shape[1]
    if active_mask is not None:
        mk = np.ascontiguousarray(active_mask, dtype=np.uint8).reshape(-1)
        keep.append(mk)
        p.active_mask = mk.ctypes.data_as(C.POINTER(C.c_uint8))
        p.active_mask_len = mk.size
    if region_mask is not None:  # region ids per cell and the optional 256 x 256 A_ij table
        rg = np.ascontiguousarray(region_mask, dtype=np.uint32).reshape(-1)
        keep.append(rg)
        p.region_mask = rg.ctypes.data_as(C.POINTER(C.c_uint32))
        p.region_mask_len = rg.size
        if exchange_lut is not None:
            lt = np.ascontiguousarray(exchange_lut, dtype=np.float64).reshape(-1)
            keep.append(lt)
            p.exchange_lut = _dptr(lt)
            p.exchange_lut_len = lt.size
    if boundary is not None:
        def arr(a, dt=np.float64):
            a = np.ascontiguousarray(a, dtype=dt).reshape(-1)
            keep.append(a)
            return a
        p.boundary_correction = int(boundary.get("tier", 0))
        p.boundary_phi_floor = float(boundary.get("phi_floor", 0.0))
        p.boundary_delta_min = float(boundary.get("delta_min", 0.0))
        if boundary.get("volume_fraction") is not None:
            vf = arr(boundary["volume_fraction"])
            p.volume_fraction = _dptr(vf)
            p.volume_fraction_len = vf.size
        names = ("xp", "xm", "yp", "ym", "zp", "zm")
        for q, a in enumerate(boundary.get("face") or []):
            setattr(p, "face_link_" + names[q], _dptr(arr(a)))
        for q, a in enumerate(boundary.get("delta") or []):
            setattr(p, "delta_" + names[q], _dptr(arr(a)))
        if boundary.get("corr") is not None:
            t, src, ten = boundary["corr"]
            t = arr(t, np.int32)
            src = arr(src, np.int32)
            ten = arr(ten)
            p.has_demag_boundary_corr = 1
            p.demag_corr_target_idx = t.ctypes.data_as(C.POINTER(C.c_int32))
            p.demag_corr_source_idx = src.ctypes.data_as(C.POINTER(C.c_int32))
            p.demag_corr_tensor = _dptr(ten)
            p.demag_corr_target_count = t.size
            p.demag_corr_stencil_size = src.size // max(t.size, 1)
    m = np.ascontiguousarray(m0, dtype=np.float64).reshape(-1)
    keep.append(m)
    p.initial_magnetization_xyz = _dptr(m)
    p.initial_magnetization_len = m.size
    p.adaptive_max_error = adaptive_max_error
    p.adaptive_dt_min = adaptive_dt_min
    p.adaptive_dt_max = adaptive_dt_max
    p.adaptive_headroom = adaptive_headroom
    return p, keep


class FdmBackend:
    """One FDM problem on the GPU behind the C ABI (keyword arguments: ``make_plan``).

    ``periodic`` (x, y, z flags) selects periodic axes and ``image_counts`` the demag
    images per periodic axis (default 10), the reference CPU engine's FdmBoundaryPolicy
    and demag_image_counts (crates/fullmag-engine/src/fdm_problem.rs:19-23); the problem
    is then created through fullmag_fdm_backend_create_periodic."""

    def __init__(self, periodic: Optional[Sequence[int]] = None, image_counts: Optional[Sequence[int]] = None,
                 **plan_kwargs):
        self.lib = load_library()
        p, keep = make_plan(**plan_kwargs)
        self.n = p.grid.nx * p.grid.ny * p.grid.nz
        self.shape = (p.grid.nz, p.grid.ny, p.grid.nx)
        self._poll = None
        if periodic is not None or image_counts is not None:
            d = _abi.PeriodicityDesc()
            for a, v in enumerate(periodic or (0, 0, 0)):
                d.periodic[a] = int(v)
            if image_counts is not None:
                d.has_image_counts = 1
                for a, v in enumerate(image_counts):
                    d.image_counts[a] = int(v)
            self.handle = self.lib.fullmag_fdm_backend_create_periodic(C.byref(p), C.byref(d))
        else:
            self.handle = self.lib.fullmag_fdm_backend_create(C.byref(p))
        del keep
        if not self.handle:
            raise FdmError(_abi.ERR_INTERNAL, "fullmag_fdm_backend_create returned NULL")
        err = self.lib.fullmag_fdm_backend_last_error(self.handle)
        if err:
            msg = err.decode()
            self.lib.fullmag_fdm_backend_destroy(self.handle)
            self.handle = None
            raise FdmError(_abi.ERR_INVALID, msg)

    # -- lifetime --
    def close(self):
        if getattr(self, "handle", None):
            self.lib.fullmag_fdm_backend_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int, what: str):
        if rc == _abi.OK:
            return
        err = self.lib.fullmag_fdm_backend_last_error(self.handle)
        msg = f"{what}: {err.decode() if err else 'no detail'}"
        if rc == _abi.ERR_INTERRUPTED:
            raise FdmInterrupted(rc, msg)
        raise FdmError(rc, msg)

    # -- stepping --
    def step(self, dt: float) -> dict:
        st = StepStats()
        rc = self.lib.fullmag_fdm_backend_step(self.handle, dt, C.byref(st))
        self._check(rc, "step")
        return st.as_dict()

    def step_many(self, dt: float, n_steps: int) -> dict:
        st = StepStats()
        rc = self.lib.fullmag_fdm_backend_step_many(self.handle, dt, n_steps, C.byref(st))
        self._check(rc, "step_many")
        return st.as_dict()

    def set_interrupt_poll(self, fn):
        """fn() -> bool, polled between device passes; True interrupts the step."""
        if fn is None:
            self._poll = None
            rc = self.lib.fullmag_fdm_backend_set_interrupt_poll(self.handle, _abi.POLL_FN(), None)
        else:
            self._poll = _abi.POLL_FN(lambda _ud: 1 if fn() else 0)
            rc = self.lib.fullmag_fdm_backend_set_interrupt_poll(self.handle, self._poll, None)
        self._check(rc, "set_interrupt_poll")

    def stats(self) -> dict:
        st = StepStats()
        self._check(self.lib.fullmag_fdm_backend_snapshot_stats(self.handle, C.byref(st)), "snapshot_stats")
        return st.as_dict()

    # -- fields --
    def copy_field(self, observable: int, dtype=np.float64) -> np.ndarray:
        if np.dtype(dtype) == np.float64:
            out = np.empty(3 * self.n, dtype=np.float64)
            rc = self.lib.fullmag_fdm_backend_copy_field_f64(self.handle, observable, _dptr(out), out.size)
        else:
            out = np.empty(3 * self.n, dtype=np.float32)
            rc = self.lib.fullmag_fdm_backend_copy_field_f32(
                self.handle, observable, out.ctypes.data_as(C.POINTER(C.c_float)), out.size)
        self._check(rc, "copy_field")
        return out.reshape(self.n, 3)

    def magnetization(self):
        return self.copy_field(_abi.OBSERVABLE_M)

    def preview(self, observable: int, pnx: int, pny: int, pnz: int, z_origin: int = 0, z_stride: int = 1):
        out = np.empty(3 * pnx * pny * pnz, dtype=np.float64)
        rc = self.lib.fullmag_fdm_backend_copy_field_preview_f64(
            self.handle, observable, pnx, pny, pnz, z_origin, z_stride, _dptr(out), out.size)
        self._check(rc, "copy_field_preview")
        return out.reshape(-1, 3)

    def upload(self, m: np.ndarray):
        a = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
        self._check(self.lib.fullmag_fdm_backend_upload_magnetization_f64(self.handle, _dptr(a), a.size),
                    "upload_magnetization")

    def refresh(self):
        self._check(self.lib.fullmag_fdm_backend_refresh_observables(self.handle), "refresh_observables")

    # -- adjoint (additive entry points) --
    def set_field_map(self, h: Optional[np.ndarray]):
        """Per-cell applied field (n, 3) in A/m added to H_eff; None removes it."""
        if h is None:
            rc = self.lib.fullmag_fdm_backend_set_field_map(self.handle, None, 0)
        else:
            a = np.ascontiguousarray(h, dtype=np.float64).reshape(-1)
            rc = self.lib.fullmag_fdm_backend_set_field_map(self.handle, _dptr(a), a.size)
        self._check(rc, "set_field_map")

    def adjoint_forward(self, dt: float, n_steps: int, checkpoint_every: int = 0):
        """n_steps fixed RK4 steps from the current state, keeping checkpoints for
        adjoint_backward (checkpoint_every 0: ceil(sqrt(n_steps)))."""
        self._check(self.lib.fullmag_fdm_adjoint_forward(self.handle, dt, n_steps, checkpoint_every),
                    "adjoint_forward")

    def adjoint_backward(self, lam: np.ndarray, want_lambda0: bool = True):
        """Given d loss / d m_final (n, 3), returns (d loss / d field map in per A/m,
        d loss / d m_initial or None), both (n, 3) float64."""
        a = np.ascontiguousarray(lam, dtype=np.float64).reshape(-1)
        grad = np.empty(3 * self.n)
        lam0 = np.empty(3 * self.n) if want_lambda0 else None
        rc = self.lib.fullmag_fdm_adjoint_backward(self.handle, _dptr(a), a.size, _dptr(grad),
                                                   _dptr(lam0) if lam0 is not None else None)
        self._check(rc, "adjoint_backward")
        return grad.reshape(self.n, 3), (lam0.reshape(self.n, 3) if lam0 is not None else None)

    def device_info(self) -> dict:
        info = _abi.DeviceInfo()
        self._check(self.lib.fullmag_fdm_backend_get_device_info(self.handle, C.byref(info)), "get_device_info")
        return {"name": info.name.decode(), "cc": (info.compute_capability_major, info.compute_capability_minor),
                "driver": info.driver_version, "runtime": info.runtime_version}

    def fft_shape(self):
        a, b, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self._check(self.lib.fullmag_fdm_backend_fft_shape(self.handle, C.byref(a), C.byref(b), C.byref(c)),
                    "fft_shape")
        return a.value, b.value, c.value

    def tuning(self) -> dict:
        a = (C.c_uint32 * 9)()
        self._check(self.lib.fullmag_fdm_backend_tuning(self.handle, a), "tuning")
        return {"rows_per_cta": a[0], "tx_y_forward": a[1], "tx_z": a[2], "tx_y_inverse": a[3], "tx_thin": a[4],
                "z_pair": a[5], "split_y_forward": a[6], "split_z": a[7], "split_y_inverse": a[8]}

    def launch_count(self) -> int:
        c = C.c_uint64()
        self._check(self.lib.fullmag_fdm_backend_launch_count(self.handle, C.byref(c)), "launch_count")
        return c.value

    KERNEL_KINDS = ("row_pass", "y_forward", "z_convolve", "y_inverse", "yz_convolve", "y_convolve_2d",
                    "finalize_stats", "extra_field")

    def set_kernel_timing(self, enable: bool):
        """Per-launch CUDA-event timing of every kernel (fixed steps then run without graphs)."""
        self._check(self.lib.fullmag_fdm_backend_set_kernel_timing(self.handle, int(bool(enable))),
                    "set_kernel_timing")

    def kernel_times(self) -> dict:
        """{kind: (total_ms, launches)} since timing was enabled."""
        k = len(self.KERNEL_KINDS)
        ms = (C.c_double * k)()
        cnt = (C.c_uint64 * k)()
        self._check(self.lib.fullmag_fdm_backend_kernel_times(self.handle, ms, cnt, k), "kernel_times")
        return {name: (ms[i], cnt[i]) for i, name in enumerate(self.KERNEL_KINDS)}

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.fullmag_fdm_backend_stream(self.handle, C.byref(s)), "stream")
        return s.value or 0


class FdmBatch:
    """Many independent problems advanced together (fullmag_fdm_batch_*)."""

    def __init__(self, plans: Sequence[dict]):
        self.lib = load_library()
        built = [make_plan(**kw) for kw in plans]
        arr = (PlanDesc * len(built))(*[b[0] for b in built])
        self.ns = [b[0].grid.nx * b[0].grid.ny * b[0].grid.nz for b in built]
        self.handle = self.lib.fullmag_fdm_batch_create(arr, len(built))
        del built
        if not self.handle:
            raise FdmError(_abi.ERR_INTERNAL, "fullmag_fdm_batch_create returned NULL")
        err = self.lib.fullmag_fdm_batch_last_error(self.handle)
        if err:
            self.close()
            raise FdmError(_abi.ERR_INVALID, err.decode())

    def __len__(self):
        return len(self.ns)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fullmag_fdm_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step_until(self, t_end: float, dt0: float):
        n = len(self.ns)
        steps = (C.c_uint64 * n)()
        wall = (C.c_uint64 * n)()
        rc = self.lib.fullmag_fdm_batch_step_until(self.handle, t_end, dt0, steps, wall)
        if rc != _abi.OK:
            err = self.lib.fullmag_fdm_batch_last_error(self.handle)
            raise FdmError(rc, f"batch step_until: {err.decode() if err else 'no detail'}")
        return np.array(steps[:], dtype=np.int64), np.array(wall[:], dtype=np.float64) * 1e-9

    def stats(self, i: int) -> dict:
        st = StepStats()
        rc = self.lib.fullmag_fdm_batch_get_stats(self.handle, i, C.byref(st))
        if rc != _abi.OK:
            raise FdmError(rc, "batch get_stats")
        return st.as_dict()

    def copy_field(self, i: int, observable: int = _abi.OBSERVABLE_M) -> np.ndarray:
        out = np.empty(3 * self.ns[i], dtype=np.float64)
        rc = self.lib.fullmag_fdm_batch_copy_field_f64(self.handle, i, observable, _dptr(out), out.size)
        if rc != _abi.OK:
            raise FdmError(rc, "batch copy_field")
        return out.reshape(-1, 3)
