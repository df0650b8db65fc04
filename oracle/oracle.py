"""ctypes front end of the FP64 oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
this module, as the checker.  The product path never imports it.  The C code it
wraps restates crates/fullmag-engine (fields, integrators) and
crates/fullmag-fdm-demag (Newell tensor) of the reference in FP64.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libfdm_oracle.so"

HEUN, DP45, ABM3, RK4, RK23 = 1, 2, 3, 4, 5


def build(force: bool = False) -> Path:
    """Compile the oracle with the committed Makefile (gcc, OpenMP)."""
    src = HERE / "fdm_oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("integrator", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("ms", C.c_double), ("a_ex", C.c_double), ("alpha", C.c_double), ("gamma", C.c_double),
        ("enable_exchange", C.c_int32), ("enable_demag", C.c_int32),
        ("has_external_field", C.c_int32), ("disable_precession", C.c_int32),
        ("h_ext", C.c_double * 3),
        ("has_uniaxial", C.c_int32), ("has_cubic", C.c_int32),
        ("ku1", C.c_double), ("ku2", C.c_double), ("u_axis", C.c_double * 3),
        ("kc1", C.c_double), ("kc2", C.c_double), ("kc3", C.c_double),
        ("c1", C.c_double * 3), ("c2", C.c_double * 3),
        ("max_error", C.c_double), ("dt_min", C.c_double), ("dt_max", C.c_double),
        ("headroom", C.c_double), ("rtol", C.c_double), ("growth_limit", C.c_double),
        ("shrink_limit", C.c_double),
        ("dp45_norm", C.c_int32), ("pad0", C.c_int32),
        ("active_mask", C.c_void_p),
        ("region_mask", C.c_void_p), ("exchange_lut", C.c_void_p),
        ("has_interfacial_dmi", C.c_int32), ("has_bulk_dmi", C.c_int32),
        ("dmi_d_interfacial", C.c_double), ("dmi_d_bulk", C.c_double),
        ("has_magnetoelastic", C.c_int32), ("pad1", C.c_int32),
        ("mel_b1", C.c_double), ("mel_b2", C.c_double), ("mel_strain", C.c_double * 6),
        ("current_density", C.c_double * 3), ("stt_degree", C.c_double), ("stt_beta", C.c_double),
        ("stt_p", C.c_double * 3), ("stt_lambda", C.c_double), ("stt_epsilon_prime", C.c_double),
        ("has_sot", C.c_int32), ("pad2", C.c_int32),
        ("sot_je", C.c_double), ("sot_xi_dl", C.c_double), ("sot_xi_fl", C.c_double),
        ("sot_sigma", C.c_double * 3), ("sot_thickness", C.c_double),
        ("ku1_field", C.c_void_p), ("ku2_field", C.c_void_p), ("kc1_field", C.c_void_p),
        ("kc2_field", C.c_void_p), ("kc3_field", C.c_void_p),
        ("has_oersted", C.c_int32), ("oersted_kind", C.c_int32),
        ("oersted_current", C.c_double), ("oersted_radius", C.c_double), ("oersted_center", C.c_double * 3),
        ("oersted_freq", C.c_double), ("oersted_phase", C.c_double), ("oersted_offset", C.c_double),
        ("oersted_t_on", C.c_double), ("oersted_t_off", C.c_double),
        ("temperature", C.c_double), ("thermal_seed", C.c_uint64),
        ("boundary_tier", C.c_int32), ("pad3", C.c_int32), ("phi_floor", C.c_double), ("delta_min", C.c_double),
        ("volume_fraction", C.c_void_p), ("face", C.c_void_p * 6), ("delta", C.c_void_p * 6),
        ("corr_target_idx", C.c_void_p), ("corr_source_idx", C.c_void_p), ("corr_tensor", C.c_void_p),
        ("corr_targets", C.c_uint32), ("corr_stencil", C.c_uint32),
        ("periodic", C.c_int32 * 3), ("image_counts", C.c_uint32 * 3),
    ]


class Stats(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "step", "time", "dt_used", "suggested_next_dt",
        "e_exchange", "e_exchange_field", "e_demag", "e_external", "e_uniaxial", "e_cubic",
        "e_anis_cpu", "e_total", "max_h_eff", "max_h_demag", "max_rhs", "rejected_attempts", "e_dmi")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = C.CDLL(str(path))
        dp = C.POINTER(C.c_double)
        L.fo_newell_f.restype = C.c_double
        L.fo_newell_f.argtypes = [C.c_double] * 3
        L.fo_newell_g.restype = C.c_double
        L.fo_newell_g.argtypes = [C.c_double] * 3
        L.fo_newell_kernels.argtypes = [C.c_int] * 3 + [C.c_double] * 3 + [dp]
        L.fo_newell_spectra.argtypes = [C.c_int] * 3 + [C.c_double] * 3 + [C.c_int, dp]
        L.fo_periodic_newell_kernels.argtypes = [C.c_int] * 3 + [C.c_double] * 3 + [
            C.POINTER(C.c_int32), C.POINTER(C.c_uint32), dp]
        L.fo_fft1d.argtypes = [dp, C.c_int, C.c_int]
        L.fo_fft3d.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.fo_create.restype = C.c_void_p
        L.fo_create.argtypes = [C.POINTER(Params), dp]
        L.fo_destroy.argtypes = [C.c_void_p]
        L.fo_set_m.argtypes = [C.c_void_p, dp]
        L.fo_get_m.argtypes = [C.c_void_p, dp]
        L.fo_set_field_map.argtypes = [C.c_void_p, dp]
        L.fo_tangent_rk4.argtypes = [C.c_void_p, C.c_double, C.c_uint64, dp, dp, dp]
        L.fo_fields.argtypes = [C.c_void_p] + [dp] * 6
        L.fo_observe.argtypes = [C.c_void_p, C.POINTER(Stats)]
        L.fo_step.argtypes = [C.c_void_p, C.c_double, C.POINTER(Stats)]
        L.fo_demag_direct.argtypes = [C.c_void_p, dp, dp]
        L.fo_num_threads.restype = C.c_int
        L.fo_set_num_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _dp(a):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def newell_f(x, y, z):
    return lib().fo_newell_f(x, y, z)


def newell_g(x, y, z):
    return lib().fo_newell_g(x, y, z)


def newell_kernels(nx, ny, nz, dx, dy, dz):
    """Real-space padded tensors, shape (6, 2nz, 2ny, 2nx): xx yy zz xy xz yz."""
    out = np.zeros(6 * 8 * nx * ny * nz)
    rc = lib().fo_newell_kernels(nx, ny, nz, dx, dy, dz, _dp(out))
    assert rc == 0
    return out.reshape(6, 2 * nz, 2 * ny, 2 * nx)


def periodic_newell_kernels(nx, ny, nz, dx, dy, dz, periodic, images):
    """Truncated-image tensors of a grid with periodic axes, shape (6, pz, py, px) with
    p = n on a periodic axis and 2n on an open one: xx yy zz xy xz yz."""
    pd = [n if per else 2 * n for n, per in zip((nx, ny, nz), periodic)]
    out = np.zeros(6 * pd[0] * pd[1] * pd[2])
    per = (C.c_int32 * 3)(*[int(bool(v)) for v in periodic])
    img = (C.c_uint32 * 3)(*[int(v) for v in images])
    rc = lib().fo_periodic_newell_kernels(nx, ny, nz, dx, dy, dz, per, img, _dp(out))
    assert rc == 0
    return out.reshape(6, pd[2], pd[1], pd[0])


def newell_spectra(nx, ny, nz, dx, dy, dz, thin_film_2d=False):
    """Interleaved complex spectra as the C ABI receives them: shape (6, 2P)."""
    P = 4 * nx * ny if thin_film_2d else 8 * nx * ny * nz
    out = np.zeros(6 * 2 * P)
    rc = lib().fo_newell_spectra(nx, ny, nz, dx, dy, dz, int(thin_film_2d), _dp(out))
    assert rc == 0
    return out.reshape(6, 2 * P)


def fft1d(x, inverse=False):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.complex128)).copy()
    buf = a.view(np.float64)
    assert lib().fo_fft1d(_dp(buf), a.size, int(inverse)) == 0
    return a


def fft3d(x, inverse=False):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.complex128)).copy()
    pz, py, px = a.shape
    assert lib().fo_fft3d(_dp(a.view(np.float64)), px, py, pz, int(inverse)) == 0
    return a


class Problem:
    """FP64 oracle problem.  Arrays are AoS (n, 3)."""

    def __init__(self, *, nx, ny, nz, dx, dy, dz, ms, a_ex, alpha, gamma=2.211e5,
                 integrator=HEUN, enable_exchange=True, enable_demag=True, h_ext=None,
                 disable_precession=False, ku1=None, ku2=0.0, u_axis=(0, 0, 1),
                 kc1=None, kc2=0.0, kc3=0.0, c1=(1, 0, 0), c2=(0, 1, 0),
                 max_error=1e-5, dt_min=1e-18, dt_max=1e-10, headroom=0.8, rtol=0.0,
                 growth_limit=float("inf"), shrink_limit=0.0, dp45_norm=0,
                 active_mask=None, m0=None, region_mask=None, exchange_lut=None,
                 dmi_d_interfacial=None, dmi_d_bulk=None, mel_b1=None, mel_b2=0.0, mel_strain=(0.0,) * 6,
                 current_density=(0.0, 0.0, 0.0), stt_degree=0.0, stt_beta=0.0, stt_p=(0.0, 0.0, 0.0),
                 stt_lambda=0.0, stt_epsilon_prime=0.0, sot_je=None, sot_xi_dl=0.0, sot_xi_fl=0.0,
                 sot_sigma=(0.0, 0.0, 1.0), sot_thickness=0.0,
                 ku1_field=None, ku2_field=None, kc1_field=None, kc2_field=None, kc3_field=None,
                 oersted_current=None, oersted_radius=0.0, oersted_center=(0.0, 0.0, 0.0), oersted_kind=0,
                 oersted_freq=0.0, oersted_phase=0.0, oersted_offset=0.0, oersted_t_on=0.0, oersted_t_off=0.0,
                 temperature=0.0, thermal_seed=42, boundary=None, periodic=None, image_counts=None):
        p = Params()
        p.nx, p.ny, p.nz, p.integrator = nx, ny, nz, integrator
        p.dx, p.dy, p.dz = dx, dy, dz
        p.ms, p.a_ex, p.alpha, p.gamma = ms, a_ex, alpha, gamma
        p.enable_exchange, p.enable_demag = int(enable_exchange), int(enable_demag)
        p.has_external_field = int(h_ext is not None)
        p.disable_precession = int(disable_precession)
        p.h_ext[:] = list(h_ext) if h_ext is not None else [0.0, 0.0, 0.0]
        p.has_uniaxial = int(ku1 is not None)
        p.ku1, p.ku2 = (ku1 or 0.0), ku2
        p.u_axis[:] = list(u_axis)
        p.has_cubic = int(kc1 is not None)
        p.kc1, p.kc2, p.kc3 = (kc1 or 0.0), kc2, kc3
        p.c1[:] = list(c1)
        p.c2[:] = list(c2)
        p.max_error, p.dt_min, p.dt_max, p.headroom = max_error, dt_min, dt_max, headroom
        p.rtol, p.growth_limit, p.shrink_limit = rtol, growth_limit, shrink_limit
        p.dp45_norm = dp45_norm
        p.has_interfacial_dmi = int(dmi_d_interfacial is not None)
        p.dmi_d_interfacial = dmi_d_interfacial or 0.0
        p.has_bulk_dmi = int(dmi_d_bulk is not None)
        p.dmi_d_bulk = dmi_d_bulk or 0.0
        p.has_magnetoelastic = int(mel_b1 is not None)
        p.mel_b1, p.mel_b2 = (mel_b1 or 0.0), mel_b2
        p.mel_strain[:] = list(mel_strain)
        p.current_density[:] = list(current_density)
        p.stt_degree, p.stt_beta = stt_degree, stt_beta
        p.stt_p[:] = list(stt_p)
        p.stt_lambda, p.stt_epsilon_prime = stt_lambda, stt_epsilon_prime
        p.has_sot = int(sot_je is not None)
        p.sot_je, p.sot_xi_dl, p.sot_xi_fl = (sot_je or 0.0), sot_xi_dl, sot_xi_fl
        p.sot_sigma[:] = list(sot_sigma)
        p.sot_thickness = sot_thickness
        if oersted_current is not None and not oersted_radius > 0.0:
            raise ValueError("oersted_radius must be positive")
        p.has_oersted = int(oersted_current is not None)
        p.oersted_current, p.oersted_radius = (oersted_current or 0.0), oersted_radius
        p.oersted_center[:] = list(oersted_center)
        p.oersted_kind, p.oersted_freq, p.oersted_phase = oersted_kind, oersted_freq, oersted_phase
        p.oersted_offset, p.oersted_t_on, p.oersted_t_off = oersted_offset, oersted_t_on, oersted_t_off
        p.temperature, p.thermal_seed = temperature, thermal_seed
        # periodic axes (x, y, z flags) and demag images per periodic axis (default 10)
        p.periodic[:] = [int(bool(v)) for v in (periodic or (0, 0, 0))]
        p.image_counts[:] = [int(v) for v in (image_counts if image_counts is not None else (10, 10, 10))]
        self._kmaps = {}
        for name, arr in (("ku1_field", ku1_field), ("ku2_field", ku2_field), ("kc1_field", kc1_field),
                          ("kc2_field", kc2_field), ("kc3_field", kc3_field)):
            if arr is not None:
                a = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
                if a.size != nx * ny * nz:
                    raise ValueError(f"{name} needs one value per cell")
                self._kmaps[name] = a
                setattr(p, name, a.ctypes.data)
        self._mask = None
        if active_mask is not None:
            self._mask = np.ascontiguousarray(active_mask, dtype=np.uint8)
            p.active_mask = self._mask.ctypes.data
        if region_mask is not None:
            self._regions = np.ascontiguousarray(region_mask, dtype=np.uint32).reshape(-1)
            if self._regions.size != nx * ny * nz or (self._regions.size and self._regions.max() >= 256):
                raise ValueError("region_mask needs one id below 256 per cell")
            p.region_mask = self._regions.ctypes.data
            if exchange_lut is not None:
                self._lut = np.ascontiguousarray(exchange_lut, dtype=np.float64).reshape(-1)
                if self._lut.size != 256 * 256:
                    raise ValueError("exchange_lut needs 256 x 256 entries")
                p.exchange_lut = self._lut.ctypes.data
        self._bnd = []
        if boundary is not None:
            # boundary correction of the double-precision path: dict with tier (1 T0, 2 T1),
            # volume_fraction, face (6 arrays) or delta (6 arrays), phi_floor, delta_min, and
            # optionally corr = (target_idx, source_idx, tensor (targets x stencil x 6))
            def keep(a, dt=np.float64):
                a = np.ascontiguousarray(a, dtype=dt).reshape(-1)
                self._bnd.append(a)
                return a.ctypes.data
            p.boundary_tier = int(boundary.get("tier", 0))
            p.phi_floor = float(boundary.get("phi_floor", 0.0))
            p.delta_min = float(boundary.get("delta_min", 0.0))
            if boundary.get("volume_fraction") is not None:
                p.volume_fraction = keep(boundary["volume_fraction"])
            for q, a in enumerate(boundary.get("face") or []):
                p.face[q] = keep(a)
            for q, a in enumerate(boundary.get("delta") or []):
                p.delta[q] = keep(a)
            if boundary.get("corr") is not None:
                t, src, ten = boundary["corr"]
                t = np.asarray(t)
                p.corr_target_idx = keep(t, np.int32)
                p.corr_source_idx = keep(src, np.int32)
                p.corr_tensor = keep(ten)
                p.corr_targets = t.size
                p.corr_stencil = np.asarray(src).size // max(t.size, 1)
        self.n = nx * ny * nz
        self.shape = (nz, ny, nx)
        self.params = p
        m0a = None if m0 is None else np.ascontiguousarray(m0, dtype=np.float64).reshape(-1)
        self._h = lib().fo_create(C.byref(p), _dp(m0a))
        if not self._h:
            raise RuntimeError("oracle create failed")

    def close(self):
        if self._h:
            lib().fo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_m(self, m):
        a = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
        lib().fo_set_m(self._h, _dp(a))

    def get_m(self):
        a = np.zeros(3 * self.n)
        lib().fo_get_m(self._h, _dp(a))
        return a.reshape(self.n, 3)

    def set_field_map(self, h):
        """Per-cell applied field (n, 3) in A/m added at active cells; None removes it."""
        if h is None:
            lib().fo_set_field_map(self._h, None)
            return
        self._hmap = np.ascontiguousarray(h, dtype=np.float64).reshape(-1)
        lib().fo_set_field_map(self._h, _dp(self._hmap))

    def fields(self, m=None):
        if m is None:
            m = self.get_m()
        m = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
        outs = {k: np.zeros(3 * self.n) for k in ("h_ex", "h_demag", "h_ext", "h_eff", "rhs")}
        lib().fo_fields(self._h, _dp(m), _dp(outs["h_ex"]), _dp(outs["h_demag"]),
                        _dp(outs["h_ext"]), _dp(outs["h_eff"]), _dp(outs["rhs"]))
        return {k: v.reshape(self.n, 3) for k, v in outs.items()}

    def observe(self):
        st = Stats()
        lib().fo_observe(self._h, C.byref(st))
        return st.as_dict()

    def step(self, dt):
        st = Stats()
        rc = lib().fo_step(self._h, dt, C.byref(st))
        if rc != 0:
            raise RuntimeError(f"oracle step failed ({rc})")
        return st.as_dict()

    def tangent_rk4(self, dt, n_steps, dh=None, dm0=None):
        """Advance n_steps RK4 steps and return d m_final along (dm0, dh) in FP64, (n, 3)."""
        a = None if dh is None else np.ascontiguousarray(dh, dtype=np.float64).reshape(-1)
        b = None if dm0 is None else np.ascontiguousarray(dm0, dtype=np.float64).reshape(-1)
        out = np.zeros(3 * self.n)
        if lib().fo_tangent_rk4(self._h, dt, n_steps, _dp(a), _dp(b), _dp(out)) != 0:
            raise RuntimeError("oracle tangent failed (cubic anisotropy is not differentiated)")
        return out.reshape(self.n, 3)

    def demag_direct(self, m=None):
        if m is None:
            m = self.get_m()
        m = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
        out = np.zeros(3 * self.n)
        lib().fo_demag_direct(self._h, _dp(m), _dp(out))
        return out.reshape(self.n, 3)


def set_threads(n: int):
    lib().fo_set_num_threads(int(n))


def threads() -> int:
    return lib().fo_num_threads()
