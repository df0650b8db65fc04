"""ctypes mirror of include/fullmag_fdm.h.

Field order and types follow the C header exactly (the header in turn keeps the
layout of the reference interface, native/include/fullmag_fdm.h:84-307, so that
crates/fullmag-fdm-sys/src/lib.rs can bind the same library).  This is the binding
a Python caller uses; tests/test_abi_layout.py checks every offset against the C
compiler's.
"""
from __future__ import annotations

import ctypes as C

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_INTERNAL = -3
ERR_INTERRUPTED = -4
MAX_EXCHANGE_REGIONS = 256

PRECISION_SINGLE = 1
PRECISION_DOUBLE = 2
BOUNDARY_NONE, BOUNDARY_VOLUME, BOUNDARY_FULL = 0, 1, 2

INTEGRATOR_HEUN = 1
INTEGRATOR_DP45 = 2
INTEGRATOR_ABM3 = 3
INTEGRATOR_RK4 = 4
INTEGRATOR_RK23 = 5

OBSERVABLE_M = 1
OBSERVABLE_H_EX = 2
OBSERVABLE_H_DEMAG = 3
OBSERVABLE_H_EXT = 4
OBSERVABLE_H_EFF = 5

SNAPSHOT_SCALAR_F32 = 1
SNAPSHOT_SCALAR_F64 = 2

_d = C.c_double
_i = C.c_int
_u32 = C.c_uint32
_u64 = C.c_uint64
_pd = C.POINTER(C.c_double)


class GridDesc(C.Structure):
    _fields_ = [("nx", _u32), ("ny", _u32), ("nz", _u32), ("dx", _d), ("dy", _d), ("dz", _d)]


class MaterialDesc(C.Structure):
    _fields_ = [("saturation_magnetisation", _d), ("exchange_stiffness", _d), ("damping", _d),
                ("gyromagnetic_ratio", _d)]


class PlanDesc(C.Structure):
    _fields_ = [
        ("grid", GridDesc),
        ("material", MaterialDesc),
        ("precision", _i),
        ("integrator", _i),
        ("disable_precession", _i),
        ("enable_exchange", _i),
        ("enable_demag", _i),
        ("has_external_field", _i),
        ("external_field_am", _d * 3),
        ("has_uniaxial_anisotropy", _i),
        ("uniaxial_anisotropy_constant", _d),
        ("uniaxial_anisotropy_k2", _d),
        ("anisotropy_axis", _d * 3),
        ("ku1_field", _pd),
        ("ku2_field", _pd),
        ("has_cubic_anisotropy", _i),
        ("cubic_Kc1", _d),
        ("cubic_Kc2", _d),
        ("cubic_Kc3", _d),
        ("cubic_axis1", _d * 3),
        ("cubic_axis2", _d * 3),
        ("kc1_field", _pd),
        ("kc2_field", _pd),
        ("kc3_field", _pd),
        ("has_interfacial_dmi", _i),
        ("dmi_D_interfacial", _d),
        ("has_bulk_dmi", _i),
        ("dmi_D_bulk", _d),
        ("has_magnetoelastic", _i),
        ("mel_b1", _d),
        ("mel_b2", _d),
        ("mel_strain", _d * 6),
        ("temperature", _d),
        ("current_density_x", _d),
        ("current_density_y", _d),
        ("current_density_z", _d),
        ("stt_degree", _d),
        ("stt_beta", _d),
        ("stt_p_x", _d),
        ("stt_p_y", _d),
        ("stt_p_z", _d),
        ("stt_lambda", _d),
        ("stt_epsilon_prime", _d),
        ("has_sot", _i),
        ("sot_je", _d),
        ("sot_xi_dl", _d),
        ("sot_xi_fl", _d),
        ("sot_sigma", _d * 3),
        ("sot_thickness", _d),
        ("has_oersted_cylinder", _i),
        ("oersted_current", _d),
        ("oersted_radius", _d),
        ("oersted_center", _d * 3),
        ("oersted_axis", _d * 3),
        ("oersted_time_dep_kind", _u32),
        ("oersted_time_dep_freq", _d),
        ("oersted_time_dep_phase", _d),
        ("oersted_time_dep_offset", _d),
        ("oersted_time_dep_t_on", _d),
        ("oersted_time_dep_t_off", _d),
        ("demag_kernel_xx_spectrum", _pd),
        ("demag_kernel_yy_spectrum", _pd),
        ("demag_kernel_zz_spectrum", _pd),
        ("demag_kernel_xy_spectrum", _pd),
        ("demag_kernel_xz_spectrum", _pd),
        ("demag_kernel_yz_spectrum", _pd),
        ("demag_kernel_spectrum_len", _u64),
        ("active_mask", C.POINTER(C.c_uint8)),
        ("active_mask_len", _u64),
        ("region_mask", C.POINTER(C.c_uint32)),
        ("region_mask_len", _u64),
        ("exchange_lut", _pd),
        ("exchange_lut_len", _u64),
        ("boundary_correction", _i),
        ("boundary_phi_floor", _d),
        ("boundary_delta_min", _d),
        ("volume_fraction", _pd),
        ("volume_fraction_len", _u64),
        ("face_link_xp", _pd),
        ("face_link_xm", _pd),
        ("face_link_yp", _pd),
        ("face_link_ym", _pd),
        ("face_link_zp", _pd),
        ("face_link_zm", _pd),
        ("delta_xp", _pd),
        ("delta_xm", _pd),
        ("delta_yp", _pd),
        ("delta_ym", _pd),
        ("delta_zp", _pd),
        ("delta_zm", _pd),
        ("has_demag_boundary_corr", _i),
        ("demag_corr_target_idx", C.POINTER(C.c_int32)),
        ("demag_corr_source_idx", C.POINTER(C.c_int32)),
        ("demag_corr_tensor", _pd),
        ("demag_corr_target_count", _u32),
        ("demag_corr_stencil_size", _u32),
        ("initial_magnetization_xyz", _pd),
        ("initial_magnetization_len", _u64),
        ("adaptive_max_error", _d),
        ("adaptive_dt_min", _d),
        ("adaptive_dt_max", _d),
        ("adaptive_headroom", _d),
    ]


class StepStats(C.Structure):
    _fields_ = [
        ("step", _u64),
        ("time_seconds", _d),
        ("dt_seconds", _d),
        ("exchange_energy_joules", _d),
        ("demag_energy_joules", _d),
        ("external_energy_joules", _d),
        ("anisotropy_energy_joules", _d),
        ("cubic_energy_joules", _d),
        ("dmi_energy_joules", _d),
        ("total_energy_joules", _d),
        ("max_effective_field_amplitude", _d),
        ("max_demag_field_amplitude", _d),
        ("max_rhs_amplitude", _d),
        ("suggested_next_dt", _d),
        ("wall_time_ns", _u64),
    ]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class DeviceInfo(C.Structure):
    _fields_ = [("name", C.c_char * 128), ("compute_capability_major", _i),
                ("compute_capability_minor", _i), ("driver_version", _i), ("runtime_version", _i)]


class SnapshotDesc(C.Structure):
    _fields_ = [("cell_count", _u64), ("component_count", _u32), ("scalar_bytes", _u32),
                ("scalar_type", _i)]


class PeriodicityDesc(C.Structure):
    _fields_ = [("periodic", _u32 * 3), ("has_image_counts", _u32), ("image_counts", _u32 * 3)]


POLL_FN = C.CFUNCTYPE(C.c_int, C.c_void_p)

# (name, restype, argtypes) of every exported entry point, in header order.
_vp = C.c_void_p
_pss = C.POINTER(StepStats)
SIGNATURES = [
    ("fullmag_fdm_is_available", _i, []),
    ("fullmag_fdm_backend_create", _vp, [C.POINTER(PlanDesc)]),
    ("fullmag_fdm_backend_step", _i, [_vp, _d, _pss]),
    ("fullmag_fdm_backend_set_interrupt_poll", _i, [_vp, POLL_FN, _vp]),
    ("fullmag_fdm_backend_copy_field_f64", _i, [_vp, _i, _pd, _u64]),
    ("fullmag_fdm_backend_copy_field_f32", _i, [_vp, _i, C.POINTER(C.c_float), _u64]),
    ("fullmag_fdm_backend_copy_field_preview_f64", _i, [_vp, _i, _u32, _u32, _u32, _u32, _u32, _pd, _u64]),
    ("fullmag_fdm_backend_copy_field_preview_f32", _i,
     [_vp, _i, _u32, _u32, _u32, _u32, _u32, C.POINTER(C.c_float), _u64]),
    ("fullmag_fdm_backend_begin_field_snapshot", _vp, [_vp, _i]),
    ("fullmag_fdm_backend_begin_preview_snapshot", _vp, [_vp, _i, _u32, _u32, _u32, _u32, _u32]),
    ("fullmag_fdm_field_snapshot_wait", _i, [_vp, C.POINTER(_vp), C.POINTER(_u64), C.POINTER(SnapshotDesc)]),
    ("fullmag_fdm_preview_snapshot_wait", _i, [_vp, C.POINTER(_vp), C.POINTER(_u64), C.POINTER(SnapshotDesc)]),
    ("fullmag_fdm_field_snapshot_destroy", None, [_vp]),
    ("fullmag_fdm_preview_snapshot_destroy", None, [_vp]),
    ("fullmag_fdm_backend_upload_magnetization_f64", _i, [_vp, _pd, _u64]),
    ("fullmag_fdm_backend_upload_magnetization_f32", _i, [_vp, C.POINTER(C.c_float), _u64]),
    ("fullmag_fdm_backend_refresh_observables", _i, [_vp]),
    ("fullmag_fdm_backend_refresh_demag_observable", _i, [_vp]),
    ("fullmag_fdm_backend_snapshot_stats", _i, [_vp, _pss]),
    ("fullmag_fdm_backend_get_device_info", _i, [_vp, C.POINTER(DeviceInfo)]),
    ("fullmag_fdm_backend_last_error", C.c_char_p, [_vp]),
    ("fullmag_fdm_backend_destroy", None, [_vp]),
    # additive
    ("fullmag_fdm_backend_step_many", _i, [_vp, _d, _u64, _pss]),
    ("fullmag_fdm_backend_device_magnetization", _i, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp)]),
    ("fullmag_fdm_backend_stream", _i, [_vp, C.POINTER(_vp)]),
    ("fullmag_fdm_backend_tuning", _i, [_vp, C.POINTER(_u32)]),
    ("fullmag_fdm_backend_launch_count", _i, [_vp, C.POINTER(_u64)]),
    ("fullmag_fdm_backend_set_kernel_timing", _i, [_vp, _i]),
    ("fullmag_fdm_backend_kernel_times", _i, [_vp, _pd, C.POINTER(_u64), _u32]),
    ("fullmag_fdm_backend_set_field_map", _i, [_vp, _pd, _u64]),
    ("fullmag_fdm_adjoint_forward", _i, [_vp, _d, _u64, _u32]),
    ("fullmag_fdm_adjoint_backward", _i, [_vp, _pd, _u64, _pd, _pd]),
    ("fullmag_fdm_batch_create", _vp, [C.POINTER(PlanDesc), _u32]),
    ("fullmag_fdm_batch_last_error", C.c_char_p, [_vp]),
    ("fullmag_fdm_batch_size", _u32, [_vp]),
    ("fullmag_fdm_batch_step_until", _i, [_vp, _d, _d, C.POINTER(_u64), C.POINTER(_u64)]),
    ("fullmag_fdm_batch_get_stats", _i, [_vp, _u32, _pss]),
    ("fullmag_fdm_batch_copy_field_f64", _i, [_vp, _u32, _i, _pd, _u64]),
    ("fullmag_fdm_batch_destroy", None, [_vp]),
    ("fullmag_fdm_backend_fft_shape", _i, [_vp, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32)]),
    ("fullmag_fdm_backend_upload_magnetization_f64_noalloc", _i, [_vp, _pd, _u64]),
    ("fullmag_fdm_backend_create_periodic", _vp, [C.POINTER(PlanDesc), C.POINTER(PeriodicityDesc)]),
]

REFERENCE_SYMBOLS = [s[0] for s in SIGNATURES[:22]]


def bind(lib: C.CDLL) -> C.CDLL:
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
