"""The C ABI without a GPU: struct layouts (ctypes mirror vs the C compiler) and the
exported symbol set of libfullmag_fdm.so (every entry point include/fullmag_fdm.h declares)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from fullmag_gb300 import _abi

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "fullmag_fdm.h"


def _c_offsets(tmp_path, struct_name, ctype):
    lines = [f'#include "{HEADER}"', "#include <stdio.h>", "#include <stddef.h>", "int main(void){"]
    lines.append(f'printf("sizeof %zu\\n", sizeof({struct_name}));')
    for name, _ in ctype._fields_:
        lines.append(f'printf("{name} %zu\\n", offsetof({struct_name}, {name}));')
    lines.append("return 0;}")
    src = tmp_path / f"{struct_name}.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / struct_name
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (l.split() for l in out.strip().splitlines())}


@pytest.mark.parametrize("sname,ctype", [
    ("fullmag_fdm_plan_desc", _abi.PlanDesc), ("fullmag_fdm_step_stats", _abi.StepStats),
    ("fullmag_fdm_device_info", _abi.DeviceInfo), ("fullmag_fdm_snapshot_desc", _abi.SnapshotDesc),
    ("fullmag_fdm_grid_desc", _abi.GridDesc), ("fullmag_fdm_material_desc", _abi.MaterialDesc),
    ("fullmag_fdm_periodicity_desc", _abi.PeriodicityDesc)])
def test_struct_layout_matches_c(tmp_path, sname, ctype):
    off = _c_offsets(tmp_path, sname, ctype)
    assert off.pop("sizeof") == C.sizeof(ctype)
    for name, _ in ctype._fields_:
        assert off[name] == getattr(ctype, name).offset, name


def test_reference_layout_invariants():
    # fixed by the reference interface (native/include/fullmag_fdm.h:273-289, :293-299)
    assert C.sizeof(_abi.StepStats) == 120
    assert C.sizeof(_abi.DeviceInfo) == 128 + 16
    assert _abi.MAX_EXCHANGE_REGIONS == 256
    assert (_abi.INTEGRATOR_HEUN, _abi.INTEGRATOR_DP45, _abi.INTEGRATOR_ABM3, _abi.INTEGRATOR_RK4,
            _abi.INTEGRATOR_RK23) == (1, 2, 3, 4, 5)


def _declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fullmag_fdm_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from fullmag_gb300 import build
    lib_path = build.build()
    lib = C.CDLL(str(lib_path))
    declared = _declared_functions()
    assert len(declared) >= 22
    for name in declared:
        assert hasattr(lib, name), name
    names = {s[0] for s in _abi.SIGNATURES}
    assert set(declared) == names
    assert len(_abi.REFERENCE_SYMBOLS) == 22


def test_libraries_resolve_every_symbol():
    # dlopen with RTLD_NOW fails on any undefined symbol, in both the engine and the
    # plain baseline library (which links the shared Newell builder)
    from fullmag_gb300 import build
    lib_path = build.build()
    for path in (lib_path, build.PLAIN_LIB):
        C.CDLL(str(path), mode=C.RTLD_GLOBAL | 2)  # RTLD_NOW


def test_library_has_no_torch_dependency():
    from fullmag_gb300 import build
    out = subprocess.run(["ldd", str(build.build())], capture_output=True, text=True).stdout
    assert "torch" not in out and "c10" not in out


def test_null_safety_without_gpu():
    from fullmag_gb300 import load_library
    lib = load_library()
    assert lib.fullmag_fdm_backend_create(None) is None
    assert lib.fullmag_fdm_backend_create_periodic(None, None) is None
    lib.fullmag_fdm_backend_destroy(None)
    lib.fullmag_fdm_field_snapshot_destroy(None)
    lib.fullmag_fdm_preview_snapshot_destroy(None)
    assert lib.fullmag_fdm_backend_last_error(None) == b"null handle"
    st = _abi.StepStats()
    assert lib.fullmag_fdm_backend_step(None, 1e-13, C.byref(st)) == _abi.ERR_INVALID


def test_plan_builder_keeps_every_caller_value():
    """make_plan fills each plan field from its argument (native_fdm.rs:132-499): the SOT
    polarisation and thickness, the Oersted axis, region ids and the stiffness table reach
    the plan unchanged."""
    import numpy as np
    from fullmag_gb300.backend import make_plan
    reg = np.array([0, 1, 1, 2], dtype=np.uint32)
    lut = np.arange(256 * 256, dtype=np.float64) * 1e-15
    p, keep = make_plan(nx=4, ny=1, nz=1, dx=1e-9, dy=1e-9, dz=1e-9, ms=8e5, a_ex=1e-11, alpha=0.1,
                        m0=np.tile([1.0, 0.0, 0.0], 4), sot_je=1.0, sot_sigma=(0.0, 1.0, 0.0),
                        sot_thickness=2e-9, oersted_current=1.0, oersted_radius=1e-9,
                        oersted_axis=(1.0, 0.0, 0.0), region_mask=reg, exchange_lut=lut)
    assert list(p.sot_sigma) == [0.0, 1.0, 0.0] and p.sot_thickness == 2e-9
    assert list(p.oersted_axis) == [1.0, 0.0, 0.0]
    assert p.region_mask_len == 4 and [p.region_mask[i] for i in range(4)] == [0, 1, 1, 2]
    assert p.exchange_lut_len == 256 * 256 and p.exchange_lut[257] == lut[257]


def test_header_matches_reference_layout(tmp_path):
    """include/fullmag_fdm.h against the reference header's own layout, recorded by
    tests/golden/make_abi_golden.py from native/include/fullmag_fdm.h: every struct of
    the reference has the same size, the same fields in the same order at the same
    offsets; every enum constant has the same value; every reference function is
    declared."""
    import json
    import sys
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from make_abi_golden import parse_header, probe
    gold = json.loads((ROOT / "tests" / "golden" / "abi_layout.json").read_text())
    structs, constants, functions = parse_header(HEADER.read_text())
    for s, fields in gold["field_order"].items():
        assert s in structs, s
        # the reference's fields, in its order, lead each struct (no field is inserted)
        assert structs[s][:len(fields)] == fields, s
    mine = probe(HEADER, gold["field_order"], list(gold["constants"]), tmp_path)
    for s, d in gold["structs"].items():
        assert mine["structs"][s]["size"] == d["size"], s
        assert mine["structs"][s]["fields"] == d["fields"], s
    assert mine["constants"] == gold["constants"]
    assert set(gold["functions"]) <= set(functions)
    assert len(gold["functions"]) == 22


def _plan(nx, ny, nz):
    import numpy as np
    from fullmag_gb300.backend import make_plan
    m0 = np.tile([1.0, 0.0, 0.0], (nx * ny * nz, 1))
    return make_plan(nx=nx, ny=ny, nz=nz, dx=2e-9, dy=2e-9, dz=2e-9, ms=8e5, a_ex=1.3e-11, alpha=0.5, m0=m0)


@pytest.mark.parametrize("shape,periodic,images,message", [
    ((8, 8, 2), (2, 0, 0), None, b"periodic[] entries must be 0 (open) or 1 (periodic)"),
    ((8, 8, 2), (1, 0, 0), (5000, 0, 0), b"image_counts above 4096"),
    ((9, 8, 2), (1, 0, 0), None, b"a periodic x axis needs an even number of cells"),
])
def test_periodic_create_refusals_without_gpu(shape, periodic, images, message):
    # the periodic entry point validates its descriptor and the periodic geometry on the
    # host, before any device work: a handle comes back with last_error set
    from fullmag_gb300 import load_library
    lib = load_library()
    p, keep = _plan(*shape)
    d = _abi.PeriodicityDesc()
    for a, v in enumerate(periodic):
        d.periodic[a] = v
    if images is not None:
        d.has_image_counts = 1
        for a, v in enumerate(images):
            d.image_counts[a] = v
    h = lib.fullmag_fdm_backend_create_periodic(C.byref(p), C.byref(d))
    try:
        assert h
        assert lib.fullmag_fdm_backend_last_error(h) == message
    finally:
        lib.fullmag_fdm_backend_destroy(h)
    del keep


@pytest.mark.parametrize("edit,message", [
    (lambda p: setattr(p, "initial_magnetization_len", 5), b"initial_magnetization_len mismatch: expected 384, got 5"),
    (lambda p: setattr(p.grid, "dx", 0.0), b"cell sizes must be positive"),
    (lambda p: setattr(p.material, "saturation_magnetisation", -1.0), b"saturation_magnetisation must be positive"),
    (lambda p: setattr(p, "active_mask_len", 7), b"active_mask_len mismatch: expected 128, got 7"),
])
def test_create_refusals_without_gpu(edit, message):
    # the plan validation of create runs on the host before any device work and reports
    # through last_error on a non-NULL handle (api.cpp:170-180, 324-395)
    import numpy as np
    from fullmag_gb300 import load_library
    lib = load_library()
    p, keep = _plan(8, 8, 2)
    mask = np.ones(8 * 8 * 2, dtype=np.uint8)
    p.active_mask = mask.ctypes.data_as(C.POINTER(C.c_uint8))
    p.active_mask_len = mask.size
    edit(p)
    h = lib.fullmag_fdm_backend_create(C.byref(p))
    try:
        assert h
        assert lib.fullmag_fdm_backend_last_error(h) == message
    finally:
        lib.fullmag_fdm_backend_destroy(h)
    del keep


@pytest.mark.parametrize("edit,periodic,message", [
    (lambda p: (setattr(p, "has_interfacial_dmi", 1), setattr(p, "dmi_D_interfacial", 1e-3)), None,
     b"DMI is not available with double-precision state (use SINGLE)"),
    (lambda p: setattr(p, "temperature", 300.0), None, b"thermal noise is not available with double-precision state (use SINGLE)"),
    (lambda p: None, (1, 0, 0), None),
])
def test_double_precision_refusals_without_gpu(edit, periodic, message):
    # the double-precision path refuses the terms it does not carry before any device work;
    # with periodic axes it refuses the boundary-correction tiers
    import numpy as np
    from fullmag_gb300 import load_library
    lib = load_library()
    p, keep = _plan(8, 8, 2)
    p.precision = _abi.PRECISION_DOUBLE
    edit(p)
    if periodic is None:
        h = lib.fullmag_fdm_backend_create(C.byref(p))
    else:
        n = 8 * 8 * 2
        phi = np.ones(n)
        p.boundary_correction = _abi.BOUNDARY_VOLUME
        p.volume_fraction = phi.ctypes.data_as(C.POINTER(C.c_double))
        p.volume_fraction_len = n
        faces = [np.ones(n) for _ in range(6)]
        for name, f in zip(("face_link_xp", "face_link_xm", "face_link_yp", "face_link_ym", "face_link_zp",
                            "face_link_zm"), faces):
            setattr(p, name, f.ctypes.data_as(C.POINTER(C.c_double)))
        d = _abi.PeriodicityDesc()
        for a, v in enumerate(periodic):
            d.periodic[a] = v
        h = lib.fullmag_fdm_backend_create_periodic(C.byref(p), C.byref(d))
        message = b"boundary correction is not available with periodic boundaries"
    try:
        assert h
        assert lib.fullmag_fdm_backend_last_error(h) == message
    finally:
        lib.fullmag_fdm_backend_destroy(h)
    del keep
