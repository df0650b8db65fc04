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
    ("fullmag_fdm_grid_desc", _abi.GridDesc), ("fullmag_fdm_material_desc", _abi.MaterialDesc)])
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


def test_library_has_no_torch_dependency():
    from fullmag_gb300 import build
    out = subprocess.run(["ldd", str(build.build())], capture_output=True, text=True).stdout
    assert "torch" not in out and "c10" not in out


def test_null_safety_without_gpu():
    from fullmag_gb300 import load_library
    lib = load_library()
    assert lib.fullmag_fdm_backend_create(None) is None
    lib.fullmag_fdm_backend_destroy(None)
    lib.fullmag_fdm_field_snapshot_destroy(None)
    lib.fullmag_fdm_preview_snapshot_destroy(None)
    assert lib.fullmag_fdm_backend_last_error(None) == b"null handle"
    st = _abi.StepStats()
    assert lib.fullmag_fdm_backend_step(None, 1e-13, C.byref(st)) == _abi.ERR_INVALID
