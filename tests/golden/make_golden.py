"""Extract the reference's own known-answer values for the FDM path into newell_kat.json.

Reads the reference test sources as text (no reference code is run):
  crates/fullmag-fdm-demag/src/newell.rs:676-908   Newell tensor known answers
  native/backends/fdm/tests/tier_a_compare.cu      Tier A case definition and tolerances
  native/backends/fdm/tests/tier_b_compare.cu      Tier B tolerances
Usage: python tests/golden/make_golden.py /path/to/fullmag
"""
import json
import re
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_golden.py <path of a mzrptu/fullmag checkout>")
root = Path(sys.argv[1])
newell = (root / "crates/fullmag-fdm-demag/src/newell.rs").read_text()


def ref_value(tag):
    # lines like "// Reference: -4.55648226e-02" that follow the N_xy(i,j,0) comment
    m = re.search(r"// N_xy\(" + tag + r"\)[^\n]*\n\s*// Reference:\s*([-0-9.e+]+)", newell)
    return float(m.group(1))


def assert_tol(name):
    # `(nxy_11 - (-4.5565e-2)).abs() < 1e-5` -> (check value, tolerance)
    m = re.search(r"\(" + name + r" - \(([-0-9.e+]+)\)\)\.abs\(\) < ([0-9.e+-]+)", newell)
    return float(m.group(1)), float(m.group(2))


kat = {
    "source": "crates/fullmag-fdm-demag/src/newell.rs (tests module)",
    "nxy_10x10x1_unit": {},
}
for tag, var in (("1,1,0", "nxy_11"), ("2,2,0", "nxy_22"), ("5,5,0", "nxy_55")):
    chk, tol = assert_tol(var)
    kat["nxy_10x10x1_unit"][tag] = {"reference": ref_value(tag), "check": chk, "tol": tol}
kat["self_trace_tol"] = 1e-10
kat["cubic_self_third_tol"] = 1e-6
kat["offdiag_self_zero_tol"] = 1e-12
kat["asymptotic_rel_tol_8_8_0"] = 1e-3

tier_a = (root / "native/backends/fdm/tests/tier_a_compare.cu").read_text()
tier_b = (root / "native/backends/fdm/tests/tier_b_compare.cu").read_text()
kat["tier_a_source"] = "native/backends/fdm/tests/tier_a_compare.cu"
kat["tier_b_source"] = "native/backends/fdm/tests/tier_b_compare.cu"
nums = {}
for key, pat in (("nx", r"\bnx\s*=\s*(\d+)"), ("ny", r"\bny\s*=\s*(\d+)"), ("nz", r"\bnz\s*=\s*(\d+)"),
                 ("steps", r"\bnsteps\s*=\s*(\d+)"), ("dt", r"\bdt\s*=\s*([0-9.e+-]+);"),
                 ("m_tol", r"TIER_A_M_TOL\s*=\s*([0-9.e+-]+)"), ("e_tol", r"TIER_A_E_TOL\s*=\s*([0-9.e+-]+)")):
    m = re.search(pat, tier_a)
    if m:
        nums[key] = float(m.group(1))
kat["tier_a_case"] = nums
kat["tier_b_tolerances"] = {
    "m_tol": float(re.search(r"TIER_B_M_TOL\s*=\s*([0-9.e+-]+)", tier_b).group(1)),
    "e_tol": float(re.search(r"TIER_B_E_TOL\s*=\s*([0-9.e+-]+)", tier_b).group(1)),
}
out = Path(__file__).with_name("newell_kat.json")
out.write_text(json.dumps(kat, indent=2) + "\n")
print(out.read_text())
