"""Record the reference C ABI's binary layout into abi_layout.json.

Reads native/include/fullmag_fdm.h of a mzrptu/fullmag checkout as text to list every
typedef'd struct with its field names, every enum constant and every declared
function, then compiles a small probe against that header with the host C compiler
and records what the compiler lays out: sizeof and offsetof of every field, and the
value of every enum constant.  No reference code runs; the probe only includes the
header.  tests/test_abi_layout.py compiles the same probe against include/fullmag_fdm.h
and compares it with this file.

Usage: python tests/golden/make_abi_golden.py <path of a mzrptu/fullmag checkout>
"""
import json
import re
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
HEADER_REL = "native/include/fullmag_fdm.h"


def strip_comments(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def parse_header(text):
    """(structs, enums, functions) of a header's text: struct name -> field names in
    order, enum constant names in order, function names."""
    text = strip_comments(text)
    structs = {}
    for body, name in re.findall(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            for part in decl.split(","):
                m = re.search(r"(\w+)\s*(\[[^\]]*\])*\s*$", part.strip())
                fields.append(m.group(1))
        structs[name] = fields
    enums = []
    for body in re.findall(r"typedef\s+enum\s*\{(.*?)\}\s*\w+\s*;", text, flags=re.S):
        for item in body.split(","):
            m = re.match(r"\s*(\w+)", item)
            if m:
                enums.append(m.group(1))
    defines = re.findall(r"#define\s+(FULLMAG_FDM_[A-Z0-9_]+)\s+-?\d+", text)
    functions = sorted(set(re.findall(r"\b(fullmag_fdm_[a-z0-9_]+)\s*\(", text)))
    return structs, enums + defines, functions


def probe(header, structs, constants, workdir):
    """Compile and run the layout probe against `header`; returns the JSON-ready dict."""
    lines = [f'#include "{header}"', "#include <stdio.h>", "#include <stddef.h>", "int main(void){"]
    for s, fields in structs.items():
        lines.append(f'printf("S {s} %zu\\n", sizeof({s}));')
        for f in fields:
            lines.append(f'printf("F {s} {f} %zu\\n", offsetof({s}, {f}));')
    for c in constants:
        lines.append(f'printf("C {c} %lld\\n", (long long)({c}));')
    lines.append("return 0;}")
    src = Path(workdir) / "abi_probe.c"
    exe = Path(workdir) / "abi_probe"
    src.write_text("\n".join(lines))
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    res = {"structs": {}, "constants": {}}
    for line in out.splitlines():
        t = line.split()
        if t[0] == "S":
            res["structs"].setdefault(t[1], {"fields": {}})["size"] = int(t[2])
        elif t[0] == "F":
            res["structs"][t[1]]["fields"][t[2]] = int(t[3])
        else:
            res["constants"][t[1]] = int(t[2])
    return res


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_abi_golden.py <path of a mzrptu/fullmag checkout>")
    header = Path(sys.argv[1]) / HEADER_REL
    structs, constants, functions = parse_header(header.read_text())
    with tempfile.TemporaryDirectory() as d:
        res = probe(header, structs, constants, d)
    res["field_order"] = structs
    res["functions"] = functions
    res["source"] = HEADER_REL
    (HERE / "abi_layout.json").write_text(json.dumps(res, indent=1, sort_keys=True) + "\n")
    print(f"{len(structs)} structs, {sum(map(len, structs.values()))} fields, {len(constants)} constants, "
          f"{len(functions)} functions")


if __name__ == "__main__":
    main()
