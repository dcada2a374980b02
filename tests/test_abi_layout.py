"""The Python mirror's view of the C ABI equals the header's: every
constant `include/krabgpu.h` defines has the same value in `_lib`, and every
public struct has the same size and field offsets as `ctypes` lays it out.
The header is compiled as plain C by the host compiler (no GPU needed)."""
import ctypes as C
import json
import os
import re
import shutil
import subprocess

import pytest

from krabmaga_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "krabgpu.h")

STRUCTS = {
    "kb_field_desc": L.FieldDesc,
    "kb_flock_params": L.FlockParamsC,
    "kb_replica_desc": L.ReplicaDesc,
    "kb_server_desc": L.ServerDesc,
    "kb_request": L.RequestC,
    "kb_server_report": L.ServerReport,
}


def header_constants():
    out = {}
    for m in re.finditer(r"^#define\s+(KB_[A-Z0-9_]+)\s+(0x[0-9a-fA-F]+|\d+)u?\b", open(HEADER).read(), re.M):
        out[m.group(1)] = int(m.group(2), 0)
    return out


def test_every_header_constant_is_mirrored():
    consts = header_constants()
    assert len(consts) >= 25
    for name, value in consts.items():
        assert getattr(L, name, None) == value, name


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "krabgpu.h"', "int main(void) {",
             '  printf("{");']
    first = True
    for sname, cls in STRUCTS.items():
        parts = [f'\\"size\\": %zu']
        args = [f"sizeof({sname})"]
        for fname, _ in cls._fields_:
            parts.append(f'\\"{fname}\\": %zu')
            args.append(f"offsetof({sname}, {fname})")
        sep = "" if first else ", "
        first = False
        lines.append(f'  printf("{sep}\\"{sname}\\": {{{", ".join(parts)}}}", {", ".join(args)});')
    lines += ['  printf("}\\n");', "  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    return json.loads(subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout)


@pytest.mark.parametrize("sname", sorted(STRUCTS))
def test_struct_layout_matches_ctypes(c_layout, sname):
    cls = STRUCTS[sname]
    got = c_layout[sname]
    assert got["size"] == C.sizeof(cls), sname
    for fname, _ in cls._fields_:
        assert got[fname] == getattr(cls, fname).offset, (sname, fname)


def _header_arities():
    h = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(kb_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", h):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


RUST_SYS = os.path.join(ROOT, "rust", "krabgpu-sys", "src", "lib.rs")


def _rust_externs():
    src = open(RUST_SYS).read()
    bound = {}
    for m in re.finditer(r"pub fn (kb_[a-z0-9_]+)\s*\(([^;]*?)\)\s*(->[^;]*)?;", src, flags=re.S):
        args = re.sub(r"//[^\n]*", "", m.group(2)).strip().rstrip(",")
        bound[m.group(1)] = 0 if not args else args.count(",") + 1
    return src, bound


def test_rust_binding_covers_the_header():
    # the extern "C" block of the Rust crate a maintainer adds to the reference
    # names every entry point of the header, each with the header's parameter count
    hdr = _header_arities()
    _, bound = _rust_externs()
    assert set(bound) == set(hdr), (set(hdr) - set(bound), set(bound) - set(hdr))
    for name, n in bound.items():
        assert hdr[name] == n, name


def test_rust_structs_and_constants_match_the_header():
    # every #[repr(C)] struct lists the ctypes mirror's fields in the same order,
    # and every constant the crate defines has the header's value
    src, _ = _rust_externs()
    for sname, cls in STRUCTS.items():
        m = re.search(r"pub struct " + sname + r"\s*\{(.*?)\n\}", src, flags=re.S)
        assert m, sname
        fields = re.findall(r"pub ([a-z0-9_]+)\s*:", m.group(1))
        assert fields == [f for f, _ in cls._fields_], sname
    consts = header_constants()
    found = re.findall(r"pub const (KB_[A-Z0-9_]+)\s*:\s*[a-z0-9_]+\s*=\s*(0x[0-9a-fA-F]+|\d+)\s*;", src)
    assert {n for n, _ in found} == set(consts), set(consts) ^ {n for n, _ in found}
    for name, v in found:
        assert consts[name] == int(v, 0), name


def test_rust_facade_keeps_the_reference_names():
    # the safe crate implements the reference's State and Field traits and keeps
    # Field2D's method names
    src = open(os.path.join(ROOT, "rust", "krabmaga-gpu", "src", "lib.rs")).read()
    assert "impl State for GpuFlocker" in src and "impl Field for GpuField2D" in src
    for name in ["set_object_location", "lazy_update", "get_neighbors_within_relax_distance",
                 "get_neighbors_within_distance", "get_objects", "num_objects_at_location",
                 "get_empty_bags", "iter_objects", "remove_object_location", "get_location"]:
        assert re.search(r"fn " + name + r"\b", src), name
    hdr = _header_arities()
    for fn in re.findall(r"sys::(kb_[a-z0-9_]+)\s*\(", src):
        assert fn in hdr, fn


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "krabgpu.h"

int main(void) {
    uint32_t ids[64];
    float xy[128], dxy[128];
    kb_field* f = NULL;
    kb_field_desc desc = {10.0f, 10.0f, 0.5f, 1, 0, 0, KB_CELL_WRAP_CLAMP};
    if (strstr(kb_version(), "sm_103a") == NULL) return 1;
    if (kb_gen_uniform(64, 50.0f, 40.0f, 7, 1.0f, ids, xy, dxy) != KB_OK) return 2;
    if (kb_field_create(NULL, &f) != KB_ERR_ARG || f != NULL) return 3;
    if (strlen(kb_last_error()) == 0) return 4;
    if (kb_device_count() == 0 && kb_field_create(&desc, &f) != KB_ERR_NO_DEVICE) return 5;
    for (int i = 0; i < 64; ++i) printf("%u %a %a %a %a\n", ids[i], xy[2 * i], xy[2 * i + 1], dxy[2 * i], dxy[2 * i + 1]);
    return 0;
}
"""


def test_plain_c_caller_links_and_agrees_with_ctypes(tmp_path):
    # the library as a C program links it: header compiled as C99, no C++ name
    # mangling; the host generator gives the same bits through either caller
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(L.LIB_PATH)
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.dirname(HEADER), str(src),
                    "-L", libdir, "-lkrabgpu", "-Wl,-rpath," + libdir, "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.returncode
    import numpy as np
    import krabmaga_gb300 as kg
    ids, xy, dxy = kg.gen_uniform(64, 50.0, 40.0, 7, 1.0)
    rows = [ln.split() for ln in out.stdout.strip().splitlines()]
    assert [int(r[0]) for r in rows] == ids.tolist()
    got = np.array([[float.fromhex(v) for v in r[1:]] for r in rows], np.float32)
    assert np.array_equal(got[:, :2], xy) and np.array_equal(got[:, 2:], dxy)
