"""CPU tests of the C-ABI library: it builds for sm_103a, loads without a
GPU, exports every entry point include/metada_gb300.h declares, and rejects
bad arguments with status codes (no compute call is made here)."""
import ctypes
import re

import pytest

from conftest import ROOT

from metada_gb300 import _lib


def declared_entry_points():
    text = (ROOT / "include" / "metada_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_bound_entry_points():
    declared = declared_entry_points()
    assert declared, "no entry points found in the header"
    assert set(declared) == set(_lib.EXPORTED), (set(declared) ^ set(_lib.EXPORTED))


def test_library_exports_every_declared_symbol(built):
    lib = _lib.load()
    for name in declared_entry_points():
        assert hasattr(lib, name), f"{name} not exported"


def test_version_and_null_context(built):
    lib = _lib.load()
    assert b"sm_103a" in lib.mg_version()
    assert lib.mg_last_error(None) == b"null context"
    assert lib.mg_ens_mean(None, None, 10, 2, 10, None) == _lib.MG_ERR_ARG
    assert lib.mg_letkf_batched(None, None) == _lib.MG_ERR_ARG
    assert lib.mg_create(None, 0) == _lib.MG_ERR_ARG


def test_create_without_gpu_reports_cuda_error(built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present; covered by the GPU tests")
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.mg_create(ctypes.byref(h), 0)
    assert rc == _lib.MG_ERR_CUDA and not h.value


def test_descriptor_layout_matches_header(tmp_path):
    """The ctypes mirrors have the C structs' sizes and field offsets, as a
    C compiler lays out include/metada_gb300.h."""
    import subprocess

    structs = {"mg_letkf_desc": _lib.LetkfDesc, "mg_letkf_stats": _lib.LetkfStats, "mg_etkf_case": _lib.EtkfCase}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "metada_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(line.split()[:2]): int(line.split()[2]) for line in out if line.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
