"""CPU test: the C++ drop-in policies compile and link against the
reference's own adapter headers (skipped where the reference tree is absent,
e.g. on the GPU host)."""
import os
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

REF = Path(os.environ["METADA_REFERENCE"]) if os.environ.get("METADA_REFERENCE") else None


@pytest.mark.skipif(REF is None or not (REF / "src").is_dir(),
                    reason="METADA_REFERENCE does not name the reference tree")
@pytest.mark.parametrize("src", ["dropin_reference.cpp", "dropin_gb300_reference.cpp"])
def test_dropin_policies_compile_against_reference_adapters(built, tmp_path, src):
    """dropin_reference.cpp: the policies over the reference's Simple backend;
    dropin_gb300_reference.cpp: the Gb300BackendTag backend set (device
    state) with the reference's adapters, including the StateBackendImpl
    concept check."""
    incs = []
    for d in ("traits", "framework/base", "framework/algorithms", "framework/adapters",
              "framework/adapters/common/utils/config", "framework/adapters/common/utils/logger",
              "backends/simple", "backends/common/observation", "backends/common/obsoperator",
              "backends/common/utils/logger/console"):
        incs += ["-I", str(REF / "src" / d)]
    cuda = Path("/usr/local/cuda")
    out = tmp_path / "dropin_reference"
    cmd = ["g++", "-std=c++20", "-O1", "-w", "-include", "algorithm", "-include", "numeric",
           "-I", str(ROOT / "include"), "-I", str(ROOT / "oracle"), "-I", str(cuda / "include"), *incs,
           str(ROOT / "tests" / "cpp" / src), "-o", str(out),
           "-L", str(ROOT / "metada_gb300" / "_lib"), "-lmetada_gb300",
           "-L", str(cuda / "lib64"), "-lcudart", f"-Wl,-rpath,{ROOT / 'metada_gb300' / '_lib'}"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-4000:]
    assert out.exists()
