"""GPU: the C++ drop-in policies (include/metada_gb300/analysis.hpp) run
through adapter stand-ins and reproduce the reference's golden analyses."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, rel_err

pytestmark = pytest.mark.gpu


def _cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    return Path(nvcc).resolve().parent.parent if nvcc else Path("/usr/local/cuda")


@pytest.fixture(scope="module")
def dropin_exe(built, tmp_path_factory):
    out = tmp_path_factory.mktemp("cpp") / "dropin_mock"
    cuda = _cuda_home()
    lib = ROOT / "metada_gb300" / "_lib"
    cmd = ["g++", "-std=c++20", "-O2", "-I", str(ROOT / "include"), "-I", str(cuda / "include"),
           str(ROOT / "tests" / "cpp" / "dropin_mock.cpp"), "-o", str(out), "-L", str(lib), "-lmetada_gb300",
           "-L", str(cuda / "lib64"), "-lcudart", f"-Wl,-rpath,{lib}", f"-Wl,-rpath,{cuda / 'lib64'}"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-3000:]
    return out


def _write_case(d: Path, g, rho_key="rho"):
    X = g["X"]
    k, n = X.shape
    p = len(g["yo"])
    radius = float(g["radius"]) if "radius" in g else 0.0
    (d / "meta.txt").write_text(f"{int(g['nx'])} {int(g['ny'])} {k} {p} {float(g['sigma'])!r} "
                                f"{float(g[rho_key])!r} {radius!r}\n")
    np.ascontiguousarray(X, dtype="<f8").tofile(d / "X.bin")
    np.ascontiguousarray(g["obs_xy"], dtype="<i4").tofile(d / "obs_xy.bin")
    np.ascontiguousarray(g["yo"], dtype="<f8").tofile(d / "yo.bin")
    return k, n


def _run(exe, d, mode, k, n):
    out = d / mode
    out.mkdir()
    proc = subprocess.run([str(exe), str(d), mode, str(out)], capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr
    members = np.fromfile(out / "members.bin", dtype="<f8").reshape(k, n)
    mean = np.fromfile(out / "mean.bin", dtype="<f8")
    return members, mean


@pytest.mark.parametrize("name,rho_key,golden", [("tutorial", "rho", "letkf"), ("tutorial", "rho11", "letkf_rho11"),
                                                 ("letkf_grid24", "rho", None), ("letkf_grid20", "rho", None)])
def test_cpp_letkf_sequential_matches_reference(dropin_exe, tmp_path, name, rho_key, golden):
    g = np.load(GOLDEN / f"{name}.npz")
    k, n = _write_case(tmp_path, g, rho_key)
    members, mean = _run(dropin_exe, tmp_path, "letkf_sequential", k, n)
    want = g[f"{golden}_members"] if golden else g["members"]
    wmean = g[f"{golden}_mean"] if golden else g["mean"]
    assert rel_err(members, want) <= 1e-10
    assert rel_err(mean, wmean) <= 1e-10


@pytest.mark.parametrize("mode", ["etkf_reference", "etkf_reference_host_h"])
def test_cpp_etkf_matches_reference(dropin_exe, tmp_path, mode):
    g = np.load(GOLDEN / "tutorial.npz")
    k, n = _write_case(tmp_path, g)
    members, mean = _run(dropin_exe, tmp_path, mode, k, n)
    assert rel_err(members, g["etkf_members"]) <= 1e-10
    assert np.array_equal(mean, g["etkf_mean"])  # background mean left in Mean()


def test_cpp_letkf_batched_modes_run(dropin_exe, tmp_path):
    import oracle.bind as ob

    g = np.load(GOLDEN / "letkf_grid24.npz")
    k, n = _write_case(tmp_path, g)
    X, nx, ny = g["X"], int(g["nx"]), int(g["ny"])
    s = float(g["sigma"])
    HX = ob.hx_idw4(X, nx, ny, g["obs_xy"])
    off, idx = ob.select_grid(nx, ny, g["obs_xy"], float(g["radius"]))
    for mode, flags, tol in (("letkf_batched_reference", ob.ORC_COMPAT, 1e-10), ("letkf_batched_hunt_mixed", 0, 1e-5)):
        members, _ = _run(dropin_exe, tmp_path, mode, k, n)
        want = ob.letkf_points(X, np.arange(nx * ny), 1, 0, HX, g["yo"], np.full(len(g["yo"]), s * s), off, idx, None,
                               float(g["rho"]), flags)[:, 0, :].T
        assert rel_err(members, want) <= tol, mode


def test_cpp_enkf_seeded_matches_reference(dropin_exe, tmp_path):
    """metada_gb300::EnKF with seed 1234 draws the perturbations the
    reference's EnKF.hpp draws when its random_device returns 1234."""
    g = np.load(GOLDEN / "tutorial.npz")
    e = np.load(GOLDEN / "enkf.npz")
    k, n = _write_case(tmp_path, g)
    members, mean = _run(dropin_exe, tmp_path, "enkf_seed1234", k, n)
    assert rel_err(members, e["tut_members"]) <= 1e-10
    assert rel_err(mean, e["tut_mean"]) <= 1e-10
    diag = np.fromfile(tmp_path / "enkf_seed1234" / "diag.bin", dtype="<f8")
    np.testing.assert_allclose(diag, e["tut_diag"][:3], rtol=1e-10)


@pytest.fixture(scope="module")
def device_exe(built, tmp_path_factory):
    out = tmp_path_factory.mktemp("cppdev") / "dropin_device"
    cuda = _cuda_home()
    lib = ROOT / "metada_gb300" / "_lib"
    cmd = ["g++", "-std=c++20", "-O2", "-I", str(ROOT / "include"), "-I", str(cuda / "include"),
           str(ROOT / "tests" / "cpp" / "dropin_device.cpp"), "-o", str(out), "-L", str(lib), "-lmetada_gb300",
           "-L", str(cuda / "lib64"), "-lcudart", f"-Wl,-rpath,{lib}", f"-Wl,-rpath,{cuda / 'lib64'}"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-3000:]
    return out


def test_device_state_two_letkf_cycles_stay_on_device(device_exe, tmp_path):
    """The device-resident state backend (Gb300BackendTag's state): members
    parsed from SimpleState text on the device, two reference-order LETKF
    cycles with the members kept in device memory (no upload or download of
    state data during either Analyse), the ensemble mean recomputed on the
    device (bit-identical to the reference's member-order sum), and the
    mean written by the device formatter."""
    import oracle.bind as ob

    g = np.load(GOLDEN / "tutorial.npz")
    X, nx, ny = g["X"], int(g["nx"]), int(g["ny"])
    k, n = X.shape
    p = len(g["yo"])
    (tmp_path / "meta.txt").write_text(f"{nx} {ny} {k} {p} {float(g['sigma'])!r} {float(g['rho'])!r} "
                                       f"{float(g['radius'])!r}\n")
    for i in range(k):
        rows = X[i].reshape(ny, nx)
        (tmp_path / f"ens_{i + 1}.txt").write_text("\n".join(" ".join(f"{v:.17g}" for v in r) for r in rows) + "\n")
    np.ascontiguousarray(g["obs_xy"], dtype="<i4").tofile(tmp_path / "obs_xy.bin")
    np.ascontiguousarray(g["yo"], dtype="<f8").tofile(tmp_path / "yo.bin")
    out = tmp_path / "out"
    out.mkdir()
    proc = subprocess.run([str(device_exe), str(tmp_path), str(out)], capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr
    c1 = np.fromfile(out / "cycle1.bin", dtype="<f8").reshape(k, n)
    c2 = np.fromfile(out / "cycle2.bin", dtype="<f8").reshape(k, n)
    assert rel_err(c1, g["letkf_members"]) <= 1e-10  # the reference's own LETKF (golden)
    want2, _ = ob.letkf_compat_grid(c1, nx, ny, g["obs_xy"], g["yo"], float(g["radius"]), float(g["rho"]))
    assert rel_err(c2, want2) <= 1e-10
    t0, t1, t1b, t2 = map(int, (out / "transfers.txt").read_text().split())
    assert t1 == t0 and t2 == t1b  # no state data crossed to or from the host inside Analyse
    mean = np.zeros(n)
    for i in range(k):
        mean = mean + c2[i]
    mean = mean * (1.0 / k)
    text = "".join(" ".join(f"{v:12.6f}" for v in mean[y * nx:(y + 1) * nx]) + "\n" for y in range(ny))
    assert (out / "mean.txt").read_text() == text
