"""Generates the golden fixtures in this directory by running the reference's
own analysis headers (oracle/_ref/ref_harness, built by oracle/build_ref.sh
from the reference tree) on:

  * the reference tutorial data (src/backends/simple/tutorial: 9 members on
    a 36 x 18 grid, 28 grid observations, error 0.1), ETKF and LETKF
    (radius 10) with inflation 1.0 as in etkf.yaml / letkf.yaml, and the
    LETKF again with inflation 1.1;
  * the seeded 64 x 64, 32-member, 1024-observation global ETKF case
    (inflation 1.05, error 0.5);
  * two seeded small-grid LETKF cases (some grid points without local
    observations);
  * the stochastic EnKF (EnKF.hpp) on the tutorial data and on the seeded
    64 x 64 case, with the harness's seeded generator in place of the
    reference's std::random_device; the perturbations it drew are stored
    with the outputs.

Run from the repository root, in a checkout that has the reference tree:
    python tests/golden/make_golden.py [REFERENCE_ROOT]
The fixtures are small .npz files holding inputs and reference outputs.
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from metada_gb300 import synthetic as syn  # noqa: E402
from metada_gb300.build import build_reference_harness  # noqa: E402

HARNESS = ROOT / "oracle" / "_ref" / "ref_harness"


def read_simple_state(path: Path) -> np.ndarray:
    return np.array([float(v) for v in path.read_text().split()], dtype=np.float64)


def read_grid_obs(path: Path, missing: float = -999.0):
    """Parses the GridObservation text format (GridObservation.hpp:416-469)."""
    xy, vals = [], []
    header = started = False
    for line in path.read_text().splitlines():
        if not line:
            continue
        if "Time" in line and "XLONG_U" in line:
            header = True
            continue
        if "---" in line and not line.strip("- \t"):
            if header:
                started = True
            continue
        if not started:
            continue
        parts = line.split()
        if len(parts) < 8:
            continue
        x, y = int(parts[3]), int(parts[2])
        v = float(parts[7])
        if v != missing:
            xy.append((x, y))
            vals.append(v)
    return np.array(xy, dtype=np.int32), np.array(vals, dtype=np.float64)


def run_harness(algo: str, nx: int, ny: int, k: int, ens_prefix: str, obs_file: str, error: float,
                rho: float, radius: float, out: Path, seed: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    out.mkdir(parents=True, exist_ok=True)
    cmd = [str(HARNESS), algo, str(nx), str(ny), str(k), ens_prefix, obs_file, repr(error), repr(rho),
           repr(radius), str(out)] + ([str(seed)] if seed is not None else [])
    subprocess.run(cmd, check=True)
    n = nx * ny
    members = np.stack([np.fromfile(out / f"member_{i}.bin", dtype="<f8", count=n) for i in range(k)])
    mean = np.fromfile(out / "mean.bin", dtype="<f8", count=n)
    return members, mean


def run_nearest(lat, lon, nx, ny, vc, olat, olon, olev, tmp: Path) -> np.ndarray:
    """The reference's IdentityObsOperator geographic branch (nearest node and
    level, IdentityObsOperator.hpp:484-520) through the harness: (i, j, k)
    per observation."""
    fin, fout = tmp / "near_in.bin", tmp / "near_out.bin"
    with open(fin, "wb") as f:
        np.array([nx, ny, len(vc), len(olat)], dtype="<i8").tofile(f)
        for a in (lat, lon, vc, olat, olon, olev):
            np.ascontiguousarray(a, dtype="<f8").tofile(f)
    subprocess.run([str(HARNESS), "nearest", str(fin), str(fout)], check=True)
    return np.fromfile(fout, dtype="<i8").reshape(-1, 3)


def make_nearest(tmp: Path) -> None:
    """Golden nearest nodes: a curvilinear grid (obs inside and outside it,
    on nodes, at midpoints of two nodes) and a regular 0.5 degree grid whose
    midpoints are exact ties; levels with exact midpoint ties."""
    out = {}
    g = np.random.default_rng(20261203 + 600)
    nx, ny = 40, 30
    lon, lat = np.meshgrid(np.linspace(70.0, 140.0, nx), np.linspace(5.0, 55.0, ny))
    lon = lon + 0.8 * np.sin(np.deg2rad(lat) * 3.0) + 0.05 * g.standard_normal(lon.shape)
    lat = lat + 0.4 * np.cos(np.deg2rad(lon) * 2.0)
    lat, lon = lat.ravel(), lon.ravel()
    p = 800
    oa, ol = g.uniform(0.0, 60.0, p), g.uniform(60.0, 150.0, p)
    oa[:60], ol[:60] = 0.5 * (lat[:60] + lat[1:61]), 0.5 * (lon[:60] + lon[1:61])
    oa[60:120], ol[60:120] = lat[300:360], lon[300:360]
    vc = np.array([1000.0, 925.0, 850.0, 700.0, 500.0, 300.0, 100.0])
    lev = g.uniform(50.0, 1050.0, p)
    lev[:30] = 0.5 * (1000.0 + 925.0)
    lev[30:40] = 700.0
    out.update(curv_lat=lat, curv_lon=lon, curv_nx=nx, curv_ny=ny, curv_vc=vc, curv_olat=oa, curv_olon=ol,
               curv_olev=lev, curv_ijk=run_nearest(lat, lon, nx, ny, vc, oa, ol, lev, tmp))
    nx, ny = 20, 15
    lon, lat = np.meshgrid(-100.0 + 0.5 * np.arange(nx), 20.0 + 0.5 * np.arange(ny))
    lat, lon = lat.ravel(), lon.ravel()
    i, j = g.integers(0, nx - 1, 300), g.integers(0, ny - 1, 300)
    ol = -100.0 + 0.5 * i + 0.25  # exact midpoints in longitude (ties between i and i + 1)
    oa = 20.0 + 0.5 * j + np.where(np.arange(300) % 2 == 0, 0.25, 0.0)  # and in both directions
    vc = np.array([0.95, 0.85, 0.75, 0.65])
    lev = np.where(np.arange(300) % 3 == 0, 0.9, g.uniform(0.6, 1.0, 300))
    out.update(reg_lat=lat, reg_lon=lon, reg_nx=nx, reg_ny=ny, reg_vc=vc, reg_olat=oa, reg_olon=ol, reg_olev=lev,
               reg_ijk=run_nearest(lat, lon, nx, ny, vc, oa, ol, lev, tmp))
    np.savez_compressed(HERE / "nearest.npz", **out)
    print("nearest.npz", {k2: np.shape(v) for k2, v in out.items() if k2.endswith("ijk")})


def grid_case_to_files(case: syn.GridCase, tmp: Path) -> tuple[str, str]:
    k = case.X.shape[0]
    for i in range(k):
        syn.write_simple_state(tmp / f"ens_{i + 1}.txt", case.X[i], case.nx, case.ny)
    syn.write_grid_obs(tmp / "obs.txt", case.obs_xy, case.yo)
    return str(tmp / "ens_"), str(tmp / "obs.txt")


def main(ref_root: str | None = None, only: str | None = None) -> None:
    import os

    if ref_root:
        os.environ["METADA_REFERENCE"] = ref_root
    if build_reference_harness() is None:
        raise SystemExit("set METADA_REFERENCE (or pass the reference root) to regenerate the golden fixtures")
    ref = Path(os.environ["METADA_REFERENCE"])
    tut = ref / "src" / "backends" / "simple" / "tutorial"
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        if only == "nearest":
            make_nearest(tmp)
            return
        # --- tutorial ---
        nx, ny, k = 36, 18, 9
        X = np.stack([read_simple_state(tut / f"ens_{i}.txt") for i in range(1, k + 1)])
        obs_xy, yo = read_grid_obs(tut / "obs_format.txt")
        sigma = syn.float_config(0.1)
        outs = {}
        for name, algo, rho, radius in (("etkf", "etkf", 1.0, 0.0), ("letkf", "letkf", 1.0, 10.0),
                                        ("letkf_rho11", "letkf", 1.1, 10.0)):
            m, mu = run_harness(algo, nx, ny, k, str(tut / "ens_"), str(tut / "obs_format.txt"), 0.1, rho,
                                radius, tmp / name)
            outs[f"{name}_members"] = m
            outs[f"{name}_mean"] = mu
        np.savez_compressed(HERE / "tutorial.npz", X=X, obs_xy=obs_xy, yo=yo, sigma=sigma, nx=nx, ny=ny,
                            radius=syn.float_config(10.0), rho=1.0, rho11=syn.float_config(1.1), **outs)
        print("tutorial.npz", {k2: v.shape for k2, v in outs.items()})

        # --- seeded 64 x 64 global ETKF ---
        c = syn.global_etkf_grid()
        d = tmp / "c1"
        d.mkdir()
        ens, obsf = grid_case_to_files(c, d)
        m, mu = run_harness("etkf", c.nx, c.ny, c.X.shape[0], ens, obsf, 0.5, 1.05, 0.0, d / "out")
        # inputs are re-read from text by the harness: store exactly what it read
        Xr = np.stack([read_simple_state(d / f"ens_{i + 1}.txt") for i in range(c.X.shape[0])])
        _, yor = read_grid_obs(Path(obsf))
        np.savez_compressed(HERE / "etkf_grid64.npz", X=Xr, obs_xy=c.obs_xy, yo=yor, sigma=c.sigma_o,
                            rho=c.rho, nx=c.nx, ny=c.ny, members=m, mean=mu)
        print("etkf_grid64.npz", m.shape)

        # --- seeded small LETKF grids ---
        for name, args in (("letkf_grid24", dict(nx=24, ny=16, k=8, p=60, radius=5.0, rho=1.05, case=11)),
                           ("letkf_grid20", dict(nx=20, ny=12, k=12, p=30, radius=3.0, rho=1.2, case=12))):
            c = syn.grid_letkf_case(**args)
            d = tmp / name
            d.mkdir()
            ens, obsf = grid_case_to_files(c, d)
            m, mu = run_harness("letkf", c.nx, c.ny, c.X.shape[0], ens, obsf, 0.5, args["rho"], args["radius"],
                                d / "out")
            Xr = np.stack([read_simple_state(d / f"ens_{i + 1}.txt") for i in range(c.X.shape[0])])
            _, yor = read_grid_obs(Path(obsf))
            np.savez_compressed(HERE / f"{name}.npz", X=Xr, obs_xy=c.obs_xy, yo=yor, sigma=c.sigma_o, rho=c.rho,
                                radius=c.radius, nx=c.nx, ny=c.ny, members=m, mean=mu)
            print(f"{name}.npz", m.shape)

        # --- stochastic EnKF (seeded perturbations) ---
        outs = {}
        m, mu = run_harness("enkf", nx, ny, k, str(tut / "ens_"), str(tut / "obs_format.txt"), 0.1, 1.0, 0.0,
                            tmp / "enkf_tut", seed=1234)
        p = len(yo)
        outs.update(tut_members=m, tut_mean=mu,
                    tut_eps=np.fromfile(tmp / "enkf_tut" / "obs_pert.bin", dtype="<f8").reshape(p, k),
                    tut_diag=np.fromfile(tmp / "enkf_tut" / "enkf_diag.bin", dtype="<f8"))
        c = syn.global_etkf_grid(case=5)
        d = tmp / "enkf_c1"
        d.mkdir()
        ens, obsf = grid_case_to_files(c, d)
        kc = c.X.shape[0]
        m, mu = run_harness("enkf", c.nx, c.ny, kc, ens, obsf, 0.5, 1.05, 0.0, d / "out", seed=7)
        Xr = np.stack([read_simple_state(d / f"ens_{i + 1}.txt") for i in range(kc)])
        _, yor = read_grid_obs(Path(obsf))
        pc = len(yor)
        outs.update(c1_X=Xr, c1_obs_xy=c.obs_xy, c1_yo=yor, c1_sigma=c.sigma_o, c1_rho=syn.float_config(1.05),
                    c1_members=m, c1_mean=mu,
                    c1_eps=np.fromfile(d / "out" / "obs_pert.bin", dtype="<f8").reshape(pc, kc),
                    c1_diag=np.fromfile(d / "out" / "enkf_diag.bin", dtype="<f8"))
        np.savez_compressed(HERE / "enkf.npz", tut_X=X, tut_obs_xy=obs_xy, tut_yo=yo, tut_sigma=sigma, nx=nx, ny=ny,
                            c1_nx=c.nx, c1_ny=c.ny, **outs)
        print("enkf.npz", {k2: np.shape(v) for k2, v in outs.items()})
        make_nearest(tmp)


if __name__ == "__main__":
    # usage: make_golden.py [REFERENCE_ROOT] [nearest]
    main(sys.argv[1] if len(sys.argv) > 1 else None, sys.argv[2] if len(sys.argv) > 2 else None)
