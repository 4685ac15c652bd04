"""Times the reference's own analysis code: oracle/_ref/ref_harness, which
compiles ETKF.hpp / LETKF.hpp / EnKF.hpp and their adapters unmodified
(built by oracle/build_ref.sh against the Eigen subset written in
oracle/eigen_subset), on

  * the 64 x 64 grid, 32-member, 1024-observation global ETKF (the seeded
    case of tests/golden/etkf_grid64.npz: sigma 0.5, inflation 1.05), and
  * the reference tutorial (36 x 18, 9 members, 28 observations): ETKF and
    LETKF (radius 10), as in its etkf.yaml / letkf.yaml.

The time is the harness's own clock around the policy's construction and
Analyse() (the text inputs already read), on the host this runs on, single
threaded as the reference is.  Test infrastructure: needs METADA_REFERENCE
(the harness is built from the reference tree).  Prints one JSON line.

    python oracle/time_ref.py [--reps N]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests" / "golden"))

from metada_gb300 import synthetic as syn  # noqa: E402
from metada_gb300.build import build_reference_harness  # noqa: E402

import make_golden as mg  # noqa: E402


def _time(cmd_args: list[str], out: Path, reps: int) -> list[float]:
    ts = []
    for _ in range(reps):
        out.mkdir(parents=True, exist_ok=True)
        subprocess.run([str(mg.HARNESS), *cmd_args, str(out)], check=True)
        ts.append(float((out / "analyse_seconds.txt").read_text()))
    return ts


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    if build_reference_harness() is None:
        raise SystemExit("set METADA_REFERENCE to the reference tree to build and time its harness")
    tut = Path(os.environ["METADA_REFERENCE"]) / "src" / "backends" / "simple" / "tutorial"
    cpu = platform.processor() or platform.machine()
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.startswith("model name"):
                cpu = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    rows = {}
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        c = syn.global_etkf_grid()
        d = tmp / "c1"
        d.mkdir()
        ens, obsf = mg.grid_case_to_files(c, d)
        k = c.X.shape[0]
        ts = _time(["etkf", str(c.nx), str(c.ny), str(k), ens, obsf, "0.5", "1.05", "0.0"], d / "out", args.reps)
        rows["global_etkf_64x64_k32_p1024"] = {"seconds_median": statistics.median(ts), "seconds": ts,
                                               "analyses_per_s": 1.0 / statistics.median(ts)}
        for name, algo, radius in (("tutorial_etkf", "etkf", "0.0"), ("tutorial_letkf_r10", "letkf", "10.0")):
            ts = _time([algo, "36", "18", "9", str(tut / "ens_"), str(tut / "obs_format.txt"), "0.1", "1.0",
                        radius], tmp / name, args.reps)
            rows[name] = {"seconds_median": statistics.median(ts), "seconds": ts,
                          "analyses_per_s": 1.0 / statistics.median(ts)}
    print(json.dumps({"what": "the reference's own ETKF/LETKF (ref_harness), construction + Analyse()",
                      "threads": 1, "cpu": cpu, "reps": args.reps, **rows}))


if __name__ == "__main__":
    main()
