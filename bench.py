"""Benchmark: batched LETKF on the 360 x 180 x 10-level x 4-variable lat-lon
configuration with 64 members and 500k observations (Gaspari-Cohn support
500 km / 2 levels), mixed precision against the FP64 path on one GB300.

A step is one full analysis cycle of the hot path on inputs resident in HBM:
restore the background ensemble (device copy), H(X) for every member,
the spatial-hash local search, and the 648,000 local analyses (perturbations,
obs-space prior, Gram, eigen-solve, update, write-back).  The metric is local
analyses per second; the mixed path is the headline, the FP64 path is timed
beside it, and the mixed analysis is checked against FP64 (max relative
error of mean and perturbations <= 1e-5).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 (torchrun, one rank per GPU) runs independent replicas: the analysis
has no exchange step on one GPU per problem, so there is no collective on the
data path; barrier and max-over-ranks timing only.

Beside the headline, the default line carries the other configurations'
summaries (skipped by --no-extras): the 512-case uneven batch, the global
ETKF of the 64 x 64 case, the learned column operator, and one cycle of the
1440 x 720 x 30 x 4, 80-member high-resolution LETKF (FP32 members, 5M
clustered obs) with its oracle check.

--impl reference times the reference algorithm's CPU implementation (the
oracle restatement, OpenMP on all host cores) on a bounded sample of the same
workload's local analyses; rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "local ETKF analyses/s @k=64: mixed vs FP64 on 1 GB300, rel err ≤1e-5"
UNIT = "analyses/s"
WORKLOAD = "batched LETKF, lat-lon 360x180x10 levels x4 vars (2.59M values), k=64, 500k obs, GC 500 km / 2 levels"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-points", type=int, default=40000, help="local analyses in the CPU sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the uneven-batch, global-ETKF, learned-operator and high-resolution summaries "
                         "of the default line")
    ap.add_argument("--extra-train-steps", type=int, default=6000,
                    help="Adam steps of the surrogate trained for the default line's learned-operator summary")
    ap.add_argument("--workload", choices=["latlon", "uneven", "column", "next", "highres"], default="latlon",
                    help="latlon: the headline LETKF configuration; uneven: 512 global-ETKF cases of "
                         "uneven sizes in one captured graph (reports analyses/s and p50/p99 latency); "
                         "column: the learned column operator (training, H(x) plain vs surrogate, LETKF); "
                         "next: the rows beside the analysis (EnKF, diagnostics, nearest node, text I/O); "
                         "highres: the 1440x720x30x4, 80-member FP32-storage LETKF with 5M clustered obs")
    ap.add_argument("--train-steps", type=int, default=6000, help="column workload: Adam steps")
    ap.add_argument("--train-batch", type=int, default=4096, help="column workload: columns per Adam step")
    ap.add_argument("--profile-case", default=None,
                    choices=["mixed", "fp64", "uneven", "uneven-small", "enkf", "metrics", "column",
                             "column-small", "highres-small"],
                    help="run a profiler case and exit: mixed/fp64 = one batched LETKF on the reduced "
                         "180x90x10x4 case (125k obs); uneven = the 512-case mixed batch run twice without "
                         "the graph; uneven-small = its first 64 cases; enkf = the mixed EnKF (2.59M values, "
                         "k=64, 500k obs) twice; metrics = Metrics::CalculateAll of that ensemble twice; column = "
                         "H(x) of 200k column obs x 64 members (720x360 columns, 30 levels), plain and "
                         "surrogate (untrained weights), twice each; column-small = the same on 360x180 columns with "
                         "50k obs (2 GB state); highres-small = two cycles of the high-resolution LETKF (k=80, FP32 "
                         "members, RTPS) on a 180x90x10x4 grid with 1.67M obs, 60%% clustered (the full "
                         "configuration's obs per level)")
    return ap.parse_args()


# ------------------------------------------------------------- plumbing ----
def dist_setup(n_gpus: int):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if _cuda_ok() else "gloo")
    return rank, world, local


def _cuda_ok() -> bool:
    import torch

    return torch.cuda.is_available()


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if _cuda_ok() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return None
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM bytes per launch of the tensor-core analysis kernel, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the reduced
# 180 x 90 x 10 x 4 case (162,000 analyses, 125k obs), scaled to this
# workload by its analyses (x4): every stream of the kernel (perturbations
# read, analysis written, lists, obs rows) grows with the analysis count.
# A constant of the build, not a measurement of this run.
TC_TRAFFIC_REDUCED_BYTES = 5.311e8
TC_TRAFFIC_REDUCED_ANALYSES = 162_000


# ------------------------------------------------------------- workload ----
def make_case():
    from metada_gb300 import synthetic as syn

    return syn.latlon_letkf_case()


class Workload:
    def __init__(self, case, device):
        import torch

        from metada_gb300 import kernels as K

        self.c = case
        self.K = K
        T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)  # noqa: E731
        c = case
        self.X0 = T(c.X)
        self.X = torch.empty_like(self.X0)
        self.olat, self.olon, self.olev = T(c.obs_lat), T(c.obs_lon), T(c.obs_lev)
        self.ovar = T(c.obs_var)
        self.yo = T(c.yo)
        self.rvar = torch.full_like(self.yo, c.sigma_o ** 2)
        la, lo = c.col_lat_lon()
        self.clat, self.clon = T(la), T(lo)
        self.col_base = T(c.col_base())
        self.npoints = c.nlat * c.nlon * c.nlev

    def step(self, precision):
        c, K = self.c, self.K
        self.X.copy_(self.X0)
        HX = K.hx_latlon(self.X, c.nlon, c.nlat, c.nlev, self.olat, self.olon, self.olev, self.ovar)
        off, idx, dist = K.select_geo(self.clat, self.clon, self.olat, self.olon, c.hsupport_km)
        _, st = K.letkf_batched(self.X, col_base=self.col_base, nlev=c.nlev, n_var=c.nvar, lev_stride=c.lev_stride,
                                var_stride=c.var_stride, HX=HX, yo=self.yo, rvar=self.rvar, loc_off=off,
                                loc_idx=idx, loc_dist=dist, obs_lev=self.olev, hsupport=c.hsupport_km,
                                vsupport=c.vsupport, rho=c.rho, flags=0, precision=precision, want_mean=False)
        return st


def timed(fn, steps, world):
    import torch

    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    out = [fn() for _ in range(steps)]
    e1.record()
    torch.cuda.synchronize()
    barrier(world)
    return e0.elapsed_time(e1) / 1e3, out


def tc_issued_flop(st, k, n_var):
    """Tensor-core FLOP the tensor-core kernel issues per launch: 3 passes per
    product, M = 128 tiles; Gram chunks of 32 obs (N = 80), per Newton-Schulz
    step two 64-wide products (the first step one), the finish three, the
    update one per 16 variables (N = 16)."""
    active = st.n_points - st.n_empty
    mma = lambda n, kdim: 3 * 2.0 * 128 * n * kdim  # noqa: E731
    chunks = st.total_local / 32.0 + 0.5 * active
    ns = 2 * st.total_sweeps - active
    upd = -(-n_var // 16)
    return chunks * mma(80, 32) + (ns + 3 * active) * mma(64, 64) + upd * active * mma(16, 64)


def flops_per_step(st, k, n_var):
    """Algorithmic FLOPs of the local analyses: Gram 2k^2 p_loc, Y'^T R^-1 d
    2k p_loc, update 2 n_var k^2 and the eigen-solve counted as 9k^3 per
    analysis (Golub-Van Loan symmetric QR with vectors, a fixed convention)."""
    return (2.0 * k * k + 2.0 * k) * st.total_local + (st.n_points - st.n_empty) * (2.0 * n_var * k * k + 9.0 * k ** 3)


# ---------------------------------------------------------- CPU baseline ----
def cpu_baseline(case, npoints: int, seed: int = 0):
    """The oracle (the reference algorithm restated in C++, OpenMP, all host
    threads) on a seeded sample of the workload's local analyses."""
    import oracle.bind as ob
    from oracle.lists import point_lists

    c = case
    la, lo = c.col_lat_lon()
    rng = np.random.default_rng(seed)
    ncols = max(1, npoints // c.nlev)
    cols = rng.choice(c.nlat * c.nlon, ncols, replace=False)
    # the sample's local search (oracle restatement of LETKF.hpp:159-165)
    off, idx, dist = ob.select_geo(la[cols], lo[cols], c.obs_lat, c.obs_lon, c.hsupport_km)
    pts, poff, pidx, pw = point_lists(np.arange(ncols), c.nlev, off, idx, dist, c.obs_lev, c.hsupport_km, c.vsupport)
    # obs-space prior of the needed obs only
    need = np.unique(pidx)
    HXs = ob.hx_latlon(c.X, c.nlon, c.nlat, c.nlev, c.obs_lat[need], c.obs_lon[need], c.obs_lev[need],
                       c.obs_var[need])
    remap = np.full(c.yo.shape[0], -1, dtype=np.int64)
    remap[need] = np.arange(need.size)
    base = cols[pts[:, 0]] + pts[:, 1] * c.lev_stride
    t0 = time.perf_counter()
    ob.letkf_points(c.X, base, c.nvar, c.var_stride, HXs, c.yo[need], c.rvar[need], poff,
                    remap[pidx].astype(np.int32), pw, c.rho, 0)
    el = time.perf_counter() - t0
    return {"value": len(base) / el, "unit": UNIT, "cores": ob.num_threads(), "kind": "port", "analyses": len(base),
            "sample": f"{len(base)} local analyses ({ncols} seeded columns x {c.nlev} levels) of the same workload, "
                      f"{el:.1f} s of CPU work"}


# ------------------------------------------------------------------ main ----
def run_reference(args, rank, world):
    if rank != 0:
        return
    case = make_case()
    import oracle.bind as ob

    steps = []
    npts = max(100, args.cpu_points // 2)
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(case, npts, seed=i)
        if i >= args.warmup:
            steps.append(cb)
    v = statistics.median(s["value"] for s in steps)
    # a step is one timed sample of the workload's local analyses
    ms_step = statistics.mean(1e3 * s["analyses"] / s["value"] for s in steps)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "step": f"one seeded sample of {steps[-1]['analyses']} of the "
                                                    f"{case.nlat * case.nlon * case.nlev} local analyses",
                       "sample": steps[-1]["sample"]},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": ob.num_threads(), "kind": "port",
                             "sample": steps[-1]["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def profile_case(precision_name: str) -> None:
    """One analysis of a reduced configuration (inputs ~170 MB, above L2; a
    few hundred MB on the device) for profiler captures, or one of the other
    workloads' cases."""
    import torch

    from metada_gb300 import _lib
    from metada_gb300 import kernels as K
    from metada_gb300 import synthetic as syn

    dev = torch.device("cuda", 0)
    if precision_name.startswith("uneven"):
        cases = syn.uneven_batch(ncases=64 if precision_name == "uneven-small" else 512)
        dc = [{"X": torch.tensor(c.X, device=dev), "obs_node": torch.tensor(c.obs_node, device=dev),
               "yo": torch.tensor(c.yo, device=dev),
               "rvar": torch.full((len(c.yo),), c.sigma_o ** 2, dtype=torch.float64, device=dev), "rho": c.rho}
              for c in cases]
        b = K.EtkfBatch(dc, flags=0, precision=_lib.MG_PREC_MIXED)
        ms = []
        for _ in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b.run(graph=False)
            b.finish()
            ms.append(1e3 * (time.perf_counter() - t0))
        b.close()
        print(json.dumps({"profile_case": precision_name, "cases": len(cases), "ms": ms}))
        return
    if precision_name.startswith("column"):
        g = torch.Generator(device=dev)
        g.manual_seed(7)
        ncol, nlev, k, p = (360 * 180, 30, 64, 50_000) if precision_name == "column-small" else (720 * 360, 30, 64,
                                                                                              200_000)
        Tm = (255.0 + 15.0 * torch.randn((k, nlev * ncol), generator=g, device=dev, dtype=torch.float64)).clamp(200, 310)
        lq = (np.log(2e-3) + torch.randn((k, nlev * ncol), generator=g, device=dev, dtype=torch.float64)).clamp(
            np.log(1e-6), np.log(2e-2))
        X = torch.cat([Tm, lq], dim=1).contiguous()
        del Tm, lq
        oc = torch.randint(0, ncol, (p,), generator=g, device=dev)
        och = torch.randint(0, 16, (p,), generator=g, device=dev).to(torch.int32)
        op = syn.column_operator()
        w, tau = torch.tensor(op.w, device=dev), torch.tensor(op.tau, device=dev)
        mlp = K.MLP(64, 256, 16)
        mlp.set_params(mlp.init_params(seed=7), torch.zeros(16, device=dev), torch.ones(16, device=dev))
        ms = {"plain": [], "surrogate": []}
        for _ in range(2):
            for name, fn in (("plain", lambda: K.hx_column(X, ncol, nlev, oc, och, w, tau)),
                             ("surrogate", lambda: mlp.hx_column(X, ncol, nlev, oc, och))):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                fn()
                torch.cuda.synchronize()
                ms[name].append(1e3 * (time.perf_counter() - t0))
        print(json.dumps({"profile_case": precision_name, "ms": ms}))
        return
    if precision_name in ("enkf", "metrics"):
        g = torch.Generator(device=dev)
        g.manual_seed(1234)
        n, k, p = 360 * 180 * 10 * 4, 64, 500_000
        truth = torch.randn(n, generator=g, device=dev, dtype=torch.float64)
        X0 = truth[None, :] + torch.randn((k, n), generator=g, device=dev, dtype=torch.float64)
        ms = []
        if precision_name == "metrics":
            for _ in range(2):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                K.ens_metrics(X0, truth)
                torch.cuda.synchronize()
                ms.append(1e3 * (time.perf_counter() - t0))
        else:
            nodes = torch.randint(0, n, (p,), generator=g, device=dev)
            yo = truth[nodes] + 0.5 * torch.randn(p, generator=g, device=dev, dtype=torch.float64)
            rvar = torch.full((p,), 0.25, dtype=torch.float64, device=dev)
            eps = 0.5 * torch.randn((p, k), generator=g, device=dev, dtype=torch.float64)
            HX = X0[:, nodes].T.contiguous()
            X = X0.clone()
            for _ in range(2):
                X.copy_(X0)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                K.enkf(X, HX, yo, rvar, eps, 1.05, precision=_lib.MG_PREC_MIXED)
                torch.cuda.synchronize()
                ms.append(1e3 * (time.perf_counter() - t0))
        print(json.dumps({"profile_case": precision_name, "ms": ms}))
        return

    if precision_name == "highres-small":
        # the high-resolution configuration's analysis on a 180 x 90 x 10 x 4
        # grid (k = 80 stored as FP32: 207 MB) with its obs density per level:
        # 5M obs over 30 levels -> 1.67M over 10 (60 % in patches)
        c = syn.highres_letkf_case(dev, nlon=180, nlat=90, nlev=10, p=1_670_000)
        la, lo = c.col_lat_lon()
        clat, clon = torch.tensor(la, device=dev), torch.tensor(lo, device=dev)
        col_base = torch.tensor(c.col_base(), device=dev)
        rvar = torch.full_like(c.yo, c.sigma_o ** 2)
        out = []
        for _ in range(2):
            HX = K.hx_latlon(c.X, c.nlon, c.nlat, c.nlev, c.obs_lat, c.obs_lon, c.obs_lev, c.obs_var)
            off, idx, dist = K.select_geo(clat, clon, c.obs_lat, c.obs_lon, c.hsupport_km)
            _, st = K.letkf_batched(c.X, col_base=col_base, nlev=c.nlev, n_var=c.nvar, lev_stride=c.lev_stride,
                                    var_stride=c.var_stride, HX=HX, yo=c.yo, rvar=rvar, loc_off=off, loc_idx=idx,
                                    loc_dist=dist, obs_lev=c.obs_lev, hsupport=c.hsupport_km, vsupport=c.vsupport,
                                    rho=c.rho, flags=_lib.MG_RTPS, precision=_lib.MG_PREC_MIXED, want_mean=False)
            torch.cuda.synchronize()
            out.append({"ms_analysis": st.ms_analysis, "handed_back": st.n_fallback,
                        "mean_local": st.total_local / max(1, st.n_points - st.n_empty), "max_local": st.max_local})
        print(json.dumps({"profile_case": precision_name, "analyses": st.n_points, "cycles": out}))
        return
    c = syn.latlon_letkf_case(nlon=180, nlat=90, nlev=10, nvar=4, k=64, p=125_000, T=45, case=40)
    w = Workload(c, dev)
    st = w.step(_lib.MG_PREC_MIXED if precision_name == "mixed" else _lib.MG_PREC_FP64)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": precision_name, "analyses": st.n_points, "ms_analysis": st.ms_analysis,
                      "mean_local": st.total_local / st.n_points, "mean_sweeps": st.total_sweeps / st.n_points}))


def run_uneven(args) -> None:
    """512 independent global ETKF analyses (n log-uniform 1k-200k, k in
    {20,32,48,64,100}, p log-uniform 100-50k, identity interpolation), one
    autotuned plan replayed as a CUDA graph."""
    out = uneven_results(args.warmup, args.steps)
    line = {"metric": "uneven-batch global ETKF analyses/s (512 cases, one captured graph)",
            "value": out["mixed"]["analyses_per_s"], "unit": "analyses/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": out["mixed"]["ms_per_batch"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": out.pop("dtype"), "data": "synthetic",
            "config": out.pop("config"), **out}
    print(json.dumps(line), flush=True)


def global_etkf_results(warmup: int, steps: int) -> dict:
    """The global ETKF of the 64 x 64 grid, k = 32, p = 1024 configuration
    (ETKF.hpp:100-179): one analysis = IDW4 H(X) of the members plus the ETKF
    update, per call on device-resident inputs, with the reference's
    semantics (Cholesky W) in FP64 and the Hunt form (symmetric W from a
    Jacobi eigen-solve) in FP64 and mixed precision; the oracle's
    restatement of the reference's ETKF timed on the host beside it."""
    import torch

    from metada_gb300 import _lib
    from metada_gb300 import kernels as K
    from metada_gb300 import synthetic as syn
    from oracle import bind as ob

    dev = torch.device("cuda", 0)
    c = syn.global_etkf_grid(case=1)
    k, n = c.X.shape
    X0 = torch.tensor(c.X, device=dev)
    X = X0.clone()
    oxy = torch.tensor(c.obs_xy, device=dev)
    yo = torch.tensor(c.yo, device=dev)
    rvar = torch.full((len(c.yo),), c.sigma_o * c.sigma_o, dtype=torch.float64, device=dev)
    res = {}
    for name, flags, prec in (("reference_semantics_fp64", _lib.MG_COMPAT, _lib.MG_PREC_FP64),
                              ("hunt_fp64", 0, _lib.MG_PREC_FP64), ("hunt_mixed", 0, _lib.MG_PREC_MIXED)):
        def call():
            HX = K.hx_idw4(X, c.nx, c.ny, oxy)
            K.etkf(X, HX, yo, rvar, c.rho, flags=flags, precision=prec)
        for _ in range(warmup):
            X.copy_(X0)
            call()
        ts = []
        for _ in range(steps):
            X.copy_(X0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            call()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        t = statistics.median(ts)
        res[name] = {"ms_per_analysis": 1e3 * t, "analyses_per_s": 1.0 / t}
    # parity of the FP64 reference-semantics call against the oracle
    X.copy_(X0)
    HX = K.hx_idw4(X, c.nx, c.ny, oxy)
    K.etkf(X, HX, yo, rvar, c.rho, flags=_lib.MG_COMPAT, precision=_lib.MG_PREC_FP64)
    HXo = ob.hx_idw4(c.X, c.nx, c.ny, c.obs_xy)
    rv = np.full(len(c.yo), c.sigma_o * c.sigma_o)
    want, _ = ob.etkf_compat(c.X, HXo, c.yo, rv, c.rho)
    got = X.cpu().numpy()
    err = float(np.abs(got - want).max() / np.abs(want).max())
    t0 = time.perf_counter()
    reps = 0
    while True:
        ob.etkf_compat(c.X, ob.hx_idw4(c.X, c.nx, c.ny, c.obs_xy), c.yo, rv, c.rho)
        reps += 1
        if time.perf_counter() - t0 >= 3.0:
            break
    tc = (time.perf_counter() - t0) / reps
    return {"workload": f"global ETKF, {c.nx}x{c.ny} grid (n={n}), k={k}, p={len(c.yo)}, IDW4 H, sigma 0.5, "
                        f"rho 1.05 (as float)",
            "step": "H(X) and one ETKF analysis per call, inputs on the device", "steps": steps, "warmup": warmup,
            **res, "rel_err_fp64_vs_oracle": err,
            "cpu_baseline": {"value": 1.0 / tc, "unit": "analyses/s", "cores": int(ob.load().orc_num_threads()),
                             "kind": "port", "sample": "the whole case: the oracle's restatement of ETKF.hpp "
                                                       "(dense p x p R, LU inverses)"}}


def uneven_results(warmup: int, steps: int) -> dict:
    """The uneven batch (mixed and FP64): analyses/s, per-case p50/p99
    latency, the autotuned plan, and the mixed path's error against FP64."""
    import torch

    from metada_gb300 import _lib
    from metada_gb300 import kernels as K
    from metada_gb300 import synthetic as syn

    dev = torch.device("cuda", 0)
    cases = syn.uneven_batch()
    out = {}
    for prec_name, prec in (("mixed", _lib.MG_PREC_MIXED), ("fp64", _lib.MG_PREC_FP64)):
        dc = []
        for c in cases:
            dc.append({"X": torch.tensor(c.X, device=dev), "obs_node": torch.tensor(c.obs_node, device=dev),
                       "yo": torch.tensor(c.yo, device=dev),
                       "rvar": torch.full((len(c.yo),), c.sigma_o ** 2, dtype=torch.float64, device=dev),
                       "rho": c.rho})
        X0 = [d["X"].clone() for d in dc]
        b = K.EtkfBatch(dc, flags=0, precision=prec)
        chunk, mode = b.autotune()
        times, lat = [], None
        for it in range(warmup + steps):
            for d, x0 in zip(dc, X0):
                d["X"].copy_(x0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            b.run(graph=True)
            e1.record()
            lat = b.finish()
            if it >= warmup:
                times.append(e0.elapsed_time(e1) / 1e3)
        t = statistics.mean(times)
        out[prec_name] = {"analyses_per_s": len(cases) / t, "ms_per_batch": 1e3 * t,
                          "case_latency_ms_p50": float(np.percentile(lat, 50)),
                          "case_latency_ms_p99": float(np.percentile(lat, 99)),
                          "autotuned": {"gram_obs_chunk": chunk, "bucket_mode": mode}}
        if prec_name == "mixed":
            Xmx = [d["X"].clone() for d in dc]
        else:
            err = 0.0
            for a, w in zip(Xmx, [d["X"] for d in dc]):
                ma, mw = a.mean(0), w.mean(0)
                err = max(err, float(((a - ma) - (w - mw)).abs().max() / (w - mw).abs().max()),
                          float((ma - mw).abs().max() / mw.abs().max()))
            out["max_rel_err_mixed_vs_fp64"] = err
        b.close()
        del dc, X0
        torch.cuda.empty_cache()
    out["dtype"] = "f32 (two-stage Jacobi + Daleckii-Krein; FP64 values as FP32 pairs)"
    out["config"] = {"workload": "512 cases: n log-uniform 1k-200k, k in {20,32,48,64,100}, p log-uniform "
                                 "100-50k, identity interpolation, sigma_o = 1",
                     "total_state_values": int(sum(c.X.size for c in cases))}
    return out


def run_next(args) -> None:
    """The rows beside the analysis, each on device-resident inputs, timed per
    call (CUDA-synchronised wall clock over --steps calls after --warmup),
    with the oracle timed on a bounded host sample:
      enkf     stochastic EnKF, lat-lon state 360x180x10x4 (2.59M values),
               k=64, 500k obs at state nodes (mixed and FP64)
      metrics  Metrics::CalculateAll of the same ensemble against a truth
      nearest  nearest node of 500k obs on a 1000x1000 curvilinear grid
               (with the vertical index among 40 levels)
      io       GridObservation text (500k lines) and the state written as
               SimpleState text ("%12.6f") and read back
    Bandwidths are algorithmic bytes per call over the call time, against the
    measured HBM copy rate."""
    import torch

    import oracle.bind as ob
    from metada_gb300 import _lib
    from metada_gb300 import kernels as K

    dev = torch.device("cuda", 0)
    ctx = K.context(0)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    g = torch.Generator(device=dev)
    g.manual_seed(1234)

    def per_call(fn, reset=None):
        for _ in range(args.warmup):
            if reset:
                reset()
            fn()
        ts = []
        for _ in range(args.steps):
            if reset:
                reset()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return statistics.mean(ts)

    def cpu_time(fn, min_s=2.0):
        t0 = time.perf_counter()
        reps = 0
        while True:
            fn()
            reps += 1
            if time.perf_counter() - t0 >= min_s:
                return (time.perf_counter() - t0) / reps

    rows = {}
    threads = ob.load().orc_num_threads()
    # ---------------------------------------------------------------- EnKF
    nlon, nlat, nlev, nvar, k, p = 360, 180, 10, 4, 64, 500_000
    n = nlon * nlat * nlev * nvar
    truth = torch.randn(n, generator=g, device=dev, dtype=torch.float64)
    X0 = truth[None, :] + torch.randn((k, n), generator=g, device=dev, dtype=torch.float64)
    nodes = torch.randint(0, n, (p,), generator=g, device=dev)
    sigma = 0.5
    yo = truth[nodes] + sigma * torch.randn(p, generator=g, device=dev, dtype=torch.float64)
    rvar = torch.full((p,), sigma * sigma, dtype=torch.float64, device=dev)
    eps = sigma * torch.randn((p, k), generator=g, device=dev, dtype=torch.float64)
    X = torch.empty_like(X0)
    HX = X0[:, nodes].T.contiguous()
    enkf_bytes = 2 * n * k * 8 + 2 * p * k * 8 + 2 * p * 8
    res = {}
    for name, prec in (("mixed", _lib.MG_PREC_MIXED), ("fp64", _lib.MG_PREC_FP64)):
        l0 = ctx.launches()
        t = per_call(lambda: K.enkf(X, HX, yo, rvar, eps, 1.05, precision=prec), reset=lambda: X.copy_(X0))
        launches = (ctx.launches() - l0) // (args.warmup + args.steps)
        res[name] = {"ms_per_call": 1e3 * t, "analyses_per_s": 1.0 / t, "hbm_gbs": enkf_bytes / t / 1e9,
                     "frac_of_hbm": enkf_bytes / t / 1e9 / hbm, "gpu_launches": int(launches)}
    # like-for-like at the reference's tutorial-sized ETKF configuration (64x64, k=32, p=1024)
    from metada_gb300 import synthetic as syn
    c1 = syn.global_etkf_grid(case=1)
    HX1 = ob.hx_idw4(c1.X, 64, 64, c1.obs_xy)
    eps1 = c1.sigma_o * np.random.default_rng(1).standard_normal((len(c1.yo), c1.X.shape[0]))
    tc = cpu_time(lambda: ob.enkf(c1.X, HX1, c1.yo, c1.rvar, eps1, c1.rho))
    X1 = torch.tensor(c1.X, device=dev)
    X10 = X1.clone()
    d1 = [torch.tensor(a, device=dev) for a in (HX1, c1.yo, c1.rvar, eps1)]
    tg1 = per_call(lambda: K.enkf(X1, *d1, c1.rho, precision=_lib.MG_PREC_FP64), reset=lambda: X1.copy_(X10))
    rows["enkf"] = {"metric": "global EnKF analyses/s", "unit": "analyses/s", "value": res["mixed"]["analyses_per_s"],
                    "config": f"{nlon}x{nlat}x{nlev}x{nvar} state ({n} values), k={k}, p={p}, obs at nodes",
                    "bound": "hbm", "algorithmic_bytes_per_call": enkf_bytes, **res,
                    "small_case": {"config": "64x64, k=32, p=1024 (FP64)", "gpu_analyses_per_s": 1.0 / tg1,
                                   "cpu_analyses_per_s": 1.0 / tc},
                    "cpu_baseline": {"value": 1.0 / tc, "unit": "analyses/s", "cores": threads, "kind": "port",
                                     "sample": "the oracle's dense p x p EnKF (the reference's algorithm) on the "
                                               "64x64, k=32, p=1024 case; the full-size case has a 500k x 500k S"}}
    del X, HX, eps, yo, rvar, nodes
    # ------------------------------------------------------------- metrics
    met_bytes = n * k * 8 + n * 8 + 2 * n * 8
    l0 = ctx.launches()
    t = per_call(lambda: K.ens_metrics(X0, truth))
    launches = (ctx.launches() - l0) // (args.warmup + args.steps)
    ns = 65_536
    Xs, ts_ = X0[:, :ns].cpu().numpy(), truth[:ns].cpu().numpy()
    tcm = cpu_time(lambda: ob.ens_metrics(Xs, ts_))
    rows["metrics"] = {"metric": "member values/s (Metrics::CalculateAll)", "unit": "values/s", "value": n * k / t,
                       "ms_per_call": 1e3 * t, "bound": "hbm", "algorithmic_bytes_per_call": met_bytes,
                       "hbm_gbs": met_bytes / t / 1e9, "frac_of_hbm": met_bytes / t / 1e9 / hbm,
                       "gpu_launches": int(launches), "config": f"k={k}, n={n}",
                       "cpu_baseline": {"value": ns * k / tcm, "unit": "values/s", "cores": threads, "kind": "port",
                                        "sample": f"the oracle on the first {ns} state values"}}
    del X0, truth
    torch.cuda.empty_cache()
    # ------------------------------------------------------------- nearest
    nx = ny = 1000
    ii = torch.arange(nx, device=dev, dtype=torch.float64)[None, :].expand(ny, nx)
    jj = torch.arange(ny, device=dev, dtype=torch.float64)[:, None].expand(ny, nx)
    nlon_ = (-100.0 + 0.05 * ii + 0.01 * torch.sin(0.1 * jj)).contiguous().reshape(-1)
    nlat_ = (20.0 + 0.04 * jj + 0.01 * torch.cos(0.1 * ii)).contiguous().reshape(-1)
    po = 500_000
    olon = -100.0 + 50.0 * torch.rand(po, generator=g, device=dev, dtype=torch.float64)
    olat = 20.0 + 40.0 * torch.rand(po, generator=g, device=dev, dtype=torch.float64)
    vc = torch.linspace(1.0, 0.0, 40, device=dev, dtype=torch.float64)
    olev = torch.rand(po, generator=g, device=dev, dtype=torch.float64)
    l0 = ctx.launches()
    t = per_call(lambda: K.nearest_node(nlat_, nlon_, nx, ny, olat, olon, vc, olev))
    launches = (ctx.launches() - l0) // (args.warmup + args.steps)
    xy, kk = K.nearest_node(nlat_, nlon_, nx, ny, olat, olon, vc, olev)
    pc = 500
    hl, hn = nlat_.cpu().numpy(), nlon_.cpu().numpy()
    ola, olo, ole, vch = olat[:pc].cpu().numpy(), olon[:pc].cpu().numpy(), olev[:pc].cpu().numpy(), vc.cpu().numpy()
    tcn = cpu_time(lambda: ob.nearest_node(hl, hn, nx, ny, ola, olo, vch, ole))
    wxy, wk = ob.nearest_node(hl, hn, nx, ny, ola, olo, vch, ole)
    same = bool(np.array_equal(wxy, xy[:pc].cpu().numpy()) and np.array_equal(wk, kk[:pc].cpu().numpy()))
    rows["nearest"] = {"metric": "geographic obs located/s", "unit": "obs/s", "value": po / t, "ms_per_call": 1e3 * t,
                       "bound": "FP64 pipe (exact distance arithmetic per visited node; nodes and hash fit in L2)", "gpu_launches": int(launches),
                       "config": f"{nx}x{ny} curvilinear grid, {po} obs, 40 levels",
                       "sample_identical_to_oracle": same,
                       "cpu_baseline": {"value": pc / tcn, "unit": "obs/s", "cores": threads, "kind": "port",
                                        "sample": f"the reference's scan over all nodes for the first {pc} obs"}}
    # ------------------------------------------------------------------ io
    rng = np.random.default_rng(5)
    lines = ["-" * 80, "Time Z   Y   X   ZNU      XLONG_U    XLAT_U     Simple", "-" * 80]
    zz, yy, xx = rng.integers(1, 40, po), rng.integers(0, 360, po), rng.integers(0, 720, po)
    vals = rng.standard_normal((po, 4)) * [0.3, 50.0, 30.0, 2.0]
    lines += [f"0 {a:4d} {b:4d} {c:4d} {v0:8.4f} {v1:10.4f} {v2:10.4f} {v3:10.4f}"
              for a, b, c, (v0, v1, v2, v3) in zip(zz, yy, xx, vals)]
    obs_text = ("\n".join(lines) + "\n").encode()
    l0 = ctx.launches()
    t_obs = per_call(lambda: K.parse_grid_obs(obs_text))
    launches_obs = (ctx.launches() - l0) // (args.warmup + args.steps)
    xyz, ov = K.parse_grid_obs(obs_text)
    ok_obs = bool(xyz.shape[0] == po and np.array_equal(xyz[:, 0].cpu().numpy(), xx))
    state = (torch.randn(n, generator=g, device=dev, dtype=torch.float64) * 15.0 + 280.0)
    t_fmt = per_call(lambda: K.format_state(state, nlon, n // nlon))
    st_text = K.format_state(state, nlon, n // nlon)
    t_par = per_call(lambda: K.parse_values(st_text))
    back = K.parse_values(st_text).cpu().numpy()
    sample = st_text[: 2_000_000]
    sample = sample[: sample.rfind(b"\n") + 1]
    tco = cpu_time(lambda: ob.parse_values(sample))
    ok_state = bool(np.array_equal(back[: 10_000], ob.parse_values(st_text[: 200_000])[: 10_000]) and
                    np.abs(back - state.cpu().numpy()).max() <= 5e-7)
    rows["io"] = {"metric": "text MB/s (parse, host text in; format, host text out)", "unit": "MB/s",
                  "value": len(st_text) / t_par / 1e6, "bound": "host link + latency of the line index scan",
                  "parse_grid_obs": {"mb_per_s": len(obs_text) / t_obs / 1e6, "ms_per_call": 1e3 * t_obs,
                                     "bytes": len(obs_text), "lines": po, "gpu_launches": int(launches_obs),
                                     "ok": ok_obs},
                  "parse_values": {"mb_per_s": len(st_text) / t_par / 1e6, "ms_per_call": 1e3 * t_par,
                                   "bytes": len(st_text), "values": n, "ok": ok_state},
                  "format_state": {"mb_per_s": len(st_text) / t_fmt / 1e6, "ms_per_call": 1e3 * t_fmt,
                                   "bytes": len(st_text), "values": n},
                  "cpu_baseline": {"value": len(sample) / tco / 1e6, "unit": "MB/s", "cores": 1, "kind": "port",
                                   "sample": f"the reference's getline + istringstream >> double loop "
                                             f"(SimpleState::readFromFile) over the first {len(sample)} bytes"}}
    line = {"metric": "rows beside the analysis (EnKF, diagnostics, nearest node, text I/O)", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "data": "synthetic (seeded)", "rows": rows}
    print(json.dumps(line), flush=True)


def run_column(args) -> None:
    """Learned column operator on the 720 x 360 column grid (30 levels, T and
    ln q, 64 members, 200k single-channel column obs): train the surrogate
    (64-padded 60 -> 256 -> 256 -> 16, SiLU, BF16 weights) by Adam on 2M
    operator-labelled columns, time H(x) of all 12.8M (obs, member) columns
    through the plain operator and through the surrogate on the tensor cores,
    and run the LETKF with each H(x)."""
    print(json.dumps(column_results(args.train_steps, args.train_batch)), flush=True)


def column_results(train_steps: int, train_batch: int) -> dict:
    """The learned-column-operator workload as one result dict (see run_column)."""
    import torch

    from metada_gb300 import _lib
    from metada_gb300 import kernels as K
    from metada_gb300 import synthetic as syn

    dev = torch.device("cuda", 0)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    op = syn.column_operator()
    w, tau = torch.tensor(op.w, device=dev), torch.tensor(op.tau, device=dev)
    # ---- training on 2M columns, shuffled once; one epoch = ncol / batch steps
    T, q = syn.random_columns(2_000_000, stream=7)
    Td, qd = torch.tensor(T, device=dev), torch.tensor(q, device=dev)
    Y = K.column_op(Td, qd, w, tau)
    Xf = K.column_features(Td, qd, 64)
    shift, scale = Y.mean(0), Y.std(0)
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    perm = torch.randperm(Xf.shape[0], device=dev, generator=g)
    Xs, Ys = Xf[perm].contiguous(), Y[perm].contiguous()
    mlp = K.MLP(64, 256, 16)
    mlp.set_params(mlp.init_params(seed=7), shift, scale)
    B, S = train_batch, train_steps
    per_epoch = Xs.shape[0] // B
    first_loss = mlp.gradients(Xs[:B], Ys[:B])[1]
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    e0.record()
    for st in range(S):
        o = (st % per_epoch) * B
        lr = 2e-3 * 0.5 * (1 + np.cos(np.pi * st / S)) + 1e-5
        mlp.train_step(Xs[o:o + B], Ys[o:o + B], lr)
    e1.record()
    torch.cuda.synchronize()
    t_train = e0.elapsed_time(e1) / 1e3
    # held-out columns: surrogate against the plain operator
    Th, qh = syn.random_columns(200_000, stream=99)
    Thd, qhd = torch.tensor(Th, device=dev), torch.tensor(qh, device=dev)
    yh = K.column_op(Thd, qhd, w, tau)
    ynet = mlp.forward(K.column_features(Thd, qhd, 64)) * scale + shift
    held_err = float(((ynet - yh).pow(2).mean() / yh.pow(2).mean()).sqrt())
    # ---- H(x) of 200k obs x 64 members, plain vs surrogate
    c = syn.column_letkf_case()
    X0 = torch.tensor(c.X, device=dev)
    oc, och = torch.tensor(c.obs_col, device=dev), torch.tensor(c.obs_ch, device=dev)
    k = X0.shape[0]
    ncols_eval = len(c.obs_col) * k

    def time_it(fn, reps=5):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record()
        for _ in range(reps):
            out = fn()
        b.record()
        torch.cuda.synchronize()
        return out, a.elapsed_time(b) / 1e3 / reps

    HXp, t_plain = time_it(lambda: K.hx_column(X0, c.ncol, c.nlev, oc, och, w, tau))
    HXs, t_sur = time_it(lambda: mlp.hx_column(X0, c.ncol, c.nlev, oc, och))
    hx_err = float(((HXs - HXp).pow(2).mean() / HXp.pow(2).mean()).sqrt())
    hx_err_sigma = float((HXs - HXp).pow(2).mean().sqrt()) / c.sigma_o
    flop_col = 2 * (60 * 256 + 256 * 256 + 256 * 16)
    # ---- the LETKF with each H(x)
    la, lo = c.col_lat_lon()
    off, idx, dist = K.select_geo(torch.tensor(la, device=dev), torch.tensor(lo, device=dev),
                                  torch.tensor(la[c.obs_col], device=dev), torch.tensor(lo[c.obs_col], device=dev),
                                  c.hsupport_km)
    yo = torch.tensor(c.yo, device=dev)
    rvar = torch.full_like(yo, c.sigma_o ** 2)
    truth = torch.tensor(c.truth, device=dev)
    nT = c.nlev * c.ncol
    res = {}
    for name, HX in (("plain", HXp), ("surrogate", HXs)):
        X = X0.clone()
        a, b = ev(), ev()
        a.record()
        K.letkf_batched(X, col_base=torch.arange(c.ncol, dtype=torch.int64, device=dev), nlev=1, n_var=2 * c.nlev,
                        lev_stride=0, var_stride=c.ncol, HX=HX, yo=yo, rvar=rvar, loc_off=off, loc_idx=idx,
                        loc_dist=dist, hsupport=c.hsupport_km, rho=c.rho, flags=0, precision=_lib.MG_PREC_MIXED,
                        want_mean=False)
        b.record()
        torch.cuda.synchronize()
        m = X.mean(0)
        res[name] = {"ms_letkf": a.elapsed_time(b),
                     "rmse_T_analysis_K": float((m[:nT] - truth[:nT]).pow(2).mean().sqrt()), "mean": m}
        del X
    rb = float((X0.mean(0)[:nT] - truth[:nT]).pow(2).mean().sqrt())
    gain_kept = (rb - res["surrogate"]["rmse_T_analysis_K"]) / (rb - res["plain"]["rmse_T_analysis_K"])
    line = {"metric": "learned column operator: surrogate H(x) columns/s on the tensor cores (plain beside)",
            "value": ncols_eval / t_sur, "unit": "columns/s", "n_gpus": 1, "steps": 5, "warmup": 2,
            "ms_per_step": 1e3 * t_sur, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 x bf16 -> f32 (surrogate); f32 (plain operator)", "data": "synthetic",
            "config": {"workload": "720x360 column grid, 30 levels (T, ln q), k=64, 200k column obs, 16 channels; "
                                   "MLP 60(64)->256->256->16 SiLU trained on 2M columns",
                       "train_steps": S, "train_batch": B},
            "training": {"s": t_train, "columns_per_s": S * B / t_train, "loss_first": first_loss,
                         "loss_last": mlp.gradients(Xs[:B], Ys[:B])[1],
                         "heldout_rel_rms_err": held_err},
            "hx": {"plain_ms": 1e3 * t_plain, "surrogate_ms": 1e3 * t_sur, "columns": ncols_eval,
                   "plain_columns_per_s": ncols_eval / t_plain, "surrogate_tflops": ncols_eval * flop_col / t_sur / 1e12,
                   "surrogate_vs_plain_rel_rms": hx_err, "surrogate_vs_plain_rms_over_sigma_o": hx_err_sigma},
            "letkf": {"background_rmse_T_K": rb,
                      **{f"{n}_{key}": v for n, r in res.items() for key, v in r.items() if key != "mean"},
                      "gain_kept_by_surrogate": gain_kept,
                      "max_abs_diff_T_K": float((res["plain"]["mean"][:nT] - res["surrogate"]["mean"][:nT]).abs().max())}}
    return line


def highres_results() -> dict:
    """High-resolution LETKF: 1440 x 720 grid, 30 levels, 4 variables (124M
    values), 80 members stored as FP32 (39.8 GB), 5M obs (60 % in 20 Gaussian
    patches of 800 km), 300 km horizontal support, 2 levels vertical, RTPS
    with alpha 0.9, mixed precision.  Cycles run back to back on the same
    obs, each analysing the previous cycle's output; a cycle is H(X), the
    spatial-hash local search and the local analyses.  The first cycle is the
    warm-up.  The analysis of a seeded sample of columns (the longest lists
    among them) is checked against the oracle (FP64, Jacobi eigen-solve) run
    on the same background, lists and H(X)."""
    import torch

    import oracle.bind as ob
    from oracle.lists import point_lists
    from metada_gb300 import _lib
    from metada_gb300 import kernels as K
    from metada_gb300 import synthetic as syn

    dev = torch.device("cuda", 0)
    t0 = time.perf_counter()
    c = syn.highres_letkf_case(dev)
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    k = c.X.shape[0]
    la, lo = c.col_lat_lon()
    clat, clon = torch.tensor(la, device=dev), torch.tensor(lo, device=dev)
    col_base = torch.tensor(c.col_base(), device=dev)
    rvar = torch.full_like(c.yo, c.sigma_o ** 2)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def cycle():
        e = [ev() for _ in range(4)]
        e[0].record()
        HX = K.hx_latlon(c.X, c.nlon, c.nlat, c.nlev, c.obs_lat, c.obs_lon, c.obs_lev, c.obs_var)
        e[1].record()
        off, idx, dist = K.select_geo(clat, clon, c.obs_lat, c.obs_lon, c.hsupport_km)
        e[2].record()
        _, st = K.letkf_batched(c.X, col_base=col_base, nlev=c.nlev, n_var=c.nvar, lev_stride=c.lev_stride,
                                var_stride=c.var_stride, HX=HX, yo=c.yo, rvar=rvar, loc_off=off, loc_idx=idx,
                                loc_dist=dist, obs_lev=c.obs_lev, hsupport=c.hsupport_km, vsupport=c.vsupport,
                                rho=c.rho, flags=_lib.MG_RTPS, precision=_lib.MG_PREC_MIXED, want_mean=False)
        e[3].record()
        torch.cuda.synchronize()
        return HX, off, idx, dist, st, [e[i].elapsed_time(e[i + 1]) for i in range(3)]

    _, off0, _, _, _, _ = cycle()  # warm-up cycle
    # background of the timed cycle at a seeded sample of columns plus the
    # ten longest lists (patch centres), for the oracle
    rng = np.random.default_rng(11)
    ncol = c.nlat * c.nlon
    longest = np.argsort(np.diff(off0.cpu().numpy()))[-10:]
    sample_cols = np.unique(np.concatenate([rng.choice(ncol, 60, replace=False), longest]))
    del off0
    pts_state = (sample_cols[:, None, None] + np.arange(c.nlev)[None, :, None] * c.lev_stride
                 + np.arange(c.nvar)[None, None, :] * c.var_stride)  # col, lev, var
    Xbg = c.X[:, torch.tensor(pts_state.reshape(-1), device=dev)].double().cpu().numpy()
    torch.cuda.reset_peak_memory_stats()
    HX, off, idx, dist, st, ms = cycle()
    free, total = torch.cuda.mem_get_info()
    Xan = c.X[:, torch.tensor(pts_state.reshape(-1), device=dev)].double().cpu().numpy()
    offh = off.cpu().numpy()
    counts = np.diff(offh)
    # oracle on the sampled columns: lists by the oracle's own search, H(X)
    # rows from the device operator (bit-exact with the oracle's in the tests)
    soff, sidx, sdist = ob.select_geo(la[sample_cols], lo[sample_cols], c.obs_lat.cpu().numpy(),
                                      c.obs_lon.cpu().numpy(), c.hsupport_km)
    same_lists = all(np.array_equal(idx[offh[cc]:offh[cc + 1]].cpu().numpy(), sidx[soff[j]:soff[j + 1]])
                     for j, cc in enumerate(sample_cols))
    need = np.unique(sidx)
    HXs = HX[torch.tensor(need, device=dev)].cpu().numpy()
    remap = np.full(c.yo.shape[0], -1, dtype=np.int64)
    remap[need] = np.arange(need.size)
    olev = c.obs_lev.cpu().numpy()
    pts, poff, pidx, pw = point_lists(np.arange(len(sample_cols)), c.nlev, soff, sidx, sdist, olev, c.hsupport_km,
                                      c.vsupport)
    m = len(sample_cols) * c.nlev
    # compact background: value (col j, lev l, var v) at column j*nlev + l of var block v
    Xc = Xbg.reshape(k, len(sample_cols), c.nlev, c.nvar).transpose(0, 3, 1, 2).reshape(k, c.nvar * m)
    base = pts[:, 0] * c.nlev + pts[:, 1]
    want = ob.letkf_points(np.ascontiguousarray(Xc), base, c.nvar, m, HXs, c.yo.cpu().numpy()[need],
                           np.full(need.size, c.sigma_o ** 2), poff, remap[pidx].astype(np.int32), pw, c.rho,
                           ob.ORC_RTPS)  # npt x nvar x k
    got = Xan.reshape(k, len(sample_cols), c.nlev, c.nvar).transpose(1, 2, 3, 0).reshape(m, c.nvar, k)
    err = float(np.abs(got - want).max() / np.abs(want).max())
    hist, edges = np.histogram(counts, bins=[0, 250, 500, 1000, 2000, 4000, 8000, 16000, 32768])
    ms_cycle = sum(ms)
    return {"metric": "local analyses/s, high-resolution LETKF (FP32 members)", "value": st.n_points / (ms_cycle / 1e3),
            "unit": "analyses/s", "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": ms_cycle,
            "higher_is_better": True,
            "dtype": ("f32 storage; 3-pass TF32 tensor-core Gram, Newton-Schulz solve and update (96-slot layout), "
                      "handed-back points on the SIMT two-stage solve; FP64 means and innovations"
                      if st.tensor_path else
                      "f32 storage; FP32 anomalies and SIMT two-stage Jacobi solve; FP64 means and innovations"),
            "data": "synthetic (seeded Gaussian random fields on the GPU)",
            "config": {"workload": "1440x720 grid, 30 levels, 4 vars (124.4M values), k=80 (FP32), 5M obs "
                                   "(60% in 20 Gaussian patches of 800 km), 300 km / 2 levels, RTPS 0.9",
                       "step": "H(X), spatial-hash local search, local analyses (each cycle analyses the previous "
                               "cycle's output with the same obs)"},
            "ms": {"hx": ms[0], "search": ms[1], "analysis_call": ms[2], "analysis_kernel": st.ms_analysis,
                   "generation_s": t_gen},
            "analyses": st.n_points, "tensor_path": st.tensor_path, "handed_back_to_simt": st.n_fallback,
            "solver_iterations_per_analysis": st.total_sweeps / max(1, st.n_points - st.n_empty),
            "local_obs": {"mean_per_analysis": st.total_local / max(1, st.n_points - st.n_empty),
                          "max_per_analysis": st.max_local, "empty_points": st.n_empty,
                          "column_candidates_histogram": {"edges": edges.tolist(), "counts": hist.tolist()},
                          "column_candidates_max": int(counts.max()), "list_entries": int(offh[-1])},
            "device_memory_gb": {"in_use_after_cycle": (total - free) / 1e9, "device_total": total / 1e9,
                                 "members_fp32": c.X.numel() * 4 / 1e9},
            "oracle_check": {"columns": int(len(sample_cols)), "analyses": int(m), "lists_identical": bool(same_lists),
                             "rel_err_vs_fp64_oracle": err}}


def run_highres(args) -> None:
    """The high-resolution LETKF as its own bench line."""
    print(json.dumps(highres_results()), flush=True)


def main():
    args = parse()
    if args.profile_case:
        profile_case(args.profile_case)
        return
    if args.workload == "uneven":
        run_uneven(args)
        return
    if args.workload == "column":
        run_column(args)
        return
    if args.workload == "next":
        run_next(args)
        return
    if args.workload == "highres":
        run_highres(args)
        return
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch

    from metada_gb300 import _lib
    from metada_gb300 import algorithms as A
    from metada_gb300 import kernels as K

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    case = make_case()
    w = Workload(case, dev)
    c = case
    k = c.X.shape[0]

    # warm-up (mixed and FP64 once each)
    for _ in range(args.warmup):
        w.step(_lib.MG_PREC_MIXED)
    w.step(_lib.MG_PREC_FP64)
    ctx = K.context(local)
    l0 = ctx.launches()
    with ClockSampler(local) as clk:
        t_mixed, sts = timed(lambda: w.step(_lib.MG_PREC_MIXED), args.steps, world)
    launches = (ctx.launches() - l0) // max(1, args.steps)
    clocks = clk.summary()
    Xmixed = w.X.clone()
    t_mixed = max_over_ranks(t_mixed, world)

    # End to end through the public API with host buffers, measured next to
    # the device-resident steps (before the long FP64 comparison run).
    e2e = None
    if args.e2e_steps > 0:
        Xh = torch.from_numpy(c.X).pin_memory()
        out = torch.empty_like(Xh).pin_memory()
        geom = A.LatLonGeometry(c.nlon, c.nlat, c.nlev, c.nvar)
        cfg = {"inflation": c.rho, "localization_radius": c.hsupport_km, "vertical_radius": c.vsupport,
               "precision": "mixed", "semantics": "hunt"}
        obs_host = dict(values=c.yo, error=c.sigma_o, lat=c.obs_lat, lon=c.obs_lon, lev=c.obs_lev, var=c.obs_var)

        def e2e_step():
            ens = A.Ensemble(Xh, geom, device=dev)
            obs = A.Observation(device=dev, **obs_host)
            A.LETKF(ens, obs, A.ObsOperator(), cfg).Analyse()
            out.copy_(ens.X, non_blocking=True)
            return out

        e2e_step()
        # The clock sampler (an nvidia-smi process) starts before the window
        # opens and stops after it closes: its start-up and shut-down are not
        # part of the API call being timed.
        with ClockSampler(local) as clk_e2e:
            barrier(world)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            te, _ = timed(e2e_step, args.e2e_steps, world)
            te = max(te, (time.perf_counter() - t0))
        te = max_over_ranks(te, world)
        h2d = Xh.numel() * 8 + c.yo.size * (8 * 5 + 4)
        e2e = {"value": world * w.npoints * args.e2e_steps / te, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(out.numel() * 8), "clocks": clk_e2e.summary()}
        del Xh, out

    t64, sts64 = timed(lambda: w.step(_lib.MG_PREC_FP64), args.fp64_steps, world)
    t64 = max_over_ranks(t64, world)
    X64 = w.X.clone()

    # accuracy of the mixed path against FP64 (analysis mean and perturbations)
    m64 = X64.mean(0)
    mmx = Xmixed.mean(0)
    err_mean = float((mmx - m64).abs().max() / m64.abs().max())
    err_pert = float(((Xmixed - mmx) - (X64 - m64)).abs().max() / (X64 - m64).abs().max())
    del X64, Xmixed

    npts = w.npoints
    value = world * npts * args.steps / t_mixed
    v64 = world * npts * args.fp64_steps / t64
    st = sts[-1]
    ms_an = statistics.mean(s.ms_analysis for s in sts)
    fl = flops_per_step(st, k, c.nvar)
    peaks = {}
    pf = ROOT / "MEASURED_PEAKS.json"
    if pf.exists():
        peaks = json.loads(pf.read_text())
    achieved_tf = fl / (ms_an / 1e3) / 1e12
    if st.tensor_path:
        # kind::tf32 runs at half the dense BF16 rate on this part; the BF16
        # rate is the measured one (burst: the kernel is timed on its own).
        bf16 = peaks.get("bf16_tflops")
        peak_tf = (bf16 if bf16 else 1900.0) / 2.0
        roof = {"kernel": "letkf_tc_kernel", "bound": "tensor",
                "peak_basis": ("measured" if bf16 else "fallback") + " dense BF16 / 2 (the TF32 rate)",
                "traffic": TC_TRAFFIC_REDUCED_BYTES * st.n_points / TC_TRAFFIC_REDUCED_ANALYSES,
                "traffic_from": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on the reduced "
                                "180x90x10x4 case (162,000 analyses), scaled by analyses",
                "tensor_tflop_issued": tc_issued_flop(st, k, c.nvar) / (ms_an / 1e3) / 1e12,
                "tensor_ctas": st.tensor_ctas, "fallback_analyses": st.n_fallback,
                "newton_schulz_steps_mean": st.total_sweeps / max(1, st.n_points - st.n_empty)}
    else:
        peak_tf = 152 * 128 * 2 * 2.07e9 / 1e12  # FP32 FMA lanes at the maximum SM clock (nominal)
        roof = {"kernel": "letkf_batched_kernel<float,64>", "bound": "fp32 simt",
                "peak_basis": "nominal FP32 FMA rate (152 SMs x 128 lanes x 2 x 2070 MHz)", "traffic": None}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(case, args.cpu_points)

    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        del w
        torch.cuda.empty_cache()

        def extra(name, fn):
            # One configuration's summary; a failure is recorded in its key
            # and does not cost the headline line.
            try:
                extras[name] = fn()
            except Exception as exc:  # noqa: BLE001
                extras[name] = {"error": f"{type(exc).__name__}: {exc}"}
            torch.cuda.empty_cache()

        def uneven():
            u = uneven_results(warmup=1, steps=3)
            return {"workload": u["config"]["workload"], "metric": "analyses/s (512 cases, one captured graph)",
                    "mixed": u["mixed"], "fp64": {kk: u["fp64"][kk] for kk in ("analyses_per_s", "ms_per_batch")},
                    "max_rel_err_mixed_vs_fp64": u["max_rel_err_mixed_vs_fp64"], "steps": 3, "warmup": 1}

        def column():
            col = column_results(args.extra_train_steps, 4096)
            return {"workload": col["config"]["workload"],
                    "surrogate_training": f"{args.extra_train_steps} Adam steps of 4096 columns in this run "
                                          f"(--workload column trains 6000)",
                    "hx": col["hx"], "heldout_rel_rms_err": col["training"]["heldout_rel_rms_err"],
                    "letkf_gain_kept_by_surrogate": col["letkf"]["gain_kept_by_surrogate"]}

        def highres():
            hr = highres_results()
            return {kk: hr[kk] for kk in ("metric", "value", "unit", "ms_per_step", "dtype", "config", "ms",
                                         "analyses", "tensor_path", "handed_back_to_simt", "local_obs",
                                         "device_memory_gb", "oracle_check")}

        extra("uneven_batch", uneven)
        extra("global_etkf_small", lambda: global_etkf_results(warmup=3, steps=20))
        extra("column_operator", column)
        extra("highres_letkf", highres)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_mixed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 means, innovations, outputs)",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "members": k, "obs": int(c.yo.size), "analyses_per_step": npts,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (1.33 GB FP64 ensemble)",
                       "step": "restore background, H(X), spatial-hash local search, batched local analyses"},
            "fp64": {"value": v64, "unit": UNIT, "ms_per_step": 1e3 * t64 / args.fp64_steps,
                     "ms_analysis_kernel": sts64[-1].ms_analysis},
            "mixed_over_fp64": value / v64,
            "rel_err_vs_fp64": {"mean": err_mean, "perturbations": err_pert},
            "local_obs": {"mean": st.total_local / st.n_points, "max": st.max_local, "empty_points": st.n_empty},
            "roofline": {**roof, "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
                         "frac": achieved_tf / peak_tf, "ms_per_launch": ms_an,
                         "basis": f"{fl:.4g} algorithmic FLOP per launch (Gram 2k^2 p_loc + 2k p_loc + update "
                                  f"2 n_var k^2 + eigen 9k^3, the reference's counting convention)"},
            "clocks": clocks,
            "gpu_launches": int(launches),
        }
        if e2e:
            line["e2e"] = e2e
        if cpu:
            line["cpu_baseline"] = cpu
        line.update(extras)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
