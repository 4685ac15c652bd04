"""The N > 1 path of bench.py on CPU with the gloo backend (world size 2):
the path runs independent replicas, so ranks share only the start barrier and
the max-over-ranks timing; the reference arm runs on rank 0 alone."""
import importlib.util
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    bench = _load_bench()
    r, w, local = bench.dist_setup(world)
    bench.barrier(w)
    # each rank's "time": the job's time is the slowest rank's
    t = bench.max_over_ranks(0.5 + rank, w)
    import torch.distributed as dist

    backend = dist.get_backend()
    dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"rank": r, "world": w, "local": local, "t": t,
                                                             "backend": backend}))


def test_rank_helpers_gloo_world2(tmp_path):
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    res = [json.loads(Path(tmp_path, f"rank{r}.json").read_text()) for r in range(2)]
    assert [x["rank"] for x in res] == [0, 1]
    assert all(x["world"] == 2 and x["backend"] == "gloo" for x in res)
    assert all(x["t"] == 1.5 for x in res)  # max over ranks, seen by every rank


def test_reference_arm_prints_once_under_torchrun():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--cpu-points", "200"]
    import time

    t0 = time.perf_counter()
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    wall = time.perf_counter() - t0
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
    # the printed step time is the sample step that ran, so the steps fit in the run
    assert 0 < line["ms_per_step"] * line["steps"] / 1e3 <= wall
    assert "local analyses" in line["config"]["step"]
