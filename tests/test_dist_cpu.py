"""Multi-rank bench path on CPU (gloo, world size 2): ranks time their own domains, the job time
is the max over ranks, and the job value sums the ranks' cells."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(1.0 + rank, dist)       # rank 1 is the slow one
    g = bench.job_glups(4096 * 4096, 100, t, world)
    r, w, _ = bench.dist_env()
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, g, r, w))


def test_two_ranks_max_and_sum():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for rank, t, g, r, w in out:
        assert t == 2.0 and r == rank and w == 2
        assert abs(g - 2 * 4096 * 4096 * 100 / 2.0 / 1e9) < 1e-9


def test_reference_arm_prints_one_contract_line():
    """`bench.py --impl reference` runs on the host cores alone (no GPU) and prints one JSON line
    with the keys of the bench contract, on the same metric and workload as the GPU arm."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "3", "--warmup", "3"],
                       cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == "GLUPS" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert "4096x4096" in d["config"]["workload"]


def test_gpus_flag_without_torchrun_spawns_ranks():
    """`bench.py --gpus 2` started without torchrun launches one process per rank itself: rank 0
    prints the one line (n_gpus 2), the other rank exits cleanly.  The reference arm runs on the
    host cores, so the whole spawn path runs here without a GPU."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "3",
                        "--warmup", "3"], cwd=root, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["impl"] == "reference"
    sys.path.insert(0, root)
    import bench
    assert d["config"] == bench.bench_config(2)


RANK_SCRIPT = r'''
import json, os, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
rank, world, local = bench.dist_env()
dist.init_process_group("gloo")
ms = bench.max_over_ranks(10.0 * (1 + rank), dist)   # rank r takes 10 (r + 1) ms for its 100 steps
value = bench.job_glups(4096 * 4096, 100, ms * 1e-3, world)
if rank == 0:
    print(json.dumps({"n_gpus": world, "ms": ms, "value": value, "local": local}))
dist.barrier()
dist.destroy_process_group()
'''


def test_spawned_ranks_aggregate_max_time_and_sum_of_cells(tmp_path):
    """The spawn path's ranks meet over gloo: the job time is the slowest rank's, the value the
    cells of all ranks over that time (each rank here stands in for one GPU's timed steps)."""
    import io
    import json
    import sys
    from contextlib import redirect_stdout
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    script = tmp_path / "rank.py"
    script.write_text(RANK_SCRIPT)
    buf = io.StringIO()
    with redirect_stdout(buf):
        rc = bench.spawn_ranks(3, [root], script=str(script), timeout=300)
    assert rc == 0
    d = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert d["n_gpus"] == 3 and d["ms"] == 30.0 and d["local"] == 0
    assert abs(d["value"] - 3 * 4096 * 4096 * 100 / 0.030 / 1e9) < 1e-9
