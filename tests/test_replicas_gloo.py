"""The N>1 path runs independent replicas (no data-path collective): each rank
times its own population and the job value is the units of all ranks over
the max time.  Two gloo ranks on CPU exercise bench.py's barrier and max."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(world)
    d.barrier()
    mx = d.max(float(rank + 1) * 1.5)
    # each replica runs a small CPU oracle sample; the job value sums replicas
    from clotho_gb300.workloads import NEUTRAL_WF
    v, dt, info, _ = bench.run_cpu_oracle(NEUTRAL_WF, 200, 2, 0, 1)
    d.barrier()
    q.put((rank, mx, v > 0, info["N"]))
    dist.destroy_process_group()


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [3.0, 3.0]          # max over ranks
    assert all(o[2] for o in out) and all(o[3] == 200 for o in out)


def test_bare_gpus_flag_starts_its_ranks():
    # `bench.py --gpus 2` without an outer launcher starts two ranks itself; on the reference arm rank 0
    # alone prints its line and the other rank exits 0 without work
    import json
    import subprocess
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--n", "200", "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=300,
                       env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["config"]["N"] == 200
