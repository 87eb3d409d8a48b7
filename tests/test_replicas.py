"""The multi-GPU path is replicas only: each rank renders its own copy of the workload and the ranks
exchange nothing but the timing barrier and the max-over-ranks step time.  Exercised here with two gloo
ranks on the CPU (the per-rank render is the CPU oracle, standing in for the GPU queue)."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import hashlib
    import torch.distributed as dist
    from kazan_gb300 import replicas, scenes
    from oracle import kz_oracle
    rk = replicas.from_env()
    replicas.init(rk, "gloo")
    replicas.barrier(rk)
    scene = scenes.small_soup(n=256, width=64, height=64)
    color, depth, st = kz_oracle.render(scene)
    digest = hashlib.sha256(color.tobytes() + depth.tobytes()).hexdigest()
    digests = [None] * world
    dist.all_gather_object(digests, digest)
    local_ms = 10.0 + 5.0 * rank
    ms = replicas.max_over_ranks(rk, local_ms)
    rate = replicas.aggregate_rate(rk, scene.triangles, ms)
    replicas.barrier(rk)
    replicas.finish(rk)
    q.put((rank, digests, ms, rate, rk.leader))


def test_two_gloo_replicas():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, d0, ms0, rate0, lead0), (r1, d1, ms1, rate1, lead1) = out
    assert d0 == d1 and d0[0] == d0[1], "replicas must render identical images"
    assert ms0 == ms1 == 15.0, "every rank sees the slowest rank's time"
    assert rate0 == rate1 == pytest.approx(256 * 2 / 0.015)
    assert lead0 and not lead1


def test_reference_arm_runs_on_rank_zero_only():
    """under torchrun the reference arm prints from rank 0; other ranks exit 0 without work"""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "soup",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    import json
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "Mtris/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
