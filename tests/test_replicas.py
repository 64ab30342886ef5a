"""Replica bookkeeping of bench.py for N>1, on CPU with gloo ranks.

The solver does not shard a mesh: N GPUs run N independent replicas and the
job's time is the slowest rank's.  These tests run that host logic with two
gloo ranks (world size 2) and check the reference arm's rank handling.
"""
from __future__ import annotations

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as tdist

    import bench
    try:
        tdist.init_process_group("gloo", rank=rank, world_size=world)
        env = bench.dist_env()
        t = bench.max_over_ranks(1.0 + 0.5 * rank, "cpu")
        v = bench.whole_job_value(env[0], 3000.0, t)
        tdist.barrier()
        tdist.destroy_process_group()
        q.put((rank, env, t, v, None))
    except Exception as e:  # reported to the parent
        q.put((rank, None, None, None, repr(e)))


def test_max_over_ranks_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=120) for _ in range(2))
    finally:
        for p in procs:
            p.join(30)
            if p.is_alive():
                p.kill()
    for rank, env, t, v, err in res:
        assert err is None, err
        assert env == (2, rank, rank)
        assert t == 1.5  # the slowest rank's time, on every rank
        assert v == pytest.approx(2 * 3000.0 / 1.5)
    assert all(p.exitcode == 0 for p in procs)


def test_single_process_is_identity():
    import bench
    assert bench.max_over_ranks(2.25, "cpu") == 2.25
    assert bench.whole_job_value(1, 100.0, 4.0) == 25.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import argparse

    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = argparse.Namespace(steps=1, warmup=1)
    assert bench.run_reference(args) is None


def test_timed_oracle_falls_back_to_the_checker_build(monkeypatch):
    """The CPU baseline runs the -O3 -ffast-math oracle build; where that
    build fails it runs the checker's -O2 build and says so."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cases
    import oracle_lib  # puts oracle/ on the path

    import bench
    import build_oracle
    real = build_oracle.build

    def no_timed(force=False, timed=False):
        if timed:
            raise RuntimeError("timed build unavailable")
        return real(force=force)

    monkeypatch.setattr(build_oracle, "build", no_timed)
    monkeypatch.setattr(oracle_lib, "_LIBS", {})
    mesh, opt = cases.airfoil(24, 8)
    orc = oracle_lib.Oracle(mesh, opt, timed=True)
    try:
        assert orc.timed is False
        assert "-O2" in bench.oracle_build(orc)
    finally:
        orc.close()


def test_reference_arm_json_line():
    """`bench.py --impl reference` (the oracle port on the host cores) prints
    one JSON line with the contract's keys, its e2e equal to its value."""
    import json
    import subprocess
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
