"""bench.py's multi-rank logic on CPU with the gloo backend, world size 2:
each rank owns a disjoint block of walkers, the step time is the maximum over
ranks and the job's pair count is the sum over ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = bench.rank_walkers(rank, 16)
        t = bench.reduce_over_ranks(0.5 + rank, "max")
        n = bench.reduce_over_ranks(1000 * (rank + 1), "sum")
        q.put((rank, w, t, n))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, t0, n0), (r1, w1, t1, n1) = got
    assert (r0, r1) == (0, 1)
    assert w0 == list(range(16)) and w1 == list(range(16, 32))
    assert t0 == t1 == 1.5
    assert n0 == n1 == 3000


def test_single_process_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(2.5, "max") == 2.5
    assert bench.rank_walkers(0, 3) == [0, 1, 2]


def _run_reference(env_extra, steps, warmup):
    import json
    import subprocess
    env = dict(os.environ, **env_extra)
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--quick",
                        "--steps", str(steps), "--warmup", str(warmup)], env=env, capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [x for x in p.stdout.splitlines() if x.startswith("{")]
    return [json.loads(x) for x in lines]


def test_reference_arm_line():
    """--impl reference on the host cores: one JSON line with the arm's own
    metric, a cpu_baseline describing the run and an e2e with no transfers;
    each step carries a tenth of the list build whatever the timed window."""
    sys.path.insert(0, ROOT)
    import bench
    (d,) = _run_reference({}, 2, 1)
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "pair-evals/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["cores"] >= 1 and "1/10 of the serial list build" in d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "pair-evals/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_silent():
    assert _run_reference({"RANK": "1", "WORLD_SIZE": "2"}, 1, 1) == []


def _fake_smi(tmp_path, loop_body):
    """An nvidia-smi stand-in: with -lms it runs loop_body, else prints one
    line in the query's format."""
    f = tmp_path / "nvidia-smi"
    f.write_text("#!/bin/sh\nfor a in \"$@\"; do case \"$a\" in -lms) %s;; esac; done\n"
                 "echo '0, 2070, 2070, 500.00, 0x0, Not Active, Not Active, Not Active, Not Active'\n" % loop_body)
    f.chmod(0o755)
    return str(tmp_path)


def test_clocks_one_shot_when_the_loop_has_no_sample(tmp_path, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("PATH", _fake_smi(tmp_path, "exec sleep 30") + os.pathsep + os.environ["PATH"])
    monkeypatch.setenv("COORD_BENCH_CLOCKS_DIR", str(tmp_path))
    c = bench.Clocks(0)
    c.start()
    out = c.stop()
    assert out["samples"] == 1 and out["sm_mhz"] == 2070.0 and out["one_shot_at_end"] is True
    assert out["reasons"] == []


def test_clocks_loop_samples_and_reasons(tmp_path, monkeypatch):
    import time
    sys.path.insert(0, ROOT)
    import bench
    body = ("while true; do echo '0, 1980, 2070, 900.00, 0x4, Not Active, Not Active, Not Active, Active'; "
            "sleep 0.05; done")
    monkeypatch.setenv("PATH", _fake_smi(tmp_path, body) + os.pathsep + os.environ["PATH"])
    monkeypatch.setenv("COORD_BENCH_CLOCKS_DIR", str(tmp_path))
    c = bench.Clocks(0)
    c.start()
    time.sleep(0.5)
    out = c.stop()
    assert out["samples"] >= 2 and out["sm_mhz"] == 1980.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"] and "one_shot_at_end" not in out
