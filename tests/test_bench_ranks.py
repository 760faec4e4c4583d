"""bench.py under torchrun, on CPU: two gloo ranks each trace their own views
(no shared rays, nothing exchanged on the data path), and the job's rate is
all ranks' rays over the slowest rank's time."""
import importlib.util
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WORKER = os.path.join(ROOT, "tests", "dist_worker.py")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks():
    pytest.importorskip("torch")
    port = _free_port()
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2")
    procs = [subprocess.Popen([sys.executable, WORKER], env=dict(env, RANK=str(r), LOCAL_RANK=str(r)),
                              stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    try:
        for p in procs:
            outs.append(p.communicate(timeout=300))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    for p, (_, err) in zip(procs, outs):
        assert p.returncode == 0, err[-2000:]
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o, _ in outs), key=lambda d: d["rank"])
    assert [d["rank"] for d in res] == [0, 1] and all(d["world"] == 2 for d in res)
    for d in res:
        assert d["units"] == (1000 + 0) + (1000 + 7)  # rays summed over ranks
        assert d["secs"] == 1.5                        # the slowest rank's time
    assert res[0]["cams"] != res[1]["cams"]           # every rank draws its own views


def test_single_process_is_a_pass_through():
    torch = pytest.importorskip("torch")
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert bench.reduce_over_ranks(torch, 123, 0.25, "cpu") == (123, 0.25)
