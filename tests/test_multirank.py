"""The multi-process path of bench.py on the CPU: two ranks over gloo on
127.0.0.1, with the environment torchrun gives each rank.

* barrier and max_over_ranks: every rank gets the largest value (the
  timing the bench reports is the maximum over ranks);
* the reference arm (--impl reference) runs on rank 0 alone, which prints
  the one JSON line; rank 1 exits 0 without output.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _spawn(args, world=2):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE=str(world), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, *args], cwd=ROOT, env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=300) for p in procs]
    return [(p.returncode, o, e) for p, (o, e) in zip(procs, outs)]


def test_barrier_and_max_over_ranks():
    code = ("import os, bench, torch.distributed as dist\n"
            "r = int(os.environ['RANK'])\n"
            "dist.init_process_group('gloo')\n"
            "bench.barrier(2)\n"
            "print(bench.max_over_ranks(1.5 + r, 2))\n"
            "dist.destroy_process_group()\n")
    for rc, out, err in _spawn(["-c", code]):
        assert rc == 0, err
        assert float(out.strip()) == 2.5


def test_reference_arm_prints_on_rank_zero_only():
    (rc0, out0, err0), (rc1, out1, err1) = _spawn(
        ["bench.py", "--impl", "reference", "--workload", "chain64", "--steps", "1", "--warmup", "3"])
    assert rc0 == 0, err0
    assert rc1 == 0, err1
    line = json.loads(out0.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert out1.strip() == ""


def test_reference_arm_line_carries_the_contract_keys():
    """One process, no torchrun: the reference arm's JSON line has the keys
    the benchmark contract lists, with e2e and cpu_baseline describing this
    run."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "chain64", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 3
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["unit"] == line["unit"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    assert "workload" in line["config"]
