"""``bench.py --impl reference``: the CPU restatement of the path timed on the
host cores, printed as one JSON line with the GPU arm's metric, unit and
config.  Runs on the CPU (the small 500-510 nm workload, about 10 s each)."""

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
ARGS = ["--impl", "reference", "--workload", "window_500_510", "--steps", "1", "--warmup", "0"]


def _env():
    env = dict(os.environ)
    env["CUDA_VISIBLE_DEVICES"] = ""
    return env


def _check_line(line: dict, n_gpus: int):
    sys.path.insert(0, str(ROOT))
    import bench

    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC
    assert line["unit"] == "evals/s" and line["higher_is_better"] is True
    assert line["n_gpus"] == n_gpus and line["steps"] == 1 and line["warmup"] == 0
    assert line["config"]["workload"] == "window_500_510"
    assert line["value"] > 0 and line["ms_per_step"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_single_process():
    out = subprocess.run([sys.executable, "bench.py", *ARGS], cwd=ROOT, env=_env(), capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    _check_line(json.loads(lines[0]), 1)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_under_torchrun_prints_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--gpus", "2",
           *ARGS]
    out = subprocess.run(cmd, cwd=ROOT, env=_env(), capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    _check_line(line, 2)
    # the port runs on every host core even though torchrun sets OMP_NUM_THREADS=1
    assert line["cpu_baseline"]["cores"] == len(os.sched_getaffinity(0))


def test_reference_arm_loads_nothing_of_the_product():
    """The CPU arm runs the oracle only: the product's native library is never
    mapped and its ctypes loader is never imported (lines come from the
    restated gfall reader, the grid from the restated grid routine)."""
    code = (
        "import sys, json\n"
        f"sys.argv = ['bench.py', *{ARGS!r}]\n"
        "import bench\n"
        "rc = bench.main()\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'rc': rc, 'mapped': 'libkurucz_gb300' in maps,\n"
        "                  'native_imported': 'kurucz_py_joss_submission_gb300._native' in sys.modules,\n"
        "                  'oracle_mapped': 'libks_oracle' in maps}))\n"
    )
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=_env(), capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert res["rc"] == 0
    assert res["oracle_mapped"]
    assert not res["mapped"], "the reference arm mapped the product library"
    assert not res["native_imported"], "the reference arm imported the product's ctypes loader"
