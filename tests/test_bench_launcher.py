"""bench.py's --gpus launcher and rank plumbing, on CPU: `--gpus 2` without
torchrun re-launches the bench under torch.distributed.run with two ranks
(gloo in --dry-run), both join, the timing reductions run, and rank 0 prints
one line naming two ranks."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_gpus_flag_launches_ranks():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--dry-run"],
                       capture_output=True, text=True, timeout=240, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["n_gpus"] == 2 and line["ranks_reporting"] == 2
    assert line["slowest"] == 2.0  # the max over ranks of (1 + rank)
    assert line["config"]["parallelism"] == "replicas x2"


def test_reference_arm_loads_only_the_oracle():
    """The reference arm builds its inputs with the oracle's generators: the
    library is never loaded, and it times the GPU arm's step numbers."""
    code = ("import runpy, sys, io, contextlib\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--config', '0', '--steps', '2', '--warmup', '3']\n"
            "buf = io.StringIO()\n"
            "with contextlib.redirect_stdout(buf):\n"
            f"    runpy.run_path({str(ROOT / 'bench.py')!r}, run_name='__main__')\n"
            "maps = open('/proc/self/maps').read()\n"
            "print(buf.getvalue().strip())\n"
            "print(int('libcwa.so' in maps), int('libcwa_oracle' in maps),"
            " int('coupledwateranimation_gb300' in sys.modules))\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=240, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout.strip().splitlines()
    line = json.loads(out[-2])
    assert out[-1].split() == ["0", "1", "0"]
    assert line["impl"] == "reference" and line["steps"] == 2
    assert line["config"]["timed_steps"] == [4, 200]
