"""The index-checked build (CWA_DEBUG_CHECKS, libcwa_debug.so): the device
index checks of the grid, neighbour, integrate and wave kernels stand in for
a memory checker.  A mixed workload (tests/_debug_workload.py) runs under
both libraries in child processes: no check may fire (a fired check returns
CWA_ERR_BOUNDS and the child exits non-zero), and every result must be
bit-identical to the release build's."""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu


def _run(env_extra: dict) -> str:
    script = Path(__file__).with_name("_debug_workload.py")
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, str(script)], env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("digest ")]
    assert lines, r.stdout[-2000:]
    return lines[-1]


def test_debug_checks_stay_silent_and_match_release(lib):
    from coupledwateranimation_gb300 import build
    build.build(debug=True)
    release = _run({"CWA_LIBRARY": "release"})
    debug = _run({"CWA_LIBRARY": "debug"})
    assert debug == release
