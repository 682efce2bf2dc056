"""The C ABI from a plain C host (tests/c_host/host_cycle.c): build a scene
with the library's generators, upload, step through the graph path, check
FP64 mass conservation, size errors and a checkpoint round trip, destroy —
no Python in the loop."""
from __future__ import annotations

import subprocess

import pytest

from test_abi import _build_c_host

pytestmark = pytest.mark.gpu


def test_c_host_full_cycle(lib, tmp_path):
    exe = _build_c_host(tmp_path)
    r = subprocess.run([str(exe), "gpu", str(tmp_path / "host.ckpt")], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.startswith("ok gpu")
