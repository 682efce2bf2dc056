"""The exclusive scan that allocates nothing (cwa_exclusive_scan_i32_noalloc).

It is for callers that cannot lend a workspace or call cudaMalloc — code
running inside a host application that owns the device-memory budget, or a
real-time loop that cannot risk an allocation's device synchronisation.  Its
scratch is a fixed array inside the library, shared by every call on a
device.  This file is collected last so a run that stops at the first
failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from coupledwateranimation_gb300 import _abi

pytestmark = pytest.mark.gpu


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _with_workspace(lib, torch, d_in, n):
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.cwa_scan_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    assert lib.cwa_exclusive_scan_i32(_abi.ptr(d_in), _abi.ptr(out), n, _abi.ptr(ws), ws.numel(),
                                      _stream(torch)) == 0, _abi.last_error()
    return out


def _no_alloc(lib, torch, d_in, n):
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    assert lib.cwa_exclusive_scan_i32_noalloc(_abi.ptr(d_in), _abi.ptr(out), n, _stream(torch)) == 0, \
        _abi.last_error()
    return out


@pytest.mark.parametrize("n", [16, 2049, 300_763])
def test_no_alloc_scan_matches_workspace_scan_twice(lib, n):
    import torch
    assert torch.cuda.is_available()
    rng = np.random.default_rng(n)
    # two calls in a row: the second must not see the first call's leftovers
    for call in range(2):
        x = torch.from_numpy(rng.integers(0, 50, n).astype(np.int32)).cuda()
        want = _with_workspace(lib, torch, x, n)
        got = _no_alloc(lib, torch, x, n)
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"call {call}: no-allocation scan differs"


def test_no_alloc_scan_rejects_sizes_above_its_limit(lib):
    # The size check comes first, so nothing is launched (null buffers are
    # passed on purpose: were the check missing, the call would stop at the
    # null-pointer check instead of launching).
    n = 16_777_216 + 1  # CWA_NOALLOC_SCAN_MAX_N + 1
    assert lib.cwa_exclusive_scan_i32_noalloc(None, None, n, None) == _abi.CWA_ERR_CAPACITY
    assert "CWA_NOALLOC_SCAN_MAX_N" in _abi.last_error()
