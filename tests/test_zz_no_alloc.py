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


def _no_alloc(lib, torch, d_in, n, out=None):
    out = torch.empty(n, dtype=torch.int32, device="cuda") if out is None else out
    assert lib.cwa_exclusive_scan_i32_noalloc(_abi.ptr(d_in), _abi.ptr(out), n, _stream(torch)) == 0, \
        _abi.last_error()
    # the look-back's bounded waits all ended in time
    assert lib.cwa_scan_noalloc_status(_stream(torch)) == 0, _abi.last_error()
    return out


# 16_777_216 = CWA_NOALLOC_SCAN_MAX_N: the scratch array's tightest fit
@pytest.mark.parametrize("n", [16, 2049, 300_763, 16_777_216])
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


def test_no_alloc_scan_unaligned_buffers(lib):
    """Input and output one element past a 16-byte boundary: the scan takes
    its scalar load / store path; two calls in a row, as above."""
    import torch
    n = 100_003
    rng = np.random.default_rng(7)
    for call in range(2):
        xs = torch.from_numpy(rng.integers(0, 50, n + 1).astype(np.int32)).cuda()
        x = xs[1:]
        want = _with_workspace(lib, torch, x, n)
        outs = torch.full((n + 1,), -1, dtype=torch.int32, device="cuda")
        got = _no_alloc(lib, torch, x, n, out=outs[1:])
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"call {call}: unaligned no-allocation scan differs"
        assert int(outs[0]) == -1, "wrote before the output"


def test_no_alloc_scan_rejects_sizes_above_its_limit(lib):
    # The size check comes first, so nothing is launched (null buffers are
    # passed on purpose: were the check missing, the call would stop at the
    # null-pointer check instead of launching).
    n = 16_777_216 + 1  # CWA_NOALLOC_SCAN_MAX_N + 1
    assert lib.cwa_exclusive_scan_i32_noalloc(None, None, n, None) == _abi.CWA_ERR_CAPACITY
    assert "CWA_NOALLOC_SCAN_MAX_N" in _abi.last_error()


@pytest.mark.parametrize("name", ["scan_kat", "scan_1k", "scan_16k"])
def test_no_alloc_scan_matches_the_reference_scan_shader(lib, name):
    """The reference's prefix_sum_cs.glsl dispatched as ParallelScan::Compute
    (UniformGrid2D/ParallelScan.cpp:43-95), compiled for the CPU: its
    outputs are tests/golden/ref_shader_outputs.npz."""
    import torch
    from pathlib import Path

    from oracle import ref
    golden = np.load(Path(__file__).resolve().parent / "golden" / "ref_shader_outputs.npz")
    x = torch.from_numpy(ref.scan_inputs()[name]).cuda()
    got = _no_alloc(lib, torch, x, x.numel())
    assert np.array_equal(got.cpu().numpy(), golden[f"{name}_out"])
