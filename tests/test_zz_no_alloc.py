"""The allocation-free plain permanent entry point (gbperm_perm_noalloc).

Some callers cannot allocate device memory: their whole pool belongs to
another allocator, or they must not pay cudaMalloc's device-wide
synchronisation.  gbperm_perm_noalloc runs the plain permanent with scratch
held in a fixed library-owned device array, so it needs no workspace.  This
test calls it through the C ABI twice in a row and checks each result
against the workspace-taking entry point gbperm_perm_dev.  It sits in its own
file, collected last, and also passes when run alone.
"""
import ctypes

import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_block

pytestmark = pytest.mark.gpu
TOL = 1e-10
_P = ctypes.c_void_p


def _reference(lib, torch, dA, n, arith, stream):
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    ws_bytes = int(lib.gbperm_perm_workspace_size(n, n))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    nat.check(lib.gbperm_perm_dev(_P(dA.data_ptr()), n, n, n, arith, _P(out.data_ptr()), None, _P(ws.data_ptr()),
                                  ws_bytes, stream))
    torch.cuda.synchronize()
    return complex(out[0].item(), out[1].item())


@pytest.mark.parametrize("mode", ["fp64", "fast"])
def test_noalloc_two_calls_match_workspace_entry_point(mode):
    torch = pytest.importorskip("torch")
    lib = nat.load()
    nat.require_device()
    arith = nat.arith_of(mode)
    stream = _P(torch.cuda.current_stream().cuda_stream)
    # two calls in a row on different matrices, then the first one again:
    # the shared scratch must not carry anything over between calls
    cases = [(20, 1), (23, 2), (20, 1)]
    for n, seed in cases:
        A = haar_block(n, seed=seed)
        dA = torch.from_numpy(A).to("cuda")
        out = torch.zeros(2, dtype=torch.float64, device="cuda")
        rc = lib.gbperm_perm_noalloc(_P(dA.data_ptr()), n, n, n, arith, _P(out.data_ptr()), None, stream)
        nat.check(rc)
        torch.cuda.synchronize()
        got = complex(out[0].item(), out[1].item())
        ref = _reference(lib, torch, dA, n, arith, stream)
        assert abs(got - ref) <= TOL * abs(ref), (n, seed, got, ref)


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    lib = nat.load()
    # rejected by the size check before any device work
    dA = torch.zeros(65 * 65, dtype=torch.complex128, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    rc = lib.gbperm_perm_noalloc(_P(dA.data_ptr()), 65, 65, 65, 0, _P(out.data_ptr()), None, None)
    assert rc == nat.GBPERM_ERR_TOO_LARGE
