"""The allocation-free plain permanent entry point (gbperm_perm_noalloc).

Some callers cannot allocate device memory: their whole pool belongs to
another allocator, or they must not pay cudaMalloc's device-wide
synchronisation.  gbperm_perm_noalloc runs the plain permanent with scratch
held in a fixed library-owned device array, so it needs no workspace.  This
test calls it through the C ABI twice in a row and checks each result
against the workspace-taking entry point gbperm_perm_dev and, at n = 20,
against the binary128 oracle; then the shapes with the largest scratch
that run in seconds (26 rows, so the grid is full, by up to 64 columns),
a rows = cols - 1 shape and the trivial shapes.  It sits in its own file,
collected last, and also passes when run alone.
"""
import ctypes

import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_block

pytestmark = pytest.mark.gpu
TOL = 1e-10
_P = ctypes.c_void_p


def _reference(lib, torch, dA, n, arith, stream, cols=None):
    cols = n if cols is None else cols
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    ws_bytes = int(lib.gbperm_perm_workspace_size(n, cols))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    nat.check(lib.gbperm_perm_dev(_P(dA.data_ptr()), n, cols, cols, arith, _P(out.data_ptr()), None,
                                  _P(ws.data_ptr()), ws_bytes, stream))
    torch.cuda.synchronize()
    return complex(out[0].item(), out[1].item())


def _noalloc(lib, torch, dA, rows, cols, arith, stream):
    out = torch.full((2,), -7.0, dtype=torch.float64, device="cuda")
    nat.check(lib.gbperm_perm_noalloc(_P(dA.data_ptr()) if dA is not None else None, rows, cols, cols, arith,
                                      _P(out.data_ptr()), None, stream))
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
        if n == 20:
            from tests import oracle_bind as orc
            _, q = orc.bbfg(A, prec=1)
            assert orc.rel_err(got, q) <= TOL


@pytest.mark.parametrize("mode", ["fp64", "fast"])
@pytest.mark.parametrize("shape", [(26, 26), (26, 48), (26, 64), (19, 20), (25, 24)])
def test_noalloc_large_scratch_shapes(mode, shape):
    # the largest fixed-point tables and a full grid of block partials that
    # run in a fraction of a second: 26 rows (2^25 Gray steps) by up to 64
    # columns (48 is the double-float product's column limit); rows =
    # cols - 1 and cols + 1 take the rectangular path
    torch = pytest.importorskip("torch")
    lib = nat.load()
    nat.require_device()
    rows, cols = shape
    rng = np.random.default_rng(rows * 100 + cols)
    A = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(rows)
    dA = torch.from_numpy(np.ascontiguousarray(A)).to("cuda")
    stream = _P(torch.cuda.current_stream().cuda_stream)
    arith = nat.arith_of(mode)
    for _ in range(2):
        got = _noalloc(lib, torch, dA, rows, cols, arith, stream)
        ref = _reference(lib, torch, dA, rows, arith, stream, cols=cols)
        assert abs(got - ref) <= TOL * abs(ref), (shape, got, ref)


def test_noalloc_trivial_shapes():
    # 0 x 0 -> 1 and rows >= cols + 2 -> 0, written on the stream by the
    # entry point itself (no matrix is read)
    torch = pytest.importorskip("torch")
    lib = nat.load()
    nat.require_device()
    stream = _P(torch.cuda.current_stream().cuda_stream)
    assert _noalloc(lib, torch, None, 0, 0, 0, stream) == 1
    dA = torch.zeros(7 * 3, dtype=torch.complex128, device="cuda")
    assert _noalloc(lib, torch, dA, 7, 3, 0, stream) == 0


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    lib = nat.load()
    nat.require_device()
    # rejected by the size check before any device work
    dA = torch.zeros(65 * 65, dtype=torch.complex128, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    rc = lib.gbperm_perm_noalloc(_P(dA.data_ptr()), 65, 65, 65, 0, _P(out.data_ptr()), None, None)
    assert rc == nat.GBPERM_ERR_TOO_LARGE
