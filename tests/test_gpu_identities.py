"""Full-size checks of the plain permanent through exactly known relations
(n = 36 and 40, where no extended-precision oracle finishes): block-diagonal
factorisation, row/column permutation invariance and diagonal scaling; and
agreement of the three products at n = 34.  At n = 40 a permanent takes
about 3 min on the FP64 kernel, 1 min on the integer-mantissa one.

Errors are stated both ways the accuracy bar is defined: relative to |perm|
and relative to the product of the row 2-norms.  For a Haar block at n = 36
|perm| is ~1e-9 of that product (the Gray sum cancels heavily), so the
|perm|-relative error is the demanding one, and both products meet 1e-10 on
every relation: rows are balanced by exact powers of two before the sum, and
a double-float result whose error estimate is above the bar is recomputed in
FP64."""
import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_block
from tests import oracle_bind as orc

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _row_norm_product(A):
    return float(np.prod(np.linalg.norm(A, axis=1)))


def test_block_diagonal_n36_factorises():
    # perm(B1 (+) B2) = perm(B1) perm(B2); the factors from the binary128 oracle
    b1 = haar_block(18, seed=361)
    b2 = haar_block(18, seed=362)
    A = np.zeros((36, 36), dtype=np.complex128)
    A[:18, :18] = b1
    A[18:, 18:] = b2
    v = nat.perm(A, mode="fast")
    p1, _ = orc.bbfg(b1, prec=1)
    p2, _ = orc.bbfg(b2, prec=1)
    ref = p1 * p2
    assert abs(v - ref) <= TOL * abs(ref), (v, ref)


def test_permutation_invariance_n36():
    rng = np.random.default_rng(37)
    A = haar_block(36, seed=3636)
    v0 = nat.perm(A, mode="fast")
    v2 = nat.perm(A[rng.permutation(36)][:, rng.permutation(36)], mode="fast")
    assert abs(v2 - v0) <= TOL * abs(v0), (v2, v0)


def _scaled(seed):
    rng = np.random.default_rng(seed)
    A = haar_block(36, seed=3636)
    d1 = rng.uniform(0.5, 2.0, 36) * np.exp(2j * np.pi * rng.random(36))
    d2 = rng.uniform(0.5, 2.0, 36) * np.exp(2j * np.pi * rng.random(36))
    return A, d1[:, None] * A * d2[None, :], np.prod(d1) * np.prod(d2)


def test_diagonal_scaling_n36_fp64():
    # perm(D1 A D2) = prod(d1) prod(d2) perm(A), |perm|-relative, FP64 product
    A, S, scale = _scaled(36)
    v0 = nat.perm(A, mode="fp64")
    v1 = nat.perm(S, mode="fp64") / scale
    assert abs(v1 - v0) <= TOL * abs(v0), (v1, v0)


def test_diagonal_scaling_n36_fast():
    # the fast path on the rescaled matrix, against the FP64 value of the
    # unscaled one: within 1e-10 of |perm| (and so of the row-norm product)
    A, S, scale = _scaled(36)
    ref = nat.perm(A, mode="fp64")
    st = nat.Stats()
    v1 = nat.perm(S, mode="fast", stats=st)
    assert abs(v1 - ref * scale) <= TOL * abs(ref * scale), (v1, ref * scale, st.arith, st.err_est)
    assert abs(v1 - ref * scale) <= TOL * _row_norm_product(S)


def _block_diag(b1, b2):
    n1, n2 = b1.shape[0], b2.shape[0]
    A = np.zeros((n1 + n2, n1 + n2), dtype=np.complex128)
    A[:n1, :n1] = b1
    A[n1:, n1:] = b2
    return A


@pytest.mark.parametrize("mode", ["fx", "fp64", "fast"])
def test_block_diagonal_n40_factorises(mode):
    # the full 2^39-step sweep of a 40 x 40 matrix whose permanent is the
    # product of two 20 x 20 permanents from the binary128 oracle
    b1 = haar_block(20, seed=401)
    b2 = haar_block(20, seed=402)
    A = _block_diag(b1, b2)
    p1, _ = orc.bbfg(b1, prec=1)
    p2, _ = orc.bbfg(b2, prec=1)
    ref = p1 * p2
    v = nat.perm(A, mode=mode)
    assert abs(v - ref) <= TOL * abs(ref), (mode, v, ref)


def test_permutation_invariance_n40_fx():
    # a Haar block of the n = 40 configuration, rows and columns permuted
    rng = np.random.default_rng(41)
    A = haar_block(40, seed=40)
    v0 = nat.perm(A, mode="fx")
    v1 = nat.perm(A[rng.permutation(40)][:, rng.permutation(40)], mode="fx")
    assert abs(v1 - v0) <= TOL * abs(v0), (v1, v0)
    assert abs(v1 - v0) <= TOL * _row_norm_product(A)


@pytest.mark.parametrize("mode", ["fx", "fast"])
def test_products_agree_n34(mode):
    # the n = 34 block of the single-permanent configuration: each product
    # against the FP64 kernel
    for seed in (34, 3434):
        A = haar_block(34, seed=seed)
        ref = nat.perm(A, mode="fp64")
        v = nat.perm(A, mode=mode)
        assert abs(v - ref) <= TOL * abs(ref), (mode, seed, v, ref)
