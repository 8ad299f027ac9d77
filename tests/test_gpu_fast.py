"""GPU parity of the double-float (FP32-pipe) product path.

Bar: relative error <= 1e-10 (normalised by |perm|) against the binary128
oracle for n <= 24, and against the FP64 kernel (itself ~1e-13 accurate) at
n = 26..32 on Haar blocks.
"""
import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_block
from tests import oracle_bind as orc

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.mark.parametrize("n", list(range(1, 25)))
def test_fast_haar_vs_quad_oracle(n):
    A = haar_block(n, seed=500 + n)
    st = nat.Stats()
    v = nat.perm(A, mode="fast", stats=st)
    _, q = orc.bbfg(A, prec=1 if n <= 20 else 0)
    assert orc.rel_err(v, q) <= TOL
    if n >= 2:
        assert st.arith == nat.ARITH_DF32


@pytest.mark.parametrize("n", [4, 9, 15, 21])
def test_fast_gaussian_vs_quad_oracle(n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    v = nat.perm(A, mode="fast")
    _, q = orc.bbfg(A, prec=1)
    assert orc.rel_err(v, q) <= TOL


@pytest.mark.parametrize("n", [26, 28, 30, 32])
def test_fast_vs_fp64_kernel(n):
    A = haar_block(n, seed=n)
    a = nat.perm(A, mode="fast")
    b = nat.perm(A, mode="fp64")
    assert abs(a - b) <= TOL * abs(b)


@pytest.mark.parametrize("shape", [(3, 5), (4, 3), (6, 9), (10, 9), (1, 4)])
def test_fast_rectangular(shape):
    rng = np.random.default_rng(sum(shape) + 5)
    A = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    v = nat.perm(A, mode="fast")
    _, q = orc.bbfg(A, prec=1)
    assert orc.rel_err(v, q) <= TOL


def test_fast_all_ones():
    import math
    for n in (8, 16, 24):
        v = nat.perm(np.ones((n, n)), mode="fast")
        assert abs(v - math.factorial(n)) <= TOL * math.factorial(n)
