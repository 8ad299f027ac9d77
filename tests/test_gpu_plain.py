"""GPU parity of the plain Glynn/BBFG kernel against the CPU oracle.

Tolerance: relative error <= 1e-10 against the binary128 oracle (the bar the
path is held to); the oracle's own double result is compared too.
"""
import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_block
from tests import oracle_bind as orc

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.mark.parametrize("n", list(range(1, 21)))
def test_plain_random_gaussian(n):
    rng = np.random.default_rng(100 + n)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    v = nat.perm(A)
    _, q = orc.bbfg(A, prec=1)
    assert orc.rel_err(v, q) <= TOL


@pytest.mark.parametrize("n", [8, 16, 20, 24])
def test_plain_haar_block(n):
    A = haar_block(n, seed=n)
    v = nat.perm(A)
    ref, dref = orc.bbfg(A, prec=1 if n <= 20 else 0)
    assert orc.rel_err(v, dref) <= TOL


@pytest.mark.parametrize("shape", [(2, 3), (3, 5), (4, 3), (5, 3), (1, 4), (3, 1), (2, 1), (1, 1), (6, 9), (10, 9)])
def test_plain_rectangular(shape):
    rng = np.random.default_rng(sum(shape))
    A = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    v = nat.perm(A)
    ref, dref = orc.bbfg(A, prec=1)
    if abs(ref) == 0.0:
        assert v == 0
    else:
        assert orc.rel_err(v, dref) <= TOL


def test_plain_trivial():
    assert nat.perm(np.zeros((0, 0))) == 1
    assert nat.perm(np.ones((5, 3))) == 0


def test_plain_all_ones_factorial():
    import math
    for n in (5, 10, 15, 20):
        v = nat.perm(np.ones((n, n)))
        assert abs(v - math.factorial(n)) / math.factorial(n) <= 1e-13
