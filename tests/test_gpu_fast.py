"""GPU parity of the double-float (FP32-pipe) product path.

Bar: relative error <= 1e-10 (normalised by |perm|) against the binary128
oracle for n <= 24, and against the FP64 kernel (itself ~1e-13 accurate) at
n = 26..32 on Haar blocks.
"""
import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_block, haar_unitary, repeated_instance
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


def test_fast_escalates_to_fx_when_estimate_exceeds_bar():
    # a positive matrix: its Gray terms are huge next to the permanent, so the
    # double-float estimate exceeds 1e-10 and the integer-mantissa twin
    # recomputes on the device; the result is then that kernel's, bit for bit
    rng = np.random.default_rng(28)
    G = np.abs(rng.standard_normal((28, 28))) + 0.1
    st = nat.Stats()
    v = nat.perm(G, mode="fast", stats=st)
    assert st.arith == nat.ARITH_FX64 and not (st.err_est <= 1e-10)
    assert v == nat.perm(G, mode="fx")
    r = nat.perm(G, mode="fp64")
    assert abs(v - r) <= TOL * abs(r)
    # with escalation off the double-float result stands, with its estimate
    nat.set_option("df.escalate", 0)
    try:
        st2 = nat.Stats()
        nat.perm(G, mode="fast", stats=st2)
        assert st2.arith == 1 and st2.err_est == st.err_est
    finally:
        nat.set_option("df.escalate", 1)


@pytest.mark.parametrize("n", [20, 24, 28])
def test_fast_error_estimate_covers_the_error(n):
    # well-conditioned inputs stay on the double-float product, and its
    # error against the FP64 kernel is within a few times the estimate
    for seed in range(3):
        A = haar_block(n, seed=100 * n + seed)
        st = nat.Stats()
        v = nat.perm(A, mode="fast", stats=st)
        r = nat.perm(A, mode="fp64")
        if st.arith == 1:
            assert 0.0 < st.err_est <= 1e-10
            assert abs(v - r) <= 3.0 * st.err_est * abs(r) + 1e-14 * abs(r)
        else:
            assert st.arith == nat.ARITH_FX64
            assert v == nat.perm(A, mode="fx")


@pytest.mark.parametrize("mode", ["fp64", "fast"])
def test_row_scaled_matrix_meets_bar(mode):
    # rows scaled by factors up to ~10: without the exact power-of-two row
    # balancing the Gray sum cancels catastrophically (the double-float
    # product was off by 1e-5 .. 1e-2 here)
    for seed in range(4):
        rng = np.random.default_rng(400 + seed)
        A = np.exp(rng.uniform(-2.3, 2.3, 18))[:, None] * haar_block(18, seed=400 + seed)
        v = nat.perm(A, mode=mode)
        _, q = orc.bbfg(A, prec=1)
        assert orc.rel_err(v, q) <= TOL


def test_fast_size_rule_runs_fx_alone():
    # above df.max_rows (square plain) and df.max_photons (repeated, pmf)
    # the double-float pass is skipped: the accurate product runs alone
    assert nat.get_option("df.max_rows") == 36 and nat.get_option("df.max_photons") == 24
    A = haar_block(22, seed=22)
    U, cin, rout = repeated_instance(seed=3, modes=24, photons=12, max_mult=3)
    nat.set_option("df.max_rows", 20)
    nat.set_option("df.max_photons", 10)
    try:
        st = nat.Stats()
        v = nat.perm(A, mode="fast", stats=st)
        assert st.arith == nat.ARITH_FX64 and st.err_est == 0.0 and st.launches == 2
        assert v == nat.perm(A, mode="fx")
        st = nat.Stats()
        r = nat.perm_repeated(U, cin, rout, mode="fast", stats=st)
        assert st.arith == nat.ARITH_FX64 and st.launches == 2
        assert r == nat.perm_repeated(U, cin, rout, mode="fx")
    finally:
        nat.set_option("df.max_rows", 36)
        nat.set_option("df.max_photons", 24)
    st = nat.Stats()
    nat.perm(A, mode="fast", stats=st)
    assert st.arith == nat.ARITH_DF32


def test_fast_repeated_escalates_to_fx_twin():
    # a Fourier interferometer near a suppressed output (the exact Fourier
    # amplitude of this output vanishes): the terms are O(1) while the
    # permanent is ~1e-7, so the double-float estimate (~2.5e-9) exceeds
    # 1e-10 and the integer-mantissa twin recomputes on the device
    m = 12
    F = np.exp(2j * np.pi * np.outer(np.arange(m), np.arange(m)) / m) / np.sqrt(m)
    U = F + 1e-4 * haar_unitary(m, 5)
    cin = np.ones(m, dtype=np.int64)
    rout = np.array([2, 0, 1, 0, 1, 1, 0, 3, 1, 0, 2, 1])
    st = nat.Stats()
    v = nat.perm_repeated(U, cin, rout, mode="fast", stats=st)
    assert st.arith == nat.ARITH_FX64 and not (st.err_est <= 1e-10)
    _, q = orc.bbfg_repeated(U, cin, rout, prec=1)
    assert orc.rel_err(v, q) <= TOL
