"""GPU parity of the integer-mantissa ("fx") product path of the plain
permanent.

The fx product keeps 55-57 significant bits per complex multiply (the FP64
product keeps 53), so it is held to the same bars as the FP64 kernel:
relative error <= 1e-10 (normalised by |perm|) against the binary128 oracle
for n <= 20 and the double oracle up to 24, agreement with the FP64 kernel
within 1e-10 at n = 26..34, and an accuracy at least that of the FP64
kernel over a set of Haar blocks measured against the binary128 oracle.
"""
import math

import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_block
from tests import oracle_bind as orc

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.mark.parametrize("n", list(range(1, 25)))
def test_fx_haar_vs_oracle(n):
    A = haar_block(n, seed=700 + n)
    st = nat.Stats()
    v = nat.perm(A, mode="fx", stats=st)
    _, q = orc.bbfg(A, prec=1 if n <= 20 else 0)
    assert orc.rel_err(v, q) <= TOL
    assert st.arith == nat.ARITH_FX64


@pytest.mark.parametrize("n", [3, 9, 17, 20])
def test_fx_gaussian_vs_quad_oracle(n):
    rng = np.random.default_rng(900 + n)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    v = nat.perm(A, mode="fx")
    _, q = orc.bbfg(A, prec=1)
    assert orc.rel_err(v, q) <= TOL


@pytest.mark.parametrize("shape", [(2, 3), (3, 5), (4, 3), (5, 3), (1, 4), (3, 1), (2, 1), (1, 1), (6, 9),
                                   (10, 9), (9, 10), (17, 18)])
def test_fx_rectangular(shape):
    rng = np.random.default_rng(sum(shape) + 11)
    A = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    v = nat.perm(A, mode="fx")
    ref, dref = orc.bbfg(A, prec=1)
    if abs(ref) == 0.0:
        assert v == 0
    else:
        assert orc.rel_err(v, dref) <= TOL


def test_fx_trivial_shapes():
    assert nat.perm(np.zeros((0, 0)), mode="fx") == 1
    assert nat.perm(np.ones((5, 3)), mode="fx") == 0


def test_fx_all_ones_factorial():
    for n in (5, 10, 15, 20):
        v = nat.perm(np.ones((n, n)), mode="fx")
        assert abs(v - math.factorial(n)) <= 1e-13 * math.factorial(n)


def test_fx_real_and_zero_column():
    # a real matrix (imaginary limbs all zero) and a matrix with a zero
    # column (its factor is 0 in every term: permanent 0)
    rng = np.random.default_rng(5)
    A = rng.standard_normal((12, 12)).astype(np.complex128)
    _, q = orc.bbfg(A, prec=1)
    assert orc.rel_err(nat.perm(A, mode="fx"), q) <= TOL
    A[:, 4] = 0.0
    assert nat.perm(A, mode="fx") == 0


def test_fx_row_scaled_matrix_meets_bar():
    for seed in range(4):
        rng = np.random.default_rng(410 + seed)
        A = np.exp(rng.uniform(-2.3, 2.3, 18))[:, None] * haar_block(18, seed=410 + seed)
        v = nat.perm(A, mode="fx")
        _, q = orc.bbfg(A, prec=1)
        assert orc.rel_err(v, q) <= TOL


def test_fx_wide_dynamic_range():
    # entries spanning 2^-300 .. 2^300 across columns: no FP32 range limit
    # applies to the integer product (the double-float path hands such
    # matrices to the FP64 kernel)
    rng = np.random.default_rng(77)
    A = haar_block(14, seed=77) * np.exp2(rng.integers(-300, 300, 14))[None, :]
    v = nat.perm(A, mode="fx")
    r = nat.perm(A, mode="fp64")
    assert abs(v - r) <= TOL * abs(r)


@pytest.mark.parametrize("n", [26, 28, 30, 32, 34])
def test_fx_vs_fp64_kernel(n):
    A = haar_block(n, seed=n)
    a = nat.perm(A, mode="fx")
    b = nat.perm(A, mode="fp64")
    assert abs(a - b) <= TOL * abs(b)


@pytest.mark.parametrize("shape", [(12, 41), (12, 48), (10, 57), (8, 64), (14, 40), (13, 33)])
def test_fx_wide_lane_groups(shape):
    # 33..64 columns (lane pairs up to 40, lane quads above) with few rows,
    # so the 2^(rows-1) Gray sum is short; the rectangular Glynn sum is the
    # reference's polynomial for rows < cols, computed by the oracle too
    rng = np.random.default_rng(shape[1])
    A = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(shape[0])
    v = nat.perm(A, mode="fx")
    _, q = orc.bbfg(A, prec=1)
    assert orc.rel_err(v, q) <= TOL


def test_fx_at_least_as_accurate_as_fp64():
    # RMS relative error against the binary128 oracle over Haar blocks
    errs = {"fx": [], "fp64": []}
    for seed in range(12):
        A = haar_block(20, seed=2000 + seed)
        _, q = orc.bbfg(A, prec=1)
        for mode in errs:
            errs[mode].append(orc.rel_err(nat.perm(A, mode=mode), q))
    rms = {m: float(np.sqrt(np.mean(np.square(e)))) for m, e in errs.items()}
    assert rms["fx"] <= rms["fp64"], rms


def test_dropin_ids_route_to_fx():
    # id 22 and the reference's long-double ids (plain 0, 8, 11; repeated
    # 1, 8) run the integer-mantissa product, lists of matrices too (one
    # integer-mantissa batched launch)
    from piquassoboost_gb300.sampling import Boson_Sampling_Utilities as bsu
    from piquassoboost_gb300.workloads import haar_unitary, repeated_instance

    A = haar_block(14, seed=14)
    v = nat.perm(A, mode="fx")
    for cls in (bsu.GB300FxPermanent, bsu.GlynnPermanent, bsu.BBFGPermanentLongDouble,
                bsu.GlynnPermanentSimpleLongDouble):
        assert cls(A).calculate() == v, cls.__name__
    assert bsu.BBFGPermanentDouble(A, backend="fx").calculate() == v
    U, cin, rout = repeated_instance(seed=5, modes=16, photons=8, max_mult=3)
    r = nat.perm_repeated(U, cin, rout, mode="fx")
    for cls in (bsu.GB300FxRepeatedPermanentCalculator, bsu.GlynnRepeatedPermanentCalculator,
                bsu.BBFGRepeatedPermanentCalculatorLongDouble):
        assert cls(U, cin, rout).calculate() == r, cls.__name__
    mats = [haar_block(k, seed=k) for k in (6, 9, 12)]
    st = nat.Stats()
    got = bsu.GB300FxPermanent(mats).calculate()
    nat.perm_batched(mats, mode="fx", stats=st)
    assert st.arith == nat.ARITH_FX64
    for m, g in zip(mats, got):
        ref = nat.perm(m, mode="fp64")
        assert abs(g - ref) <= TOL * abs(ref)
