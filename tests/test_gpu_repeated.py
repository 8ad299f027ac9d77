"""GPU parity of the repeated-multiplicity kernel against the CPU oracle."""
import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_unitary, repeated_instance
from tests import oracle_bind as orc

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _random_case(seed):
    rng = np.random.default_rng(seed)
    m = int(rng.integers(1, 9))
    A = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    k = int(rng.integers(1, 12))
    cin = rng.multinomial(k, np.ones(m) / m).astype(np.int64)
    rout = rng.multinomial(k, np.ones(m) / m).astype(np.int64)
    return A, cin, rout


@pytest.mark.parametrize("mode", ["fp64", "fast", "fx"])
@pytest.mark.parametrize("seed", range(60))
def test_repeated_random(seed, mode):
    A, cin, rout = _random_case(seed)
    v = nat.perm_repeated(A, cin, rout, mode=mode)
    ref, dref = orc.bbfg_repeated(A, cin, rout, prec=1)
    if abs(ref) < 1e-300:
        assert abs(v) < 1e-12
    else:
        assert orc.rel_err(v, dref) <= TOL, (v, ref)


def test_repeated_matches_expanded_plain():
    # permanent with multiplicities == plain permanent of the expanded matrix
    rng = np.random.default_rng(7)
    U = haar_unitary(8, 3)
    cin = np.array([2, 0, 1, 3, 0, 1, 1, 0])
    rout = np.array([1, 1, 0, 2, 2, 0, 1, 1])
    E = orc.adapt_interferometer_multiplied(U, cin, rout)
    v = nat.perm_repeated(U, cin, rout)
    _, dref = orc.bbfg(E, prec=1)
    assert orc.rel_err(v, dref) <= TOL


@pytest.mark.parametrize("mode", ["fp64", "fast", "fx"])
def test_repeated_24_modes_12_photons(mode):
    U, inp, out = repeated_instance(seed=11, modes=24, photons=12, max_mult=4)
    st = nat.Stats()
    v = nat.perm_repeated(U, inp, out, mode=mode, stats=st)
    _, dref = orc.bbfg_repeated(U, inp, out, prec=1)
    assert orc.rel_err(v, dref) <= TOL
    if mode == "fast":
        assert st.arith == nat.ARITH_DF32
    if mode == "fx":
        assert st.arith == nat.ARITH_FX64


@pytest.mark.parametrize("seed", range(4))
def test_repeated_fx_vs_fp64_60_modes_30_photons(seed):
    # the repeated configuration (60-mode Haar, 30 photons, multiplicities up
    # to 4): the integer-mantissa product against the FP64 kernel, where the
    # double-float product misses the bar on most instances
    U, inp, out = repeated_instance(seed=seed, modes=60, photons=30, max_mult=4)
    a = nat.perm_repeated(U, inp, out, mode="fx")
    b = nat.perm_repeated(U, inp, out, mode="fp64")
    assert abs(a - b) <= TOL * abs(b), (a, b)


@pytest.mark.parametrize("seed", range(6))
def test_repeated_fx_column_powers(seed):
    # input multiplicities above 1 on the column side (powers by repeated
    # normalised multiplies), several lane shapes
    rng = np.random.default_rng(500 + seed)
    m = int(rng.integers(6, 26))
    U = haar_unitary(m, 500 + seed)
    k = int(rng.integers(4, 12))
    cin = rng.multinomial(k, np.ones(m) / m).astype(np.int64)
    rout = rng.multinomial(k, np.ones(m) / m).astype(np.int64)
    v = nat.perm_repeated(U, cin, rout, mode="fx")
    _, dref = orc.bbfg_repeated(U, cin, rout, prec=1)
    if abs(complex(dref[0], dref[1])) < 1e-300:
        assert abs(v) < 1e-12
    else:
        assert orc.rel_err(v, dref) <= TOL


def test_repeated_fast_vs_fp64_boson_sampling_shape():
    # 40 modes, 20 photons (the 60-mode / 30-photon shape at a size the FP64
    # kernel finishes in well under a second)
    U, inp, out = repeated_instance(seed=5, modes=40, photons=20, max_mult=4)
    a = nat.perm_repeated(U, inp, out, mode="fast")
    b = nat.perm_repeated(U, inp, out, mode="fp64")
    assert abs(a - b) <= TOL * abs(b)


def test_repeated_state_sum_error():
    with pytest.raises(nat.GBPermError) as e:
        nat.perm_repeated(np.eye(3), [1, 1, 1], [1, 1, 0])
    assert e.value.code == nat.GBPERM_ERR_STATE_SUM


def test_repeated_zero_photons():
    assert nat.perm_repeated(np.eye(3), [0, 0, 0], [0, 0, 0]) == 1


@pytest.mark.parametrize("force_q", [0, 1, 2, 3])
def test_repeated_low_digit_override(force_q):
    A, cin, rout = _random_case(1234)
    cin = np.array([1, 2, 1, 0, 3]); rout = np.array([2, 1, 1, 2, 1])
    A = haar_unitary(5, 9)
    nat.set_option("repeated.low_digits", force_q)
    try:
        v = nat.perm_repeated(A, cin, rout)
    finally:
        nat.set_option("repeated.low_digits", -1)
    _, dref = orc.bbfg_repeated(A, cin, rout, prec=1)
    assert orc.rel_err(v, dref) <= TOL


@pytest.mark.parametrize("mode", ["fp64", "fast"])
def test_repeated_batched_matches_single(mode):
    # sampler-style pairs on one interferometer: mostly single occupations
    # (expanded into the batched plain launch) and some bunched states (run
    # as repeated launches)
    rng = np.random.default_rng(5)
    m = 16
    U = haar_unitary(m, 9)
    pairs = []
    for q in range(60):
        k = int(rng.integers(0, 11))
        if q % 5 == 0:
            inp = rng.multinomial(k, np.ones(3) / 3)
            inp = np.concatenate([inp, np.zeros(m - 3, dtype=np.int64)])
        else:
            inp = np.zeros(m, dtype=np.int64)
            inp[rng.choice(m, size=k, replace=False)] = 1
        out = rng.multinomial(k, np.ones(m) / m).astype(np.int64)
        pairs.append((inp, out))
    st = nat.Stats()
    vals = nat.perm_repeated_many(U, pairs, mode=mode, stats=st)
    for (i, o), v in zip(pairs, vals):
        ref = nat.perm_repeated(U, i, o, mode=mode)
        assert abs(v - ref) <= 1e-10 * max(abs(ref), 1e-300) + 1e-15, (i, o, v, ref)
    _, dref = orc.bbfg_repeated(U, pairs[1][0], pairs[1][1], prec=1)
    assert orc.rel_err(vals[1], dref) <= TOL


def test_repeated_batched_mismatch_raises():
    U = haar_unitary(6, 1)
    pairs = [([1, 1, 0, 0, 0, 0], [0, 1, 1, 0, 0, 0]), ([1, 1, 1, 0, 0, 0], [0, 1, 1, 0, 0, 0])]
    with pytest.raises(nat.GBPermError):
        nat.perm_repeated_many(U, pairs)


def test_repeated_list_branch_uses_batch():
    from piquassoboost_gb300.sampling.Boson_Sampling_Utilities import BBFGRepeatedPermanentCalculatorDouble
    U = haar_unitary(8, 4)
    inp = [np.array([1, 1, 0, 1, 0, 0, 0, 0])]
    # one input state against a 2-D array of output states (one per row)
    outs = [np.array([[0, 1, 0, 0, 1, 1, 0, 0], [3, 0, 0, 0, 0, 0, 0, 0], [0, 0, 0, 0, 0, 0, 1, 2]])]
    res = BBFGRepeatedPermanentCalculatorDouble(U, inp, outs).calculate()
    assert len(res) == 1 and len(res[0]) == 3
    for v, o in zip(res[0], outs[0]):
        ref, _ = orc.bbfg_repeated(U, inp[0], o, prec=1)
        assert abs(v - ref) <= TOL * abs(ref)


def test_dropin_backend_keyword_selects_the_arithmetic():
    from piquassoboost_gb300.sampling import Boson_Sampling_Utilities as bsu
    U = haar_unitary(10, 6)
    cin = np.array([1, 1, 0, 2, 0, 1, 0, 0, 1, 0])
    rout = np.array([0, 2, 1, 0, 1, 0, 1, 1, 0, 0])
    # the keyword gives the same call as the library id of that arithmetic (both deterministic)
    assert bsu.BBFGRepeatedPermanentCalculatorDouble(U, cin, rout, backend="fast").calculate() == \
        bsu.GB300FastRepeatedPermanentCalculator(U, cin, rout).calculate()
    assert bsu.GB300FastRepeatedPermanentCalculator(U, cin, rout, backend="fp64").calculate() == \
        nat.perm_repeated(U, cin, rout, mode="fp64")
    A = U[:7, :7]
    assert bsu.BBFGPermanentDouble(A, backend="fast").calculate() == bsu.GB300FastPermanent(A).calculate()
    ref, _ = orc.bbfg(A, prec=1)
    assert abs(bsu.GlynnPermanent(A, backend="fast").calculate() - ref) <= TOL * abs(ref)


@pytest.mark.parametrize("mode", ["fp64", "fast"])
def test_chinhuh_form_vs_reference_build(mode):
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "reference_calculators.json")) as f:
        cases = json.load(f)["repeated"]
    for case in cases:
        vals = {int(k): complex(*v) for k, v in case["values"].items()}
        if 0 not in vals:
            continue
        A = np.array([complex(r, i) for r, i in case["matrix"]]).reshape(case["shape"])
        v = nat.perm_repeated(A, case["input_state"], case["output_state"], mode=mode, form="chinhuh")
        assert abs(v - vals[0]) <= TOL * max(abs(vals[0]), 1e-300), (v, vals[0])


@pytest.mark.parametrize("seed", range(20))
def test_chinhuh_form_vs_oracle(seed):
    A, cin, rout = _random_case(seed)
    v = nat.perm_repeated(A, cin, rout, form="chinhuh")
    ref, dref = orc.chinhuh(A, cin, rout, prec=1)
    if abs(ref) < 1e-300:
        assert abs(v) < 1e-12
    else:
        assert orc.rel_err(v, dref) <= TOL, (v, ref)
