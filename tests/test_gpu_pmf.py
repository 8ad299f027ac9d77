"""GPU parity of the boson-sampling pmf layer (gbperm_compute_pmf) against
the CPU oracle's restatement of compute_pmf
(samplingHelperFunctions.cpp:78-342) and the reference build's outputs."""
import json
import os

import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_unitary
from tests import oracle_bind as orc

pytestmark = pytest.mark.gpu
TOL = 1e-10
HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_calculators.json")) as _f:
    PMF_GOLD = json.load(_f).get("pmf", [])


@pytest.fixture(autouse=True)
def _double_float_layers():
    # the fast mode's pmf rule (df.pmf_max_photons, default 0) sends every
    # layer to the integer-mantissa kernel; lifted here so that "fast"
    # exercises the double-float layer and its FP64 twin
    nat.require_device()
    nat.set_option("df.pmf_max_photons", 64)
    yield
    nat.set_option("df.pmf_max_photons", 0)


def test_pmf_fast_default_rule_runs_fx():
    # beyond df.pmf_max_photons (default 0: every layer) a double-float
    # request runs the integer-mantissa layer
    nat.set_option("df.pmf_max_photons", 0)
    U = haar_unitary(12, 3)
    cin = np.array([1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0])
    sample = np.array([0, 2, 0, 1, 0, 0, 0, 1, 0, 0, 1, 0])
    st = nat.Stats()
    a, x = nat.compute_pmf(U, sample, cin, mode="fast", stats=st)
    assert st.arith == nat.ARITH_FX64
    b, y = nat.compute_pmf(U, sample, cin, mode="fx")
    assert np.array_equal(a, b) and np.array_equal(x, y)


def _check(U, sample, cin, mode="fp64"):
    pmf, add = nat.compute_pmf(U, sample, cin, mode=mode)
    rpmf, radd = orc.compute_pmf(U, sample, cin, prec=1)
    assert pmf.shape == rpmf.shape
    assert np.allclose(pmf, rpmf, rtol=TOL, atol=1e-13), np.max(np.abs(pmf - rpmf))
    scale = np.max(np.abs(radd))
    for a, b in zip(add, radd):
        if abs(b) > 1e-6 * scale:
            assert abs(a - b) <= TOL * abs(b), (a, b)
        else:
            assert abs(a - b) <= TOL * scale
    assert abs(pmf.sum() - 1.0) < 1e-12
    assert np.all(pmf >= 0.0)
    return pmf, add


@pytest.mark.parametrize("mode", ["fp64", "fast"])
@pytest.mark.parametrize("i", range(len(PMF_GOLD)))
def test_pmf_reference_build_vectors(i, mode):
    case = PMF_GOLD[i]
    m = case["m"]
    U = np.array([complex(r, im) for r, im in case["matrix"]]).reshape(m, m)
    pmf, _ = nat.compute_pmf(U, case["sample"], case["current_input"], mode=mode)
    assert np.allclose(pmf, case["pmf"], rtol=TOL, atol=1e-13)


def _layer(seed, m, k, max_in=1, bunch=False):
    """A Clifford & Clifford layer: input with k photons, sample with k-1."""
    rng = np.random.default_rng(seed)
    U = haar_unitary(m, seed)
    cin = np.zeros(m, dtype=np.int64)
    if max_in == 1:
        cin[rng.choice(m, size=k, replace=False)] = 1
    else:
        while cin.sum() < k:
            j = rng.integers(m)
            if cin[j] < max_in:
                cin[j] += 1
    p = np.ones(m) / m if not bunch else rng.dirichlet(np.full(m, 0.2))
    sample = rng.multinomial(k - 1, p).astype(np.int64)
    return U, sample, cin


@pytest.mark.parametrize("mode", ["fp64", "fast"])
@pytest.mark.parametrize("seed", range(24))
def test_pmf_random_layers(seed, mode):
    rng = np.random.default_rng(100 + seed)
    m = int(rng.integers(2, 16))
    k = int(rng.integers(1, min(m, 12) + 1))
    U, sample, cin = _layer(seed, m, k, max_in=int(rng.integers(1, 4)), bunch=bool(seed % 2))
    _check(U, sample, cin, mode)


@pytest.mark.parametrize("mode", ["fp64", "fast"])
@pytest.mark.parametrize("k", [2, 5, 9, 17, 33])
def test_pmf_lane_group_shapes(k, mode):
    # 1, 2, 4, 8 columns per lane with 4 lanes, and 8 x 8 above 32 input modes;
    # a bunched sample keeps the Gray range small at k = 33
    m = max(2 * k, 8)
    U = haar_unitary(m, k)
    cin = np.zeros(m, dtype=np.int64)
    cin[:k] = 1
    sample = np.zeros(m, dtype=np.int64)
    if k <= 17:
        rng = np.random.default_rng(k)
        sample = rng.multinomial(k - 1, np.ones(m) / m).astype(np.int64)
    else:
        sample[3], sample[7], sample[11] = 15, 10, k - 1 - 25
    _check(U, sample, cin, mode)


def test_pmf_first_photon():
    U = haar_unitary(6, 1)
    cin = np.array([0, 1, 0, 0, 0, 0])
    pmf, add = _check(U, np.zeros(6, dtype=np.int64), cin)
    assert np.allclose(pmf, np.abs(U[:, 1]) ** 2 / np.sum(np.abs(U[:, 1]) ** 2))
    assert add[1] == 1.0 and np.all(add[[0, 2, 3, 4, 5]] == 0)


@pytest.mark.parametrize("mode", ["fp64", "fast"])
def test_pmf_repeated_input_and_sample(mode):
    U = haar_unitary(7, 5)
    cin = np.array([3, 0, 2, 0, 1, 0, 0])
    sample = np.array([0, 2, 0, 2, 0, 1, 0])
    _check(U, sample, cin, mode)


def test_pmf_fast_matches_fp64_at_size():
    # the benchmark's 60-mode / 30-photon layer shape at 40 modes / 20 photons
    U, sample, cin = _layer(21, 40, 20)
    st = nat.Stats()
    a, x = nat.compute_pmf(U, sample, cin, mode="fast", stats=st)
    b, y = nat.compute_pmf(U, sample, cin, mode="fp64")
    assert st.arith == nat.ARITH_DF32
    assert np.allclose(a, b, rtol=1e-10, atol=1e-13)
    assert np.max(np.abs(x - y)) <= 1e-10 * np.max(np.abs(y))


@pytest.mark.parametrize("mode", ["fp64", "fast"])
def test_pmf_amplitude_is_laplace_expansion_at_size(mode):
    # sum_l input[l] perm_l U[k][l] is the permanent of the sample plus one
    # photon in mode k against the input (expansion along the new row): a
    # size-independent check against the repeated-permanent kernel
    U, sample, cin = _layer(7, 48, 24)
    pmf, add = nat.compute_pmf(U, sample, cin, mode=mode)
    amps = (cin * add) @ U.T
    mags = np.abs(cin * add) @ np.abs(U.T)   # sum_l |input[l] perm_l U[k][l]|
    ref = np.zeros(48, dtype=np.complex128)
    for k in range(48):
        out = sample.copy()
        out[k] += 1
        ref[k] = nat.perm_repeated(U, cin, out)
        assert abs(amps[k] - ref[k]) <= 1e-10 * abs(ref[k]) + 1e-12 * mags[k], (k, amps[k], ref[k])
    p_ref = np.abs(ref) ** 2 / np.sum(np.abs(ref) ** 2)
    assert np.allclose(pmf, p_ref, rtol=1e-9, atol=1e-13)


def test_pmf_photon_count_mismatch_raises():
    U = haar_unitary(4, 2)
    with pytest.raises(nat.GBPermError):
        nat.compute_pmf(U, [1, 1, 0, 0], [1, 1, 0, 0])
    with pytest.raises(nat.GBPermError):
        nat.compute_pmf(U, [0, 0, 0, 0], [0, 0, 0, 0])
    with pytest.raises(nat.GBPermError):
        nat.compute_pmf(U, [-1, 1, 0, 0], [1, 1, 0, 0])


def test_pmf_reproducible():
    U, sample, cin = _layer(3, 30, 14)
    a, x = nat.compute_pmf(U, sample, cin)
    b, y = nat.compute_pmf(U, sample, cin)
    assert np.array_equal(a, b) and np.array_equal(x, y)


@pytest.mark.parametrize("seed", range(8))
def test_pmf_fx_random_layers(seed):
    # the integer-mantissa layer against the binary128 oracle, lane shapes
    # 1, 2, 4 and 8 columns per lane
    rng = np.random.default_rng(300 + seed)
    m = int(rng.integers(6, 30))
    U = haar_unitary(m, 300 + seed)
    k = int(rng.integers(1, min(m, 24)))
    cin = np.zeros(m, dtype=np.int64)
    cin[rng.choice(m, k + 1, replace=False)] = 1
    sample = rng.multinomial(k, np.ones(m) / m).astype(np.int64)
    st = nat.Stats()
    _check(U, sample, cin, "fx")
    nat.compute_pmf(U, sample, cin, mode="fx", stats=st)
    assert st.arith == nat.ARITH_FX64


def test_pmf_fx_repeated_input_and_wide():
    # input multiplicities above 1 (column powers) and more than 32 occupied
    # input modes (8 lanes x 8 columns)
    U = haar_unitary(7, 5)
    _check(U, np.array([0, 2, 0, 2, 0, 1, 0]), np.array([3, 0, 2, 0, 1, 0, 0]), "fx")
    m = 40
    U = haar_unitary(m, 41)
    cin = np.ones(m, dtype=np.int64)
    cin[34:] = 0
    rng = np.random.default_rng(41)
    sample = rng.multinomial(33, np.ones(m) / m).astype(np.int64)
    a, x = nat.compute_pmf(U, sample, cin, mode="fx")
    b, y = nat.compute_pmf(U, sample, cin, mode="fp64")
    assert np.allclose(a, b, rtol=1e-10, atol=1e-13)
    assert np.max(np.abs(x - y)) <= 1e-10 * np.max(np.abs(y))


def test_pmf_fx_matches_fp64_at_size():
    # a 40-mode / 20-photon layer: integer-mantissa against the FP64 kernel
    U, sample, cin = _layer(21, 40, 20)
    a, x = nat.compute_pmf(U, sample, cin, mode="fx")
    b, y = nat.compute_pmf(U, sample, cin, mode="fp64")
    assert np.allclose(a, b, rtol=1e-10, atol=1e-13)
    assert np.max(np.abs(x - y)) <= 1e-10 * np.max(np.abs(y))
