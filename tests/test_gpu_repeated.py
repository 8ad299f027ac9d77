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


@pytest.mark.parametrize("mode", ["fp64", "fast"])
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


@pytest.mark.parametrize("mode", ["fp64", "fast"])
def test_repeated_config3_small(mode):
    U, inp, out = repeated_instance(seed=11, modes=24, photons=12, max_mult=4)
    st = nat.Stats()
    v = nat.perm_repeated(U, inp, out, mode=mode, stats=st)
    _, dref = orc.bbfg_repeated(U, inp, out, prec=1)
    assert orc.rel_err(v, dref) <= TOL
    if mode == "fast":
        assert st.arith == nat.ARITH_DF32


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
