"""Pin the CPU oracle to the reference (no GPU needed).

* the known answers of the reference's unittests/test_permanent.py:47-251
  (extracted into golden/reference_unittests.json by golden/make_golden.py);
* outputs of the reference's own C++ calculators on seeded inputs
  (golden/reference_calculators.json), for every library id the oracle
  restates;
* adaptInterferometer outputs, bit for bit.
"""
import json
import os

import numpy as np
import pytest

from tests import oracle_bind as orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def _mat(case):
    a = np.array([complex(r, i) for r, i in case["matrix"]], dtype=np.complex128)
    return a.reshape(case["shape"])


def _c(v):
    return complex(v[0], v[1])


def _close(a, b, tol):
    scale = max(abs(b), 1e-300)
    return abs(a - b) <= tol * scale or (abs(b) < 1e-14 and abs(a) < 1e-14)


UNIT = _load("reference_unittests.json")["cases"]
CALC = _load("reference_calculators.json")


@pytest.mark.parametrize("case", UNIT, ids=[c["name"] for c in UNIT])
def test_oracle_reference_unittests(case):
    A = _mat(case)
    exp = _c(case["expected"])
    for prec in (0, 1):
        v, _ = orc.bbfg_repeated(A, case["input_state"], case["output_state"], prec=prec)
        assert _close(v, exp, 1e-12), (prec, v, exp)
    if len(case["input_state"]) == A.shape[1] and len(case["output_state"]) == A.shape[0]:
        v, _ = orc.glynn_repeated(A, case["input_state"], case["output_state"], prec=1)
        assert _close(v, exp, 1e-12)


@pytest.mark.parametrize("i", range(len(CALC["plain"])))
def test_oracle_plain_vs_reference_build(i):
    case = CALC["plain"][i]
    A = _mat(case)
    r, c = case["shape"]
    ref = {int(k): _c(v) for k, v in case["values"].items()}
    q, _ = orc.bbfg(A, prec=1)
    for lib, val in ref.items():
        assert _close(q, val, 1e-11), (lib, q, val)
    d, _ = orc.bbfg(A, prec=0)
    assert _close(d, ref[7], 1e-11)
    if r <= 16:
        g, _ = orc.glynn_recursive(A, prec=1)
        assert _close(g, ref[7], 1e-11)
    if r == c and r <= 12:
        s, _ = orc.glynn_simple(A, prec=1)
        assert _close(s, ref[10], 1e-11)


@pytest.mark.parametrize("i", range(len(CALC["repeated"])))
def test_oracle_repeated_vs_reference_build(i):
    case = CALC["repeated"][i]
    A = _mat(case)
    cin, rout = case["input_state"], case["output_state"]
    ref = {int(k): _c(v) for k, v in case["values"].items()}
    for prec in (0, 1):
        v, _ = orc.bbfg_repeated(A, cin, rout, prec=prec)
        for lib, val in ref.items():
            assert _close(v, val, 1e-10), (prec, lib, v, val)
    if len(cin) == A.shape[1] and sum(rout) <= 12:
        g, _ = orc.glynn_repeated(A, cin, rout, prec=1)
        assert _close(g, ref[7], 1e-10)


@pytest.mark.parametrize("i", range(len(CALC["adapt"])))
def test_oracle_adapt_interferometer_exact(i):
    case = CALC["adapt"][i]
    m = case["m"]
    U = np.array([complex(r, i) for r, i in case["matrix"]]).reshape(m, m)
    sub = orc.adapt_interferometer(U, case["input_state"], case["output_state"])
    exp = np.array([complex(r, i) for r, i in case["result"]]).reshape(case["shape"])
    assert sub.shape == exp.shape
    assert np.array_equal(sub, exp)


def test_oracle_expanded_equals_repeated():
    # ctests/permanents_accuracy.cpp:41-79 pattern: expanded matrix vs multiplicities
    rng = np.random.default_rng(3)
    for dim in range(2, 8):
        U = rng.standard_normal((dim, dim)) + 1j * rng.standard_normal((dim, dim))
        mult = rng.integers(1, 3, size=dim)
        E = orc.adapt_interferometer_multiplied(U, mult, mult)
        a, _ = orc.bbfg(E, prec=1)
        b, _ = orc.bbfg_repeated(U, mult, mult, prec=1)
        assert _close(a, b, 1e-12)


def test_oracle_mismatched_states_raise():
    # performance_tests/test_permanent_calculators.py:43-75
    A = np.eye(4, dtype=complex)
    with pytest.raises(RuntimeError):
        orc.bbfg_repeated(A, [1, 1, 1, 0], [1, 1, 1, 1])
    with pytest.raises(RuntimeError):
        orc.glynn_repeated(A, [1, 1, 1, 0], [1, 1, 1, 1])


def test_oracle_all_ones_factorial():
    import math
    for n in range(1, 13):
        v, _ = orc.bbfg(np.ones((n, n)), prec=1)
        assert abs(v - math.factorial(n)) <= 1e-12 * math.factorial(n)


@pytest.mark.parametrize("i", range(len(CALC.get("pmf", []))))
def test_oracle_compute_pmf_vs_reference_build(i):
    # samplingHelperFunctions.cpp:78-342
    case = CALC["pmf"][i]
    m = case["m"]
    U = np.array([complex(r, im) for r, im in case["matrix"]]).reshape(m, m)
    pmf, _ = orc.compute_pmf(U, case["sample"], case["current_input"], prec=1)
    assert np.allclose(pmf, case["pmf"], rtol=1e-10, atol=1e-14)


@pytest.mark.parametrize("i", range(len(CALC["repeated"])))
def test_oracle_chinhuh_vs_reference_build(i):
    # CChinHuhPermanentCalculator.cpp:48-201 (repeated lib 0)
    case = CALC["repeated"][i]
    ref = {int(k): _c(v) for k, v in case["values"].items()}
    if 0 not in ref:
        pytest.skip("no lib 0 value")
    A = _mat(case)
    for prec in (0, 1):
        v, _ = orc.chinhuh(A, case["input_state"], case["output_state"], prec=prec)
        assert _close(v, ref[0], 1e-10), (prec, v, ref[0])


@pytest.mark.parametrize("prec", [0, 1])
def test_range_sums_add_up_to_the_permanent(prec):
    """orc_bbfg_range_prec (the bench's CPU-baseline sampler) over a split of
    the whole Gray range gives the full sum, in double and in binary128."""
    import ctypes

    lib = orc.lib()
    P = ctypes.c_void_p
    fn = lib.orc_bbfg_range_prec
    fn.argtypes = [P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                   ctypes.c_uint64, ctypes.c_uint64, P]
    rng = np.random.default_rng(7)
    n = 12
    A = np.ascontiguousarray(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    total = 1 << (n - 1)
    cuts = [0, 1, 333, 1024, total]
    acc = 0j
    for a, b in zip(cuts[:-1], cuts[1:]):
        out = np.zeros(4)
        assert fn(A.ctypes.data_as(P), n, n, n, prec, 3, a, b, out.ctypes.data_as(P)) == 0
        acc += complex(out[0] + out[2], out[1] + out[3])
    ref, _ = orc.bbfg(A, prec=1)
    assert abs(acc / total - ref) <= 1e-12 * abs(ref)
    out = np.zeros(4)
    assert fn(A.ctypes.data_as(P), n, n, n, 2, 1, 0, total, out.ctypes.data_as(P)) != 0  # bad prec
    assert fn(A.ctypes.data_as(P), n, n, n, 0, 1, 5, 5, out.ctypes.data_as(P)) != 0  # empty range
