"""CPU-side checks of the C ABI and the drop-in API (no GPU needed).

* libgbperm.so loads and exports every function declared in include/gbperm.h;
* compute calls fail loudly without a GPU (no CPU fallback);
* trivial shapes follow the reference's semantics without touching a GPU;
* the drop-in classes keep the reference's lib-id table, messages and state
  coercion (Boson_Sampling_Utilities.py:30-335).
"""
import ctypes
import os
import re

import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(gbperm_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    return nat.load(build_if_missing=True)


def test_library_exports_every_declared_function(lib):
    declared = _declared_functions()
    assert len(declared) >= 10
    for name in sorted(declared):
        assert hasattr(lib, name), name
    # and the ctypes binding covers them all
    assert declared <= set(nat.exported_symbols())


def test_version_and_errors(lib):
    assert lib.gbperm_version() >= 100
    assert nat.get_option("plain.seg_log2") == -1
    with pytest.raises(nat.GBPermError):
        nat.set_option("no.such.key", 1)
    # double-float results above the error bar go to FP64 unless switched off
    assert nat.get_option("df.escalate") == 1
    nat.set_option("df.escalate", 0)
    try:
        assert nat.get_option("df.escalate") == 0
    finally:
        nat.set_option("df.escalate", 1)
    # the stats record carries the error estimate after the four int32 fields
    assert nat.Stats.err_est.offset == 40 and ctypes.sizeof(nat.Stats) == 48


def test_trivial_shapes_need_no_gpu():
    assert nat.perm(np.zeros((0, 0))) == 1
    assert nat.perm(np.zeros((4, 0))) == 1
    assert nat.perm(np.ones((5, 3))) == 0
    assert nat.perm_repeated(np.eye(3), [0, 0, 0], [0, 0, 0]) == 1
    assert nat.perm_batched([]) == []


def test_state_sum_mismatch_is_reported(lib):
    with pytest.raises(nat.GBPermError) as e:
        nat.perm_repeated(np.eye(3), [1, 1, 1], [1, 1, 0])
    assert e.value.code == nat.GBPERM_ERR_STATE_SUM
    assert "Number of input and output states should be equal" in str(e.value)


def test_oversize_and_bad_args(lib):
    with pytest.raises(nat.GBPermError) as e:
        nat.perm_repeated(np.eye(3), [1, 1, 1, 1], [1, 1, 1, 1])
    assert e.value.code == nat.GBPERM_ERR_ARG


@pytest.mark.skipif(nat.load(build_if_missing=True).gbperm_device_count() > 0, reason="a GPU is present")
def test_no_cpu_fallback_without_gpu():
    rng = np.random.default_rng(0)
    A = rng.standard_normal((6, 6))
    with pytest.raises(nat.GBPermError) as e:
        nat.perm(A)
    assert e.value.code == nat.GBPERM_ERR_NO_DEVICE
    with pytest.raises(nat.GBPermError):
        nat.perm_repeated(A, [1] * 6, [1] * 6)


def test_dropin_lib_ids_and_messages():
    from piquassoboost_gb300.sampling import Boson_Sampling_Utilities as bsu

    A = np.eye(3)
    for cls, lib_id in [(bsu.GlynnPermanent, 0), (bsu.GlynnPermanentDouble, 6), (bsu.BBFGPermanentDouble, 7),
                        (bsu.BBFGPermanentLongDouble, 8), (bsu.GlynnPermanentSimpleDouble, 10),
                        (bsu.GlynnPermanentSimpleLongDouble, 11)]:
        assert cls(A).lib == lib_id
    for cls in (bsu.GlynnPermanentInf, bsu.GlynnPermanentSingleDFE, bsu.GlynnPermanentDualDFE):
        with pytest.raises(Exception, match="Wrong value set for permanent library."):
            cls(A)
    for cls, lib_id in [(bsu.ChinHuhPermanentCalculator, 0), (bsu.GlynnRepeatedPermanentCalculator, 1),
                        (bsu.GlynnRepeatedPermanentCalculatorDouble, 6),
                        (bsu.BBFGRepeatedPermanentCalculatorDouble, 7),
                        (bsu.BBFGRepeatedPermanentCalculatorLongDouble, 8)]:
        assert cls(A, (1, 1, 1), (1, 1, 1)).lib == lib_id
    inf = bsu.GlynnRepeatedInfPermanentCalculator(A, (1, 1, 1), (1, 1, 1))
    with pytest.raises(Exception, match="Wrong value set for permanent library."):
        inf.calculate()
    for cls in (bsu.GlynnRepeatedSingleDFEPermanentCalculator, bsu.GlynnRepeatedDualDFEPermanentCalculator):
        with pytest.raises(Exception, match="Wrong value set for permanent library."):
            cls(A, (1, 1, 1), (1, 1, 1))
    # the reference's Python class accepts lists only of numpy arrays
    with pytest.raises(Exception, match="The input state should be a numpy array"):
        bsu.BBFGRepeatedPermanentCalculatorDouble(A, [1, 1, 1], (1, 1, 1))


def test_dropin_backend_keyword():
    from piquassoboost_gb300.sampling import Boson_Sampling_Utilities as bsu

    A = np.eye(3)
    assert bsu.BBFGPermanentDouble(A).backend is None
    assert bsu.GlynnPermanent(A, backend="fast").backend == "fast"
    assert bsu.GB300FastRepeatedPermanentCalculator(A, (1, 1, 1), (1, 1, 1), backend="fp64").backend == "fp64"
    assert bsu.ChinHuhPermanentCalculator_wrapper(7, A, np.ones(3, np.int64), np.ones(3, np.int64),
                                                  backend="fast").backend == "fast"
    for bad in ("cpu", "FP64", 1):
        with pytest.raises(ValueError, match="unknown backend"):
            bsu.BBFGPermanentDouble(A, backend=bad)
        with pytest.raises(ValueError, match="unknown backend"):
            bsu.BBFGRepeatedPermanentCalculatorDouble(A, (1, 1, 1), (1, 1, 1), backend=bad)
    # the library id is still checked first, with the reference's message
    with pytest.raises(Exception, match="Wrong value set for permanent library."):
        bsu.GlynnPermanentInf(A, backend="fast")
    # keyword only: a third positional argument is not taken as the backend
    with pytest.raises(TypeError):
        bsu.BBFGPermanentDouble(A, "fast")
    # trivial shapes are answered without a device under either arithmetic
    assert bsu.BBFGPermanentDouble(np.zeros((0, 0)), backend="fast").calculate() == 1
    assert bsu.GB300Permanent(np.ones((5, 3)), backend="fast").calculate() == 0
    assert bsu.BBFGRepeatedPermanentCalculatorDouble(A, (0, 0, 0), (0, 0, 0), backend="fast").calculate() == 1


def test_dropin_state_coercion_and_lists():
    from piquassoboost_gb300.sampling import Boson_Sampling_Utilities as bsu

    A = np.eye(2)
    c = bsu.BBFGRepeatedPermanentCalculatorDouble(A, (0, 0), (0, 0))
    assert isinstance(c.input_state, np.ndarray) and c.input_state.dtype == np.int64
    assert c.calculate() == 1
    # list of input states, list of lists of output states -> nested lists
    # (the wrapper type; the reference's Python subclass accepts only flat lists)
    c = bsu.ChinHuhPermanentCalculator_wrapper(7, A, [np.zeros(2, np.int64)], [[np.zeros(2, np.int64)] * 2])
    assert c.calculate() == [[1, 1]]
    with pytest.raises(Exception, match="The input state should be a numpy array"):
        bsu.BBFGRepeatedPermanentCalculatorDouble(A, [(0, 0)], [np.zeros(2)])


def test_connector_empty_list_quirk():
    from piquassoboost_gb300.connector import cpp_permanent_function

    assert cpp_permanent_function(np.eye(2), [], []) == 1.0
    assert cpp_permanent_function(np.eye(2), np.zeros(2, np.int64), np.zeros(2, np.int64)) == 1


def test_new_entry_points_validate_before_the_device(lib):
    # argument and state errors are reported without a GPU, as for the permanents
    U = np.eye(4, dtype=np.complex128)
    with pytest.raises(nat.GBPermError) as e:
        nat.compute_pmf(U, [1, 1, 0, 0], [1, 1, 0, 0])
    assert e.value.code == nat.GBPERM_ERR_STATE_SUM
    with pytest.raises(nat.GBPermError) as e:
        nat.compute_pmf(U, [-1, 1, 0, 0], [1, 1, 0, 0])
    assert e.value.code == nat.GBPERM_ERR_ARG
    with pytest.raises(nat.GBPermError) as e:
        nat.perm_repeated_many(U, [([1, 0, 0, 0], [1, 0, 0, 0]), ([1, 1, 0, 0], [1, 0, 0, 0])])
    assert e.value.code == nat.GBPERM_ERR_STATE_SUM
    assert nat.perm_repeated_many(U, [([0, 0, 0, 0], [0, 0, 0, 0])]) == [1]
    assert nat.perm_repeated(U, [0, 0, 0, 0], [0, 0, 0, 0], form="chinhuh") == 1
    with pytest.raises(nat.GBPermError) as e:
        nat.perm_repeated(U, [1, 1, 0, 0], [1, 0, 0, 0], form="chinhuh")
    assert e.value.code == nat.GBPERM_ERR_STATE_SUM
    with pytest.raises(nat.GBPermError) as e:
        nat.perm_grad_batched(np.zeros((2, 40, 40), dtype=np.complex128))
    assert e.value.code == nat.GBPERM_ERR_TOO_LARGE


@pytest.mark.skipif(nat.load(build_if_missing=True).gbperm_device_count() > 0, reason="a GPU is present")
def test_new_entry_points_need_a_gpu():
    rng = np.random.default_rng(1)
    U = np.linalg.qr(rng.standard_normal((6, 6)) + 1j * rng.standard_normal((6, 6)))[0]
    for call in (lambda: nat.compute_pmf(U, [1, 0, 0, 0, 0, 0], [1, 1, 0, 0, 0, 0]),
                 lambda: nat.perm_repeated_many(U, [([1, 1, 0, 0, 0, 0], [0, 1, 1, 0, 0, 0])]),
                 lambda: nat.perm_repeated(U, [1, 1, 0, 0, 0, 0], [0, 1, 1, 0, 0, 0], form="chinhuh"),
                 lambda: nat.perm_grad_batched(np.stack([U, U]))):
        with pytest.raises(nat.GBPermError) as e:
            call()
        assert e.value.code == nat.GBPERM_ERR_NO_DEVICE


def test_probe_kind_is_validated_before_the_device(lib):
    v = ctypes.c_double()
    assert lib.gbperm_probe_peak(9, ctypes.byref(v)) == nat.GBPERM_ERR_ARG
    assert lib.gbperm_probe_peak(-1, ctypes.byref(v)) == nat.GBPERM_ERR_ARG
    assert set(nat._PROBES.values()) == set(range(9))
