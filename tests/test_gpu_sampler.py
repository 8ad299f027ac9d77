"""GPU boson sampler (gbperm_sampler_*, the drop-in
GeneralizedCliffordsB[UniformLosses]SimulationStrategy classes) against the
reference's seeded samples.

The pmf layers run on the GPU; the draws use the reference's std::mt19937
stream, so a seed must give the reference's samples exactly: the multisets
of unittests/test_seeding.py and the sample-by-sample sequences of the
reference's own C++ samplers (tests/golden/reference_sampler.json), and the
oracle's samples on larger fresh cases.
"""
import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.sampling.BosonSamplingSimulator import BosonSamplingSimulator
from piquassoboost_gb300.sampling.simulation_strategies.GeneralizedCliffordsSimulationStrategy import (
    GeneralizedCliffordsBSimulationStrategy,
    GeneralizedCliffordsBUniformLossesSimulationStrategy,
)
from piquassoboost_gb300.workloads import haar_unitary
from tests import oracle_bind as orc
from tests.sampler_fixtures import load

pytestmark = pytest.mark.gpu
FIX = load()


def _strategy(case, seed=None, backend=None):
    seed = case["seed"] if seed is None else seed
    if case.get("transmissivity") is None:
        return GeneralizedCliffordsBSimulationStrategy(case["U"], seed, backend=backend)
    return GeneralizedCliffordsBUniformLossesSimulationStrategy(case["U"], case["transmissivity"], seed,
                                                               backend=backend)


@pytest.mark.parametrize("case", FIX["seeding_cases"], ids=lambda c: c["name"])
def test_reproduces_test_seeding(case):
    nat.require_device()
    samples = _strategy(case).simulate(np.array(case["input_state"]), case["shots"])
    assert isinstance(samples, tuple) and len(samples) == case["shots"]
    assert all(s.dtype == np.int64 for s in samples)
    assert sorted(s.tolist() for s in samples) == case["expected_multiset"]


@pytest.mark.parametrize("case", FIX["sequences"], ids=lambda c: c["name"])
def test_reproduces_reference_sequences(case):
    nat.require_device()
    samples = _strategy(case).simulate(case["input_state"], len(case["samples"]))
    assert [s.tolist() for s in samples] == case["samples"]


@pytest.mark.parametrize("backend", ["fast", "fx"])
def test_other_backends_give_the_same_draws(backend):
    nat.require_device()
    for case in FIX["sequences"]:
        samples = _strategy(case, backend=backend).simulate(case["input_state"], len(case["samples"]))
        assert [s.tolist() for s in samples] == case["samples"], case["name"]


def test_reseed_and_stream_continuation():
    nat.require_device()
    case = FIX["sequences"][1]
    st = _strategy(case, seed=31)
    a = [s.tolist() for s in st.simulate(case["input_state"], 6)]
    st.seed(31)
    b = [s.tolist() for s in st.simulate(case["input_state"], 3)] + \
        [s.tolist() for s in st.simulate(case["input_state"], 3)]
    assert a == b
    sim = BosonSamplingSimulator(_strategy(case, seed=31))
    c = [s.tolist() for s in sim.get_classical_simulation_results(case["input_state"], samples_number=6)]
    assert c == a


def test_matrix_property_and_errors():
    nat.require_device()
    U = haar_unitary(6, 1)
    st = GeneralizedCliffordsBSimulationStrategy(U, 2)
    assert np.array_equal(st.interferometer_matrix, U)
    V = haar_unitary(6, 2)
    st.interferometer_matrix = V
    st.seed(4)
    got = [s.tolist() for s in st.simulate([1, 1, 0, 1, 0, 0], 5)]
    assert got == orc.sample_b(V, [1, 1, 0, 1, 0, 0], 5, 4).tolist()
    with pytest.raises(nat.GBPermError):
        st.simulate([1, 1, 0], 2)            # one entry per mode
    with pytest.raises(nat.GBPermError):
        st.simulate([1, -1, 0, 0, 0, 0], 2)  # negative occupation
    assert st.simulate([1, 0, 0, 0, 0, 0], 0) == ()


@pytest.mark.parametrize("m,photons,seed,loss", [(30, 10, 1, None), (24, 12, 2, None), (20, 9, 3, 0.7)])
def test_matches_oracle_on_larger_cases(m, photons, seed, loss):
    # fresh seeds and interferometers beyond the fixtures, against the
    # oracle's restatement of the same sampler
    nat.require_device()
    U = haar_unitary(m, 100 + seed)
    inp = np.zeros(m, dtype=np.int64)
    inp[:photons] = 1
    case = {"U": U, "seed": seed, "transmissivity": loss}
    got = np.array([s for s in _strategy(case).simulate(inp, 3)])
    ref = orc.sample_b(U, inp, 3, seed, loss, threads=0)
    assert got.tolist() == ref.tolist()
