"""The oracle's boson sampler (oracle/perm_oracle.c: orc_sample_b, a C
restatement of the reference's generalised Clifford & Clifford B strategy
with its own MT19937) against the reference's samples: the seeded cases of
unittests/test_seeding.py (a multiset of 20 samples each) and sequences of
the reference's own C++ samplers (exact, sample by sample).  CPU only."""
import numpy as np
import pytest

from tests import oracle_bind as orc
from tests.sampler_fixtures import load

FIX = load()


@pytest.mark.parametrize("case", FIX["seeding_cases"], ids=lambda c: c["name"])
def test_oracle_reproduces_test_seeding(case):
    got = orc.sample_b(case["U"], case["input_state"], case["shots"], case["seed"], case.get("transmissivity"))
    assert sorted(got.tolist()) == case["expected_multiset"]


@pytest.mark.parametrize("case", FIX["sequences"], ids=lambda c: c["name"])
def test_oracle_reproduces_reference_sequences(case):
    got = orc.sample_b(case["U"], case["input_state"], len(case["samples"]), case["seed"], case["transmissivity"])
    assert got.tolist() == case["samples"]


def test_oracle_photon_counts():
    # lossless: every sample holds all photons; uniform losses: at most all
    U = FIX["sequences"][0]["U"]
    inp = FIX["sequences"][0]["input_state"]
    a = orc.sample_b(U, inp, 8, 3)
    assert (a.sum(axis=1) == sum(inp)).all()
    b = orc.sample_b(U, inp, 8, 3, transmissivity=0.5)
    assert (b.sum(axis=1) <= sum(inp)).all() and (b >= 0).all()
    # transmissivity 0: no photon survives
    c = orc.sample_b(U, inp, 4, 3, transmissivity=0.0)
    assert (c == 0).all()
