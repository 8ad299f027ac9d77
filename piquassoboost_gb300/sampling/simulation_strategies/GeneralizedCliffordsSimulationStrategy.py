"""Generalised Clifford & Clifford boson samplers, drop-in for the
reference's classes of the same names
(piquassoboost/sampling/simulation_strategies/GeneralizedCliffordsSimulation
Strategy.py, wrappers GeneralizedCliffordsBSimulationStrategy_wrapper.cpp and
GeneralizedCliffordsBUniformLossesSimulationStrategy_wrapper.cpp).

Same constructors, ``seed()``, ``simulate(input_state, samples_number)``
returning a tuple of int64 numpy arrays (one occupation vector per sample)
and the ``interferometer_matrix`` property.  The per-photon probability
layers run on the GPU (gbperm_compute_pmf), the sampling loop and the
random stream in the native library (gbperm_sampler_*), with the
reference's std::mt19937 so that a seed gives the reference's samples.

Deliberate deviations:
  * each strategy object owns its generator; the reference shares one
    generator between all strategy objects of the process;
  * ``seed=None`` seeds from the clock, as the reference's constructor does
    before a seed is set;
  * the keyword-only ``backend`` ("fx" default: the integer-mantissa
    product, at least as accurate as FP64 and faster on GB300; "fp64"; or
    "fast") selects the arithmetic of the pmf layers.  Every backend
    reproduces the reference's seeded samples in the tests.
"""
from __future__ import annotations

import time

import numpy as np

from ... import _native as nat


def _clock_seed() -> int:
    return int(time.time())


class GeneralizedCliffordsBSimulationStrategy:
    """CGeneralizedCliffordsBSimulationStrategy
    (simulation_strategies/source/CGeneralizedCliffordsBSimulationStrategy.cpp
    :137-316)."""

    _transmissivity = None

    def __init__(self, interferometer_matrix, seed=None, *, backend=None):
        self._backend = backend or "fx"
        if self._backend not in ("fp64", "fx", "fast"):
            raise ValueError(f"unknown backend {backend!r}: expected None, 'fp64', 'fx' or 'fast'")
        self._matrix = np.ascontiguousarray(interferometer_matrix, dtype=np.complex128)
        self._sampler = nat.Sampler(self._matrix, _clock_seed() if seed is None else seed, mode=self._backend,
                                    transmissivity=self._transmissivity)

    @property
    def interferometer_matrix(self):
        return self._matrix

    @interferometer_matrix.setter
    def interferometer_matrix(self, value):
        m = np.ascontiguousarray(value, dtype=np.complex128)
        self._sampler.set_matrix(m)
        self._matrix = m

    def seed(self, value):
        """Reseed the random stream (std::mt19937 with the low 32 bits)."""
        self._sampler.seed(value)

    def simulate(self, input_state, samples_number: int = 1):
        """Samples of the output occupation for the input occupation
        ``input_state`` (one entry per mode); a tuple of int64 arrays."""
        out = self._sampler.simulate(input_state, samples_number)
        return tuple(np.array(row) for row in out)


class GeneralizedCliffordsBUniformLossesSimulationStrategy(GeneralizedCliffordsBSimulationStrategy):
    """CGeneralizedCliffordsBUniformLossesSimulationStrategy
    (simulation_strategies/source/CGeneralizedCliffordsBUniformLossesSimulation
    Strategy.cpp:110-322): every photon survives with probability
    transmissivity^2; each sample first draws how many do."""

    def __init__(self, interferometer_matrix, transmissivity, seed=None, *, backend=None):
        self._transmissivity = float(transmissivity)
        super().__init__(interferometer_matrix, seed, backend=backend)
