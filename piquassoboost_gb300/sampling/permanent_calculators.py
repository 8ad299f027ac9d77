"""Free functions of the reference's ``permanent_calculators`` module
(sampling/permanent_calculators_wrapper.cpp:28-168): the repeated Glynn
permanent in double / long double, computed on the GB300."""
from __future__ import annotations

from .. import _native as nat


def permanent_CPU_repeated_double(matrix, input_state, output_state):
    """GlynnPermanentCalculatorRepeatedDouble semantics; returns complex."""
    return nat.perm_repeated(matrix, input_state, output_state)


def permanent_CPU_repeated_long_double(matrix, input_state, output_state):
    """GlynnPermanentCalculatorRepeatedLongDouble semantics; returns complex."""
    return nat.perm_repeated(matrix, input_state, output_state)
