"""Permanent calculator classes with the reference's names, constructor
signatures, library ids and return conventions
(piquassoboost/sampling/Boson_Sampling_Utilities.py:30-335), computed on the
GB300 by libgbperm.

Plain calculators take ``(matrix)``; ``calculate()`` returns a Python complex,
or a list of complex when ``matrix`` is a list of matrices
(GlynnPermanentCalculator_Wrapper.hpp:204-294).  Repeated calculators take
``(matrix, input_state, output_state)`` where input_state holds the column
multiplicities and output_state the row multiplicities; lists of states give
nested lists (ChinHuhPermanentCalculator_Wrapper.hpp:233-323).

Library ids (the reference's tables, GlynnPermanentCalculator_Wrapper.hpp
:34-44 and ChinHuhPermanentCalculator_Wrapper.hpp:36-47) all select the same
GPU Glynn/BBFG sum; the ids whose reference backend is absent from a build
without MPFR or FPGA support fail the same way the reference does ("Wrong
value set for permanent library.").  Three ids are added: 20 (GB300 FP64),
21 (GB300 fast: FP32-pipe double-float product) and 22 (GB300 integer-mantissa
product).  The reference's "long double" ids (plain 0, 8, 11; repeated 1, 8)
run the integer-mantissa product: 55-57 significant bits per complex
multiply, more than the FP64 product's 53 (it does not reach the x87
extended type's 64).  Lists of states run through one persistent
multiplicity launch with that product; lists of matrices run through the
plain batched launch in the same product.

Every class also takes a keyword-only ``backend``: None (default) keeps the
arithmetic of its library id, "fp64" selects the FP64 product, "fx" the
integer-mantissa product and "fast" the double-float product (whose results
above a 1e-10 error estimate are recomputed on the device: single
permanents by the integer-mantissa product, plain batches in FP64).  The
reference has no such argument; an unknown value raises ValueError.

Deliberate deviations: arrays are converted to complex128 / int64 (the
reference reinterprets a C-contiguous array's memory whatever its dtype), and
states longer than the matrix raise instead of reading past it.
"""
from __future__ import annotations

from typing import List

import numpy as np

from .. import _native as nat

WRONG_LIB = "Wrong value set for permanent library."

# plain ids served on the GPU; value = arithmetic mode passed to libgbperm
PLAIN_LIBS = {0: "fx", 6: "fp64", 7: "fp64", 8: "fx", 10: "fp64", 11: "fx", 20: "fp64", 21: "fast", 22: "fx"}
# repeated ids served on the GPU (lib 9 constructs but cannot calculate)
REPEATED_LIBS = {0: "fp64", 1: "fx", 6: "fp64", 7: "fp64", 8: "fx", 20: "fp64", 21: "fast", 22: "fx"}
REPEATED_CONSTRUCT_ONLY = {9}
BACKENDS = ("fp64", "fast", "fx")


# lib 0 (ChinHuhPermanentCalculator) evaluates the Chin-Huh form of the sum
# (CChinHuhPermanentCalculator.cpp:48-201) on the same kernels
REPEATED_FORM = {0: "chinhuh"}


def _check_backend(backend):
    if backend is not None and backend not in BACKENDS:
        raise ValueError(f"unknown backend {backend!r}: expected None, 'fp64', 'fx' or 'fast'")
    return backend


def _coerce_matrix(m):
    if isinstance(m, list):
        return m
    return np.ascontiguousarray(m, dtype=np.complex128) if not (
        isinstance(m, np.ndarray) and m.dtype == np.complex128 and m.flags.c_contiguous) else m


class GlynnPermanentCalculator_wrapper:
    """Plain permanent calculator (the reference's CPython type of that name)."""

    def __init__(self, matrix=None, lib: int = 7, *, backend=None):
        if matrix is None:
            raise TypeError("GlynnPermanentCalculator_wrapper: matrix is required")
        if lib not in PLAIN_LIBS:
            raise Exception(WRONG_LIB)
        self.lib = int(lib)
        self.backend = _check_backend(backend)
        self._matrix = _coerce_matrix(matrix)

    @property
    def matrix(self):
        return self._matrix

    @matrix.setter
    def matrix(self, value):
        self._matrix = _coerce_matrix(value)

    def calculate(self):
        mode = self.backend or PLAIN_LIBS[self.lib]
        if isinstance(self._matrix, list):
            return nat.perm_batched([nat.as_matrix(m) for m in self._matrix], mode=mode)
        if self.lib in (10, 11):
            a = nat.as_matrix(self._matrix)
            if a.shape[0] != a.shape[1] and a.size > 0:
                # GlynnPermanentCalculatorSimple.hpp:67-70: non-square -> 0
                return 0j
        return nat.perm(self._matrix, mode=mode)


class ChinHuhPermanentCalculator_wrapper:
    """Repeated-multiplicity calculator (the reference's CPython type of that
    name, which dispatches on ``lib``)."""

    def __init__(self, lib: int = 7, matrix=None, input_state=None, output_state=None, *, backend=None):
        if matrix is None or input_state is None or output_state is None:
            raise TypeError("ChinHuhPermanentCalculator_wrapper: matrix, input_state and output_state are required")
        if lib not in REPEATED_LIBS and lib not in REPEATED_CONSTRUCT_ONLY:
            raise Exception(WRONG_LIB)
        self.lib = int(lib)
        self.backend = _check_backend(backend)
        self._matrix = _coerce_matrix(matrix)
        self.input_state = input_state
        self.output_state = output_state

    @property
    def matrix(self):
        return self._matrix

    @matrix.setter
    def matrix(self, value):
        self._matrix = _coerce_matrix(value)

    def calculate(self):
        if self.lib not in REPEATED_LIBS:
            raise Exception(WRONG_LIB)
        mode = self.backend or REPEATED_LIBS[self.lib]
        ins, outs = self.input_state, self.output_state
        if isinstance(ins, list) and isinstance(outs, list):
            # ChinHuhPermanentCalculator_Wrapper.hpp:233-323
            multi_input = len(ins) != 0 and isinstance(ins[0], list)
            pairs = []
            shape = []
            for i in range(len(ins)):
                if multi_input:
                    fixed_out = outs[i]
                    row = [(inp, fixed_out) for inp in ins[i]]
                else:
                    fixed_in = ins[i]
                    row = [(fixed_in, out) for out in outs[i]]
                shape.append(len(row))
                pairs.extend(row)
            vals = nat.perm_repeated_many(self._matrix, pairs, mode=mode)
            res, k = [], 0
            for n in shape:
                res.append(vals[k:k + n])
                k += n
            return res
        if isinstance(ins, list) or isinstance(outs, list):
            raise TypeError("input_state and output_state must both be lists, or both arrays")
        return nat.perm_repeated(self._matrix, ins, outs, mode=mode, form=REPEATED_FORM.get(self.lib, "bbfg"))


class RepeatedPermanentCalculator(ChinHuhPermanentCalculator_wrapper):
    """Permanent of the effective scattering matrix of a boson-sampling
    instance (Boson_Sampling_Utilities.py:30-78): states that are neither numpy
    arrays nor lists are converted to int64 arrays; lists must hold arrays."""

    def __init__(self, lib, matrix, input_state, output_state, *, backend=None):
        if not isinstance(input_state, np.ndarray):
            if not isinstance(input_state, list):
                input_state = np.array(input_state, dtype=np.int64)
            else:
                for item in input_state:
                    if not isinstance(item, np.ndarray):
                        raise Exception('The input state should be a numpy array, or a list of numpy arrays')
        if not isinstance(output_state, np.ndarray):
            if not isinstance(output_state, list):
                output_state = np.array(output_state, dtype=np.int64)
            else:
                for item in output_state:
                    if not isinstance(item, np.ndarray):
                        raise Exception('The output state should be a numpy array, or a list of numpy arrays')
        super().__init__(lib=lib, matrix=matrix, input_state=input_state, output_state=output_state,
                         backend=backend)

    def calculate(self):
        return super().calculate()


class ChinHuhPermanentCalculator(RepeatedPermanentCalculator):
    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(0, matrix, input_state, output_state, backend=backend)


class GlynnRepeatedPermanentCalculator(RepeatedPermanentCalculator):
    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(1, matrix, input_state, output_state, backend=backend)


class GlynnRepeatedInfPermanentCalculator(RepeatedPermanentCalculator):
    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(9, matrix, input_state, output_state, backend=backend)


class GlynnRepeatedSingleDFEPermanentCalculator(RepeatedPermanentCalculator):
    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(2, matrix, input_state, output_state, backend=backend)


class GlynnRepeatedDualDFEPermanentCalculator(RepeatedPermanentCalculator):
    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(3, matrix, input_state, output_state, backend=backend)


class GlynnRepeatedMultiSingleDFEPermanentCalculator(RepeatedPermanentCalculator):
    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(4, matrix, input_state, output_state, backend=backend)


class GlynnRepeatedMultiDualDFEPermanentCalculator(RepeatedPermanentCalculator):
    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(5, matrix, input_state, output_state, backend=backend)


class GlynnRepeatedPermanentCalculatorDouble(RepeatedPermanentCalculator):
    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(6, matrix, input_state, output_state, backend=backend)


class BBFGRepeatedPermanentCalculatorDouble(RepeatedPermanentCalculator):
    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(7, matrix, input_state, output_state, backend=backend)


class BBFGRepeatedPermanentCalculatorLongDouble(RepeatedPermanentCalculator):
    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(8, matrix, input_state, output_state, backend=backend)


class GB300RepeatedPermanentCalculator(RepeatedPermanentCalculator):
    """New id 20: GB300 FP64 product (exact integer column sums)."""

    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(20, matrix, input_state, output_state, backend=backend)


class GB300FastRepeatedPermanentCalculator(RepeatedPermanentCalculator):
    """New id 21: GB300 FP32-pipe double-float product."""

    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(21, matrix, input_state, output_state, backend=backend)


class GB300FxRepeatedPermanentCalculator(RepeatedPermanentCalculator):
    """New id 22: GB300 integer-mantissa product (at least FP64 accuracy)."""

    def __init__(self, matrix, input_state, output_state, *, backend=None):
        super().__init__(22, matrix, input_state, output_state, backend=backend)


class GlynnPermanent(GlynnPermanentCalculator_wrapper):
    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 0, backend=backend)


class GlynnPermanentInf(GlynnPermanentCalculator_wrapper):
    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 1, backend=backend)


class GlynnPermanentSingleDFE(GlynnPermanentCalculator_wrapper):
    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 2, backend=backend)


class GlynnPermanentDualDFE(GlynnPermanentCalculator_wrapper):
    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 3, backend=backend)


class GlynnPermanentDouble(GlynnPermanentCalculator_wrapper):
    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 6, backend=backend)


class BBFGPermanentDouble(GlynnPermanentCalculator_wrapper):
    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 7, backend=backend)


class BBFGPermanentLongDouble(GlynnPermanentCalculator_wrapper):
    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 8, backend=backend)


class GlynnPermanentSimpleDouble(GlynnPermanentCalculator_wrapper):
    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 10, backend=backend)


class GlynnPermanentSimpleLongDouble(GlynnPermanentCalculator_wrapper):
    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 11, backend=backend)


class GB300Permanent(GlynnPermanentCalculator_wrapper):
    """New id 20: GB300 FP64 product (exact integer column sums)."""

    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 20, backend=backend)


class GB300FastPermanent(GlynnPermanentCalculator_wrapper):
    """New id 21: GB300 FP32-pipe double-float product."""

    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 21, backend=backend)


class GB300FxPermanent(GlynnPermanentCalculator_wrapper):
    """New id 22: GB300 integer-mantissa product (at least FP64 accuracy)."""

    def __init__(self, matrix, *, backend=None):
        super().__init__(matrix, 22, backend=backend)


__all__: List[str] = [n for n in dir() if n[0].isupper()]
