"""piquasso connector hook (the reference's connector.py:23-39).

``cpp_permanent_function(matrix, input, output)`` is the permanent callback
piquasso calls; it runs the repeated BBFG permanent on the GB300.
``BoostConnector`` is defined only when piquasso is importable.
"""
from __future__ import annotations

from .sampling.Boson_Sampling_Utilities import BBFGRepeatedPermanentCalculatorDouble


def cpp_permanent_function(matrix, input, output):
    result = BBFGRepeatedPermanentCalculatorDouble(matrix, input, output).calculate()
    if isinstance(result, list):
        # the reference returns 1.0 when empty lists are passed
        result = 1.0
    return result


try:  # pragma: no cover - piquasso is optional
    from piquasso._simulators.connectors import NumpyConnector

    class BoostConnector(NumpyConnector):
        def __init__(self) -> None:
            super().__init__()
            self.permanent = cpp_permanent_function
            self.number_of_approximated_modes = None
except Exception:  # piquasso not installed
    BoostConnector = None
