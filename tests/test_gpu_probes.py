"""The pipe probes behind the bench's roofline denominators: every kind runs
and returns a positive rate, ordered as the GB300 pipes are (the 32-bit add
at least as fast as the variable shift, the shift at least as fast as the
64-bit add and the leading-bit search)."""
import math

import pytest

from piquassoboost_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def test_every_probe_kind_runs():
    rates = {k: nat.probe_peak(k) for k in nat._PROBES}
    for k, v in rates.items():
        assert math.isfinite(v) and v > 0.0, (k, v)
    assert rates["iadd"] >= 0.9 * rates["shf"]
    assert rates["shf"] >= 0.9 * rates["add64"]
    assert rates["shf"] >= 0.9 * rates["bfind"]
    assert rates["fp32"] > rates["fp64"]
