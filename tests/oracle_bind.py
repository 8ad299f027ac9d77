"""ctypes binding of the CPU oracle (oracle/perm_oracle.c) for the tests.

Test infrastructure only: the oracle gives the expected values, and is never
the thing tested.
Results come back as (value, dd) where dd = [re_hi, im_hi, re_lo, im_lo].
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_P = ctypes.c_void_p
_I = ctypes.c_int64
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(ROOT, "oracle", "_build", "libperm_oracle.so")
        if not os.path.exists(path):
            import sys
            sys.path.insert(0, ROOT)
            from piquassoboost_gb300.build import build_oracle
            build_oracle()
        _lib = ctypes.CDLL(path)
        _lib.orc_last_error.restype = ctypes.c_char_p
    return _lib


def _mat(A):
    a = np.asarray(A)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    return np.ascontiguousarray(a, dtype=np.complex128)


def _ret(rc, out):
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return complex(out[0], out[1]), out.copy()


def bbfg(A, prec=0, threads=0):
    a = _mat(A); out = np.zeros(4)
    rc = lib().orc_bbfg(a.ctypes.data_as(_P), _I(a.shape[0]), _I(a.shape[1]), _I(a.shape[1]),
                        ctypes.c_int(prec), ctypes.c_int(threads), out.ctypes.data_as(_P))
    return _ret(rc, out)


def bbfg_repeated(A, col_mult, row_mult, prec=0, threads=0):
    a = _mat(A); out = np.zeros(4)
    c = np.ascontiguousarray(col_mult, dtype=np.int64)
    r = np.ascontiguousarray(row_mult, dtype=np.int64)
    rc = lib().orc_bbfg_repeated(a.ctypes.data_as(_P), _I(a.shape[0]), _I(a.shape[1]), _I(a.shape[1]),
                                 c.ctypes.data_as(_P), _I(len(c)), r.ctypes.data_as(_P), _I(len(r)),
                                 ctypes.c_int(prec), ctypes.c_int(threads), out.ctypes.data_as(_P))
    return _ret(rc, out)


def glynn_recursive(A, prec=0):
    a = _mat(A); out = np.zeros(4)
    rc = lib().orc_glynn_recursive(a.ctypes.data_as(_P), _I(a.shape[0]), _I(a.shape[1]), _I(a.shape[1]),
                                   ctypes.c_int(prec), out.ctypes.data_as(_P))
    return _ret(rc, out)


def glynn_repeated(A, col_mult, row_mult, prec=0):
    a = _mat(A); out = np.zeros(4)
    c = np.ascontiguousarray(col_mult, dtype=np.int64)
    r = np.ascontiguousarray(row_mult, dtype=np.int64)
    rc = lib().orc_glynn_repeated(a.ctypes.data_as(_P), _I(a.shape[0]), _I(a.shape[1]), _I(a.shape[1]),
                                  c.ctypes.data_as(_P), r.ctypes.data_as(_P), ctypes.c_int(prec),
                                  out.ctypes.data_as(_P))
    return _ret(rc, out)


def chinhuh(A, col_mult, row_mult, prec=0):
    """The Chin-Huh form of the repeated permanent (repeated lib 0)."""
    a = _mat(A); out = np.zeros(4)
    c = np.ascontiguousarray(col_mult, dtype=np.int64)
    r = np.ascontiguousarray(row_mult, dtype=np.int64)
    rc = lib().orc_chinhuh(a.ctypes.data_as(_P), _I(a.shape[0]), _I(a.shape[1]), _I(a.shape[1]),
                           c.ctypes.data_as(_P), r.ctypes.data_as(_P), ctypes.c_int(prec), out.ctypes.data_as(_P))
    return _ret(rc, out)


def glynn_simple(A, prec=0):
    a = _mat(A); out = np.zeros(4)
    rc = lib().orc_glynn_simple(a.ctypes.data_as(_P), _I(a.shape[0]), _I(a.shape[1]), _I(a.shape[1]),
                                ctypes.c_int(prec), out.ctypes.data_as(_P))
    return _ret(rc, out)


def adapt_interferometer(U, input_state, output_state):
    u = _mat(U)
    i = np.ascontiguousarray(input_state, dtype=np.int64)
    o = np.ascontiguousarray(output_state, dtype=np.int64)
    nr = ctypes.c_int64(); nc = ctypes.c_int64()
    lib().orc_adapt_interferometer(u.ctypes.data_as(_P), _I(u.shape[0]), _I(u.shape[1]), i.ctypes.data_as(_P),
                                   o.ctypes.data_as(_P), None, ctypes.byref(nr), ctypes.byref(nc))
    out = np.zeros((nr.value, nc.value), dtype=np.complex128)
    lib().orc_adapt_interferometer(u.ctypes.data_as(_P), _I(u.shape[0]), _I(u.shape[1]), i.ctypes.data_as(_P),
                                   o.ctypes.data_as(_P), out.ctypes.data_as(_P), ctypes.byref(nr), ctypes.byref(nc))
    return out


def adapt_interferometer_multiplied(U, input_state, output_state):
    u = _mat(U)
    i = np.ascontiguousarray(input_state, dtype=np.int64)
    o = np.ascontiguousarray(output_state, dtype=np.int64)
    n = ctypes.c_int64()
    lib().orc_adapt_interferometer_multiplied(u.ctypes.data_as(_P), _I(u.shape[0]), _I(u.shape[1]),
                                              i.ctypes.data_as(_P), o.ctypes.data_as(_P), None, ctypes.byref(n))
    out = np.zeros((n.value, n.value), dtype=np.complex128)
    lib().orc_adapt_interferometer_multiplied(u.ctypes.data_as(_P), _I(u.shape[0]), _I(u.shape[1]),
                                              i.ctypes.data_as(_P), o.ctypes.data_as(_P), out.ctypes.data_as(_P),
                                              ctypes.byref(n))
    return out


def dd_value(dd):
    """Double-double complex as a (re, im) pair of Python floats plus lo parts."""
    return complex(dd[0], dd[1]), complex(dd[2], dd[3])


def rel_err(val, ref_dd):
    """|val - ref| / |ref| evaluated with the oracle's double-double value."""
    hi = complex(ref_dd[0], ref_dd[1]); lo = complex(ref_dd[2], ref_dd[3])
    d = (complex(val) - hi) - lo
    return abs(d) / abs(hi)


def compute_pmf(U, sample, current_input, prec=0, threads=0):
    """(pmf, addends) of the reference's compute_pmf restated in the oracle."""
    u = _mat(U)
    m = u.shape[0]
    s = np.ascontiguousarray(sample, dtype=np.int64)
    c = np.ascontiguousarray(current_input, dtype=np.int64)
    pmf = np.zeros(m)
    add = np.zeros(m, dtype=np.complex128)
    rc = lib().orc_compute_pmf(u.ctypes.data_as(_P), _I(m), _I(m), s.ctypes.data_as(_P), c.ctypes.data_as(_P),
                               ctypes.c_int(prec), ctypes.c_int(threads), pmf.ctypes.data_as(_P),
                               add.ctypes.data_as(_P))
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return pmf, add


def sample_b(U, input_state, nsamples, seed, transmissivity=None, prec=0, threads=1):
    """The oracle's Clifford & Clifford B sampler (orc_sample_b): nsamples
    rows of output occupations; transmissivity None = lossless."""
    u = _mat(U)
    m = u.shape[0]
    inp = np.ascontiguousarray(input_state, dtype=np.int64)
    out = np.zeros((nsamples, m), dtype=np.int64)
    f = lib().orc_sample_b
    f.argtypes = [_P, _I, _I, _P, _I, ctypes.c_uint64, ctypes.c_double, ctypes.c_int, ctypes.c_int, _P]
    rc = f(u.ctypes.data_as(_P), m, m, inp.ctypes.data_as(_P), nsamples, seed,
           -1.0 if transmissivity is None else float(transmissivity), prec, threads, out.ctypes.data_as(_P))
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return out
