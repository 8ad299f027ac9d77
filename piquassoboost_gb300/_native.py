"""ctypes binding of libgbperm.so (the C ABI declared in include/gbperm.h).

The library is loaded from the package's own ``_lib`` folder (built in-tree by
``piquassoboost_gb300.build``).  There is no CPU fallback: if the library is
missing or no CUDA device is visible, every compute call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from .build import LIB_PATH

GBPERM_OK = 0
GBPERM_ERR_ARG = 1
GBPERM_ERR_STATE_SUM = 2
GBPERM_ERR_TOO_LARGE = 3
GBPERM_ERR_CUDA = 4
GBPERM_ERR_LIB = 5
GBPERM_ERR_NO_DEVICE = 6

ARITH_FP64 = 0
ARITH_DF32 = 1
ARITH_FX64 = 2
# "fx": integer-mantissa product (at least FP64 accuracy, integer pipes)
_MODES = {"fp64": ARITH_FP64, "fast": ARITH_DF32, "df32": ARITH_DF32, "fx": ARITH_FX64}


def arith_of(mode) -> int:
    if isinstance(mode, int):
        return mode
    try:
        return _MODES[mode]
    except KeyError:
        raise ValueError(f"unknown arithmetic mode {mode!r}") from None

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32


class Stats(ctypes.Structure):
    """Mirror of gbperm_stats."""

    _fields_ = [
        ("kernel_ms", ctypes.c_double),
        ("steps", ctypes.c_double),
        ("flops", ctypes.c_double),
        ("launches", ctypes.c_int32),
        ("grid", ctypes.c_int32),
        ("seg_log2", ctypes.c_int32),
        ("arith", ctypes.c_int32),
        ("err_est", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class GBPermError(Exception):
    """Raised when a libgbperm call returns a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


# (name, restype, argtypes) of every exported entry point
_SIGNATURES = [
    ("gbperm_version", ctypes.c_int, []),
    ("gbperm_last_error", ctypes.c_char_p, []),
    ("gbperm_device_count", ctypes.c_int, []),
    ("gbperm_set_option", ctypes.c_int, [ctypes.c_char_p, _I64]),
    ("gbperm_get_option", _I64, [ctypes.c_char_p]),
    ("gbperm_perm", ctypes.c_int, [_P, _I64, _I64, _I64, ctypes.c_int, _P, _P, _P]),
    ("gbperm_perm_workspace_size", ctypes.c_size_t, [_I64, _I64]),
    ("gbperm_perm_dev", ctypes.c_int, [_P, _I64, _I64, _I64, ctypes.c_int, _P, _P, _P, ctypes.c_size_t, _P]),
    ("gbperm_probe_peak", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    ("gbperm_batch_plan_create", ctypes.c_int, [_P, _P, _I64, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    ("gbperm_batch_plan_destroy", None, [_P]),
    ("gbperm_batch_plan_run", ctypes.c_int, [_P, _P, _P, _P]),
    ("gbperm_batch_plan_run_dev", ctypes.c_int, [_P, _P, _P, _P]),
    ("gbperm_batch_plan_set_item_log2", ctypes.c_int, [_P, _I64]),
    ("gbperm_batch_plan_get_item_log2", _I64, [_P]),
    ("gbperm_perm_batched", ctypes.c_int, [_P, _P, _P, _I64, ctypes.c_int, _P, _P]),
    ("gbperm_batch_plan_autotune", ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    ("gbperm_batch_plan_get_shape", ctypes.c_int, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    ("gbperm_perm_grad", ctypes.c_int, [_P, _I64, _I64, _P, _P, _P, _P]),
    ("gbperm_perm_grad_workspace_size", ctypes.c_size_t, [_I64]),
    ("gbperm_perm_grad_dev", ctypes.c_int, [_P, _I64, _I64, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    ("gbperm_perm_grad_batched", ctypes.c_int, [_P, _I64, _I64, _P, _P, _P]),
    ("gbperm_perm_grad_batched_workspace_size", ctypes.c_size_t, [_I64, _I64]),
    ("gbperm_perm_grad_batched_dev", ctypes.c_int, [_P, _I64, _I64, _I64, _I64, _P, _P, _P, ctypes.c_size_t, _P]),
    ("gbperm_perm_noalloc", ctypes.c_int, [_P, _I64, _I64, _I64, ctypes.c_int, _P, _P, _P]),
    ("gbperm_perm_noalloc_scratch_bytes", ctypes.c_size_t, []),
    ("gbperm_perm_repeated", ctypes.c_int,
     [_P, _I64, _I64, _I64, _P, _I64, _P, _I64, ctypes.c_int, _P, _P, _P]),
    ("gbperm_perm_chinhuh", ctypes.c_int,
     [_P, _I64, _I64, _I64, _P, _I64, _P, _I64, ctypes.c_int, _P, _P, _P]),
    ("gbperm_compute_pmf", ctypes.c_int, [_P, _I64, _I64, _P, _P, ctypes.c_int, _P, _P, _P]),
    ("gbperm_perm_repeated_batched", ctypes.c_int,
     [_P, _I64, _I64, _I64, _P, _I64, _P, _I64, _I64, ctypes.c_int, _P, _P]),
    ("gbperm_rep_batch_create", ctypes.c_int, [_P, _I64, _I64, _I64, _P, _I64, _P, _I64, _I64, ctypes.c_int,
                                                ctypes.POINTER(ctypes.c_void_p)]),
    ("gbperm_rep_batch_run", ctypes.c_int, [_P, _P, _P]),
    ("gbperm_rep_batch_run_dev", ctypes.c_int, [_P, _P, _P]),
    ("gbperm_rep_batch_info", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I64)]),
    ("gbperm_rep_batch_destroy", None, [_P]),
    ("gbperm_sampler_create", ctypes.c_int, [_P, _I64, _I64, ctypes.c_uint64, ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_void_p)]),
    ("gbperm_sampler_set_matrix", ctypes.c_int, [_P, _P, _I64, _I64]),
    ("gbperm_sampler_seed", ctypes.c_int, [_P, ctypes.c_uint64]),
    ("gbperm_sampler_set_uniform_losses", ctypes.c_int, [_P, ctypes.c_double]),
    ("gbperm_sampler_simulate", ctypes.c_int, [_P, _P, _I64, _I64, _P, _P]),
    ("gbperm_sampler_destroy", None, [_P]),
    ("gbperm_mesh_workspace_size", ctypes.c_size_t, [_I64]),
    ("gbperm_mesh_unitary_dev", ctypes.c_int, [_P, _I64, _P, _P, ctypes.c_size_t, _P]),
    ("gbperm_mesh_unitary_backward_dev", ctypes.c_int, [_P, _I64, _P, _P, _P, ctypes.c_size_t, _P]),
]

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    """libgbperm.so in the package, or the file named by GBPERM_LIB (a
    differently configured build of the same sources)."""
    return os.environ.get("GBPERM_LIB", LIB_PATH)


def load(build_if_missing: bool = False):
    """Load libgbperm.so once; raise RuntimeError if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            if build_if_missing and path == LIB_PATH:
                from .build import build_native

                build_native()
            else:
                raise RuntimeError(
                    f"libgbperm.so not found at {path}; build it with "
                    "`python -m piquassoboost_gb300.build` (the GPU path has no CPU fallback)")
        lib = ctypes.CDLL(path)
        for name, res, args in _SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def exported_symbols() -> list[str]:
    return [name for name, _, _ in _SIGNATURES]


def check(rc: int) -> None:
    if rc != GBPERM_OK:
        msg = load().gbperm_last_error().decode("utf-8", "replace")
        raise GBPermError(rc, msg)


def require_device() -> None:
    if load().gbperm_device_count() <= 0:
        raise GBPermError(GBPERM_ERR_NO_DEVICE,
                          "no CUDA device visible: the GB300 permanent library needs a GPU")


def set_option(key: str, value: int) -> None:
    check(load().gbperm_set_option(key.encode(), int(value)))


def get_option(key: str) -> int:
    return int(load().gbperm_get_option(key.encode()))


def as_matrix(matrix) -> np.ndarray:
    """complex128, C-contiguous, 2-D (a 1-D array of length n is n x 1, as the
    reference's numpy2matrix does, common/numpy_interface.cpp:145-151)."""
    a = np.asarray(matrix)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    if a.ndim != 2:
        raise ValueError("numpy2matrix: Wrong matrix dimension was given")
    return np.ascontiguousarray(a, dtype=np.complex128)


def perm(matrix, mode="fp64", return_dd: bool = False, stats: Stats | None = None):
    """Plain permanent on the GPU through gbperm_perm (host buffers)."""
    lib = load()
    a = as_matrix(matrix)
    rows, cols = a.shape
    out = np.zeros(2)
    dd = np.zeros(4)
    rc = lib.gbperm_perm(a.ctypes.data_as(_P), rows, cols, cols, arith_of(mode), out.ctypes.data_as(_P),
                         dd.ctypes.data_as(_P),
                         ctypes.byref(stats) if stats is not None else None)
    check(rc)
    if return_dd:
        return complex(out[0], out[1]), dd
    return complex(out[0], out[1])


def as_state(state) -> np.ndarray:
    s = np.asarray(state)
    if s.ndim != 1:
        s = s.reshape(-1)
    return np.ascontiguousarray(s, dtype=np.int64)


def perm_repeated(matrix, input_state, output_state, mode="fp64", return_dd: bool = False,
                  stats: Stats | None = None, form: str = "bbfg"):
    """Repeated-multiplicity permanent on the GPU (gbperm_perm_repeated, or
    gbperm_perm_chinhuh with form="chinhuh").

    input_state gives the column multiplicities, output_state the row
    multiplicities (the reference's convention)."""
    lib = load()
    fn = {"bbfg": lib.gbperm_perm_repeated, "chinhuh": lib.gbperm_perm_chinhuh}[form]
    a = as_matrix(matrix)
    cm = as_state(input_state)
    rm = as_state(output_state)
    rows, cols = a.shape
    out = np.zeros(2)
    dd = np.zeros(4)
    rc = fn(a.ctypes.data_as(_P), rows, cols, cols, cm.ctypes.data_as(_P), len(cm), rm.ctypes.data_as(_P), len(rm),
            arith_of(mode), out.ctypes.data_as(_P), dd.ctypes.data_as(_P),
            ctypes.byref(stats) if stats is not None else None)
    check(rc)
    if return_dd:
        return complex(out[0], out[1]), dd
    return complex(out[0], out[1])


def perm_repeated_many(matrix, pairs, mode="fp64", stats: Stats | None = None):
    """Repeated permanents of one matrix for a list of (input, output) state
    pairs, in order, through one batched call (gbperm_perm_repeated_batched).
    States shorter than the longest are zero-padded."""
    lib = load()
    a = as_matrix(matrix)
    rows, cols = a.shape
    if len(pairs) == 0:
        return []
    ins = [as_state(i) for i, _ in pairs]
    outs = [as_state(o) for _, o in pairs]
    ncol = max(len(x) for x in ins)
    nrow = max(len(x) for x in outs)
    cm = np.zeros((len(pairs), ncol), dtype=np.int64)
    rm = np.zeros((len(pairs), nrow), dtype=np.int64)
    for k, (x, y) in enumerate(zip(ins, outs)):
        cm[k, :len(x)] = x
        rm[k, :len(y)] = y
    out = np.zeros(2 * len(pairs))
    check(lib.gbperm_perm_repeated_batched(a.ctypes.data_as(_P), rows, cols, cols, cm.ctypes.data_as(_P), ncol,
                                           rm.ctypes.data_as(_P), nrow, len(pairs), arith_of(mode),
                                           out.ctypes.data_as(_P),
                                           ctypes.byref(stats) if stats is not None else None))
    return [complex(out[2 * k], out[2 * k + 1]) for k in range(len(pairs))]


class BatchPlan:
    """A reusable batched plan (gbperm_batch_plan_*): fixed shapes, a CUDA
    graph captured at creation, one persistent launch per run."""

    def __init__(self, shapes, mode="fp64"):
        lib = load()
        self.shapes = [(int(r), int(c)) for r, c in shapes]
        self.rows = np.ascontiguousarray([r for r, _ in self.shapes], dtype=np.int64)
        self.cols = np.ascontiguousarray([c for _, c in self.shapes], dtype=np.int64)
        self.count = len(self.shapes)
        self.total = int(np.sum(self.rows * self.cols))
        self._h = ctypes.c_void_p()
        if any(r > 0 and c > 0 and r < c + 2 for r, c in self.shapes):
            require_device()
        check(lib.gbperm_batch_plan_create(self.rows.ctypes.data_as(_P), self.cols.ctypes.data_as(_P),
                                           self.count, arith_of(mode), ctypes.byref(self._h)))

    def pack(self, matrices) -> np.ndarray:
        buf = np.empty(max(self.total, 1), dtype=np.complex128)
        k = 0
        for m, (r, c) in zip(matrices, self.shapes):
            buf[k:k + r * c] = np.asarray(m, dtype=np.complex128).reshape(-1)
            k += r * c
        return buf

    def run(self, matrices=None, packed=None, stats: Stats | None = None):
        if packed is None:
            packed = self.pack(matrices)
        out = np.zeros(2 * max(self.count, 1))
        check(load().gbperm_batch_plan_run(self._h, packed.ctypes.data_as(_P), out.ctypes.data_as(_P),
                                           ctypes.byref(stats) if stats is not None else None))
        return [complex(out[2 * i], out[2 * i + 1]) for i in range(self.count)]

    def set_item_log2(self, v: int) -> None:
        check(load().gbperm_batch_plan_set_item_log2(self._h, int(v)))

    def item_log2(self) -> int:
        return int(load().gbperm_batch_plan_get_item_log2(self._h))

    def shape(self) -> tuple[int, int]:
        """(lanes per Gray segment, columns per lane) of the plan's kernel."""
        g, c = ctypes.c_int64(), ctypes.c_int64()
        check(load().gbperm_batch_plan_get_shape(self._h, ctypes.byref(g), ctypes.byref(c)))
        return int(g.value), int(c.value)

    def autotune(self, matrices=None, packed=None, reps: int = 1) -> float:
        """Time the candidate shapes on this batch and keep the fastest;
        returns its time per batch in ms (gbperm_batch_plan_autotune)."""
        if packed is None:
            packed = self.pack(matrices)
        ms = ctypes.c_double()
        check(load().gbperm_batch_plan_autotune(self._h, packed.ctypes.data_as(_P), int(reps), ctypes.byref(ms)))
        return ms.value

    def close(self):
        if self._h:
            load().gbperm_batch_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def perm_batched(matrices, mode="fp64", stats: Stats | None = None):
    """Plain permanents of a list of matrices in one persistent launch."""
    mats = [as_matrix(m) for m in matrices]
    if not mats:
        return []
    plan = BatchPlan([m.shape for m in mats], mode=mode)
    try:
        return plan.run(mats, stats=stats)
    finally:
        plan.close()


def compute_pmf(interferometer, sample, current_input, mode="fp64", stats: Stats | None = None):
    """One probability layer of the Clifford & Clifford sampler on the GPU
    (gbperm_compute_pmf): returns (pmf, addends), pmf normalised to sum 1 over
    the m output modes and addends[l] the permanent with one photon removed
    from input mode l (0 where the input mode is empty).  mode "fx" runs the
    integer-mantissa product, "fast" the double-float one (FP64 beyond the
    df.pmf_max_photons rule)."""
    lib = load()
    u = as_matrix(interferometer)
    m = u.shape[0]
    if u.shape[1] != m:
        raise ValueError("compute_pmf: square interferometer required")
    s = as_state(sample)
    c = as_state(current_input)
    if len(s) != m or len(c) != m:
        raise ValueError("compute_pmf: states must have one entry per mode")
    pmf = np.zeros(m)
    add = np.zeros(m, dtype=np.complex128)
    check(lib.gbperm_compute_pmf(u.ctypes.data_as(_P), m, m, s.ctypes.data_as(_P), c.ctypes.data_as(_P),
                                 arith_of(mode), pmf.ctypes.data_as(_P), add.ctypes.data_as(_P),
                                 ctypes.byref(stats) if stats is not None else None))
    return pmf, add


class RepBatchPlan:
    """A reusable persistent-launch plan for many repeated permanents of one
    interferometer (gbperm_rep_batch_*): pairs of (input_state,
    output_state) over the matrix's columns and rows, integer-mantissa
    product."""

    def __init__(self, matrix, pairs):
        lib = load()
        a = as_matrix(matrix)
        rows, cols = a.shape
        ins = [as_state(i) for i, _ in pairs]
        outs = [as_state(o) for _, o in pairs]
        ncol = max([len(x) for x in ins] + [0])
        nrow = max([len(x) for x in outs] + [0])
        cm = np.zeros((len(pairs), ncol), dtype=np.int64)
        rm = np.zeros((len(pairs), nrow), dtype=np.int64)
        for k, (i, o) in enumerate(zip(ins, outs)):
            cm[k, :len(i)] = i
            rm[k, :len(o)] = o
        self.count = len(pairs)
        self._a = a
        self._h = ctypes.c_void_p()
        check(lib.gbperm_rep_batch_create(a.ctypes.data_as(_P), rows, cols, cols, cm.ctypes.data_as(_P), ncol,
                                          rm.ctypes.data_as(_P), nrow, self.count, ARITH_FX64, ctypes.byref(self._h)))

    def run(self, stats: Stats | None = None) -> np.ndarray:
        out = np.zeros(2 * max(self.count, 1))
        check(load().gbperm_rep_batch_run(self._h, out.ctypes.data_as(_P),
                                          ctypes.byref(stats) if stats is not None else None))
        return out[0:2 * self.count:2] + 1j * out[1:2 * self.count:2]

    def run_dev(self, d_out_ptr: int, stream_ptr: int | None = None):
        check(load().gbperm_rep_batch_run_dev(self._h, _P(d_out_ptr), _P(stream_ptr or 0)))

    def info(self):
        steps, flops, mul_ops, items = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), _I64()
        check(load().gbperm_rep_batch_info(self._h, ctypes.byref(steps), ctypes.byref(flops), ctypes.byref(mul_ops),
                                           ctypes.byref(items)))
        return {"steps": steps.value, "flops": flops.value, "mul_ops": mul_ops.value, "items": items.value}

    def close(self):
        if self._h:
            load().gbperm_rep_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Sampler:
    """Handle of a native boson sampler (gbperm_sampler_*): the generalised
    Clifford & Clifford B form over GPU pmf layers, with the reference's
    std::mt19937 random stream.  transmissivity=None: lossless; a value in
    [0, 1]: uniform losses (each sample first draws its surviving photon
    count)."""

    def __init__(self, interferometer, seed: int, mode="fp64", transmissivity=None):
        lib = load()
        U = np.ascontiguousarray(interferometer, dtype=np.complex128)
        if U.ndim != 2 or U.shape[0] != U.shape[1]:
            raise ValueError("the interferometer must be a square matrix")
        self._h = ctypes.c_void_p()
        check(lib.gbperm_sampler_create(U.ctypes.data_as(_P), U.shape[0], U.shape[0], int(seed) & (2 ** 64 - 1),
                                        arith_of(mode), ctypes.byref(self._h)))
        self.modes = U.shape[0]
        if transmissivity is not None:
            check(lib.gbperm_sampler_set_uniform_losses(self._h, float(transmissivity)))

    def set_matrix(self, interferometer):
        U = np.ascontiguousarray(interferometer, dtype=np.complex128)
        if U.ndim != 2 or U.shape[0] != U.shape[1]:
            raise ValueError("the interferometer must be a square matrix")
        check(load().gbperm_sampler_set_matrix(self._h, U.ctypes.data_as(_P), U.shape[0], U.shape[0]))
        self.modes = U.shape[0]

    def seed(self, value: int):
        check(load().gbperm_sampler_seed(self._h, int(value) & (2 ** 64 - 1)))

    def simulate(self, input_state, samples_number: int, stats: Stats | None = None) -> np.ndarray:
        inp = np.ascontiguousarray(np.asarray(input_state).reshape(-1), dtype=np.int64)
        out = np.zeros((max(int(samples_number), 0), inp.shape[0]), dtype=np.int64)
        check(load().gbperm_sampler_simulate(self._h, inp.ctypes.data_as(_P), inp.shape[0], int(samples_number),
                                             out.ctypes.data_as(_P), ctypes.byref(stats) if stats is not None else None))
        return out

    def close(self):
        if self._h:
            load().gbperm_sampler_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_PROBES = {"fp64": 0, "fp32": 1, "dmma": 2, "imad_wide": 3, "imad": 4, "shf": 5, "add64": 6, "bfind": 7,
           "iadd": 8}


def probe_peak(kind: str) -> float:
    """Measured pipe peak: "fp64" / "fp32" FMA and "dmma" (FP64 tensor MMA)
    in TFLOP/s; "imad_wide" (mad.wide.s32), "imad" (mad.lo.s32), "shf"
    (shf.l.wrap.b32), "add64" (add.s64), "bfind" (bfind.s32) and "iadd"
    (add.s32) in tera lane-operations/s."""
    v = ctypes.c_double()
    check(load().gbperm_probe_peak(_PROBES[kind], ctypes.byref(v)))
    return v.value


_grad_lock = threading.Lock()


class grad_arithmetic:
    """Context manager selecting the gradient sweep's product (the library's
    process-wide option "grad.arith"): "fast" (double-float, recomputed with
    the integer-mantissa product on the device when its range check fails or
    its error estimate is above 1e-10; the default) or "fx" (integer-mantissa
    product throughout).  Python threads that switch it are serialised."""

    def __init__(self, mode):
        self.arith = arith_of(mode)
        if self.arith not in (ARITH_DF32, ARITH_FX64):
            raise ValueError("the gradient runs the 'fast' or the 'fx' product")

    def __enter__(self):
        _grad_lock.acquire()
        self.prev = get_option("grad.arith")
        set_option("grad.arith", self.arith)
        return self

    def __exit__(self, *exc):
        set_option("grad.arith", self.prev)
        _grad_lock.release()
        return False


def perm_grad(matrix, stats: Stats | None = None, mode: str | None = None):
    """Permanent and full gradient G[k, l] = dperm/da_kl (host buffers).
    mode None keeps the current gradient arithmetic (see grad_arithmetic)."""
    lib = load()
    a = as_matrix(matrix)
    n = a.shape[0]
    if a.shape[0] != a.shape[1]:
        raise ValueError("perm_grad: square matrix required")
    require_device()
    perm = np.zeros(2)
    g = np.zeros((n, n), dtype=np.complex128)

    def call():
        check(lib.gbperm_perm_grad(a.ctypes.data_as(_P), n, n, perm.ctypes.data_as(_P), None,
                                   g.ctypes.data_as(_P), ctypes.byref(stats) if stats is not None else None))

    if mode is None:
        call()
    else:
        with grad_arithmetic(mode):
            call()
    return complex(perm[0], perm[1]), g


def perm_grad_batched(matrices, stats: Stats | None = None, mode: str | None = None):
    """Permanents and full gradients of a batch of equal-size square matrices
    (host buffers, one set of launches): returns (perms[count], grads[count, n, n])."""
    lib = load()
    a = np.ascontiguousarray(np.asarray(matrices), dtype=np.complex128)
    if a.ndim != 3 or a.shape[1] != a.shape[2]:
        raise ValueError("perm_grad_batched: a count x n x n stack of square matrices is required")
    count, n = a.shape[0], a.shape[1]
    perms = np.zeros(count, dtype=np.complex128)
    grads = np.zeros((count, n, n), dtype=np.complex128)

    def call():
        check(lib.gbperm_perm_grad_batched(a.ctypes.data_as(_P), n, count, perms.ctypes.data_as(_P),
                                           grads.ctypes.data_as(_P),
                                           ctypes.byref(stats) if stats is not None else None))

    if mode is None:
        call()
    else:
        with grad_arithmetic(mode):
            call()
    return perms, grads
