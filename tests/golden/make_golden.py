"""Generate the golden fixtures in this folder from the reference.

Run in the development container (where the reference tree and its C++ build,
oracle/_ref/libpqbref.so from oracle/build_ref.sh, exist):

    python tests/golden/make_golden.py [--reference-root /root/reference]

It writes
  reference_unittests.json   the known answers of the reference's
                             unittests/test_permanent.py, read from that file
                             with a small literal-only AST evaluator (the file
                             is parsed, never executed);
  reference_calculators.json outputs of the reference's own C++ calculators
                             (plain lib 0/6/7/8/10/11, repeated lib 0/1/6/7/8,
                             adaptInterferometer) on seeded inputs;
  reference_sampler.json     the seeded boson samples of the reference's
                             unittests/test_seeding.py (the lossless and the
                             uniform-losses cases; literals read with the AST
                             as above), and sample sequences of the
                             reference's own C++ samplers
                             (CGeneralizedCliffordsB[UniformLosses]
                             SimulationStrategy) on seeded inputs.
The fixtures are committed; tests read them without the reference.
"""
from __future__ import annotations

import argparse
import ast
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from piquassoboost_gb300.workloads import haar_unitary  # noqa: E402

_P = ctypes.c_void_p
_I = ctypes.c_int64


# ---------------------------------------------------------------- AST side
class _Eval(ast.NodeVisitor):
    """Evaluates numpy-literal expressions: numbers, lists, +-*/, np.array,
    np.ones, np.zeros, np.sqrt, and names bound earlier in the function."""

    def __init__(self, env):
        self.env = env

    def ev(self, node):
        if isinstance(node, ast.Constant):
            if isinstance(node.value, (int, float, complex)):
                return node.value
            raise ValueError("unsupported constant")
        if isinstance(node, (ast.List, ast.Tuple)):
            return [self.ev(e) for e in node.elts]
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub):
            return -self.ev(node.operand)
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.UAdd):
            return self.ev(node.operand)
        if isinstance(node, ast.BinOp):
            a, b = self.ev(node.left), self.ev(node.right)
            a = np.asarray(a) if isinstance(a, list) else a
            b = np.asarray(b) if isinstance(b, list) else b
            ops = {ast.Add: np.add, ast.Sub: np.subtract, ast.Mult: np.multiply, ast.Div: np.divide}
            return ops[type(node.op)](a, b)
        if isinstance(node, ast.Name):
            return self.env[node.id]
        if isinstance(node, ast.Call) and isinstance(node.func, ast.Attribute):
            fn = node.func.attr
            args = [self.ev(a) for a in node.args]
            kw = {k.arg: k.value for k in node.keywords}
            dtype = None
            if "dtype" in kw and isinstance(kw["dtype"], ast.Attribute):
                dtype = {"int64": np.int64, "complex128": np.complex128, "float64": np.float64}[kw["dtype"].attr]
            if fn == "array":
                return np.array(args[0], dtype=dtype)
            if fn == "asarray":
                return np.asarray(args[0], dtype=dtype)
            if fn == "ones":
                return np.ones(args[0], dtype=dtype)
            if fn == "zeros":
                return np.zeros(args[0], dtype=dtype)
            if fn == "sqrt":
                return np.sqrt(args[0])
        raise ValueError(f"unsupported expression {ast.dump(node)[:80]}")


def extract_unittests(path):
    tree = ast.parse(open(path).read())
    cases = []
    for fn in tree.body:
        if not (isinstance(fn, ast.FunctionDef) and fn.name.startswith("test_")):
            continue
        env = {}
        ev = _Eval(env)
        for st in fn.body:
            if isinstance(st, ast.Assign):
                val = ev.ev(st.value)
                for t in st.targets:
                    if isinstance(t, ast.Name):
                        env[t.id] = val
                    elif isinstance(t, ast.Tuple):  # no tuple unpacking in literals
                        pass
                # chained assignment `input = output = ...`
            elif isinstance(st, ast.Assert):
                call = st.test
                # assert np.isclose(_perm(M, cols, rows), expected)
                if isinstance(call, ast.Call) and getattr(call.func, "attr", "") == "isclose":
                    inner, expected = call.args
                    m, cols, rows = (ev.ev(a) for a in inner.args)
                    cases.append({
                        "name": fn.name,
                        "matrix": _cplx_list(np.asarray(m, dtype=np.complex128)),
                        "shape": list(np.asarray(m).shape),
                        "input_state": [int(x) for x in np.asarray(cols).ravel()],
                        "output_state": [int(x) for x in np.asarray(rows).ravel()],
                        "expected": _cplx(complex(ev.ev(expected))),
                        "source": f"unittests/test_permanent.py:{fn.lineno}",
                    })
    return cases


def _cplx(z):
    return [float(np.real(z)), float(np.imag(z))]


def _cplx_list(a):
    a = np.asarray(a, dtype=np.complex128)
    return [[float(v.real), float(v.imag)] for v in a.ravel()]


# ----------------------------------------------------------- reference side
class Ref:
    def __init__(self, path):
        self.lib = ctypes.CDLL(path)
        self.lib.ref_last_error.restype = ctypes.c_char_p

    def perm(self, lib_id, A):
        A = np.ascontiguousarray(A, dtype=np.complex128)
        out = np.zeros(2)
        rc = self.lib.ref_perm(lib_id, A.ctypes.data_as(_P), _I(A.shape[0]), _I(A.shape[1]), out.ctypes.data_as(_P))
        if rc:
            raise RuntimeError(self.lib.ref_last_error())
        return complex(out[0], out[1])

    def perm_rep(self, lib_id, A, cin, rout):
        A = np.ascontiguousarray(A, dtype=np.complex128)
        cin = np.ascontiguousarray(cin, dtype=np.int64)
        rout = np.ascontiguousarray(rout, dtype=np.int64)
        out = np.zeros(2)
        rc = self.lib.ref_perm_repeated(lib_id, A.ctypes.data_as(_P), _I(A.shape[0]), _I(A.shape[1]),
                                        cin.ctypes.data_as(_P), _I(len(cin)), rout.ctypes.data_as(_P),
                                        _I(len(rout)), out.ctypes.data_as(_P))
        if rc:
            raise RuntimeError(self.lib.ref_last_error())
        return complex(out[0], out[1])

    def compute_pmf(self, U, sample, current_input):
        U = np.ascontiguousarray(U, dtype=np.complex128)
        s = np.ascontiguousarray(sample, dtype=np.int64)
        c = np.ascontiguousarray(current_input, dtype=np.int64)
        out = np.zeros(U.shape[0])
        rc = self.lib.ref_compute_pmf(U.ctypes.data_as(_P), _I(U.shape[0]), s.ctypes.data_as(_P),
                                      c.ctypes.data_as(_P), out.ctypes.data_as(_P))
        if rc:
            raise RuntimeError(self.lib.ref_last_error())
        return out

    def adapt(self, U, cin, rout):
        U = np.ascontiguousarray(U, dtype=np.complex128)
        cin = np.ascontiguousarray(cin, dtype=np.int64)
        rout = np.ascontiguousarray(rout, dtype=np.int64)
        r, c = ctypes.c_int64(), ctypes.c_int64()
        self.lib.ref_adapt_interferometer(U.ctypes.data_as(_P), _I(U.shape[0]), cin.ctypes.data_as(_P),
                                          rout.ctypes.data_as(_P), None, ctypes.byref(r), ctypes.byref(c))
        out = np.zeros((r.value, c.value), dtype=np.complex128)
        self.lib.ref_adapt_interferometer(U.ctypes.data_as(_P), _I(U.shape[0]), cin.ctypes.data_as(_P),
                                          rout.ctypes.data_as(_P), out.ctypes.data_as(_P), ctypes.byref(r),
                                          ctypes.byref(c))
        return out


def reference_calculators(ref):
    cases = {"plain": [], "repeated": [], "adapt": [], "pmf": []}
    rng = np.random.default_rng(20240611)
    # plain: Gaussian and Haar blocks, square and rectangular
    shapes = [(n, n) for n in range(1, 15)] + [(2, 3), (3, 5), (4, 3), (5, 3), (1, 4), (3, 1), (2, 1),
                                                (6, 9), (10, 9), (7, 7)]
    for i, (r, c) in enumerate(shapes):
        if i % 2 == 0:
            A = rng.standard_normal((r, c)) + 1j * rng.standard_normal((r, c))
        else:
            A = haar_unitary(max(2 * r, 2 * c, 2), 1000 + i)[:r, :c]
        libs = [0, 6, 7, 8] + ([10, 11] if r == c and r <= 12 else [])
        cases["plain"].append({
            "shape": [r, c], "matrix": _cplx_list(A),
            "values": {str(l): _cplx(ref.perm(l, A)) for l in libs},
        })
    for n in (16, 18, 20):
        A = haar_unitary(2 * n, 2000 + n)[:n, :n]
        cases["plain"].append({"shape": [n, n], "matrix": _cplx_list(A),
                               "values": {str(l): _cplx(ref.perm(l, A)) for l in (7, 8)}})
    # repeated: random multiplicities on Gaussian / Haar matrices
    for t in range(40):
        m = int(rng.integers(2, 9))
        if t % 2:
            A = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
        else:
            A = haar_unitary(m, 3000 + t)
        k = int(rng.integers(1, 10))
        cin = rng.multinomial(k, np.ones(m) / m).astype(np.int64)
        rout = rng.multinomial(k, np.ones(m) / m).astype(np.int64)
        vals = {str(l): _cplx(ref.perm_rep(l, A, cin, rout)) for l in (0, 1, 6, 7, 8)}
        cases["repeated"].append({"shape": [m, m], "matrix": _cplx_list(A), "input_state": cin.tolist(),
                                  "output_state": rout.tolist(), "values": vals})
    # repeated with a boson-sampling shape (30 modes, 12 photons)
    U = haar_unitary(30, 4242)
    cin = np.zeros(30, dtype=np.int64); cin[:12] = 1
    rout = rng.multinomial(12, np.ones(30) / 30).astype(np.int64)
    cases["repeated"].append({"shape": [30, 30], "matrix": _cplx_list(U), "input_state": cin.tolist(),
                              "output_state": rout.tolist(),
                              "values": {str(l): _cplx(ref.perm_rep(l, U, cin, rout)) for l in (7, 8)}})
    # adaptInterferometer
    for t in range(5):
        m = 6 + t
        U = haar_unitary(m, 5000 + t)
        cin = rng.multinomial(m // 2, np.ones(m) / m).astype(np.int64)
        rout = rng.multinomial(m // 2, np.ones(m) / m).astype(np.int64)
        sub = ref.adapt(U, cin, rout)
        cases["adapt"].append({"m": m, "matrix": _cplx_list(U), "input_state": cin.tolist(),
                               "output_state": rout.tolist(), "shape": list(sub.shape),
                               "result": _cplx_list(sub)})
    # compute_pmf: a Clifford-Clifford layer (k input photons, k-1 sampled)
    for t in range(12):
        m = int(rng.integers(4, 16))
        U = haar_unitary(m, 6000 + t)
        k = int(rng.integers(1, 9))
        inp = rng.multinomial(k, np.ones(m) / m).astype(np.int64)
        smp = rng.multinomial(k - 1, np.ones(m) / m).astype(np.int64)
        cases["pmf"].append({"m": m, "matrix": _cplx_list(U), "sample": smp.tolist(), "current_input": inp.tolist(),
                             "pmf": [float(x) for x in ref.compute_pmf(U, smp, inp)]})
    return cases


# ------------------------------------------------------------ sampler side
def _literal(node):
    """Python literals, unary minus and complex sums like -0.1 - 0.2j."""
    if isinstance(node, ast.Constant):
        return node.value
    if isinstance(node, (ast.List, ast.Tuple)):
        return [_literal(e) for e in node.elts]
    if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.USub, ast.UAdd)):
        v = _literal(node.operand)
        return -v if isinstance(node.op, ast.USub) else v
    if isinstance(node, ast.BinOp) and isinstance(node.op, (ast.Add, ast.Sub)):
        a, b = _literal(node.left), _literal(node.right)
        return a + b if isinstance(node.op, ast.Add) else a - b
    if isinstance(node, ast.BinOp) and isinstance(node.op, ast.Mult):
        a, b = _literal(node.left), _literal(node.right)
        return a * b  # list repetition, as Python evaluates it
    raise ValueError(f"not a literal: {ast.dump(node)[:80]}")


def extract_seeding(path):
    """The lossless and uniform-losses boson-sampling cases of
    unittests/test_seeding.py: interferometer, input occupation, seed,
    shots, singular values and the expected samples (a multiset: piquasso
    lists the samples grouped from its outcome counts, not in drawing
    order)."""
    tree = ast.parse(open(path).read())
    U = None
    for st in tree.body:
        if isinstance(st, ast.Assign) and st.targets[0].id == "_U":
            U = np.array(_literal(st.value.args[0]), dtype=np.complex128)
    cases = []
    for fn in tree.body:
        if not isinstance(fn, ast.FunctionDef) or fn.name not in (
                "test_boson_sampling_seeded", "test_LossyInterferometer_boson_sampling_uniform_losses"):
            continue
        vals = {}
        for node in ast.walk(fn):
            if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name):
                name = node.targets[0].id
                if name in ("seed_sequence", "expected_samples"):
                    vals[name] = _literal(node.value)
                if name == "singular_values":
                    vals[name] = _literal(node.value.args[0])
            if isinstance(node, ast.Call) and getattr(node.func, "attr", "") == "StateVector":
                vals["input_state"] = _literal(node.args[0])
            if isinstance(node, ast.Call) and getattr(node.func, "attr", "") == "execute":
                for kw in node.keywords:
                    if kw.arg == "shots":
                        vals["shots"] = _literal(kw.value)
        case = {"name": fn.name, "source": f"unittests/test_seeding.py:{fn.lineno}", "seed": vals["seed_sequence"],
                "input_state": vals["input_state"], "shots": vals["shots"],
                "expected_multiset": sorted(list(map(list, vals["expected_samples"])))}
        if "singular_values" in vals:
            # the test's lossy matrix _U diag(s) _U _U^T; its singular values are
            # uniform, so the reference's boosted path divides it by the first
            # one and runs the uniform-losses strategy with that transmissivity
            M = U @ np.diag(np.array(vals["singular_values"])) @ U @ U.T
            sv = np.linalg.svd(M)[1]
            case["transmissivity"] = float(sv[0])
            case["interferometer"] = _cplx_list(M / sv[0])
        else:
            case["interferometer"] = _cplx_list(U)
        case["modes"] = len(vals["input_state"])
        cases.append(case)
    return cases


def reference_sampler(ref_so, seeding_cases):
    lib = ctypes.CDLL(ref_so)
    lib.ref_sample_b.argtypes = [_P, _I, _P, _I, ctypes.c_uint64, _P]
    lib.ref_sample_b_uniform_losses.argtypes = [_P, _I, ctypes.c_double, _P, _I, ctypes.c_uint64, _P]

    def run(U, inp, seed, n, t=None):
        U = np.ascontiguousarray(U, dtype=np.complex128)
        m = U.shape[0]
        inp = np.ascontiguousarray(inp, dtype=np.int64)
        out = np.zeros((n, m), dtype=np.int64)
        if t is None:
            rc = lib.ref_sample_b(U.ctypes.data_as(_P), m, inp.ctypes.data_as(_P), n, seed, out.ctypes.data_as(_P))
        else:
            rc = lib.ref_sample_b_uniform_losses(U.ctypes.data_as(_P), m, t, inp.ctypes.data_as(_P), n, seed,
                                                 out.ctypes.data_as(_P))
        if rc != 0:
            raise RuntimeError("reference sampler failed")
        return out.tolist()

    seqs = []
    for c in seeding_cases:
        U = np.array([complex(a, b) for a, b in c["interferometer"]]).reshape(c["modes"], c["modes"])
        got = run(U, c["input_state"], c["seed"], c["shots"], c.get("transmissivity"))
        if sorted(got) != c["expected_multiset"]:
            raise RuntimeError(f"the reference build does not reproduce {c['name']}")
        seqs.append({"name": c["name"], "interferometer": c["interferometer"], "modes": c["modes"],
                     "input_state": c["input_state"], "seed": c["seed"], "transmissivity": c.get("transmissivity"),
                     "samples": got})
    # seeded Haar interferometers: (modes, unitary seed, input occupation,
    # sampler seed, samples, transmissivity or None)
    plan = [
        (8, 3, [1, 1, 1, 1, 0, 0, 0, 0], 5, 12, None),
        (12, 4, [1, 0, 1, 0, 2, 0, 1, 0, 0, 0, 0, 0], 77, 10, None),
        (16, 5, [1] * 8 + [0] * 8, 2024, 6, None),
        (20, 6, [1] * 10 + [0] * 10, 9, 4, None),
        (10, 7, [1] * 5 + [0] * 5, 11, 15, 0.8),
        (14, 8, [2, 0, 1, 1, 0, 1, 0, 0, 1, 0, 0, 0, 0, 0], 123, 10, 0.6),
    ]
    for m, useed, inp, seed, n, t in plan:
        U = haar_unitary(m, useed)
        seqs.append({"name": f"haar{m}_seed{seed}", "interferometer": _cplx_list(U), "modes": m,
                     "input_state": inp, "seed": seed, "transmissivity": t, "samples": run(U, inp, seed, n, t)})
    return seqs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", default=os.environ.get("PQB_REFERENCE_ROOT", "/root/reference"))
    args = ap.parse_args()
    ut = os.path.join(args.reference_root, "unittests", "test_permanent.py")
    cases = extract_unittests(ut)
    with open(os.path.join(HERE, "reference_unittests.json"), "w") as f:
        json.dump({"source": "unittests/test_permanent.py", "cases": cases}, f, indent=1)
    print(f"{len(cases)} unittest known answers")
    so = os.path.join(ROOT, "oracle", "_ref", "libpqbref.so")
    if not os.path.exists(so):
        os.environ["PQB_REFERENCE_ROOT"] = args.reference_root
        import subprocess
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    calc = reference_calculators(Ref(so))
    with open(os.path.join(HERE, "reference_calculators.json"), "w") as f:
        json.dump({"source": "reference C++ calculators built by oracle/build_ref.sh", **calc}, f)
    print({k: len(v) for k, v in calc.items()})
    seeding = extract_seeding(os.path.join(args.reference_root, "unittests", "test_seeding.py"))
    seqs = reference_sampler(so, seeding)
    with open(os.path.join(HERE, "reference_sampler.json"), "w") as f:
        json.dump({"source": "unittests/test_seeding.py and the reference C++ samplers built by oracle/build_ref.sh",
                   "seeding_cases": seeding, "sequences": seqs}, f)
    print(f"{len(seeding)} seeding cases, {len(seqs)} sampler sequences")


if __name__ == "__main__":
    main()
