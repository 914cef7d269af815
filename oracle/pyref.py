"""TEST INFRASTRUCTURE: the checking tools built from the reference's own
sources (oracle/_ref/, by rank_structured_cholesky_gb300/_build.py
build_reference_tools, only where the reference sources are present).

* ``septree(points, max_leaf)``: the reference's SeparatorTree order and leaf
  ranges, built as NestedDissection::ReorderNestedSeparators builds them
  (src/rschol/ordering/NestedDissection.cpp:811-817).
* ``pcg(colptr, rowind, vals, b, apply, eps, maxit)``: the reference's
  PCG_SOLVER::solvePCG (src/rschol/linearalgebra/PCG_SOLVER.cpp:226-363) from
  x = 0 with ``apply(b) -> x`` as its preconditioner.

Used by tests/golden/make_golden.py to write the committed fixtures and by
CPU tests that re-check them live; never by the library.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(_HERE, "_ref")
SEPTREE = os.path.join(REF_OUT, "ref_septree_kat")
PCG_LIB = os.path.join(REF_OUT, "libref_pcg.so")

APPLY_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                            ctypes.c_int)
_lib = None


def available():
    return os.path.exists(SEPTREE) and os.path.exists(PCG_LIB)


def septree(points, max_leaf):
    """(order, leaf_first) of the reference's separator tree over points (n x 3)."""
    pts = np.asarray(points, np.float64).reshape(-1, 3)
    inp = "%d %d\n" % (len(pts), max_leaf) + "".join("%.17g %.17g %.17g\n" % tuple(p) for p in pts)
    out = subprocess.run([SEPTREE], input=inp, text=True, stdout=subprocess.PIPE, check=True).stdout.split()
    n = len(pts)
    order = np.array(out[:n], np.int32)
    nl = int(out[n])
    ranges = np.array(out[n + 1:n + 1 + 2 * nl], np.int64).reshape(nl, 2)
    assert np.all(ranges[1:, 0] == ranges[:-1, 1] + 1) and ranges[0, 0] == 0 and ranges[-1, 1] == n - 1
    first = np.concatenate([ranges[:, 0], [n]]).astype(np.int32)
    return order, first


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(PCG_LIB)
        lib.ref_pcg_solve.restype = ctypes.c_int
        lib.ref_pcg_solve.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int, APPLY_FN,
                                      ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        _lib = lib
    return _lib


def pcg(colptr, rowind, vals, b, apply, eps=1e-8, maxit=10000):
    """x, iterations, final ||b - A x|| / ||b|| from the reference's PCG loop."""
    colptr = np.ascontiguousarray(colptr, np.int32)
    rowind = np.ascontiguousarray(rowind, np.int32)
    vals = np.ascontiguousarray(vals, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    n = len(colptr) - 1
    x = np.zeros(n)

    def cb(_user, pb, px, m):
        src = np.ctypeslib.as_array(pb, shape=(m,))
        dst = np.ctypeslib.as_array(px, shape=(m,))
        dst[:] = apply(src.copy())

    fn = APPLY_FN(cb)
    res = ctypes.c_double()
    it = _load().ref_pcg_solve(n, colptr.ctypes.data, rowind.ctypes.data, vals.ctypes.data, b.ctypes.data,
                               x.ctypes.data, eps, maxit, fn, None, ctypes.byref(res))
    return x, it, res.value
