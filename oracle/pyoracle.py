"""TEST INFRASTRUCTURE: ctypes binding of the CPU oracle (oracle/oracle.cpp).

The oracle is the FP64 CPU restatement of the reference's factor + PCG path
and is used only as the checker in tests/, by the smoke check and as the
CPU baseline in bench.py.  It is never imported by the library itself.

Dense kernels go through scipy's bundled BLAS/LAPACK (the reference links
CBLAS/LAPACKE); the function pointers come from scipy's Cython capsules.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

_lib = None


def _capsule_ptr(capsule):
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(capsule, get_name(capsule))


def load(use_blas=True):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("oracle library not built: %s (run __graft_entry__.build())" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    pI, pD = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    lib.oracle_create.restype = P
    lib.oracle_create.argtypes = [I, pI, pI, pD, pD, pI, pD]
    lib.oracle_free.argtypes = [P]
    lib.oracle_factor.restype = I
    lib.oracle_factor.argtypes = [P]
    lib.oracle_apply.argtypes = [P, pD, pD, I]
    lib.oracle_pcg.restype = I
    lib.oracle_pcg.argtypes = [P, pD, pD, D, I, pD, pD]
    lib.oracle_num_nodes.restype = I
    lib.oracle_num_nodes.argtypes = [P]
    lib.oracle_node_info.argtypes = [P, I, pI]
    lib.oracle_node_l11.argtypes = [P, I, pD]
    lib.oracle_node_l21.argtypes = [P, I, pD]
    lib.oracle_perm.argtypes = [P, pI]
    lib.oracle_node_rows.argtypes = [P, I, pI]
    lib.oracle_times.argtypes = [P, pD]
    lib.oracle_gaussians.argtypes = [P, ctypes.c_longlong, pD]
    lib.oracle_set_blas.argtypes = [P, P, P, P, P]
    lib.oracle_problem_diffusion.restype = P
    lib.oracle_problem_diffusion.argtypes = [I, I, I, I, D, ctypes.c_uint, I]
    lib.oracle_problem_elasticity.restype = P
    lib.oracle_problem_elasticity.argtypes = [I, D, D, ctypes.c_uint, I]
    lib.oracle_problem_sizes.argtypes = [P, ctypes.POINTER(ctypes.c_longlong)]
    lib.oracle_problem_get.argtypes = [P, P, P, P, P, P]
    lib.oracle_problem_free.argtypes = [P]
    if use_blas:
        try:
            import scipy.linalg.cython_blas as cb
            import scipy.linalg.cython_lapack as cl
            lib.oracle_set_blas(
                _capsule_ptr(cb.__pyx_capi__["dgemm"]),
                _capsule_ptr(cb.__pyx_capi__["dtrsm"]),
                _capsule_ptr(cl.__pyx_capi__["dpotrf"]),
                _capsule_ptr(cl.__pyx_capi__["dgeqrf"]),
                _capsule_ptr(cl.__pyx_capi__["dorgqr"]),
            )
        except Exception:  # plain-loop fallback inside the oracle
            pass
    _lib = lib
    return lib


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Problem:
    """A synthetic system built by the oracle library (the same generators as
    the GPU library's rschol_problem_*), with the fields of
    rank_structured_cholesky_gb300.Problem."""

    def __init__(self, handle):
        lib = load()
        if not handle:
            raise RuntimeError("problem generation failed")
        sz = (ctypes.c_longlong * 3)()
        lib.oracle_problem_sizes(handle, sz)
        n, nnz, nrhs = int(sz[0]), int(sz[1]), int(sz[2])
        self.n, self.nrhs = n, nrhs
        self.colptr = np.zeros(n + 1, np.int32)
        self.rowind = np.zeros(nnz, np.int32)
        self.vals = np.zeros(nnz)
        self.xyz = np.zeros(3 * n)
        rhs = np.zeros(n * max(nrhs, 1))
        lib.oracle_problem_get(handle, self.colptr.ctypes.data, self.rowind.ctypes.data, self.vals.ctypes.data,
                               self.xyz.ctypes.data, rhs.ctypes.data)
        lib.oracle_problem_free(handle)
        self.rhs = rhs.reshape(max(nrhs, 1), n)


def diffusion(dim, nx, sigma=0.0, seed=0, nrhs=1):
    nz = nx if dim == 3 else 1
    return Problem(load().oracle_problem_diffusion(dim, nx, nx, nz, sigma, seed, nrhs))


def elasticity(ne, E=1.0, nu=0.3, seed=2, nrhs=1):
    return Problem(load().oracle_problem_elasticity(ne, E, nu, seed, nrhs))


class OracleFactor:
    """Ordering + symbolic + FP64 numeric factor of the reference algorithm."""

    def __init__(self, colptr, rowind, vals, xyz=None, params=None):
        lib = load()
        p = dict(DEFAULT_PARAMS)
        if params:
            p.update(params)
        self.params = p
        self.colptr = np.ascontiguousarray(colptr, dtype=np.int32)
        self.rowind = np.ascontiguousarray(rowind, dtype=np.int32)
        self.vals = np.ascontiguousarray(vals, dtype=np.float64)
        self.n = len(self.colptr) - 1
        ip = np.array([p["max_dense_block"], p["max_diag_block"], p["explicit_threshold"], p["nd_leaf"],
                       p["oversampling"], p["rank_cap"], p["power_iters"], p["reorder_separators"]],
                      dtype=np.int32)
        dp = np.array([p["rank_constant"], p["diag_rank_constant"]], dtype=np.float64)
        xyz_p = None
        if xyz is not None:
            self._xyz = np.ascontiguousarray(xyz, dtype=np.float64)
            xyz_p = _dp(self._xyz)
        self.h = lib.oracle_create(self.n, _ip(self.colptr), _ip(self.rowind), _dp(self.vals), xyz_p,
                                   _ip(ip), _dp(dp))
        if not self.h:
            raise RuntimeError("oracle_create failed")
        self.status = None

    def factor(self):
        self.status = load().oracle_factor(self.h)
        return self.status

    def apply(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        load().oracle_apply(self.h, _dp(b), _dp(x), nrhs)
        return x

    def pcg(self, b, eps=1e-8, maxit=10000):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        rec = ctypes.c_double()
        true = ctypes.c_double()
        it = load().oracle_pcg(self.h, _dp(b), _dp(x), eps, maxit, ctypes.byref(rec), ctypes.byref(true))
        return x, it, rec.value, true.value

    def num_nodes(self):
        return load().oracle_num_nodes(self.h)

    def node_info(self, j):
        info = np.zeros(8, dtype=np.int32)
        load().oracle_node_info(self.h, j, _ip(info))
        keys = ["c0", "c1", "compressed", "m", "n_stored", "rank", "hodlr_nodes", "interior"]
        return dict(zip(keys, info.tolist()))

    def node_l11(self, j):
        inf = self.node_info(j)
        n = inf["c1"] - inf["c0"] + 1
        out = np.zeros((n, n))
        load().oracle_node_l11(self.h, j, _dp(out))
        return out

    def node_l21(self, j):
        inf = self.node_info(j)
        n = inf["c1"] - inf["c0"] + 1
        rows = inf["m"] if inf["compressed"] else inf["n_stored"]
        out = np.zeros((rows, n))
        if rows:
            load().oracle_node_l21(self.h, j, _dp(out))
        return out

    def node_rows(self, j):
        out = np.zeros(self.node_info(j)["m"], dtype=np.int32)
        if out.size:
            load().oracle_node_rows(self.h, j, _ip(out))
        return out

    def perm(self):
        out = np.zeros(self.n, dtype=np.int32)
        load().oracle_perm(self.h, _ip(out))
        return out

    def times(self):
        t = np.zeros(4)
        load().oracle_times(self.h, _dp(t))
        return {"symbolic_s": t[0], "numeric_s": t[1], "attempts": int(t[2]), "diag_rank_constant": t[3]}

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle_free(self.h)
            self.h = None


DEFAULT_PARAMS = {
    "max_dense_block": 200,
    "max_diag_block": 400,
    "explicit_threshold": 4000,
    "nd_leaf": 64,
    "oversampling": 5,
    "rank_cap": 0,
    "power_iters": 1,
    "reorder_separators": 1,
    "rank_constant": 0.4,
    "diag_rank_constant": 0.5,
}
