"""GB300-native rank-structured Cholesky preconditioner + PCG.

Python host mirror of the reference's interface for this path
(jeffchadwick/rank_structured_cholesky):

* ``FactorPreconditioner.initialize / solve``  -- src/rschol/solver/FactorPreconditioner.h:92-113
* ``PCGSolver(A, eps, iterations).solve_pcg``   -- src/rschol/linearalgebra/PCG_SOLVER.h:52-65
* ``solve(A, b)``                               -- src/python/rschol.pyx:38-53 (``rschol.solve``)

All compute runs in the native library (``_build/librschol_gb300.so``, C ABI
declared in ``include/rschol_gpu.h``) on the GPU.  There is no CPU fallback:
if the library or a CUDA device is missing the calls raise.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "librschol_gb300.so")

RSCHOL_OK = 0
STATUS_NAMES = {
    0: "RSCHOL_OK", 1: "RSCHOL_E_BAD_INPUT", 2: "RSCHOL_E_NOT_PD_AFTER_RETRY", 3: "RSCHOL_E_OOM",
    4: "RSCHOL_E_CUDA", 5: "RSCHOL_E_BREAKDOWN", 6: "RSCHOL_E_TIMEOUT", 7: "RSCHOL_E_NO_DEVICE",
    8: "RSCHOL_E_UNSUPPORTED", 9: "RSCHOL_E_NOT_PD",
}
FP64, MIXED = 0, 1

# Every entry point declared in include/rschol_gpu.h.
EXPORTED = [
    "rschol_default_params", "rschol_create", "rschol_destroy", "rschol_last_error", "rschol_factor_create",
    "rschol_check_structure",
    "rschol_refactor", "rschol_refactor_device", "rschol_stream", "rschol_profile", "rschol_factor_free", "rschol_precond_apply", "rschol_precond_apply_device",
    "rschol_precond_apply_device_noalloc", "rschol_selftest_gemm", "rschol_bench_gemm", "rschol_step_timing", "rschol_pcg",
    "rschol_pcg_device", "rschol_pcg_pysolve", "rschol_factor_n", "rschol_factor_device_bytes", "rschol_factor_num_nodes",
    "rschol_factor_node_info", "rschol_factor_node_l11", "rschol_factor_node_l21", "rschol_factor_perm",
    "rschol_factor_describe", "rschol_factor_stats", "rschol_problem_diffusion", "rschol_problem_elasticity",
    "rschol_problem_n", "rschol_problem_nnz", "rschol_problem_nrhs", "rschol_problem_get", "rschol_problem_free",
    "rschol_mt_draws", "rschol_mt_gaussians", "rschol_block_rank", "rschol_separator_tree", "rschol_etree_counts",
    "rschol_relaxed_supernodes", "rschol_factor_autotune", "rschol_factor_tune_schedule", "rschol_session_create", "rschol_session_columns", "rschol_session_add",
    "rschol_session_step", "rschol_session_result", "rschol_session_counts", "rschol_session_destroy",
    "rschol_server_create", "rschol_server_submit", "rschol_server_wait",
    "rschol_server_stats", "rschol_server_destroy",
]


class RscholError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


class Params(ctypes.Structure):
    _fields_ = [
        ("max_dense_block", ctypes.c_int), ("max_diag_block", ctypes.c_int), ("explicit_threshold", ctypes.c_int),
        ("nd_leaf", ctypes.c_int), ("oversampling", ctypes.c_int), ("rank_cap", ctypes.c_int),
        ("power_iters", ctypes.c_int), ("reorder_separators", ctypes.c_int), ("rank_constant", ctypes.c_double),
        ("diag_rank_constant", ctypes.c_double), ("max_factor_attempts", ctypes.c_int),
        ("rank_alpha", ctypes.c_double), ("seed", ctypes.c_uint), ("precision", ctypes.c_int),
        ("device", ctypes.c_int), ("root_fp64", ctypes.c_int), ("schur_bf16", ctypes.c_int),
    ]


class PcgInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("residual", ctypes.c_double), ("true_residual", ctypes.c_double),
                ("seconds", ctypes.c_double)]


_lib = None


def load_library():
    """Load the native library (built by ``_build.build_library``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("native library missing: %s -- run __graft_entry__.build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    P, I, D, LL = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
    pI, pD = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    sig = {
        "rschol_default_params": (None, [ctypes.POINTER(Params)]),
        "rschol_create": (P, [ctypes.POINTER(Params)]),
        "rschol_destroy": (None, [P]),
        "rschol_last_error": (ctypes.c_char_p, [P]),
        "rschol_factor_create": (I, [P, I, pI, pI, pD, pD, ctypes.POINTER(P)]),
        "rschol_check_structure": (I, [I, pI, pI, pD, ctypes.POINTER(Params), ctypes.c_char_p, I]),
        "rschol_refactor": (I, [P, pD]),
        "rschol_refactor_device": (I, [P, P]),
        "rschol_stream": (P, [P]),
        "rschol_profile": (I, [P, P, P]),
        "rschol_factor_free": (None, [P]),
        "rschol_precond_apply": (I, [P, pD, pD, I]),
        "rschol_precond_apply_device": (I, [P, P, P, I]),
        "rschol_precond_apply_device_noalloc": (I, [P, P, P, I]),
        "rschol_selftest_gemm": (I, [I, I, I, I, I, I, I, pD]),
        "rschol_bench_gemm": (I, [I, I, I, I, I, pD]),
        "rschol_step_timing": (I, [P, I, P]),
        "rschol_pcg": (I, [P, pD, pD, I, D, I, ctypes.POINTER(PcgInfo)]),
        "rschol_pcg_device": (I, [P, P, P, I, D, I, ctypes.POINTER(PcgInfo)]),
        "rschol_pcg_pysolve": (None, [I, pI, pI, pD, pD, pD]),
        "rschol_factor_n": (I, [P]),
        "rschol_factor_device_bytes": (D, [P]),
        "rschol_factor_num_nodes": (I, [P]),
        "rschol_factor_node_info": (I, [P, I, pI]),
        "rschol_factor_node_l11": (I, [P, I, pD]),
        "rschol_factor_node_l21": (I, [P, I, pD]),
        "rschol_factor_perm": (I, [P, pI]),
        "rschol_factor_describe": (ctypes.c_char_p, [P]),
        "rschol_factor_stats": (I, [P, pD]),
        "rschol_problem_diffusion": (P, [I, I, I, I, D, ctypes.c_uint, I]),
        "rschol_problem_elasticity": (P, [I, D, D, ctypes.c_uint, I]),
        "rschol_problem_n": (I, [P]),
        "rschol_problem_nnz": (LL, [P]),
        "rschol_problem_nrhs": (I, [P]),
        "rschol_problem_get": (None, [P, P, P, P, P, P]),
        "rschol_problem_free": (None, [P]),
        "rschol_mt_draws": (None, [ctypes.c_uint, LL, P]),
        "rschol_mt_gaussians": (None, [ctypes.c_uint, LL, P]),
        "rschol_block_rank": (I, [I, I, D, I, I]),
        "rschol_separator_tree": (I, [I, P, I, P, P]),
        "rschol_etree_counts": (None, [I, P, P, P, P]),
        "rschol_relaxed_supernodes": (I, [I, P, P, I, P, P, P, P, I, P, P]),
        "rschol_factor_autotune": (I, [P, I]),
        "rschol_factor_tune_schedule": (I, [P, I]),
        "rschol_session_create": (P, [P, I]),
        "rschol_session_columns": (I, [P]),
        "rschol_session_add": (I, [P, LL, I, pD, pD, D, I]),
        "rschol_session_step": (I, [P, ctypes.POINTER(LL), pI]),
        "rschol_session_result": (I, [P, LL, ctypes.POINTER(PcgInfo)]),
        "rschol_session_counts": (I, [P, pI, pI]),
        "rschol_session_destroy": (None, [P]),
        "rschol_server_create": (P, [ctypes.POINTER(Params), I, D]),
        "rschol_server_submit": (I, [P, I, I, pI, pI, pD, pD, I, pD, D, I]),
        "rschol_server_wait": (I, [P, I, pD, ctypes.POINTER(PcgInfo), pD]),
        "rschol_server_stats": (I, [P, pD]),
        "rschol_server_destroy": (None, [P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def default_params(**overrides):
    p = Params()
    load_library().rschol_default_params(ctypes.byref(p))
    for k, v in overrides.items():
        if k == "precision" and isinstance(v, str):
            v = MIXED if v.lower().startswith("mix") else FP64
        setattr(p, k, v)
    return p


# --------------------------------------------------------------------------
# Synthetic problems
class Problem:
    def __init__(self, handle):
        lib = load_library()
        n, nnz, nrhs = lib.rschol_problem_n(handle), lib.rschol_problem_nnz(handle), lib.rschol_problem_nrhs(handle)
        self.n, self.nrhs = n, nrhs
        self.colptr = np.zeros(n + 1, np.int32)
        self.rowind = np.zeros(nnz, np.int32)
        self.vals = np.zeros(nnz)
        self.xyz = np.zeros(3 * n)
        self.rhs = np.zeros(n * max(nrhs, 1))
        lib.rschol_problem_get(handle, self.colptr.ctypes.data, self.rowind.ctypes.data, self.vals.ctypes.data,
                               self.xyz.ctypes.data, self.rhs.ctypes.data)
        lib.rschol_problem_free(handle)
        self.rhs = self.rhs.reshape(max(nrhs, 1), n)

    def scipy(self):
        import scipy.sparse as sp
        return sp.csc_matrix((self.vals, self.rowind, self.colptr), shape=(self.n, self.n))


def diffusion(dim, nx, ny=None, nz=None, sigma=0.0, seed=0, nrhs=1):
    ny = nx if ny is None else ny
    nz = (nx if dim == 3 else 1) if nz is None else nz
    h = load_library().rschol_problem_diffusion(dim, nx, ny, nz, sigma, seed, nrhs)
    if not h:
        raise RuntimeError("problem generation failed")
    return Problem(h)


def elasticity(ne, E=1.0, nu=0.3, seed=2, nrhs=1):
    h = load_library().rschol_problem_elasticity(ne, E, nu, seed, nrhs)
    if not h:
        raise RuntimeError("problem generation failed")
    return Problem(h)


# --------------------------------------------------------------------------
class Context:
    def __init__(self, params=None, **overrides):
        lib = load_library()
        self.params = params if params is not None else default_params(**overrides)
        self.h = lib.rschol_create(ctypes.byref(self.params))

    def last_error(self):
        return load_library().rschol_last_error(self.h).decode()

    def close(self):
        if getattr(self, "h", None):
            load_library().rschol_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def check_structure(colptr, rowind, xyz=None, **params):
    """(status, reason): whether GpuFactor can take this pattern with these
    parameters, from the host ordering and symbolic analysis alone (no device)."""
    colptr = np.ascontiguousarray(colptr, np.int32)
    rowind = np.ascontiguousarray(rowind, np.int32)
    xp = None
    if xyz is not None:
        xyz = np.ascontiguousarray(xyz, np.float64)
        xp = _dp(xyz)
    prm = default_params(**params)
    msg = ctypes.create_string_buffer(512)
    st = load_library().rschol_check_structure(len(colptr) - 1, _ip(colptr), _ip(rowind), xp, ctypes.byref(prm),
                                               msg, len(msg))
    return st, msg.value.decode()


class GpuFactor:
    """Symbolic + numeric factorisation on the GPU (FactorPreconditioner::initialize)."""

    def __init__(self, ctx, colptr, rowind, vals, xyz=None):
        lib = load_library()
        self.ctx = ctx
        self.colptr = np.ascontiguousarray(colptr, np.int32)
        self.rowind = np.ascontiguousarray(rowind, np.int32)
        self.vals = np.ascontiguousarray(vals, np.float64)
        self.n = len(self.colptr) - 1
        xp = None
        if xyz is not None:
            self._xyz = np.ascontiguousarray(xyz, np.float64)
            xp = _dp(self._xyz)
        h = ctypes.c_void_p()
        st = lib.rschol_factor_create(ctx.h, self.n, _ip(self.colptr), _ip(self.rowind), _dp(self.vals), xp,
                                      ctypes.byref(h))
        if st != RSCHOL_OK:
            raise RscholError(st, ctx.last_error())
        self.h = h

    def refactor(self, vals):
        v = np.ascontiguousarray(vals, np.float64)
        st = load_library().rschol_refactor(self.h, _dp(v))
        if st != RSCHOL_OK:
            raise RscholError(st, self.ctx.last_error())

    def apply(self, b):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros_like(b)
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        st = load_library().rschol_precond_apply(self.h, _dp(b), _dp(x), nrhs)
        if st != RSCHOL_OK:
            raise RscholError(st, self.ctx.last_error())
        return x

    def pcg(self, b, eps=1e-8, maxit=10000):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros_like(b)
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        infos = (PcgInfo * nrhs)()
        st = load_library().rschol_pcg(self.h, _dp(b), _dp(x), nrhs, eps, maxit, infos)
        if st not in (RSCHOL_OK, 5):
            raise RscholError(st, self.ctx.last_error())
        info = [dict(iterations=i.iterations, residual=i.residual, true_residual=i.true_residual,
                     seconds=i.seconds) for i in infos]
        return x, (info[0] if nrhs == 1 else info)

    def autotune(self, max_columns=64):
        """Time the batched apply's tile shapes for every width class up to max_columns."""
        st = load_library().rschol_factor_autotune(self.h, max_columns)
        if st != RSCHOL_OK:
            raise RscholError(st, self.ctx.last_error())

    def tune_schedule(self, repeats=2):
        """Time the factor's candidate schedules (tensor-core GEMM threshold, fused or
        per-panel blocked Cholesky) and keep the fastest; the factor stays factored."""
        st = load_library().rschol_factor_tune_schedule(self.h, repeats)
        if st != RSCHOL_OK:
            raise RscholError(st, self.ctx.last_error())
        return self.describe()["schedule"]

    def num_nodes(self):
        return load_library().rschol_factor_num_nodes(self.h)

    def node_info(self, j):
        info = np.zeros(8, np.int32)
        load_library().rschol_factor_node_info(self.h, j, _ip(info))
        keys = ["c0", "c1", "compressed", "m", "n_stored", "rank", "hodlr_nodes", "interior"]
        return dict(zip(keys, info.tolist()))

    def node_l11(self, j):
        inf = self.node_info(j)
        n = inf["c1"] - inf["c0"] + 1
        out = np.zeros((n, n))
        load_library().rschol_factor_node_l11(self.h, j, _dp(out))
        return out

    def node_l21(self, j):
        inf = self.node_info(j)
        n = inf["c1"] - inf["c0"] + 1
        rows = inf["m"] if inf["compressed"] else inf["n_stored"]
        out = np.zeros((rows, n))
        if rows:
            load_library().rschol_factor_node_l21(self.h, j, _dp(out))
        return out

    def perm(self):
        out = np.zeros(self.n, np.int32)
        load_library().rschol_factor_perm(self.h, _ip(out))
        return out

    def describe(self):
        import json
        return json.loads(load_library().rschol_factor_describe(self.h).decode())

    def stats(self):
        s = np.zeros(8)
        load_library().rschol_factor_stats(self.h, _dp(s))
        return dict(symbolic_s=s[0], numeric_s=s[1], attempts=int(s[2]), diag_rank_constant=s[3],
                    factor_launches=int(s[4]), device_bytes=s[5], gaussian_draws=int(s[6]), factor_flops=s[7],
                    live_device_bytes=load_library().rschol_factor_device_bytes(self.h))

    def close(self):
        if getattr(self, "h", None):
            load_library().rschol_factor_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Session:
    """Continuous-batching PCG on one GpuFactor (rschol_session_*).

    ``add`` queues a request of right-hand sides; ``step`` runs one PCG
    iteration of every active column and returns the requests finished in
    it as {tag: (status, x, info)}.
    """

    def __init__(self, factor, max_columns=64):
        self.factor = factor
        self.h = load_library().rschol_session_create(factor.h, max_columns)
        if not self.h:
            raise RscholError(4, factor.ctx.last_error())
        self.columns = load_library().rschol_session_columns(self.h)
        self._reqs = {}

    def add(self, tag, b, eps=1e-8, maxit=10000):
        b = np.ascontiguousarray(b, np.float64)
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        x = np.zeros_like(b)
        st = load_library().rschol_session_add(self.h, tag, nrhs, _dp(b), _dp(x), eps, maxit)
        if st != RSCHOL_OK:
            raise RscholError(st, "rschol_session_add")
        self._reqs[tag] = (b, x, nrhs)   # the buffers stay alive until the request is done

    def step(self):
        lib = load_library()
        tags = (ctypes.c_longlong * self.columns)()
        nd = ctypes.c_int(0)
        st = lib.rschol_session_step(self.h, tags, ctypes.byref(nd))
        if st != RSCHOL_OK:
            raise RscholError(st, self.factor.ctx.last_error())
        out = {}
        for i in range(nd.value):
            b, x, nrhs = self._reqs.pop(tags[i])
            infos = (PcgInfo * nrhs)()
            rs = lib.rschol_session_result(self.h, tags[i], infos)
            info = [dict(iterations=q.iterations, residual=q.residual, true_residual=q.true_residual,
                         seconds=q.seconds) for q in infos]
            out[tags[i]] = (rs, x, info)
        return out

    def counts(self):
        a, q = ctypes.c_int(0), ctypes.c_int(0)
        load_library().rschol_session_counts(self.h, ctypes.byref(a), ctypes.byref(q))
        return a.value, q.value

    def close(self):
        if getattr(self, "h", None):
            load_library().rschol_session_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop over many systems on one GPU (no reference counterpart).

    Requests are (matrix id, CSC matrix, right-hand sides); factors are cached
    on the device by matrix id within ``hbm_budget_bytes`` and reused by later
    requests for the same id; ``workers`` threads serve requests concurrently.
    ``submit`` returns a request id, ``wait`` its solution, PCG info and times.
    """

    def __init__(self, params=None, workers=4, hbm_budget_bytes=64e9, **overrides):
        lib = load_library()
        self.params = params if params is not None else default_params(**overrides)
        self.h = lib.rschol_server_create(ctypes.byref(self.params), workers, float(hbm_budget_bytes))
        if not self.h:
            raise RscholError(1, "rschol_server_create: bad arguments")
        self._shapes = {}

    def submit(self, matrix_id, colptr, rowind, vals, b, xyz=None, eps=1e-8, maxit=10000):
        colptr = np.ascontiguousarray(colptr, np.int32)
        rowind = np.ascontiguousarray(rowind, np.int32)
        vals = np.ascontiguousarray(vals, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        n = len(colptr) - 1
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        xp = None
        if xyz is not None:
            xyz = np.ascontiguousarray(xyz, np.float64)
            xp = _dp(xyz)
        rid = load_library().rschol_server_submit(self.h, int(matrix_id), n, _ip(colptr), _ip(rowind), _dp(vals), xp,
                                                  nrhs, _dp(b), eps, maxit)
        if rid <= 0:
            raise RscholError(-rid, "rschol_server_submit rejected the request")
        self._shapes[rid] = b.shape
        return rid

    def wait(self, rid):
        shape = self._shapes.pop(rid)
        nrhs = 1 if len(shape) == 1 else shape[0]
        x = np.zeros(shape)
        infos = (PcgInfo * nrhs)()
        times = np.zeros(5)
        st = load_library().rschol_server_wait(self.h, rid, _dp(x), infos, _dp(times))
        info = [dict(iterations=i.iterations, residual=i.residual, true_residual=i.true_residual,
                     seconds=i.seconds) for i in infos]
        t = dict(queued=times[0], factor=times[1], pcg=times[2], latency=times[3], cache_hit=bool(times[4]))
        return st, x, info, t

    def stats(self):
        s = np.zeros(8)
        load_library().rschol_server_stats(self.h, _dp(s))
        keys = ["completed", "hits", "misses", "evictions", "cached_bytes", "peak_cached_bytes", "cached_factors",
                "queued"]
        return dict(zip(keys, s.tolist()))

    def close(self):
        if getattr(self, "h", None):
            load_library().rschol_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------------
# Reference-shaped interface
class FactorPreconditioner:
    """FactorPreconditioner (src/rschol/solver/FactorPreconditioner.h:92-113)."""

    def __init__(self, params=None, **overrides):
        self.ctx = Context(params, **overrides)
        self.factor = None

    def initialize(self, A, mesh_positions=None, max_dense_block=None, max_diagonal_block=None):
        if max_dense_block is not None:
            self.ctx.params.max_dense_block = max_dense_block
        if max_diagonal_block is not None:
            self.ctx.params.max_diag_block = max_diagonal_block
        if max_dense_block is not None or max_diagonal_block is not None:
            p = self.ctx.params
            self.ctx.close()
            self.ctx = Context(p)
        colptr, rowind, vals = _csc_arrays(A)
        xyz = None if mesh_positions is None else np.asarray(mesh_positions, np.float64).reshape(-1)
        self.factor = GpuFactor(self.ctx, colptr, rowind, vals, xyz)
        return self

    def solve(self, b):
        return self.factor.apply(b)


class PCGSolver:
    """PCG_SOLVER(A, eps, iterations) + solvePCG(x, b, M)."""

    def __init__(self, A, eps=1e-6, iterations=10000):
        self.A, self.eps, self.iterations = A, eps, iterations
        self.last = None

    def solve_pcg(self, b, M):
        x, info = M.factor.pcg(b, self.eps, self.iterations)
        self.last = info
        return x

    def residual(self):
        return None if self.last is None else self.last["true_residual"]


def _csc_arrays(A):
    if isinstance(A, tuple):
        return A
    import scipy.sparse as sp
    A = sp.csc_matrix(A)
    A.sort_indices()
    return A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float64)


def solve(A, b):
    """rschol.solve(A, b) (src/python/rschol.pyx:38-53): pcg_pysolve with the
    reference driver's settings (maxDenseBlock 200, maxDiagonalBlock 400,
    eps 1e-6, 10000 iterations, no positions)."""
    lib = load_library()
    import scipy.sparse as sp
    A = sp.csr_matrix(A)
    indptr = A.indptr.astype(np.int32)
    indices = A.indices.astype(np.int32)
    data = A.data.astype(np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = b.copy()
    lib.rschol_pcg_pysolve(A.shape[0], _ip(indptr), _ip(indices), _dp(data), _dp(b), _dp(x))
    return x
