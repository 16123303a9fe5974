"""ctypes binding of the engine's C ABI (include/igaos_pdhg.h).

This is the reference-facing boundary seen from Python: the same calls a
cgo/JNI/ctypes user makes. There is no CPU fallback: if the native library
is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
# IGAOS_PDHG_LIB selects another build of the same library (tuning variants)
LIB_PATH = os.environ.get("IGAOS_PDHG_LIB") or os.path.join(_PKG, "libigaos_pdhg.so")

OK, ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_NODEVICE, ERR_NUMERIC, ERR_TIMEOUT = range(7)
FP64, FP32_REFINE, FP32 = 0, 1, 2
PRECISIONS = {"fp64": FP64, "fp32-refine": FP32_REFINE, "fp32": FP32}
SCALINGS = {"ruiz": 0, "ruiz-pc": 1}
SCHEDULES = {"fixed": 0, "autotune": 1}
STATUS_NAMES = ["optimal", "near-optimal", "feasible", "infeasible", "unbounded",
                "iteration-limit", "time-limit", "error"]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Options(C.Structure):
    _fields_ = [
        ("time_limit_s", C.c_double), ("tolerance", C.c_double),
        ("max_iterations", C.c_int64), ("seed", C.c_int), ("presolve", C.c_int),
        ("restarts", C.c_int), ("verbosity", C.c_int), ("precision", C.c_int),
        ("check_period", C.c_int), ("inner_tolerance", C.c_double),
        ("max_refinements", C.c_int), ("use_graphs", C.c_int), ("device", C.c_int),
        ("detect_infeasibility", C.c_int), ("pdhg_presolve", C.c_int), ("crossover", C.c_int),
        ("scaling", C.c_int), ("schedule", C.c_int),
    ]


class Result(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("error_code", C.c_int), ("objective", C.c_double),
        ("pinf", C.c_double), ("dinf", C.c_double), ("rel_gap", C.c_double),
        ("prow", C.c_double), ("iterations", C.c_int64), ("attempts", C.c_int64),
        ("kkt_checks", C.c_int64), ("restarts", C.c_int64), ("kkt_passes", C.c_int64),
        ("refinements", C.c_int), ("solve_time_ms", C.c_double),
        ("setup_time_ms", C.c_double), ("device_time_ms", C.c_double),
        ("attempt_time_ms", C.c_double), ("launches", C.c_int64),
        ("rollbacks", C.c_int64), ("entries_a", C.c_int32), ("entries_at", C.c_int32),
        ("message", C.c_char * 160),
    ]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["message"] = self.message.decode(errors="replace")
        d["status_name"] = STATUS_NAMES[self.status] if 0 <= self.status < 8 else "?"
        return d


class BatchResult(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("finished_fp64", C.c_int), ("objective", C.c_double),
        ("pinf", C.c_double), ("dinf", C.c_double), ("rel_gap", C.c_double),
        ("prow", C.c_double), ("iterations", C.c_int64), ("attempts", C.c_int64),
        ("restarts", C.c_int64), ("kernel_time_ms", C.c_double), ("total_time_ms", C.c_double),
        ("instance_time_ms", C.c_double),
    ]


class CrossoverInfo(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("pad", C.c_int), ("pushes", C.c_int64), ("pivots", C.c_int64),
        ("bound_flips", C.c_int64), ("phase1_iterations", C.c_int64),
        ("refactorizations", C.c_int64), ("basis_repairs", C.c_int64),
        ("superbasic_left", C.c_int64), ("time_ms", C.c_double),
    ]


CROSSOVER_STATUS = ["optimal", "pivot-cap", "singular", "unbounded", "infeasible", "too-large"]


class UnrolledLayout(C.Structure):
    """igaos_pdhg_unrolled_layout: sizes plus DEVICE addresses of the
    concatenated CSR / CSC index arrays of a batch (differentiable layer)."""
    _fields_ = [
        ("count", C.c_int), ("precision", C.c_int), ("iterations", C.c_int),
        ("checkpoint", C.c_int), ("ridge", C.c_double), ("max_m", C.c_int), ("max_n", C.c_int),
        ("max_nnz", C.c_int64), ("total_m", C.c_int64), ("total_n", C.c_int64), ("total_nnz", C.c_int64),
        ("row_off", C.c_void_p), ("col_off", C.c_void_p), ("nz_off", C.c_void_p),
        ("ap", C.c_void_p), ("ai", C.c_void_p), ("cp", C.c_void_p), ("ci", C.c_void_p),
        ("cperm", C.c_void_p),
    ]


_LIB = None


def lib():
    """Loads libigaos_pdhg.so (raises if absent -- never falls back)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built; run igaos_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        L.igaos_pdhg_create.argtypes = [
            C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int64, _ip, _ip, _dp, _ip, _ip, _dp,
            _dp, _dp, _dp, _dp, _dp, C.c_double, C.POINTER(Options)]
        L.igaos_pdhg_solve.argtypes = [C.c_void_p, C.POINTER(Options), C.POINTER(Result), _dp, _dp]
        L.igaos_pdhg_destroy.argtypes = [C.c_void_p]
        L.igaos_pdhg_destroy.restype = None
        L.igaos_pdhg_default_options.argtypes = [C.POINTER(Options)]
        L.igaos_pdhg_default_options.restype = None
        L.igaos_pdhg_last_error.argtypes = [C.c_char_p, C.c_size_t]
        L.igaos_pdhg_solve_csr.argtypes = [
            C.c_int, C.c_int, C.c_int64, _ip, _ip, _dp, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp,
            C.c_double, C.POINTER(Options), C.POINTER(Result), _dp, _dp]
        L.igaos_pdhg_get_scaling.argtypes = [C.c_void_p, _dp, _dp]
        L.igaos_pdhg_get_step_init.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.igaos_pdhg_get_transpose.argtypes = [C.c_void_p, _ip, _ip, _dp]
        L.igaos_pdhg_iterate.argtypes = [C.c_void_p, C.c_int, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp]
        L.igaos_pdhg_evaluate.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.igaos_pdhg_set_start.argtypes = [C.c_void_p, _dp, _dp]
        L.igaos_pdhg_spmv.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp]
        L.igaos_pdhg_gather_rate.argtypes = [C.c_int, C.c_int, _dp]
        L.igaos_pdhg_ray_certificate.argtypes = [C.c_int, C.c_int] + [_dp] * 11 + [C.POINTER(C.c_int)]
        L.igaos_pdhg_presolve.argtypes = [
            C.c_int, C.c_int, C.c_int64, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double,
            C.POINTER(C.c_void_p), C.POINTER(C.c_int)]
        L.igaos_pdhg_presolved_info.argtypes = [C.c_void_p, _ip, _ip, C.POINTER(C.c_int64), _dp,
                                                C.POINTER(C.c_int64)]
        L.igaos_pdhg_presolved_lp.argtypes = [C.c_void_p, _ip, _ip] + [_dp] * 6
        L.igaos_pdhg_postsolve.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.igaos_pdhg_postsolve_ray.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.igaos_pdhg_presolved_ray.argtypes = [C.c_void_p, _dp, _dp]
        L.igaos_pdhg_presolved_destroy.argtypes = [C.c_void_p]
        L.igaos_pdhg_presolved_destroy.restype = None
        L.igaos_pdhg_crossover.argtypes = [
            C.c_int, C.c_int, C.c_int64, _ip, _ip] + [_dp] * 9 + [
            C.POINTER(C.c_byte), C.POINTER(CrossoverInfo)]
        L.igaos_pdhg_dual_repair_device.argtypes = [C.c_void_p, _dp, _dp, C.c_double,
                                                    C.c_double, _dp, C.POINTER(C.c_int), _dp]
        L.igaos_pdhg_solve_batch.argtypes = [
            C.c_int, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, C.POINTER(Options),
            C.POINTER(BatchResult), _dp, _dp]
        # device-pointer entry point: every pointer is passed as an address
        L.igaos_pdhg_evaluate_noalloc.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 15
        _lp = C.POINTER(UnrolledLayout)
        L.igaos_pdhg_unrolled_checkpoint_elems.argtypes = [_lp]
        L.igaos_pdhg_unrolled_checkpoint_elems.restype = C.c_int64
        L.igaos_pdhg_unrolled_workspace_bytes.argtypes = [_lp]
        L.igaos_pdhg_unrolled_workspace_bytes.restype = C.c_int64
        L.igaos_pdhg_unrolled_steps.argtypes = [_lp, C.c_void_p, C.c_double, C.c_void_p,
                                                C.c_void_p, C.c_void_p]
        L.igaos_pdhg_unrolled_forward.argtypes = [_lp] + [C.c_void_p] * 13
        L.igaos_pdhg_unrolled_backward.argtypes = [_lp] + [C.c_void_p] * 21
        _LIB = L
    return _LIB


def gather_rate(log2_words: int, device: int = -1) -> float:
    """Random 4-byte gathers per second the GPU serves from a resident vector
    of 2**log2_words floats (igaos_pdhg_gather_rate)."""
    out = C.c_double(0.0)
    _check(lib().igaos_pdhg_gather_rate(int(log2_words), int(device), C.byref(out)))
    return out.value


def ray_certificate(lp, x, y):
    """(kind, xray, yray): the infeasibility-certificate test of
    detect_infeasibility on host arrays (original units): 1 = y is a dual ray
    (the LP is infeasible), 2 = x is a primal ray (its dual is infeasible),
    0 = neither. Needs no GPU."""
    import scipy.sparse as sp
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    f = lambda a: np.ascontiguousarray(a, np.float64)
    x, y = f(x), f(y)
    ax, aty = f(A @ x), f(A.T @ y)
    xr, yr = np.zeros(lp.n), np.zeros(lp.m)
    kind = C.c_int(-1)
    _check(lib().igaos_pdhg_ray_certificate(
        int(lp.m), int(lp.n), *[_d(v) for v in (x, ax, y, aty, f(lp.c), f(lp.cl), f(lp.cu),
                                                  f(lp.rmin), f(lp.rmax), xr, yr)],
        C.byref(kind)))
    return kind.value, xr, yr


PRESOLVE_COUNTS = ("empty_rows", "singleton_rows", "redundant_rows", "fixed_cols", "empty_cols",
                   "free_singletons")


class Presolved:
    """The engine's presolve of an LP on the host (igaos_pdhg_presolve; no
    GPU needed): `outcome` is "reduced", "infeasible" or "unbounded"; when
    reduced, `lp` is the reduced LP (an LPData), `counts` the reductions made,
    postsolve(x_red, y_red) maps a pair of the reduced LP back and
    postsolve_ray(x_red, y_red) a ray; when infeasible or unbounded, ray() is
    the (x, y) certificate presolve found in the original LP."""

    def __init__(self, lp):
        from . import generators as G
        a = _arrays(lp, with_transpose=False)
        self.m0, self.n0 = int(lp.m), int(lp.n)
        h = C.c_void_p()
        oc = C.c_int(-1)
        _check(lib().igaos_pdhg_presolve(
            self.m0, self.n0, int(a["ap"][self.m0]), _i(a["ap"]), _i(a["ai"]), _d(a["ax"]),
            _d(a["c"]), _d(a["cl"]), _d(a["cu"]), _d(a["rmin"]), _d(a["rmax"]),
            float(getattr(lp, "obj_const", 0.0)), C.byref(h), C.byref(oc)))
        self.outcome = {0: "reduced", 3: "infeasible", 4: "unbounded"}[oc.value]
        self.h = h
        self.lp, self.counts = None, None
        if oc.value != 0:
            return
        m, n, nnz = C.c_int(), C.c_int(), C.c_int64()
        k = C.c_double()
        cnt = (C.c_int64 * 6)()
        _check(lib().igaos_pdhg_presolved_info(self.h, C.byref(m), C.byref(n), C.byref(nnz),
                                               C.byref(k), cnt))
        self.counts = dict(zip(PRESOLVE_COUNTS, list(cnt)))
        m, n, nnz = m.value, n.value, nnz.value
        ap, ai = np.zeros(m + 1, np.int32), np.zeros(max(nnz, 1), np.int32)
        ax = np.zeros(max(nnz, 1))
        v = {f: np.zeros(max(n, 1)) for f in ("c", "cl", "cu")}
        v.update({f: np.zeros(max(m, 1)) for f in ("rmin", "rmax")})
        _check(lib().igaos_pdhg_presolved_lp(self.h, _i(ap), _i(ai), _d(ax), *[
            _d(v[f]) for f in ("c", "cl", "cu", "rmin", "rmax")]))
        rows = np.repeat(np.arange(m), np.diff(ap))
        self.lp = G.from_triplets(m, n, rows, ai[:nnz], ax[:nnz], v["c"][:n], v["cl"][:n],
                                  v["cu"][:n], v["rmin"][:m], v["rmax"][:m], obj_const=k.value)

    def postsolve(self, x_red, y_red):
        f = lambda a: np.ascontiguousarray(a, np.float64)
        xr, yr = f(x_red), f(y_red)
        x, y = np.zeros(self.n0), np.zeros(self.m0)
        _check(lib().igaos_pdhg_postsolve(self.h, _d(xr), _d(yr), _d(x), _d(y)))
        return x, y

    def postsolve_ray(self, x_red, y_red):
        f = lambda a: np.ascontiguousarray(a, np.float64)
        xr, yr = f(x_red), f(y_red)
        x, y = np.zeros(self.n0), np.zeros(self.m0)
        _check(lib().igaos_pdhg_postsolve_ray(self.h, _d(xr), _d(yr), _d(x), _d(y)))
        return x, y

    def ray(self):
        x, y = np.zeros(self.n0), np.zeros(self.m0)
        _check(lib().igaos_pdhg_presolved_ray(self.h, _d(x), _d(y)))
        return x, y

    def close(self):
        if getattr(self, "h", None):
            lib().igaos_pdhg_presolved_destroy(self.h)
            self.h = None

    __del__ = close


def crossover(lp, x0):
    """(x, y, basis, info): an optimal vertex of the LP reached from the start
    point x0 by the engine's host crossover (igaos_pdhg_crossover; no GPU
    needed, m <= 2048). basis codes: 0 at lower, 1 at upper, 2 basic, 3
    inside its bounds; n structurals, then m row activities. info is a dict
    with "status" (CROSSOVER_STATUS name) and the pivot counts."""
    a = _arrays(lp, with_transpose=False)
    m, n = int(lp.m), int(lp.n)
    x0 = np.ascontiguousarray(x0, np.float64)
    x, y = np.zeros(n), np.zeros(m)
    basis = np.zeros(n + m, np.int8)
    info = CrossoverInfo()
    _check(lib().igaos_pdhg_crossover(
        m, n, int(a["ap"][m]), _i(a["ap"]), _i(a["ai"]), _d(a["ax"]),
        *[_d(a[k]) for k in ("c", "cl", "cu", "rmin", "rmax")], _d(x0), _d(x), _d(y),
        basis.ctypes.data_as(C.POINTER(C.c_byte)), C.byref(info)))
    d = {f: getattr(info, f) for f, _ in CrossoverInfo._fields_ if f != "pad"}
    d["status"] = CROSSOVER_STATUS[info.status]
    return x, y, basis, d


def last_error() -> str:
    buf = C.create_string_buffer(512)
    lib().igaos_pdhg_last_error(buf, 512)
    return buf.value.decode(errors="replace")


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"igaos_pdhg error {code}: {msg}")
        self.code = code


def _check(rc):
    if rc != OK:
        raise EngineError(rc, last_error())


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return None if a is None else a.ctypes.data_as(_ip)


# igaos.solve keyword names (python/igaos_bindings.cpp:26-28) -> option fields
_ALIASES = {"time_limit": "time_limit_s"}


def default_options(**kw) -> Options:
    o = Options()
    lib().igaos_pdhg_default_options(C.byref(o))
    for k, v in kw.items():
        k = _ALIASES.get(k, k)
        if k == "precision" and isinstance(v, str):
            v = PRECISIONS[v]
        if k == "scaling" and isinstance(v, str):
            v = SCALINGS[v]
        if k == "schedule" and isinstance(v, str):
            v = SCHEDULES[v]
        if not hasattr(o, k):
            raise TypeError(f"unknown option {k!r}")
        setattr(o, k, v)
    return o


def _arrays(lp, with_transpose=True):
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    i = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    a = dict(ap=i(lp.ap), ai=i(lp.ai), ax=f(lp.ax), c=f(lp.c), cl=f(lp.cl), cu=f(lp.cu),
             rmin=f(lp.rmin), rmax=f(lp.rmax))
    if with_transpose and getattr(lp, "cp", None) is not None:
        a.update(cp=i(lp.cp), ci=i(lp.ci), acx=f(lp.acx))
    else:
        a.update(cp=None, ci=None, acx=None)
    return a


class Problem:
    """An LP uploaded to the GPU (igaos_pdhg_create / _destroy)."""

    def __init__(self, lp, with_transpose=True, **opts):
        self.m, self.n = int(lp.m), int(lp.n)
        a = _arrays(lp, with_transpose)
        self._keep = a
        self.nnz = int(a["ap"][self.m])
        h = C.c_void_p()
        o = default_options(**opts)
        rc = lib().igaos_pdhg_create(
            C.byref(h), self.m, self.n, self.nnz, _i(a["ap"]), _i(a["ai"]), _d(a["ax"]),
            _i(a["cp"]), _i(a["ci"]), _d(a["acx"]), _d(a["c"]), _d(a["cl"]), _d(a["cu"]),
            _d(a["rmin"]), _d(a["rmax"]), float(getattr(lp, "obj_const", 0.0)), C.byref(o))
        _check(rc)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().igaos_pdhg_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def solve(self, **opts):
        o = default_options(**opts)
        r = Result()
        x = np.zeros(self.n)
        y = np.zeros(self.m)
        rc = lib().igaos_pdhg_solve(self.h, C.byref(o), C.byref(r), _d(x), _d(y))
        d = r.as_dict()
        d["rc"] = rc
        d["x"], d["y"] = x, y
        return d

    def scaling(self):
        dr, dc = np.zeros(self.m), np.zeros(self.n)
        _check(lib().igaos_pdhg_get_scaling(self.h, _d(dr), _d(dc)))
        return dr, dc

    def step_init(self):
        v = [C.c_double() for _ in range(3)]
        _check(lib().igaos_pdhg_get_step_init(self.h, *[C.byref(t) for t in v]))
        return tuple(t.value for t in v)

    def transpose(self):
        cp = np.zeros(self.n + 1, np.int32)
        ci = np.zeros(self.nnz, np.int32)
        acx = np.zeros(self.nnz)
        _check(lib().igaos_pdhg_get_transpose(self.h, _i(cp), _i(ci), _d(acx)))
        return cp, ci, acx

    def iterate(self, state: dict, iters: int, precision="fp64"):
        st = {k: np.ascontiguousarray(state[k], dtype=np.float64).copy()
              for k in ("x", "y", "xavg", "yavg", "axcur")}
        s6 = np.array([state["eta"], state["omega"], state["k"], state["hn"], 0, 0], np.float64)
        prec = PRECISIONS[precision] if isinstance(precision, str) else precision
        _check(lib().igaos_pdhg_iterate(self.h, prec, int(iters), _d(st["x"]), _d(st["y"]),
                                        _d(st["xavg"]), _d(st["yavg"]), _d(st["axcur"]), _d(s6)))
        st.update(eta=s6[0], omega=s6[1], k=int(s6[2]), hn=int(s6[3]), attempts=int(s6[4]),
                  parity=int(s6[5]))
        return st

    def set_start(self, x0=None, y0=None):
        """Start point (original units) of the following solves on this
        handle; no arguments clear it (igaos_pdhg_set_start)."""
        if x0 is None and y0 is None:
            _check(lib().igaos_pdhg_set_start(self.h, None, None))
            return
        self._x0 = np.ascontiguousarray(x0, np.float64)
        self._y0 = np.ascontiguousarray(y0, np.float64)
        _check(lib().igaos_pdhg_set_start(self.h, _d(self._x0), _d(self._y0)))

    def evaluate(self, x, y):
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        out = np.zeros(6)
        _check(lib().igaos_pdhg_evaluate(self.h, _d(x), _d(y), _d(out)))
        return dict(zip(("pinf", "dinf", "gap", "op", "od", "prow"), out.tolist()))

    def dual_repair_device(self, x, y_it, col_tol, tol):
        """(certified, y, metrics): the engine's matrix-free dual repair on the
        device at candidate x from the dual estimate y_it, original units (any
        m); metrics = dict of pinf, dinf, gap, op, od, prow of (x, y)."""
        a = [np.ascontiguousarray(v, np.float64) for v in (x, y_it)]
        y = np.zeros(self.m)
        m6 = np.zeros(6)
        ok = C.c_int(0)
        _check(lib().igaos_pdhg_dual_repair_device(self.h, _d(a[0]), _d(a[1]), C.c_double(col_tol),
                                                   C.c_double(tol), _d(y), C.byref(ok), _d(m6)))
        return bool(ok.value), y, dict(zip(("pinf", "dinf", "gap", "op", "od", "prow"), m6.tolist()))

    def spmv(self, x, transpose=False, precision="fp64"):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.n if transpose else self.m)
        prec = PRECISIONS[precision] if isinstance(precision, str) else precision
        _check(lib().igaos_pdhg_spmv(self.h, int(bool(transpose)), prec, _d(x), _d(y)))
        return y


def solve_lp(lp, **opts):
    """One-shot solve of an LP object (m, n, ap, ai, ax, [cp, ci, acx], c, cl,
    cu, rmin, rmax, obj_const) through igaos_pdhg_solve_csr."""
    a = _arrays(lp)
    m, n = int(lp.m), int(lp.n)
    o = default_options(**opts)
    r = Result()
    x, y = np.zeros(n), np.zeros(m)
    rc = lib().igaos_pdhg_solve_csr(
        m, n, int(a["ap"][m]), _i(a["ap"]), _i(a["ai"]), _d(a["ax"]), _i(a["cp"]), _i(a["ci"]),
        _d(a["acx"]), _d(a["c"]), _d(a["cl"]), _d(a["cu"]), _d(a["rmin"]), _d(a["rmax"]),
        float(getattr(lp, "obj_const", 0.0)), C.byref(o), C.byref(r), _d(x), _d(y))
    d = r.as_dict()
    d["rc"] = rc
    d["x"], d["y"] = x, y
    return d


def solve_batch(lps, want_solutions=True, **opts):
    """Solves a list of LPs (objects with m, n, ap, ai, ax, c, cl, cu, rmin,
    rmax) in one persistent launch (igaos_pdhg_solve_batch). Returns a list
    of per-instance dicts (status_name, objective, iterations, ... and x, y
    when requested)."""
    count = len(lps)
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    m = i32([lp.m for lp in lps])
    n = i32([lp.n for lp in lps])
    cat = lambda k, f: f(np.concatenate([np.asarray(getattr(lp, k)) for lp in lps]))
    ap, ai, ax = cat("ap", i32), cat("ai", i32), cat("ax", f64)
    c, cl, cu, rmin, rmax = (cat(k, f64) for k in ("c", "cl", "cu", "rmin", "rmax"))
    res = (BatchResult * count)()
    x = np.zeros(int(n.sum())) if want_solutions else None
    y = np.zeros(int(m.sum())) if want_solutions else None
    o = default_options(**opts)
    rc = lib().igaos_pdhg_solve_batch(count, _i(m), _i(n), _i(ap), _i(ai), _d(ax), _d(c), _d(cl),
                                      _d(cu), _d(rmin), _d(rmax), C.byref(o), res, _d(x), _d(y))
    _check(rc)
    out = []
    co = ro = 0
    for b in range(count):
        r = res[b]
        d = {f: getattr(r, f) for f, _ in BatchResult._fields_ if f != "pad"}
        d["status_name"] = STATUS_NAMES[r.status] if 0 <= r.status < 8 else "?"
        if want_solutions:
            d["x"] = x[co:co + lps[b].n]
            d["y"] = y[ro:ro + lps[b].m]
        co += lps[b].n
        ro += lps[b].m
        out.append(d)
    return out
