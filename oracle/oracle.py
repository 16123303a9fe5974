"""ctypes wrapper over the CPU oracle (liborc.so) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
import this module. It also loads, when they were built, the reference
helpers under oracle/_ref/ (the reference's own evaluate(), counting_sort(),
parse_mps() and CPU simplex, compiled from the reference sources).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF_EVAL = None
_REF_SIMPLEX = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


STAGED = os.path.join(HERE, "_ref", "src")


def reference_dir():
    """The reference tree: $IGAOS_REFERENCE_DIR, else a `reference` directory
    beside the repository; None when neither exists."""
    d = os.environ.get("IGAOS_REFERENCE_DIR") or os.path.join(
        os.path.dirname(os.path.dirname(HERE)), "reference")
    return d if os.path.isdir(d) else None


def build(ref: bool = False) -> None:
    """Compile liborc.so; with `ref`, also the reference helpers under _ref/:
    from the reference tree when it exists (staging the files they read into
    _ref/src on the way), else from an earlier staging in _ref/src."""
    targets, args = ["all"], []
    if ref:
        rd = reference_dir()
        if rd is not None:
            targets += ["stage", "ref"]
            args = [f"REF={rd}"]
        elif os.path.isdir(STAGED):
            targets += ["ref"]
            args = [f"REF={STAGED}"]
    subprocess.run(["make", "-s", "-C", HERE, *args, *targets], check=True)


class orc_metrics(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("pinf", "dinf", "gap", "op", "od", "prow")]


class orc_lp(C.Structure):
    _fields_ = [
        ("m", C.c_int), ("n", C.c_int), ("nnz", C.c_int64),
        ("ap", _ip), ("ai", _ip), ("ax", _dp),
        ("cp", _ip), ("ci", _ip), ("acx", _dp),
        ("c", _dp), ("cl", _dp), ("cu", _dp), ("rmin", _dp), ("rmax", _dp),
        ("obj_const", C.c_double),
    ]


class orc_options(C.Structure):
    _fields_ = [
        ("time_limit_s", C.c_double), ("tolerance", C.c_double),
        ("max_iterations", C.c_int64), ("check_period", C.c_int),
        ("threads", C.c_int), ("verbosity", C.c_int), ("perturb_at", C.c_int64),
    ]


class orc_result(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("objective", C.c_double), ("pinf", C.c_double),
        ("dinf", C.c_double), ("gap", C.c_double), ("prow", C.c_double),
        ("iterations", C.c_int64), ("attempts", C.c_int64),
        ("restarts", C.c_int64), ("checks", C.c_int64),
        ("seconds", C.c_double), ("loop_seconds", C.c_double),
        ("eta", C.c_double), ("omega", C.c_double), ("rollbacks", C.c_int64),
    ]


class orc_state(C.Structure):
    _fields_ = [
        ("x", _dp), ("y", _dp), ("xavg", _dp), ("yavg", _dp), ("axcur", _dp),
        ("eta", C.c_double), ("omega", C.c_double),
        ("k", C.c_int64), ("hn", C.c_int64),
    ]


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liborc.so")
        if not os.path.exists(path):
            build()
        _LIB = C.CDLL(path)
        _LIB.orc_power_iteration.restype = C.c_double
        _LIB.orc_iterate.restype = C.c_int64
    return _LIB


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


STATUS_NAMES = {0: "optimal", 1: "near-optimal", 2: "feasible", 3: "infeasible",
                4: "unbounded", 5: "iteration-limit", 6: "time-limit", 7: "error"}


def evaluate(lp, x, y, Ax, d):
    """FP64 KKT metrics, restatement of the reference evaluate()."""
    mt = orc_metrics()
    x, y, Ax, d = f64(x), f64(y), f64(Ax), f64(d)
    lib().orc_evaluate(lp.m, lp.n, _d(lp.rmin), _d(lp.rmax), _d(lp.cl), _d(lp.cu),
                       _d(lp.c), _d(x), _d(y), _d(Ax), _d(d), C.byref(mt))
    return {k: getattr(mt, k) for k in ("pinf", "dinf", "gap", "op", "od", "prow")}


def evaluate_arrays(rmin, rmax, cl, cu, c, x, y, Ax, d):
    mt = orc_metrics()
    arrs = [f64(a) for a in (rmin, rmax, cl, cu, c, x, y, Ax, d)]
    lib().orc_evaluate(len(arrs[0]), len(arrs[2]), *[_d(a) for a in arrs], C.byref(mt))
    return {k: getattr(mt, k) for k in ("pinf", "dinf", "gap", "op", "od", "prow")}


def counting_sort(ti, tj, tv, rows, cols):
    ti, tj, tv = i32(ti), i32(tj), f64(tv)
    nt = len(ti)
    ap = np.zeros(rows + 1, np.int32); cp = np.zeros(cols + 1, np.int32)
    ai = np.zeros(nt, np.int32); ci = np.zeros(nt, np.int32)
    ax = np.zeros(nt); acx = np.zeros(nt)
    lib().orc_counting_sort(C.c_int64(nt), _i(ti), _i(tj), _d(tv), rows, cols,
                            _i(ap), _i(ai), _d(ax), _i(cp), _i(ci), _d(acx))
    return ap, ai, ax, cp, ci, acx


def transpose(rows, cols, ap, ai, ax):
    ap, ai, ax = i32(ap), i32(ai), f64(ax)
    nnz = int(ap[rows])
    cp = np.zeros(cols + 1, np.int32); ci = np.zeros(nnz, np.int32); acx = np.zeros(nnz)
    lib().orc_transpose(rows, cols, _i(ap), _i(ai), _d(ax), _i(cp), _i(ci), _d(acx))
    return cp, ci, acx


def spmv(ptr, idx, val, x, threads=1):
    ptr, idx, val, x = i32(ptr), i32(idx), f64(val), f64(x)
    rows = len(ptr) - 1
    y = np.zeros(rows)
    lib().orc_spmv(rows, _i(ptr), _i(idx), _d(val), _d(x), _d(y), threads)
    return y


@dataclass
class LP:
    """An LP in the engine's form: rmin <= A x <= rmax, cl <= x <= cu,
    minimise c^T x + obj_const. A is held as CSR and as CSC."""
    m: int
    n: int
    ap: np.ndarray
    ai: np.ndarray
    ax: np.ndarray
    cp: np.ndarray
    ci: np.ndarray
    acx: np.ndarray
    c: np.ndarray
    cl: np.ndarray
    cu: np.ndarray
    rmin: np.ndarray
    rmax: np.ndarray
    obj_const: float = 0.0

    @property
    def nnz(self):
        return int(self.ap[self.m])

    def as_c(self):
        s = orc_lp()
        s.m, s.n, s.nnz = self.m, self.n, self.nnz
        for k in ("ap", "ai", "cp", "ci"):
            setattr(s, k, _i(getattr(self, k)))
        for k in ("ax", "acx", "c", "cl", "cu", "rmin", "rmax"):
            setattr(s, k, _d(getattr(self, k)))
        s.obj_const = self.obj_const
        return s


def lp_from(obj) -> LP:
    """Coerce any object with the LP attributes into contiguous arrays."""
    return LP(m=int(obj.m), n=int(obj.n), ap=i32(obj.ap), ai=i32(obj.ai), ax=f64(obj.ax),
              cp=i32(obj.cp), ci=i32(obj.ci), acx=f64(obj.acx), c=f64(obj.c),
              cl=f64(obj.cl), cu=f64(obj.cu), rmin=f64(obj.rmin), rmax=f64(obj.rmax),
              obj_const=float(getattr(obj, "obj_const", 0.0)))


def ruiz(lp: LP, sweeps=10):
    dr = np.zeros(lp.m); dc = np.zeros(lp.n)
    s = lp.as_c()
    lib().orc_ruiz(C.byref(s), sweeps, _d(dr), _d(dc))
    return dr, dc


def scale(lp: LP, dr, dc):
    s = lp.as_c()
    dr, dc = f64(dr), f64(dc)
    out = dict(sax=np.zeros(lp.nnz), sacx=np.zeros(lp.nnz), sc=np.zeros(lp.n),
               scl=np.zeros(lp.n), scu=np.zeros(lp.n), srmin=np.zeros(lp.m),
               srmax=np.zeros(lp.m))
    lib().orc_scale(C.byref(s), _d(dr), _d(dc), *[_d(out[k]) for k in
                    ("sax", "sacx", "sc", "scl", "scu", "srmin", "srmax")])
    return out


def power_iteration(lp: LP, sd, iters=30, threads=1):
    return lib().orc_power_iteration(lp.m, lp.n, _i(lp.ap), _i(lp.ai), _d(sd["sax"]),
                                     _i(lp.cp), _i(lp.ci), _d(sd["sacx"]), iters, threads)


def primal(tau, x, c, ata, lo, hi):
    x, c, ata, lo, hi = (f64(a) for a in (x, c, ata, lo, hi))
    n = len(x)
    xn, xb, dx = np.zeros(n), np.zeros(n), np.zeros(n)
    lib().orc_primal(n, C.c_double(tau), _d(x), _d(c), _d(ata), _d(lo), _d(hi),
                     _d(xn), _d(xb), _d(dx))
    return xn, xb, dx


def dual(sigma, y, axb, rmin, rmax, axcur):
    y, axb, rmin, rmax, axcur = (f64(a) for a in (y, axb, rmin, rmax, axcur))
    m = len(y)
    yn, dy, adx = np.zeros(m), np.zeros(m), np.zeros(m)
    lib().orc_dual(m, C.c_double(sigma), _d(y), _d(axb), _d(rmin), _d(rmax), _d(axcur),
                   _d(yn), _d(dy), _d(adx))
    return yn, dy, adx


def iterate(lp: LP, sd, state: dict, iters: int, threads=1):
    """Runs `iters` accepted iterations on the scaled problem from `state`
    (dict with x, y, xavg, yavg, axcur, eta, omega, k, hn); returns the new
    state and the attempt count."""
    st = {k: f64(state[k]).copy() for k in ("x", "y", "xavg", "yavg", "axcur")}
    cs = orc_state()
    for k in st:
        setattr(cs, k, _d(st[k]))
    cs.eta, cs.omega = state["eta"], state["omega"]
    cs.k, cs.hn = int(state["k"]), int(state["hn"])
    att = lib().orc_iterate(lp.m, lp.n, _i(lp.ap), _i(lp.ai), _d(sd["sax"]), _i(lp.cp),
                            _i(lp.ci), _d(sd["sacx"]), _d(sd["sc"]), _d(sd["scl"]),
                            _d(sd["scu"]), _d(sd["srmin"]), _d(sd["srmax"]),
                            C.byref(cs), C.c_int64(iters), threads)
    st.update(eta=cs.eta, omega=cs.omega, k=cs.k, hn=cs.hn)
    return st, att


def pdhg_solve(lp: LP, tolerance=1e-4, time_limit=120.0, max_iterations=500000,
               threads=1, check_period=64, verbosity=0, perturb_at=0):
    o = orc_options(time_limit, tolerance, max_iterations, check_period, threads, verbosity,
                    perturb_at)
    r = orc_result()
    x = np.zeros(lp.n); y = np.zeros(lp.m)
    s = lp.as_c()
    lib().orc_pdhg_solve(C.byref(s), C.byref(o), C.byref(r), _d(x), _d(y))
    out = {f: getattr(r, f) for f, _ in orc_result._fields_}
    out["status_name"] = STATUS_NAMES.get(r.status, "?")
    out["x"], out["y"] = x, y
    return out


# ----------------------------------------------------- reference helpers
def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libref_eval.so"))


def ref_simplex_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libref_simplex.so"))


def _ref_eval():
    global _REF_EVAL
    if _REF_EVAL is None:
        _REF_EVAL = C.CDLL(os.path.join(HERE, "_ref", "libref_eval.so"))
    return _REF_EVAL


def ref_evaluate(rmin, rmax, cl, cu, c, x, y, Ax, d):
    arrs = [f64(a) for a in (rmin, rmax, cl, cu, c, x, y, Ax, d)]
    out = np.zeros(6)
    _ref_eval().ref_evaluate(len(arrs[0]), len(arrs[2]), *[_d(a) for a in arrs], _d(out))
    return dict(zip(("pinf", "dinf", "gap", "op", "od", "prow"), out.tolist()))


def dual_repair(lp: LP, x, Ax, y_it, col_tol):
    """The oracle's restatement of the reference dual_repair: (certified, y)."""
    y = np.zeros(lp.m)
    s = lp.as_c()
    ok = lib().orc_dual_repair(C.byref(s), _d(f64(x)), _d(f64(Ax)), _d(f64(y_it)),
                               C.c_double(col_tol), _d(y))
    return bool(ok), y


def ref_dual_repair(lp: LP, x, Ax, y_it, col_tol):
    """The reference's own dual_repair (compiled from its sources): (certified, y)."""
    y = np.zeros(lp.m)
    L = _ref_eval()
    L.ref_dual_repair.restype = C.c_int
    ok = L.ref_dual_repair(lp.m, lp.n, _i(lp.ap), _i(lp.ai), _d(lp.ax), _i(lp.cp), _i(lp.ci),
                           _d(lp.acx), _d(lp.c), _d(lp.cl), _d(lp.cu), _d(lp.rmin),
                           _d(lp.rmax), _d(f64(x)), _d(f64(Ax)), _d(f64(y_it)),
                           C.c_double(col_tol), _d(y))
    return bool(ok), y


def ref_counting_sort(ti, tj, tv, rows, cols):
    ti, tj, tv = i32(ti), i32(tj), f64(tv)
    nt = len(ti)
    ap = np.zeros(rows + 1, np.int32); cp = np.zeros(cols + 1, np.int32)
    ai = np.zeros(nt, np.int32); ci = np.zeros(nt, np.int32)
    ax = np.zeros(nt); acx = np.zeros(nt)
    _ref_eval().ref_counting_sort(C.c_long(nt), _i(ti), _i(tj), _d(tv), rows, cols,
                                  _i(ap), _i(ai), _d(ax), _i(cp), _i(ci), _d(acx))
    return ap, ai, ax, cp, ci, acx


def ref_parse_mps(path: str) -> LP:
    L = _ref_eval()
    m, n, nnz, oc = C.c_int(), C.c_int(), C.c_long(), C.c_double()
    if L.ref_parse_mps(path.encode(), C.byref(m), C.byref(n), C.byref(nnz), C.byref(oc)):
        raise RuntimeError("reference parse_mps failed on " + path)
    m, n, nnz = m.value, n.value, nnz.value
    a = dict(ap=np.zeros(m + 1, np.int32), ai=np.zeros(nnz, np.int32), ax=np.zeros(nnz),
             cp=np.zeros(n + 1, np.int32), ci=np.zeros(nnz, np.int32), acx=np.zeros(nnz),
             c=np.zeros(n), cl=np.zeros(n), cu=np.zeros(n), rmin=np.zeros(m), rmax=np.zeros(m))
    L.ref_fetch_model(*[(_i(a[k]) if a[k].dtype == np.int32 else _d(a[k])) for k in
                        ("ap", "ai", "ax", "cp", "ci", "acx", "c", "cl", "cu", "rmin", "rmax")])
    return LP(m=m, n=n, obj_const=oc.value, **a)


def ref_last_integ(n: int) -> np.ndarray:
    """Integer flags (uint8 per column) of the model ref_parse_mps parsed last."""
    out = np.zeros(n, np.uint8)
    _ref_eval().ref_fetch_integ(out.ctypes.data_as(C.POINTER(C.c_ubyte)))
    return out


def ref_simplex_solve(lp: LP, time_limit=600.0):
    global _REF_SIMPLEX
    if _REF_SIMPLEX is None:
        _REF_SIMPLEX = C.CDLL(os.path.join(HERE, "_ref", "libref_simplex.so"))
    obj = C.c_double(); its = C.c_long()
    x = np.zeros(lp.n); y = np.zeros(lp.m)
    msg = C.create_string_buffer(256)
    st = _REF_SIMPLEX.ref_simplex_solve(
        lp.m, lp.n, C.c_long(lp.nnz), _i(lp.ap), _i(lp.ai), _d(lp.ax), _i(lp.cp), _i(lp.ci),
        _d(lp.acx), _d(lp.c), _d(lp.cl), _d(lp.cu), _d(lp.rmin), _d(lp.rmax),
        C.c_double(lp.obj_const), C.c_double(time_limit), C.byref(obj), C.byref(its),
        _d(x), _d(y), msg, 256)
    return dict(status=STATUS_NAMES.get(st, "?"), objective=obj.value, iterations=its.value,
                x=x, y=y, message=msg.value.decode())


def ref_pdhg_available() -> bool:
    """True when libref_eval.so was built with the reference's GPU solve."""
    if not ref_available():
        return False
    return hasattr(_ref_eval(), "ref_pdhg_solve")


# The reference's dense dual repair (src/pdhg/pdhg.cu:322-327) sizes and
# indexes its m x m matrix with int arithmetic; above this many rows m*m
# overflows int32, so a solve that reaches the repair schedule (k >= 5000,
# pdhg.cu:854) is only run with fewer iterations than that.
REF_REPAIR_MAX_ROWS = 46340
REF_REPAIR_FIRST_K = 5000


def ref_pdhg_solve(lp: LP, tolerance=1e-4, time_limit=120.0, max_iterations=500000,
                   verbosity=0):
    """The reference's own GPU PDHG (cuSPARSE path, compiled from its sources)
    on `lp`: dict with status_name, objective, pinf, dinf, gap, iterations,
    loop_ms (its own timer), wall_ms (the whole call), x, y, message.
    LPs above REF_REPAIR_MAX_ROWS rows must be given a finite iteration budget
    below REF_REPAIR_FIRST_K and no finite time limit."""
    if lp.m > REF_REPAIR_MAX_ROWS and not (
            max_iterations < REF_REPAIR_FIRST_K and not (0 < time_limit < 1e6)):
        raise ValueError("the reference's dense dual repair overflows int32 above "
                         f"{REF_REPAIR_MAX_ROWS} rows: give max_iterations < "
                         f"{REF_REPAIR_FIRST_K} and time_limit >= 1e6")
    L = _ref_eval()
    L.ref_pdhg_solve.restype = C.c_int
    out = np.zeros(7)
    x = np.zeros(lp.n); y = np.zeros(lp.m)
    msg = C.create_string_buffer(512)
    st = L.ref_pdhg_solve(lp.m, lp.n, _i(lp.ap), _i(lp.ai), _d(lp.ax), _i(lp.cp), _i(lp.ci),
                          _d(lp.acx), _d(lp.c), _d(lp.cl), _d(lp.cu), _d(lp.rmin),
                          _d(lp.rmax), C.c_double(lp.obj_const), C.c_double(tolerance),
                          C.c_double(time_limit), C.c_long(int(max_iterations)),
                          C.c_int(verbosity), _d(out), _d(x), _d(y), msg, 512)
    return dict(status_name=STATUS_NAMES.get(st, "exception"), objective=out[0],
                pinf=out[1], dinf=out[2], gap=out[3], iterations=int(out[4]),
                loop_ms=out[5], wall_ms=out[6], x=x, y=y, message=msg.value.decode())


def pock_chambolle(lp: LP, dr, dc):
    """One Pock-Chambolle pass with alpha = 1 (Pock & Chambolle 2011, as PDLP
    applies it after Ruiz; the reference has no such pass): on the scaled
    matrix a~_ij = a_ij dc_j / dr_i, rows are divided by the square root of
    their 1-norm and columns likewise, both norms taken from the same matrix.
    Returns the new (dr, dc); rows and columns with no positive finite norm
    keep their factor."""
    dr, dc = f64(dr).copy(), f64(dc).copy()
    rows = np.repeat(np.arange(lp.m), np.diff(lp.ap))
    v = np.abs(lp.ax) * dc[lp.ai] / dr[rows]
    rs = np.bincount(rows, weights=v, minlength=lp.m)
    cs = np.bincount(lp.ai, weights=v, minlength=lp.n)
    ok_r = (rs > 0) & np.isfinite(rs)
    ok_c = (cs > 0) & np.isfinite(cs)
    dr[ok_r] *= np.sqrt(rs[ok_r])
    dc[ok_c] /= np.sqrt(cs[ok_c])
    return dr, dc
