"""C ABI checks that need no GPU: the library loads, exports every entry point
include/igaos_pdhg.h declares, validates input before touching a device, and
reports the missing device honestly (reference: src/api/engine.hpp:35-37 and
src/pdhg/pdhg.cu:461-465 report failures as Status::Error + message)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, has_gpu

HEADER = os.path.join(ROOT, "include", "igaos_pdhg.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(igaos_pdhg_\w+)\s*\(", txt)))


def test_exports_every_declared_symbol(native):
    syms = declared_symbols()
    assert len(syms) >= 12
    missing = [s for s in syms if not hasattr(native, s)]
    assert not missing, missing


def test_abi_version_and_defaults(native):
    import ctypes as C
    from igaos_gb300 import capi
    assert native.igaos_pdhg_abi_version() == 4
    o = capi.default_options()
    # igaos::Options defaults (reference include/igaos/options.h:5-13)
    assert o.time_limit_s == 120.0 and o.tolerance == 1e-4 and o.max_iterations == 500000
    assert o.presolve == 1 and o.restarts == 0 and o.verbosity == 0 and o.seed == 0
    assert o.precision == capi.FP64 and o.check_period == 64 and o.use_graphs == 1
    assert o.detect_infeasibility == 0  # off, as the reference engine
    assert o.pdhg_presolve == 0  # off: the reference engine ignores `presolve`
    assert o.crossover == 0
    assert o.scaling == capi.SCALINGS["ruiz"]  # the reference's Ruiz scaling alone
    assert o.schedule == capi.SCHEDULES["fixed"]
    assert C.sizeof(o) == 88  # ABI 4 layout of igaos_pdhg_options


def _tiny():
    from igaos_gb300.generators import random_lp
    return random_lp(8, 12, 10, 0)


@pytest.mark.parametrize("breaker, msg", [
    (lambda a: a.update(m=0), "at least one row"),
    (lambda a: a["ai"].__setitem__(0, 99), "column index out of range"),
    (lambda a: a["ax"].__setitem__(1, np.nan), "matrix values must be finite"),
    (lambda a: a["c"].__setitem__(0, np.inf), "cost must be finite"),
    (lambda a: a["cl"].__setitem__(0, 20.0), "lower bound above upper"),
    (lambda a: a["rmin"].__setitem__(0, np.nan), "row bounds must not be NaN"),
    (lambda a: a["ap"].__setitem__(1, 1000), "non-decreasing"),
])
def test_invalid_input_rejected_before_device(native, breaker, msg):
    from igaos_gb300 import capi
    lp = _tiny()
    a = dict(m=lp.m, n=lp.n, ap=lp.ap.copy(), ai=lp.ai.copy(), ax=lp.ax.copy(),
             c=lp.c.copy(), cl=lp.cl.copy(), cu=lp.cu.copy(), rmin=lp.rmin.copy(),
             rmax=lp.rmax.copy())
    breaker(a)
    h = C.c_void_p()
    o = capi.default_options()
    d = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))
    i = lambda x: x.ctypes.data_as(C.POINTER(C.c_int))
    rc = native.igaos_pdhg_create(C.byref(h), a["m"], a["n"], int(lp.ap[lp.m]), i(a["ap"]),
                                  i(a["ai"]), d(a["ax"]), None, None, None, d(a["c"]),
                                  d(a["cl"]), d(a["cu"]), d(a["rmin"]), d(a["rmax"]), 0.0,
                                  C.byref(o))
    assert rc == capi.ERR_INVALID
    assert msg in capi.last_error()
    assert not h.value


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_device_is_an_honest_error(native):
    from igaos_gb300 import capi
    r = capi.solve_lp(_tiny())
    assert r["rc"] == capi.ERR_NODEVICE
    assert r["status_name"] == "error"
    assert "no CUDA device" in r["message"]


def test_null_handles(native):
    from igaos_gb300 import capi
    assert native.igaos_pdhg_solve(None, None, None, None, None) == capi.ERR_INVALID
    assert native.igaos_pdhg_set_start(None, None, None) == capi.ERR_INVALID
    assert "NULL" in capi.last_error()
    native.igaos_pdhg_destroy(None)  # no-op


def test_helper_entries_reject_bad_arguments(native):
    """The certificate test and the gather-rate calibration refuse bad
    arguments with IGAOS_PDHG_ERR_INVALID and a message, before any device
    work."""
    import ctypes as C
    from igaos_gb300 import capi
    kind = C.c_int(-1)
    assert native.igaos_pdhg_ray_certificate(2, 2, *([None] * 11), C.byref(kind)) == capi.ERR_INVALID
    assert "NULL" in capi.last_error()
    assert native.igaos_pdhg_ray_certificate(-1, 2, *([None] * 11), C.byref(kind)) == capi.ERR_INVALID
    out = C.c_double(0.0)
    assert native.igaos_pdhg_gather_rate(4, -1, C.byref(out)) == capi.ERR_INVALID
    assert "log2_words" in capi.last_error()


def test_presolve_entries_reject_bad_arguments(native):
    """The host presolve entries refuse NULL handles and outputs with
    IGAOS_PDHG_ERR_INVALID; a presolved problem handle refuses the
    inspection entry points (their sizes are the reduced LP's)."""
    import ctypes as C
    from igaos_gb300 import capi
    oc = C.c_int(-1)
    assert native.igaos_pdhg_presolve(2, 2, 0, *([None] * 8), 0.0, None, C.byref(oc)) == \
        capi.ERR_INVALID
    assert native.igaos_pdhg_presolved_info(None, None, None, None, None, None) == capi.ERR_INVALID
    assert native.igaos_pdhg_postsolve(None, None, None, None, None) == capi.ERR_INVALID
    native.igaos_pdhg_presolved_destroy(None)  # no-op


C_PROGRAM = r"""
#include <math.h>
#include <stdio.h>
#include "igaos_pdhg.h"
int main(void) {
    /* min x1 + 2 x2 + 3 x3 s.t. x1 + x2 + x3 = 4, x1, x2 in [0, 10], x3 free */
    const int ap[2] = {0, 3}, ai[3] = {0, 1, 2};
    const double ax[3] = {1, 1, 1}, c[3] = {1, 2, 3}, cl[3] = {0, 0, -INFINITY};
    const double cu[3] = {10, 10, INFINITY}, rmin[1] = {4}, rmax[1] = {4};
    igaos_pdhg_presolved* ps = NULL;
    int outcome = -1, m = -1, n = -1;
    int64_t nnz = -1, counts[6];
    double k = 0.0, x[3], y[1], x0[3] = {0, 0, 0}, xv[3], yv[1];
    signed char basis[4];
    igaos_pdhg_crossover_info info;
    if (igaos_pdhg_presolve(1, 3, 3, ap, ai, ax, c, cl, cu, rmin, rmax, 0.0, &ps, &outcome))
        return 1;
    igaos_pdhg_presolved_info(ps, &m, &n, &nnz, &k, counts);
    igaos_pdhg_postsolve(ps, NULL, NULL, x, y);
    igaos_pdhg_presolved_destroy(ps);
    if (igaos_pdhg_crossover(1, 3, 3, ap, ai, ax, c, cl, cu, rmin, rmax, x0, xv, yv, basis,
                             &info))
        return 2;
    printf("%d %d %d %g | %g %g %g %g | %d %g %g %g %g\n", outcome, m, n, k, x[0], x[1], x[2],
           y[0], info.status, xv[0], xv[1], xv[2], yv[0]);
    return 0;
}
"""


def test_c_program_calls_the_host_entries(native, tmp_path):
    """The header is plain C99 and the library links into a C program, which
    presolves, postsolves and crosses over an LP with no device: the binding
    a cgo / FFI user writes."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not present")
    src = tmp_path / "t.c"
    src.write_text(C_PROGRAM)
    pkg = os.path.join(ROOT, "igaos_gb300")
    exe = tmp_path / "t"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-L", pkg, "-ligaos_pdhg", f"-Wl,-rpath,{pkg}", "-lm", "-o",
                    str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert out == ["0", "0", "0", "-18", "|", "10", "10", "-16", "-3", "|", "0", "10", "10",
                   "-16", "-3"], out
