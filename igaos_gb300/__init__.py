"""GB300-native PDHG LP engine with the IGAOS engine surface.

Drop-in surface (reference python/igaos/__init__.py, python/igaos_bindings.cpp):
    solve(path, time_limit=120, tolerance=1e-4, max_iterations=500000,
          presolve=True, seed=0, engine="auto")  -> Solution
    read_mps(path) -> Model;  Model, Solution, Status, has_pdhg
Only engine="pdhg" is carried by this build; it runs hand-written sm_103a
kernels through the C ABI in include/igaos_pdhg.h.

GB300 extensions:
    solve(..., precision="fp64"|"fp32-refine"|"fp32", detect_infeasibility=False,
          pdhg_presolve=False, crossover=False)
    capi.Problem / capi.solve_lp  -- LPs given as CSR arrays (C ABI via ctypes)
    capi.Presolved                -- the engine's presolve / postsolve on the host
    capi.crossover                -- host crossover from any point to an optimal vertex
    generators                    -- seeded synthetic LPs of the benchmark shapes
"""
from __future__ import annotations

__version__ = "0.1.0"

_CORE_NAMES = ("Model", "Solution", "Status", "has_pdhg", "read_mps", "solve")


def __getattr__(name):
    if name in _CORE_NAMES:
        try:
            from . import _core
        except ImportError as e:  # pragma: no cover - depends on the build
            raise ImportError(
                "igaos_gb300._core is not built; run igaos_gb300.build.build()") from e
        return getattr(_core, name)
    raise AttributeError(name)


def solve_arrays(lp, precision="fp64", **opts):
    """Solve an LP given as arrays (see generators.LPData) on the GPU."""
    from . import capi
    return capi.solve_lp(lp, precision=precision, **opts)
