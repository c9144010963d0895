"""Solver-configuration autotuner.

Times whole solves of the assembled operator, to the caller's tolerance, for
each candidate (method, preconditioner, PCG iterations per captured CUDA
graph, and for the multigrid CG with the split operator the shape of its
outer product kernel: register-fed, or staged through shared memory with a
given number of block-column groups per stage and stages per warp) and keeps
the fastest that converged.  The device time of each trial
comes from the library's event timing (asend_solve_stats.ms_solve); a trial
that hits its iteration cap, or runs longer than `give_up` times the best so
far, is dropped.  Results are cached per problem class (element type, DOF,
block structure, right-hand sides), in memory or in a JSON file.

The other kernels' CTA shapes and the per-chunk right-hand-side count are
fixed at compile time; what is tuned here is what the library takes at run
time.
"""
from __future__ import annotations

import json
from pathlib import Path

from . import _lib

DEFAULT_GRAPH_ITERS = (4, 8, 16, 32)


def default_candidates(structured: bool) -> list[dict]:
    pcs = [_lib.PC_JACOBI, _lib.PC_BLOCK] + ([_lib.PC_MG] if structured else [])
    out = []
    for pc in pcs:
        for g in DEFAULT_GRAPH_ITERS:
            out.append({"method": _lib.METHOD_FP64, "precond": pc, "graph_iters": g})
    if structured:
        for v in _lib.PRODUCT_VARIANTS:
            out.append({"method": _lib.METHOD_SPLIT, "precond": _lib.PC_MG, "graph_iters": 8, "product": v})
    return out


def problem_key(solver) -> str:
    m = solver.p.mesh
    structured = m.elem_type in (8, 81) and m.nx * m.ny * m.nz == m.n_elems
    return f"type{m.elem_type}-dof{solver.n_dof}-{'block' if structured else 'mesh'}-rhs{max(1, solver.n_cases)}"


def tune(solver, rel_tol=1e-8, candidates=None, give_up=3.0, repeats=2, cache: dict | str | Path | None = None,
         max_iter=0):
    """Return (best options dict, trial table).  `solver` is an assembled
    GpuSolver (or any object with static_solve_device(**opts) -> (rc, stats),
    p.mesh, n_dof and n_cases)."""
    key = problem_key(solver)
    store, path = _load_cache(cache)
    if key in store:
        return dict(store[key]["best"]), store[key]["trials"]
    set_variant = getattr(solver, "set_product_variant", lambda v: None)
    m = solver.p.mesh
    structured = m.elem_type in (8, 81) and m.nx * m.ny * m.nz == m.n_elems
    cands = candidates if candidates is not None else default_candidates(structured)
    trials, best, best_ms = [], None, float("inf")
    for c in cands:
        opts = dict(c, rel_tol=rel_tol, max_iter=max_iter)
        set_variant(opts.pop("product", _lib.PRODUCT_DEFAULT))
        ms_runs, rc, st = [], 0, {}
        for _ in range(max(1, repeats)):
            rc, st = solver.static_solve_device(**opts)
            if rc != _lib.ASEND_OK:
                break
            ms_runs.append(float(st["ms_solve"]))
            if ms_runs[-1] > give_up * best_ms:
                break
        ok = rc == _lib.ASEND_OK and len(ms_runs) > 0
        ms = min(ms_runs) if ms_runs else float("inf")
        trials.append({**c, "rc": int(rc), "ms": ms if ok else None, "iterations": int(st.get("iterations", 0))})
        if ok and ms < best_ms:
            best, best_ms = dict(c), ms
    set_variant(_lib.PRODUCT_DEFAULT)
    if best is None:
        raise RuntimeError(f"no candidate configuration converged for {key}: {trials}")
    store[key] = {"best": best, "trials": trials}
    _save_cache(store, path)
    return dict(best), trials


def tune_product(solver, n_launch=20):
    """The fastest shape of the multigrid CG's split outer product on this
    operator: each shape's device time over n_launch back-to-back launches
    (asend_time_mg_kernel, the kernel alone).  The shapes give bit-identical
    results, so this changes only the time.  Installs the winner and returns
    (variant, {variant: ms per launch})."""
    times = {}
    for v in _lib.PRODUCT_VARIANTS:
        solver.set_product_variant(v)
        times[v] = solver.time_mg_kernel(0, _lib.METHOD_SPLIT, n_launch)[0]
    best = min(times, key=times.get)
    solver.set_product_variant(best)
    return best, times


def _load_cache(cache):
    if cache is None:
        return {}, None
    if isinstance(cache, dict):
        return cache, None
    path = Path(cache)
    return (json.loads(path.read_text()) if path.exists() else {}), path


def _save_cache(store, path):
    if path is not None:
        path.write_text(json.dumps(store, indent=1, sort_keys=True))
