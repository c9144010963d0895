"""Solver-configuration autotuner: selection, the give-up rule, failures and
the cache, with a stand-in solver that reports scripted device times (the
GPU run is in test_gpu_parity.py)."""
from types import SimpleNamespace

import pytest

from asend3d_gb300 import _lib, autotune


class FakeSolver:
    """static_solve_device returns scripted (rc, ms, iterations) per precond."""

    def __init__(self, table, structured=True, product_ms=None):
        n = 4 if structured else 3
        self.p = SimpleNamespace(mesh=SimpleNamespace(elem_type=8, nx=n, ny=2, nz=2, n_elems=16))
        self.n_dof = 135
        self.n_cases = 1
        self.table = table
        self.product_ms = product_ms or {v: 20.0 for v in _lib.PRODUCT_VARIANTS}
        self.variant = _lib.PRODUCT_DEFAULT
        self.calls = []

    def set_product_variant(self, v):
        self.variant = v

    def static_solve_device(self, **o):
        self.calls.append(dict(o, product=self.variant))
        if o["method"] == _lib.METHOD_SPLIT:  # None: that shape's solve hits its cap
            ms = self.product_ms[self.variant]
            return (_lib.ASEND_MAX_ITER if ms is None else _lib.ASEND_OK), {"ms_solve": ms or 0.0, "iterations": 10}
        rc, ms, it = self.table[(o["precond"], o["graph_iters"])]
        return rc, {"ms_solve": ms, "iterations": it}


def table(best=(_lib.PC_MG, 8), fail=()):
    t = {}
    for pc in (_lib.PC_JACOBI, _lib.PC_BLOCK, _lib.PC_MG):
        for g in autotune.DEFAULT_GRAPH_ITERS:
            ms = {_lib.PC_JACOBI: 50.0, _lib.PC_BLOCK: 40.0, _lib.PC_MG: 10.0}[pc] + g * 0.1
            t[(pc, g)] = (_lib.ASEND_OK, ms, 10)
    t[best] = (_lib.ASEND_OK, 1.0, 10)
    for f in fail:
        t[f] = (_lib.ASEND_MAX_ITER, t[f][1], 10)
    return t


def test_picks_fastest_converged():
    s = FakeSolver(table())
    best, trials = autotune.tune(s)
    assert best == {"method": _lib.METHOD_FP64, "precond": _lib.PC_MG, "graph_iters": 8}
    assert len(trials) == 12 + len(_lib.PRODUCT_VARIANTS) and all(c["rel_tol"] == 1e-8 for c in s.calls)
    assert s.variant == _lib.PRODUCT_DEFAULT  # restored after the trials


def test_picks_product_shape():
    """The split multigrid CG's outer-product shapes are candidates of their
    own; each trial runs with its shape installed."""
    ms = {v: 5.0 + v for v in _lib.PRODUCT_VARIANTS}
    ms[_lib.PRODUCT_STAGED_3x2] = 0.5
    s = FakeSolver(table(), product_ms=ms)
    best, trials = autotune.tune(s, repeats=1)
    assert best == {"method": _lib.METHOD_SPLIT, "precond": _lib.PC_MG, "graph_iters": 8,
                    "product": _lib.PRODUCT_STAGED_3x2}
    split_calls = [c for c in s.calls if c["method"] == _lib.METHOD_SPLIT]
    assert [c["product"] for c in split_calls] == list(_lib.PRODUCT_VARIANTS)
    assert all("product" not in t or t["method"] == _lib.METHOD_SPLIT for t in trials)


def test_failed_candidates_are_dropped():
    s = FakeSolver(table(best=(_lib.PC_MG, 8), fail=[(_lib.PC_MG, 8)]))
    best, trials = autotune.tune(s)
    assert best["precond"] == _lib.PC_MG and best["graph_iters"] == 4
    assert [t for t in trials if t["precond"] == _lib.PC_MG and t["graph_iters"] == 8][0]["ms"] is None


def test_unstructured_meshes_skip_multigrid():
    s = FakeSolver(table(best=(_lib.PC_BLOCK, 16)), structured=False)
    best, trials = autotune.tune(s)
    assert best["precond"] == _lib.PC_BLOCK and all(t["precond"] != _lib.PC_MG for t in trials)


def test_give_up_stops_repeats_of_slow_candidates():
    s = FakeSolver(table())
    autotune.tune(s, candidates=[{"method": 0, "precond": _lib.PC_MG, "graph_iters": 8},
                                 {"method": 0, "precond": _lib.PC_JACOBI, "graph_iters": 4}], repeats=3)
    jac = [c for c in s.calls if c["precond"] == _lib.PC_JACOBI]
    assert len(jac) == 1  # 50 ms > 3 x 1 ms after its first run


def test_nothing_converges_raises():
    s = FakeSolver(table(fail=[(pc, g) for pc in (0, 1, 3) for g in autotune.DEFAULT_GRAPH_ITERS]),
                   product_ms={v: None for v in _lib.PRODUCT_VARIANTS})
    with pytest.raises(RuntimeError, match="no candidate"):
        autotune.tune(s)


def test_cache_file(tmp_path):
    f = tmp_path / "tune.json"
    s = FakeSolver(table())
    best, _ = autotune.tune(s, cache=f)
    s2 = FakeSolver(table(best=(_lib.PC_JACOBI, 4)))
    best2, _ = autotune.tune(s2, cache=f)
    assert best2 == best and s2.calls == []  # served from the cache
    assert autotune.problem_key(s) in f.read_text()
