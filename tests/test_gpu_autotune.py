"""The solver-configuration autotuner on the GPU: every candidate of the
structured 20x4x4 cantilever is timed, the choice converges to the target
and is the fastest converged trial."""
import pytest

from asend3d_gb300 import _lib, autotune, configs
from asend3d_gb300.solver import GpuSolver

pytestmark = pytest.mark.gpu


def test_tune_cantilever(gpu_lib):
    g = GpuSolver(configs.cantilever_small())
    g.assemble(precision=64)
    best, trials = autotune.tune(g, rel_tol=1e-8, repeats=1)
    assert len(trials) == len(autotune.default_candidates(True)) and best in autotune.default_candidates(True)
    ok = [t for t in trials if t["ms"] is not None]
    assert min(t["ms"] for t in ok) == [t for t in ok if all(t[k] == best[k] for k in best)][0]["ms"]
    rc, st = g.static_solve_device(rel_tol=1e-8, **best)
    assert rc == _lib.ASEND_OK and st["rel_residual"] <= 1e-8
    g.close()
