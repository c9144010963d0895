"""The split-precision operator product (ASEND_METHOD_SPLIT): FP64 values held
as FP32 hi + lo pairs, products in compensated FP32 arithmetic.

Tolerances:
  * y = A x against the FP64 product: 1e-13 relative (norm-wise), and each
    row within 1e-13 of sum_j |A_ij| |x_j| (the scale of its terms);
  * solves to rel_tol 1e-10 with the split method match the FP64 method's
    solution to 1e-8 and converge in about the same iteration count (within
    3 or 15 %: the multigrid CG's FP32 V-cycle makes the paths differ).
"""
import numpy as np
import pytest

from asend3d_gb300 import _lib, configs
from asend3d_gb300.solver import GpuSolver

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def test_split_product_matches_fp64(gpu_lib, oracle_lib):
    import scipy.sparse as sp

    p = configs.block_large(nx=40, ny=8, nz=8, seed=3)
    g = GpuSolver(p)
    g.assemble(precision=64)
    rng = np.random.default_rng(0)
    o = oracle_lib.Oracle(p)
    rp, col, val = g.csr(which=0)
    Aabs = sp.csr_matrix((np.abs(val), col, rp), shape=(g.n_dof, g.n_dof))
    for x in (rng.standard_normal(g.n_dof), np.ones(g.n_dof), rng.standard_normal(g.n_dof) * 1e-3 + 1.0):
        y64 = g.apply(x, 64)
        y48 = g.apply(x, 48)
        assert rel(y48, y64) < 1e-13
        scale = Aabs @ np.abs(x)
        assert np.all(np.abs(y48 - y64) <= 1e-13 * scale + 1e-300)
        assert rel(y64, o.apply(x)) < 1e-11  # the FP64 product itself against the oracle
    g.close()


@pytest.mark.parametrize("precond", [_lib.PC_JACOBI, _lib.PC_MG])
def test_split_solve_matches_fp64(gpu_lib, precond):
    p = configs.block_large(nx=30, ny=6, nz=6, seed=9)
    g = GpuSolver(p)
    g.assemble(precision=64)
    u64, rc, st64 = g.static_solve(method=_lib.METHOD_FP64, precond=precond, rel_tol=1e-10)
    assert rc == 0
    u48, rc, st48 = g.static_solve(method=_lib.METHOD_SPLIT, precond=precond, rel_tol=1e-10)
    assert rc == 0 and st48["rel_residual"] <= 1e-10
    assert rel(u48[0], u64[0]) < 1e-8
    # the flexible CG with an FP32 V-cycle follows a slightly different path
    assert abs(st48["iterations"] - st64["iterations"]) <= max(3, st64["iterations"] // 7)
    L64, g64, _, _ = g.adjoint_gradient(method=_lib.METHOD_FP64, precond=precond, rel_tol=1e-10)
    L48, g48, _, _ = g.adjoint_gradient(method=_lib.METHOD_SPLIT, precond=precond, rel_tol=1e-10)
    assert L48 == pytest.approx(L64, rel=1e-9)
    g.close()


def test_mg_kernel_timing_entry(gpu_lib):
    p = configs.block_large(nx=20, ny=4, nz=4, seed=1)
    g = GpuSolver(p)
    g.assemble(precision=64)
    for k in range(3):
        ms, by = g.time_mg_kernel(k, _lib.METHOD_SPLIT, 3)
        assert ms > 0 and by > 0
    g.close()
