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


def _solve_with_each_product_shape(g, **kw):
    """Solve + compliance gradient with every product shape (fused V-cycle
    tail on, overlapped launches), and with the register-fed shape, the tail
    off (one launch per coarse level and step) and fully serialised launches."""
    out = {}
    runs = [(v, True) for v in _lib.PRODUCT_VARIANTS] + [(_lib.PRODUCT_REGISTERS, False)]
    for v, tail in runs:
        g.set_product_variant(v)
        g.mg_set_fused_tail(tail)
        g.set_launch_overlap(tail)  # the serialised launches ride with the unfused tail
        u, rc, st = g.static_solve(method=_lib.METHOD_SPLIT, precond=_lib.PC_MG, **kw)
        assert rc == 0, (v, tail, st)
        L, gE, rc2, _ = g.adjoint_gradient(method=_lib.METHOD_SPLIT, precond=_lib.PC_MG, **kw)
        assert rc2 == 0, (v, tail)
        out[(v, tail)] = (u, st["iterations"], L, gE)
    g.set_product_variant(_lib.PRODUCT_DEFAULT)
    g.mg_set_fused_tail(True)
    g.set_launch_overlap(True)
    return out


def _assert_identical(out):
    u0, it0, L0, g0 = out[(_lib.PRODUCT_REGISTERS, False)]
    for k, (u, it, L, gE) in out.items():
        np.testing.assert_array_equal(u, u0, err_msg=f"shape, tail {k}")
        assert it == it0 and L == L0, k
        np.testing.assert_array_equal(gE, g0, err_msg=f"shape, tail {k}")


def test_product_shapes_bit_identical_single_block(gpu_lib):
    """Every shape of the multigrid CG's outer split product -- register-fed,
    or staged through shared memory by bulk copies with 2-4 groups per stage
    and 2-3 stages per warp -- and the fused V-cycle tail against one launch
    per coarse level give the same bits: solution, iteration count,
    compliance and its gradient.  40x8x8 block: slices with ragged row
    lengths, stage counts that do not divide the slice lengths."""
    p = configs.block_large(nx=40, ny=8, nz=8, seed=5)
    g = GpuSolver(p)
    g.assemble(precision=64)
    _assert_identical(_solve_with_each_product_shape(g, rel_tol=1e-10))
    g.close()


def test_product_shapes_bit_identical_batched(gpu_lib):
    """The same on a stacked batch of three uneven instances with 4 load
    cases each (instances start on CTA boundaries; some warps of a CTA own
    no slice at the end of the stack)."""
    prob, node_ptr, elem_ptr, inst = configs.batch_uq(which=[3, 10, 17])
    dims = [(q.mesh.nx, q.mesh.ny, q.mesh.nz) for q in inst]
    g = GpuSolver(prob, instances=node_ptr, blocks=dims)
    g.assemble(precision=64)
    _assert_identical(_solve_with_each_product_shape(g, rel_tol=1e-10))
    g.close()


def test_fused_tail_bit_identical_on_many_instances(gpu_lib):
    """A stack of the sweep's 16 smallest instances (enough blocks for the
    V-cycle's fused coarse tail, one CTA per instance): solution, iterations,
    compliance and gradient equal those of one launch per level and step, and
    the fused run launches fewer kernels."""
    sizes = sorted(range(64), key=lambda k: np.prod([d + 1 for d in configs.batch_dims(k, 7)]))
    prob, node_ptr, elem_ptr, inst = configs.batch_uq(which=sorted(sizes[:16]))
    dims = [(q.mesh.nx, q.mesh.ny, q.mesh.nz) for q in inst]
    g = GpuSolver(prob, instances=node_ptr, blocks=dims)
    g.assemble(precision=64)
    out, launches = {}, {}
    for tail in (False, True):
        g.mg_set_fused_tail(tail)
        n0 = g.kernel_launches
        u, rc, st = g.static_solve(method=_lib.METHOD_SPLIT, precond=_lib.PC_MG, rel_tol=1e-10)
        assert rc == 0, st
        L, gE, rc2, _ = g.adjoint_gradient(method=_lib.METHOD_SPLIT, precond=_lib.PC_MG, rel_tol=1e-10)
        assert rc2 == 0
        launches[tail] = g.kernel_launches - n0
        out[tail] = (u, st["iterations"], L, gE)
    np.testing.assert_array_equal(out[True][0], out[False][0])
    assert out[True][1] == out[False][1] and out[True][2] == out[False][2]
    np.testing.assert_array_equal(out[True][3], out[False][3])
    assert launches[True] < launches[False]
    g.close()


def test_split_only_assembly(gpu_lib):
    """precision 48: the operator's hi / lo values summed in FP32 pairs, with
    no FP64 copy.  The split multigrid solve on it (true residuals from the
    pairs) reaches 1e-10 and its solution, compliance and gradient match the
    solve on the FP64 assembly; the FP64 copy rebuilt on demand (CSR export,
    an FP64 solve) equals the FP64 assembly's values to 1e-13 of max|K| on
    every slot without a penalty term, and to 2^-46 of the value on the
    penalty slots (K + sf C^T C with sf = 1e5 max|K|, held as a 48-bit pair
    in either assembly)."""
    p = configs.block_large(nx=40, ny=8, nz=8, seed=5)
    g = GpuSolver(p)
    kw = dict(method=_lib.METHOD_SPLIT, precond=_lib.PC_MG, rel_tol=1e-10)
    g.assemble(precision=64)
    rp0, c0, v0 = g.csr(which=0)
    rp2, c2, w0 = g.csr(which=2)
    u64, rc, st = g.static_solve(**kw)
    assert rc == 0
    L64, g64, _, _ = g.adjoint_gradient(**kw)
    g.assemble(precision=48)
    u48, rc, st48 = g.static_solve(**kw)
    assert rc == 0 and st48["rel_residual"] <= 1e-10, st48
    L48, g48, rc2, _ = g.adjoint_gradient(**kw)
    assert rc2 == 0
    assert rel(u48, u64) < 1e-9
    assert L48 == pytest.approx(L64, rel=1e-9)
    assert rel(g48, g64) < 1e-8
    kmax = np.abs(w0).max()
    rp2b, c2b, w48 = g.csr(which=2)  # rebuilds the FP64 values from the pairs
    np.testing.assert_array_equal(rp2b, rp2)
    np.testing.assert_array_equal(c2b, c2)
    rp0b, c0b, v48 = g.csr(which=0)
    np.testing.assert_array_equal(c0b, c0)
    np.testing.assert_array_equal(c0, c2)
    pen = v0 != w0  # slots holding K + sf C^T C: a pair carries K there only to 2^-48 of sf
    assert pen.any() and not pen.all()
    assert np.abs(w48 - w0)[~pen].max() <= 1e-13 * kmax
    assert np.all(np.abs(v48 - v0)[pen] <= 2.0 ** -46 * np.abs(v0)[pen])
    # an FP64 solve after a split-only assembly runs on the rebuilt values
    uf, rcf, _ = g.static_solve(method=_lib.METHOD_FP64, precond=_lib.PC_MG, rel_tol=1e-10)
    assert rcf == 0 and rel(uf, u64) < 1e-9
    g.close()
