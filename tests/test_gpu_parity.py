"""GPU parity tests: the sm_103a library through its C ABI vs the FP64 oracle.

Tolerances (written here, per quantity):
  * assembly pattern (row pointers, column indices) and element colouring
    validity: bit-exact;
  * FP64-assembled operator values: 1e-12 relative to max|K| (closed-form
    3x3 adjugate vs the reference's Givens-QR inverse differ by rounding);
  * FP32-assembled values: 2e-6 relative to max|K|;
  * displacements after a solve to rel. residual tol: 10 * tol * cond-margin
    (checked as ||u - u_ref|| / ||u_ref|| <= 1e-7 at tol 1e-10);
  * adjoint gradients: 1e-6 relative (norm-wise), as the benchmark target.
"""
from pathlib import Path

import numpy as np
import pytest

from asend3d_gb300 import _lib, configs
from asend3d_gb300.mesh import block_hex8, block_tet4
from asend3d_gb300.solver import AsendError, GpuSolver, Problem

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


@pytest.fixture(scope="module")
def small(gpu_lib, oracle_lib):
    p = configs.cantilever_small()
    g = GpuSolver(p)
    g.assemble(precision=64)
    o = oracle_lib.Oracle(p)
    yield p, g, o
    g.close()


def test_assembly_pattern_bit_exact_and_values(small):
    p, g, o = small
    rp, col, val = g.csr(which=2)  # operator without the penalty terms
    orp, ocol, oval = o.csr(which=0)
    assert np.array_equal(rp, orp)
    assert np.array_equal(col, ocol)
    scale = np.abs(oval).max()
    assert np.abs(val - oval).max() <= 2e-11 * scale


def test_assembly_fp32_values(gpu_lib, oracle_lib):
    p = configs.cantilever_small()
    g = GpuSolver(p)
    g.assemble(precision=32)
    _, _, val = g.csr(which=2)
    _, _, oval = oracle_lib.Oracle(p).csr(which=0)
    assert np.abs(val - oval).max() <= 2e-6 * np.abs(oval).max()
    g.close()


def test_penalty_and_operator(small):
    p, g, o = small
    _, _, val = g.csr(which=0)
    _, _, oval = o.csr(which=2)
    assert np.abs(val - oval).max() <= 2e-11 * np.abs(oval).max()
    x = np.random.default_rng(0).standard_normal(o.n_dof)
    y_ref = o.apply(x)
    assert rel(g.apply(x, 64), y_ref) < 1e-11
    assert rel(g.apply(x, 32), y_ref) < 2e-6


def test_colouring_valid(small):
    p, g, o = small
    colour, n = g.coloring()
    assert n == 8  # structured hex: 2 x 2 x 2 parity colouring
    conn = p.mesh.conn
    for c in range(n):
        nodes = conn[colour == c].ravel()
        assert len(np.unique(nodes)) == len(nodes), f"colour {c} has elements sharing a node"


@pytest.mark.parametrize("method,pc", [(_lib.METHOD_FP64, _lib.PC_JACOBI), (_lib.METHOD_MIXED, _lib.PC_JACOBI),
                                       (_lib.METHOD_MIXED, _lib.PC_BLOCK), (_lib.METHOD_FP64, _lib.PC_BLOCK)])
def test_static_solve_parity(small, method, pc):
    p, g, o = small
    gold = np.load(GOLD / "cantilever_small.npz")
    u, rc, st = g.static_solve(method=method, precond=pc, rel_tol=1e-10)
    assert rc == 0, st
    assert st["rel_residual"] <= 1e-10
    f = o.loads()[0] + o.penalty_rhs()
    true_res = np.linalg.norm(f - o.apply(u[0])) / np.linalg.norm(f)
    assert true_res <= 1.01e-10
    assert rel(u[0], gold["u"]) < 1e-7
    assert np.allclose(g.load_vector(0), f, rtol=1e-13, atol=0)


def test_adjoint_tip_gradient_golden(small):
    p, g, o = small
    gold = np.load(GOLD / "cantilever_small.npz")
    g.static_solve(method=_lib.METHOD_FP64, precond=_lib.PC_MG, rel_tol=1e-11)
    L, dLdE, rc, st = g.adjoint_gradient(method=_lib.METHOD_FP64, precond=_lib.PC_MG, rel_tol=1e-11)
    assert rc == 0
    assert L == pytest.approx(float(gold["L"]), rel=1e-9)
    assert rel(dLdE, gold["dLdE"]) < 1e-6
    dLdD = g.design_var_gradient(dLdE)
    assert len(dLdD) == 80
    assert rel(dLdD, gold["dLdD"]) < 1e-6


def test_compliance_gradient_lognormal(gpu_lib, oracle_lib):
    p = configs.block_large(nx=24, ny=6, nz=6, seed=5)
    g = GpuSolver(p)
    g.assemble()
    u, rc, _ = g.static_solve(method=_lib.METHOD_FP64, precond=_lib.PC_MG, rel_tol=1e-11)
    assert rc == 0
    L, dLdE, rc, _ = g.adjoint_gradient()
    o = oracle_lib.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    ur, _, _ = o.solve(f, precond=oracle_lib.PC_DIRECT)
    gr, _, _, _ = o.adjoint(ur, lam=ur)
    assert L == pytest.approx(f @ ur, rel=1e-9)
    assert rel(dLdE, gr) < 1e-6
    # homogeneity checksum: sum_e E_e dC/dE_e = -C (penalty held fixed: 1e-4)
    assert np.dot(p.E, dLdE) == pytest.approx(-L, rel=1e-4)
    g.close()


def test_multi_rhs_batch(gpu_lib, oracle_lib):
    p = configs.batch_instance(3)
    g = GpuSolver(p)
    g.assemble()
    assert g.n_cases == 4
    u, rc, st = g.static_solve(rel_tol=1e-10)
    assert rc == 0 and st["n_rhs"] == 4
    o = oracle_lib.Oracle(p)
    for k, fk in enumerate(o.loads()):
        f = fk + o.penalty_rhs()
        ur, _, _ = o.solve(f, precond=oracle_lib.PC_DIRECT)
        assert rel(u[k], ur) < 1e-7
    g.close()


def test_tet4_golden(gpu_lib):
    gold = np.load(GOLD / "tet_block.npz")
    m = block_tet4(4, 2, 2, 1.0, 0.5, 0.5)
    p = Problem(m, np.full(m.n_elems, 7.0e10), np.full(m.n_elems, 0.33), None)
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    p.add_elem_set("all", np.arange(m.n_elems, dtype=np.int32))
    p.add_surface_traction("all", (1.0, 0.0, 0.0), (0.0, 0.0, -1.0e6))
    g = GpuSolver(p)
    g.assemble()
    u, rc, _ = g.static_solve(method=_lib.METHOD_FP64, rel_tol=1e-11)
    assert rc == 0
    assert rel(u[0], gold["u"]) < 1e-8
    g.close()


def test_newmark_parity(gpu_lib, oracle_lib):
    p = configs.cantilever_small(nx=10, ny=2, nz=2)
    dt, beta, gamma = 1e-4, 0.25, 0.5
    n = 60
    t = np.arange(n) * dt
    amp = np.exp(-0.5 * ((t - 2e-3) / 5e-4) ** 2)
    tip = int(p.node_sets["tip"][0])
    g = GpuSolver(p)
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    hist, u, rc, st = g.newmark(amp, probe_dof=3 * tip + 2, rel_tol=1e-12)
    assert rc == 0
    o = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    href, uref, rc2, _ = o.newmark(n, dt, beta, gamma, o.loads()[0], amp, 3 * tip + 2, precond=oracle_lib.PC_DIRECT)
    assert rc2 == 0
    assert rel(hist, href) < 1e-8
    assert rel(u, uref) < 1e-8
    g.close()


def test_input_errors_are_reported(gpu_lib):
    m = block_hex8(2, 1, 1, 2.0, 1.0, 1.0)
    bad = Problem(m, np.array([1e9, -1.0]), np.full(2, 0.3))
    with pytest.raises(AsendError, match="modulus"):
        GpuSolver(bad)
    p = Problem(m, np.full(2, 1e9), np.full(2, 0.3))
    g = GpuSolver(p)
    with pytest.raises(AsendError, match="assemble first"):
        g.static_solve()
    g.close()


def test_zero_and_nonfinite_loads(gpu_lib):
    p = configs.cantilever_small(nx=4, ny=2, nz=2)
    p.loads = [[("vector", np.zeros(p.mesh.n_dof))]]
    g = GpuSolver(p)
    g.assemble()
    u, rc, _ = g.static_solve()
    assert rc == 0 and not np.any(u)
    f = np.zeros(p.mesh.n_dof)
    f[5] = np.nan
    p.loads = [[("vector", f)]]
    g.set_loads()
    u, rc, st = g.static_solve()
    assert rc == _lib.ASEND_NONFINITE
    g.close()


def test_full_size_block_properties(gpu_lib):
    """Full-size 200x40x40 block (1.01 M DOF): size-independent checks."""
    p = configs.block_large()
    g = GpuSolver(p)
    g.assemble(precision=64)
    rc, st = g.static_solve_device(method=_lib.METHOD_FP64, precond=_lib.PC_MG, rel_tol=1e-8)
    assert rc == 0 and st["rel_residual"] <= 1e-8
    assert st["iterations"] < 300
    u_mg = g.solution(0)
    L, dLdE, rc, _ = g.adjoint_gradient()
    assert rc == 0 and L > 0
    assert np.all(dLdE < 0)  # stiffening any element lowers the compliance
    assert np.dot(p.E, dLdE) == pytest.approx(-L, rel=1e-4)
    f = g.load_vector(0)
    res = np.linalg.norm(f - g.apply(u_mg, 64)) / np.linalg.norm(f)
    assert res <= 1.05e-8
    rc, st64 = g.static_solve_device(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-8)
    assert rc == 0
    assert rel(u_mg, g.solution(0)) < 1e-6
    g.close()


@pytest.mark.parametrize("method", [_lib.METHOD_FP64])
def test_multigrid_small_parity(small, method):
    p, g, o = small
    gold = np.load(GOLD / "cantilever_small.npz")
    u, rc, st = g.static_solve(method=method, precond=_lib.PC_MG, rel_tol=1e-10)
    assert rc == 0, st
    nl = g.mg_levels
    dims = [g.mg_level_info(l)["dims"] for l in range(nl)]
    assert dims[:2] == [(20, 4, 4), (10, 2, 2)]  # two-cell axes wait until all axes are thin
    cx, cy, cz = dims[-1]
    assert 3 * (cx + 1) * (cy + 1) * (cz + 1) <= 256
    assert st["iterations"] < 60
    f = o.loads()[0] + o.penalty_rhs()
    assert np.linalg.norm(f - o.apply(u[0])) / np.linalg.norm(f) <= 1.01e-10
    assert rel(u[0], gold["u"]) < 1e-7


def test_multigrid_lognormal_matches_oracle(gpu_lib, oracle_lib):
    p = configs.block_large(nx=30, ny=6, nz=6, seed=9)
    g = GpuSolver(p)
    g.assemble()
    u, rc, st = g.static_solve(method=_lib.METHOD_FP64, precond=_lib.PC_MG, rel_tol=1e-11)
    assert rc == 0 and st["iterations"] < 80
    o = oracle_lib.Oracle(p)
    ur, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert rel(u[0], ur) < 1e-8
    g.close()


def test_batched_instances_match_individual_solves(gpu_lib):
    """Uneven instances stacked in one operator: per-instance, per-case results
    equal separate solves (and the shared launch sequence converges every
    instance to its own tolerance)."""
    from asend3d_gb300.solver import combine

    insts = []
    for k, (nx, ny) in enumerate([(6, 2), (11, 3), (4, 2)]):
        p = configs.cantilever_small(nx=nx, ny=ny, nz=ny, E=70e9 * (1 + 0.2 * k))
        p.add_nodal_force("tip", [0.0, 500.0, 0.0], case=1)
        insts.append(p)
    prob, node_ptr, elem_ptr = combine(insts)
    assert all(v % 128 == 0 for v in node_ptr[:-1])
    g = GpuSolver(prob, instances=node_ptr)
    g.assemble()
    u, rc, st = g.static_solve(method=_lib.METHOD_FP64, precond=_lib.PC_BLOCK, rel_tol=1e-10)
    assert rc == 0, st
    for i, p in enumerate(insts):
        gi = GpuSolver(p)
        gi.assemble()
        ui, rci, _ = gi.static_solve(method=_lib.METHOD_FP64, precond=_lib.PC_BLOCK, rel_tol=1e-10)
        assert rci == 0
        o = node_ptr[i]
        for k in range(2):
            seg = u[k, 3 * o:3 * o + 3 * p.mesh.n_nodes]
            assert rel(seg, ui[k]) < 1e-8
        gi.close()
    # padding nodes stay exactly zero
    for i in range(len(insts) - 1):
        pad = u[:, 3 * (node_ptr[i] + insts[i].mesh.n_nodes):3 * node_ptr[i + 1]]
        assert not np.any(pad)
    L, dLdE, rc, _ = g.adjoint_gradient()
    assert rc == 0 and np.all(dLdE < 0)
    g.close()


def test_multigrid_semicoarsening_damping_and_symmetry(gpu_lib):
    """Stretched cells (2.5:1) coarsen only the two fine axes first; every
    smoothed level gets omega = 1.5 / lambda_est with lambda_est (power
    iteration) below the guaranteed bound ||D^-1 A||_inf; the V-cycle is a
    symmetric positive definite operator (FP32: asymmetry within 1e-5 of
    ||u|| ||V v||)."""
    g = GpuSolver(configs.learned_patch(32, 16, 16))
    g.assemble(64)
    rc, st = g.static_solve_device(method=_lib.METHOD_FP64, precond=_lib.PC_MG, rel_tol=1e-8)
    assert rc == _lib.ASEND_OK and st["rel_residual"] <= 1e-8
    nl = g.mg_levels
    info = [g.mg_level_info(l) for l in range(nl)]
    assert info[0]["dims"] == (32, 16, 16)
    assert info[1]["dims"] == (32, 8, 8)      # x not coarsened: cells were 2.5x longer in x
    assert info[2]["dims"] == (16, 4, 4)
    for l in range(nl - 1):
        lam, bound, om = info[l]["lambda_est"], info[l]["lambda_bound"], info[l]["omega"]
        assert 0 < lam <= bound * (1 + 1e-5)
        assert om == pytest.approx(1.5 / lam, rel=1e-5)
    assert info[-1]["omega"] == 0.0
    rng = np.random.default_rng(1)
    u = rng.standard_normal(g.n_dof).astype(np.float32)
    v = rng.standard_normal(g.n_dof).astype(np.float32)
    Vu, Vv = g.mg_vcycle(u).astype(np.float64), g.mg_vcycle(v).astype(np.float64)
    a, b = u.astype(np.float64) @ Vv, v.astype(np.float64) @ Vu
    assert abs(a - b) <= 1e-5 * np.linalg.norm(u) * np.linalg.norm(Vv)
    assert v.astype(np.float64) @ Vv > 0 and u.astype(np.float64) @ Vu > 0
    g.close()
