"""Quadratic tetrahedra (type 10; element_meth.rs:228-262 four-point rule,
element_soln_fields.rs:229-298 shape functions) on the GPU path against the
oracle's restatement (pinned in tests/test_oracle_tet10.py).

Tolerances: pattern bit-exact; FP64 operator and mass values 2e-11 of the
largest entry (closed-form adjugate against the reference's Givens-QR
inverse); static displacements 1e-7 (PCG to 1e-11, the level point-Jacobi
PCG reaches on this penalty-supported quadratic mesh, against the oracle's
direct solve); adjoint modulus gradients 1e-6; Newmark probe history 1e-7;
body loads 1e-11 of the largest entry (the oracle's four-point mass products
round at 1e-12); element objectives 1e-8 (values) and 1e-6 (gradients);
material strain pairs 1e-7 of the largest entry."""
import numpy as np
import pytest

from asend3d_gb300 import _lib
from asend3d_gb300.mesh import block_tet10
from asend3d_gb300.solver import GpuSolver, Problem

pytestmark = pytest.mark.gpu
KW = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-11, max_iter=200000)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def beam(nu=0.3):
    m = block_tet10(5, 2, 2, 1.5, 0.3, 0.3)
    m.coords[:, 2] += 0.01 * np.sin(3.0 * m.coords[:, 0]) * m.coords[:, 1]  # moved nodes: curved edges
    E = 70e9 * (1.0 + 0.2 * np.cos(np.arange(m.n_elems)))
    p = Problem(m, E, np.full(m.n_elems, nu), np.full(m.n_elems, 2700.0))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    tip = m.nodes_in_range(xr=(1.5 - 1e-9, 2.0))
    p.add_node_set("tip", tip)
    p.add_nodal_force("tip", [0.0, 300.0, -1000.0 / len(tip)])
    p.add_elem_set("all", np.arange(m.n_elems))
    p.objective = ("displacement", "tip", 3, 1.0 / len(tip))
    return p


def test_tet10_operator_and_mass(gpu_lib, oracle_lib):
    p = beam()
    g = GpuSolver(p)
    g.assemble(precision=64)
    o = oracle_lib.Oracle(p)
    rp, col, val = g.csr(which=2)
    orp, ocol, oval = o.csr(which=0)
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    assert np.abs(val - oval).max() <= 2e-11 * np.abs(oval).max()
    x = np.random.default_rng(1).standard_normal(o.n_dof)
    assert rel(g.apply(x, 64), o.apply(x)) < 1e-11
    # dynamic operator K + c_M M against the oracle's
    dt, beta, gamma = 1e-5, 0.25, 0.5
    g.assemble(precision=64, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    od = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    _, _, dval = g.csr(which=2)
    _, _, odval = od.csr(which=0)
    assert np.abs(dval - odval).max() <= 2e-11 * np.abs(odval).max()
    g.close()


def test_tet10_static_adjoint_and_pairs(gpu_lib, oracle_lib):
    p = beam()
    g = GpuSolver(p)
    g.assemble(precision=64)
    u, rc, _ = g.static_solve(**KW)
    assert rc == 0
    o = oracle_lib.Oracle(p)
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert rel(u[0], uo) < 1e-7
    L, gE, rc, _ = g.adjoint_gradient(**KW)
    assert rc == 0
    tip = p.node_sets["tip"]
    dLdu = np.zeros(o.n_dof)
    dLdu[3 * tip + 2] = 1.0 / len(tip)
    go, lam, _, _ = o.adjoint(uo, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
    assert L == pytest.approx(float(dLdu @ uo), rel=1e-7)
    assert rel(gE, go) < 1e-6
    P = g.strain_pairs()
    Po = o.strain_pairs(uo, lam)
    assert np.abs(P - Po).max() <= 1e-7 * np.abs(Po).max()
    # element objective (strain energy, volume integral) and its gradient
    els = np.arange(p.mesh.n_elems)
    Le = g.set_element_objective(els, "strainEnergy", 0, "volumeIntegral", 2.0, 1.0)
    Lo, dLdu_e, _, dLdE = o.element_objective(uo, els, "strainEnergy", 0, "volumeIntegral", 2.0, 1.0)
    assert Le == pytest.approx(Lo, rel=1e-8)
    _, gEe, rc, _ = g.adjoint_gradient(**KW)
    assert rc == 0
    goe, _, _, _ = o.adjoint(uo, dLdu=dLdu_e, precond=oracle_lib.PC_DIRECT)
    assert rel(gEe, dLdE + goe) < 1e-6
    g.close()


def test_tet10_body_loads_and_newmark(gpu_lib, oracle_lib):
    p = beam()
    p.add_gravity("all", [0.0, 0.0, -9.81], case=1)
    p.add_centrifugal("all", 200.0, [0.0, 0.15, 0.15], [1.0, 0.0, 0.0], case=2)
    g = GpuSolver(p)
    o = oracle_lib.Oracle(p)
    for k, fo in enumerate(o.loads()):
        fg = g.load_vector(k)
        assert np.abs(fg - fo).max() <= 1e-11 * np.abs(fo).max(), k
    g.close()
    q = beam()
    dt, beta, gamma, n = 2e-5, 0.25, 0.5, 30
    amp = np.sin(np.linspace(0.0, 3.0, n))
    probe = 3 * int(q.node_sets["tip"][0]) + 2
    g = GpuSolver(q)
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    hist, u, rc, _ = g.newmark(amp, probe_dof=probe, **KW)
    assert rc == 0
    od = oracle_lib.Oracle(q, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    href, uref, rc2, _ = od.newmark(n, dt, beta, gamma, od.loads()[0], amp, probe, precond=oracle_lib.PC_DIRECT)
    assert rc2 == 0
    assert rel(hist, href) < 1e-7
    assert rel(u, uref) < 1e-7
    g.close()
