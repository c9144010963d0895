"""GPU parity of the brickIM path (type 81: hex8 + 9 condensed incompatible
modes) against the FP64 oracle.

Tolerances (written here, per quantity):
  * element stiffness / mass (FP64 both sides; Gauss-Jordan vs the
    reference's Givens-QR condensation): 1e-11 relative to max|K_e|, max|M_e|;
  * assembled operator: pattern bit-exact, values 2e-11 relative to max|K|;
  * displacements after a solve to rel. residual 1e-8 (the thin beam's FP64
    floor): 1e-6 relative;
  * adjoint modulus gradients: 1e-5 relative (norm-wise).
"""
import ctypes as C

import numpy as np
import pytest

from asend3d_gb300 import _lib, configs
from asend3d_gb300.mesh import block_hex8
from asend3d_gb300.solver import GpuSolver, Problem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def test_brickim_element_matrices_match_oracle(gpu_lib, oracle_lib):
    rng = np.random.default_rng(8)
    m = block_hex8(3, 2, 2, 1.5, 1.0, 0.8)
    m.elem_type = 81
    m.coords += rng.uniform(-0.05, 0.05, size=m.coords.shape)
    ne = m.n_elems
    E, nu, rho = rng.uniform(50e9, 200e9, ne), rng.uniform(0.0, 0.4, ne), rng.uniform(2000, 8000, ne)
    g = GpuSolver(Problem(m, E, nu, rho))
    ke, me = g.element_matrices()
    lib = oracle_lib.load()
    P = C.POINTER(C.c_double)
    for e in range(ne):
        xyz = np.ascontiguousarray(m.coords[m.conn[e]])
        ko, mo = np.zeros(576), np.zeros(576)
        assert lib.orc_element_stiffness(81, xyz.ctypes.data_as(P), E[e], nu[e], 0.0, ko.ctypes.data_as(P)) == 0
        assert lib.orc_element_mass(81, xyz.ctypes.data_as(P), rho[e], 0.0, mo.ctypes.data_as(P)) == 0
        assert np.abs(ke[e] - ko.reshape(24, 24)).max() <= 1e-11 * np.abs(ko).max(), e
        assert np.abs(me[e] - mo.reshape(24, 24)).max() <= 1e-11 * np.abs(mo).max(), e
    g.close()


def test_brickim_beam_bending_and_adjoint(gpu_lib, oracle_lib):
    """The reference's hexBeam case with its default element: tip deflection
    F L^3 / 3EI = 8 and the tip objective's modulus gradient."""
    m = block_hex8(100, 10, 1, 10.0, 1.0, 0.1)
    m.elem_type = 81
    p = Problem(m, np.full(m.n_elems, 1e6), np.full(m.n_elems, 0.0), None)
    p.add_node_set("xMin", m.nodes_in_range(xr=(-0.01, 0.01)))  # clamp at x = 0 only
    p.fix_displacement("xMin")
    xmax = m.nodes_in_range(xr=(9.99, 10.01))
    p.add_node_set("xMax", xmax)
    p.add_nodal_force("xMax", [0.0, 0.0, 2.0 / len(xmax)])
    p.objective = ("displacement", "xMax", 3, 1.0 / len(xmax))
    g = GpuSolver(p)
    g.assemble(precision=64)
    o = oracle_lib.Oracle(p)
    rp, col, val = g.csr(0)
    rpo, colo, valo = o.csr(2)
    np.testing.assert_array_equal(rp, rpo)
    np.testing.assert_array_equal(col, colo)
    assert np.abs(val - valo).max() <= 2e-11 * np.abs(valo).max()
    # the penalty-stiffened thin beam's FP64 true residual bottoms out near
    # 1e-8 (every preconditioner), so parity is checked at that tolerance
    kw = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-8, max_iter=400000)
    u, rc, st = g.static_solve(**kw)
    assert rc == _lib.ASEND_OK, st
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert rel(u[0], uo) < 1e-6
    assert u[0][3 * xmax + 2].mean() == pytest.approx(8.0, rel=1e-3)
    L, gE, rc, st = g.adjoint_gradient(**kw)
    assert rc == _lib.ASEND_OK
    dLdu = np.zeros(o.n_dof)
    dLdu[3 * xmax + 2] = 1.0 / len(xmax)
    go, _, _, _ = o.adjoint(uo, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
    assert rel(gE, go) < 1e-5
    assert gE.sum() == pytest.approx(-8e-6, rel=1e-3)
    g.close()


def test_brickim_lognormal_block_multigrid(gpu_lib, oracle_lib):
    """A lognormal-modulus brickIM block solved with multigrid (coarse levels
    Galerkin from standard hex8 geometry integration) matches the oracle."""
    p = configs.block_large(nx=24, ny=6, nz=6, seed=3)
    p.mesh.elem_type = 81
    g = GpuSolver(p)
    g.assemble(precision=64)
    u, rc, st = g.static_solve(method=_lib.METHOD_FP64, precond=_lib.PC_MG, rel_tol=1e-10)
    assert rc == _lib.ASEND_OK, st
    o = oracle_lib.Oracle(p)
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert rel(u[0], uo) < 1e-6
    g.close()
