"""GPU parity of the shell4 path (type 41) against the FP64 oracle.

Tolerances (written here, per quantity):
  * element stiffness / mass (FP64 both sides; Gauss-Jordan vs the
    reference's Givens-QR condensation): 1e-11 relative to max|K_e|, max|M_e|;
  * assembled operator: pattern bit-exact, values 2e-11 relative to max|K|;
  * displacements after a solve to rel. residual 1e-9: 1e-6 relative (the
    thin, penalty-stiffened beam has an FP64 residual floor near 1e-8 under
    point-Jacobi CG);
  * adjoint modulus gradients: 1e-5 relative (norm-wise), same reason;
  * Newmark centre history (each step solved to 1e-12): 1e-7 relative; the
    mixed-precision run (steps to 1e-10) 1e-6.
"""
import numpy as np
import pytest

from asend3d_gb300 import _lib, configs
from asend3d_gb300.mesh import plate_quad4
from asend3d_gb300.solver import AsendError, GpuSolver, Problem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def shell_beam(F=(0.0, 0.0, 1.0)):
    m = plate_quad4(10, 1, 10.0, 1.0)
    p = Problem(m, np.full(m.n_elems, 1e6), np.full(m.n_elems, 0.0), np.full(m.n_elems, 1.0),
                thickness=np.full(m.n_elems, 0.1))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-0.1, 0.1)))
    p.add_node_set("xMax", m.nodes_in_range(xr=(9.9, 10.1)))
    p.fix_displacement("xMin", comps=(1, 2, 3, 4, 5, 6))
    p.add_nodal_force("xMax", list(F))
    p.objective = ("displacement", "xMax", 3, 0.5)
    return p


def test_shell_element_matrices_match_oracle(gpu_lib, oracle_lib):
    """Distorted flat quads (general Jacobian), E/nu/t/rho per element."""
    import ctypes as C
    rng = np.random.default_rng(3)
    m = plate_quad4(3, 2, 1.5, 1.0)
    m.coords[:, :2] += rng.uniform(-0.08, 0.08, size=(m.n_nodes, 2))
    m.coords[:, 2] = 0.25
    ne = m.n_elems
    E, nu = rng.uniform(50e9, 80e9, ne), rng.uniform(0.2, 0.35, ne)
    rho, t = rng.uniform(2000, 3000, ne), rng.uniform(0.002, 0.01, ne)
    p = Problem(m, E, nu, rho, thickness=t)
    g = GpuSolver(p)
    ke, me = g.element_matrices()
    lib = oracle_lib.load()
    P = C.POINTER(C.c_double)
    for e in range(ne):
        xyz = np.ascontiguousarray(m.coords[m.conn[e]])
        ko = np.zeros(576)
        mo = np.zeros(576)
        assert lib.orc_element_stiffness(41, xyz.ctypes.data_as(P), E[e], nu[e], t[e], ko.ctypes.data_as(P)) == 0
        assert lib.orc_element_mass(41, xyz.ctypes.data_as(P), rho[e], t[e], mo.ctypes.data_as(P)) == 0
        ko, mo = ko.reshape(24, 24), mo.reshape(24, 24)
        assert np.abs(ke[e] - ko).max() <= 1e-11 * np.abs(ko).max(), e
        assert np.abs(me[e] - mo).max() <= 1e-11 * np.abs(mo).max(), e
    g.close()


def test_shell_beam_static_and_adjoint(gpu_lib, oracle_lib):
    """The reference's shellBeam cantilever: operator, tip deflection (7.98,
    analytic 8) and the adjoint gradient of the tip objective.  The thin beam
    is badly conditioned for point Jacobi, hence the large iteration cap."""
    p = shell_beam()
    g = GpuSolver(p)
    g.assemble(precision=64)
    o = oracle_lib.Oracle(p)
    rp, col, val = g.csr(0)
    rpo, colo, valo = o.csr(2)
    np.testing.assert_array_equal(rp, rpo)
    np.testing.assert_array_equal(col, colo)
    assert np.abs(val - valo).max() <= 2e-11 * np.abs(valo).max()
    kw = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-9, max_iter=200000)
    u, rc, st = g.static_solve(**kw)
    assert rc == _lib.ASEND_OK, st
    uo, rco, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert rel(u[0], uo) < 1e-6
    tip = p.node_sets["xMax"]
    assert np.allclose(u[0][6 * tip + 2], 8.0, rtol=0.01)
    L, gE, rc, st = g.adjoint_gradient(**kw)
    assert rc == _lib.ASEND_OK
    dLdu = np.zeros(o.n_dof)
    dLdu[6 * tip + 2] = 0.5
    go, _, _, _ = o.adjoint(uo, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
    assert rel(gE, go) < 1e-5
    assert gE.sum() == pytest.approx(-8e-6, rel=0.01)
    g.close()


def test_shell_plate_newmark_matches_oracle(gpu_lib, oracle_lib):
    """20x20 plate of the transient case (same supports and pulse), 150 steps
    of 2 us: centre deflection history and final state against the oracle's
    direct-solve Newmark; the mixed-precision solve against it too."""
    p = configs.shell_plate(20)
    dt, beta, gamma, n = 2e-6, 0.25, 0.5, 150
    amp = configs.gaussian_pulse(n, dt)
    probe = 6 * int(p.node_sets["centre"][0]) + 2
    g = GpuSolver(p)
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    hist, u, rc, st = g.newmark(amp, probe_dof=probe, method=_lib.METHOD_FP64, rel_tol=1e-12)
    assert rc == _lib.ASEND_OK
    o = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    href, uref, rc2, _ = o.newmark(n, dt, beta, gamma, o.loads()[0], amp, probe, precond=oracle_lib.PC_DIRECT)
    assert rc2 == 0
    assert rel(hist, href) < 1e-7
    assert rel(u, uref) < 1e-7
    assert hist.min() < 0  # the plate moves down under the -z impulse
    hm, um, rcm, stm = g.newmark(amp, probe_dof=probe, method=_lib.METHOD_MIXED, rel_tol=1e-10)
    assert rcm == _lib.ASEND_OK
    assert rel(hm, href) < 1e-6
    # extrapolated initial increments: same history, fewer iterations
    hx, ux, rcx, stx = g.newmark(amp, probe_dof=probe, method=_lib.METHOD_FP64, rel_tol=1e-12, warm_start=2)
    assert rcx == _lib.ASEND_OK
    assert rel(hx, href) < 1e-7
    assert stx["iterations"] < st["iterations"]
    g.close()


def test_shell_input_checks(gpu_lib):
    m = plate_quad4(2, 2, 1.0, 1.0)
    p = Problem(m, np.full(4, 1e9), np.full(4, 0.3))
    with pytest.raises(AsendError, match="thickness"):
        GpuSolver(p)
    m.coords[4, 2] = 0.1  # centre node lifted: elements not flat
    p = Problem(m, np.full(4, 1e9), np.full(4, 0.3), thickness=np.full(4, 0.01))
    with pytest.raises(AsendError, match="flat"):
        GpuSolver(p)
