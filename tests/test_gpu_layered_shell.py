"""Layered shell4 sections on the GPU (per-element ABD and section mass,
asend_set_shell_sections) against the oracle and the reference's
compositePlate known answers (examples/testCases/compositePlate/notes.txt).

Tolerances: the one-element known answers as in tests/test_shell_section.py
(1e-8; ux of the laminate 1e-5, the penalty supports' share); operator and
dynamic operator values 2e-11 of the largest entry; static displacements
1e-5 for the laminate's static solve (PCG to 1e-9 on an ill-conditioned thin clamped
plate, against a direct solve); Newmark probe history 1e-7 (PCG to 1e-11 per step)."""
import numpy as np
import pytest

from asend3d_gb300 import _lib
from asend3d_gb300.mesh import plate_quad4
from asend3d_gb300.solver import AsendError, GpuSolver, Problem

from test_shell_section import HOMOG, TWOPLY, composite_plate

pytestmark = pytest.mark.gpu
KW = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-13, max_iter=100000)
# the 10 x 10 laminate (a thin clamped plate with penalty supports and stiff
# drilling terms) is ill-conditioned: its static solve runs to 1e-9; its
# mass-dominated Newmark steps to 1e-11
KW9 = dict(KW, rel_tol=1e-9)
KW11 = dict(KW, rel_tol=1e-11)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def test_composite_plate_known_answers_gpu(gpu_lib):
    p, m = composite_plate(*HOMOG)
    g = GpuSolver(p)
    g.assemble(precision=64)
    u, rc, _ = g.static_solve(**KW)
    assert rc == 0
    tip = u[0].reshape(-1, 6)[m.nodes_in_range(xr=(0.9, 1.1))]
    np.testing.assert_allclose(tip[:, 2], 1.2e-3, rtol=1e-8)
    g.close()
    p, m = composite_plate(*TWOPLY)
    g = GpuSolver(p)
    g.assemble(precision=64)
    u, rc, _ = g.static_solve(**KW)
    assert rc == 0
    corner = u[0].reshape(-1, 6)[m.nodes_in_range(xr=(0.9, 1.1), yr=(0.9, 1.1))[0]]
    assert corner[0] == pytest.approx(4.651452282161358e-06, rel=1e-5)
    assert corner[1] == pytest.approx(2.6514522821613584e-06, rel=1e-8)
    assert corner[2] == pytest.approx(-1.79253112033e-04, rel=1e-8)
    assert corner[3] == pytest.approx(-8.96265560167775e-05, rel=1e-8)
    g.close()


def laminate_plate():
    n = 10
    m = plate_quad4(n, n, 1.0, 1.0)
    ne = m.n_elems
    p = Problem(m, np.full(ne, 7e10), np.full(ne, 0.3), np.full(ne, 2700.0), thickness=np.full(ne, 4e-3))
    cf = [1.4e11, 1e10, 0.3, 5e9, 1600.0]
    half = np.arange(0, ne, 2)
    p.shell_sections = [(half, [cf + [1e-3, 0.0], cf + [1e-3, 45.0], cf + [1e-3, -45.0], cf + [1e-3, 90.0]], 0.0),
                        (np.arange(1, ne, 2), [cf + [2e-3, 30.0], cf + [1e-3, -60.0]], -1.0)]
    edge = m.nodes_in_range(xr=(-1e-9, 1e-9))
    p.add_node_set("xMin", edge)
    p.fix_displacement("xMin", comps=(1, 2, 3, 4, 5, 6))
    tip = m.nodes_in_range(xr=(1.0 - 1e-9, 2.0))
    p.add_node_set("tip", tip)
    p.add_nodal_force("tip", [10.0, 5.0, -2.0])
    p.add_elem_set("all", np.arange(ne))
    return p


def test_layered_operator_solve_and_dynamics(gpu_lib, oracle_lib):
    p = laminate_plate()
    g = GpuSolver(p)
    g.assemble(precision=64)
    o = oracle_lib.Oracle(p)
    rp, col, val = g.csr(which=2)
    orp, ocol, oval = o.csr(which=0)
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    assert np.abs(val - oval).max() <= 2e-11 * np.abs(oval).max()
    u, rc, _ = g.static_solve(**KW9)
    assert rc == 0
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert rel(u[0], uo) < 1e-5
    # per-element modulus gradients are refused; the adjoint itself runs
    with pytest.raises(AsendError, match="isotropic"):
        g.adjoint_gradient(**KW9)
    with pytest.raises(AsendError, match="layered"):
        p2 = laminate_plate()
        p2.add_gravity("all", [0.0, 0.0, -9.81])
        GpuSolver(p2).load_vector(0)
    # Newmark with the coupled section mass
    dt, beta, gamma, n = 5e-6, 0.25, 0.5, 40
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    od = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    _, _, dval = g.csr(which=2)
    _, _, odval = od.csr(which=0)
    assert np.abs(dval - odval).max() <= 2e-11 * np.abs(odval).max()
    amp = np.sin(np.linspace(0.0, 2.0, n))
    probe = 6 * int(p.node_sets["tip"][-1]) + 2
    hist, uf, rc, _ = g.newmark(amp, probe_dof=probe, **KW11)
    assert rc == 0
    href, uref, rc2, _ = od.newmark(n, dt, beta, gamma, od.loads()[0], amp, probe, precond=oracle_lib.PC_DIRECT)
    assert rc2 == 0
    assert rel(hist, href) < 1e-7
    assert rel(uf, uref) < 1e-7
    g.close()
