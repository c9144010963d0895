"""Element loads on the GPU path against the oracle's restatement of
get_app_load_dfd0 (element_equations.rs:1833-2056): body force, gravity,
centrifugal (element-centroid acceleration) and surface pressure.

Tolerances: load vectors 1e-12 of their largest entry for hex8, brickIM
and shells (closed-form node weights against the oracle's mass-matrix
products) and 1e-10 for tet4, where the oracle's one-point mass products and the
closed-form |det|/24 node weights differ by up to 3e-12 relative (measured
on this mesh on the CPU); static displacements
under gravity 1e-8 (PCG to 1e-11); the resultant of a gravity load on a box
equals rho g V to 1e-12."""
import numpy as np
import pytest

from asend3d_gb300 import _lib, configs
from asend3d_gb300.mesh import block_hex8, block_tet4
from asend3d_gb300.solver import GpuSolver, Problem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def solid(kind):
    if kind == "tet4":
        m = block_tet4(4, 2, 2, 2.0, 0.4, 0.4)
    else:
        m = block_hex8(6, 2, 2, 2.0, 0.4, 0.4)
        m.coords[:, 2] += 0.03 * np.sin(3.0 * m.coords[:, 0]) * m.coords[:, 1]  # distorted elements
        if kind == "brickIM":
            m.elem_type = 81
    rho = 2700.0 * (1.0 + 0.3 * np.arange(m.n_elems) / m.n_elems)
    p = Problem(m, np.full(m.n_elems, 70e9), np.full(m.n_elems, 0.3), rho)
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    p.add_elem_set("all", np.arange(m.n_elems))
    p.add_elem_set("half", np.arange(0, m.n_elems, 2))
    return p


@pytest.mark.parametrize("kind", ["hex8", "brickIM", "tet4"])
def test_element_loads_match_oracle(gpu_lib, oracle_lib, kind):
    p = solid(kind)
    p.add_body_force("half", [1e4, -2e4, 5e3], case=0)
    p.add_gravity("all", [0.0, 0.0, -9.81], case=1)
    p.add_centrifugal("all", 300.0, [0.0, 0.2, 0.2], [3.0, 0.0, 0.0], case=2)
    p.add_surface_pressure("all", [1.0, 0.0, 0.0], 2.5e5, norm_tol=5.0, case=3)
    p.add_gravity("half", [1.0, 2.0, -9.81], case=3)
    g = GpuSolver(p)
    o = oracle_lib.Oracle(p)
    for k, fo in enumerate(o.loads()):
        fg = g.load_vector(k)
        tol = 1e-10 if kind == "tet4" else 1e-12
        assert np.abs(fg - fo).max() <= tol * np.abs(fo).max(), (kind, k)
    g.close()


def test_gravity_static_solve_and_resultant(gpu_lib, oracle_lib):
    m = block_hex8(10, 2, 2, 2.0, 0.4, 0.4)
    m.elem_type = 81  # incompatible modes: plain hex8 locks in bending (11 % stiff here)
    p = Problem(m, np.full(m.n_elems, 70e9), np.full(m.n_elems, 0.3), np.full(m.n_elems, 2700.0))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    p.add_elem_set("all", np.arange(m.n_elems))
    p.add_gravity("all", [0.0, 0.0, -9.81])
    g = GpuSolver(p)
    f = g.load_vector(0)
    assert f[2::3].sum() == pytest.approx(-9.81 * 2700.0 * 2.0 * 0.4 * 0.4, rel=1e-12)
    g.assemble(precision=64)
    u, rc, _ = g.static_solve(method=_lib.METHOD_FP64, precond=_lib.PC_MG, rel_tol=1e-11)
    assert rc == 0
    o = oracle_lib.Oracle(p)
    ur, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert rel(u[0], ur) < 1e-8
    # cantilever under its own weight: tip deflection q L^4 / (8 E I) within 5 %
    q = 2700.0 * 9.81 * 0.4 * 0.4
    w_beam = q * 2.0 ** 4 / (8 * 70e9 * 0.4 ** 4 / 12)
    tip = m.nodes_in_range(xr=(2.0 - 1e-9, 2.0 + 1e-9))
    assert -u[0][3 * tip + 2].mean() == pytest.approx(w_beam, rel=0.05)
    g.close()


def test_shell_gravity_and_centrifugal(gpu_lib, oracle_lib):
    p = configs.shell_plate(n=6)
    p.add_elem_set("all", np.arange(p.mesh.n_elems))
    p.add_gravity("all", [0.0, 0.0, -9.81], case=1)
    p.add_centrifugal("all", 50.0, [0.5, 0.5, 0.0], [0.0, 0.0, 1.0], case=2)
    p.add_body_force("all", [0.0, 0.0, 1e3], case=3)
    g = GpuSolver(p)
    o = oracle_lib.Oracle(p)
    for k, fo in enumerate(o.loads()):
        fg = g.load_vector(k)
        assert np.abs(fg - fo).max() <= 1e-12 * np.abs(fo).max(), k
    f1 = g.load_vector(1)
    assert f1[2::6].sum() == pytest.approx(-9.81 * 2700.0 * 1.0 * 0.005, rel=1e-12)
    g.close()
