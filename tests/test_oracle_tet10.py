"""tet10 in the oracle (element_meth.rs:228-262, element_soln_fields.rs:229-298):
element properties, the linear patch test and quadratic completeness (pure
bending with nu = 0 is an exact elasticity solution with a quadratic
displacement field, so prescribing it on the boundary must reproduce it at
every free node).  Tolerances: element identities 1e-12
relative; field errors 1e-4 relative (penalty-enforced boundary values,
sf = 1e5 max|K|)."""
import ctypes as C

import numpy as np
import pytest

from asend3d_gb300.mesh import block_tet10
from asend3d_gb300.solver import Problem


def element(oracle_lib, xyz, E=2e11, nu=0.3, rho=7850.0):
    lib = oracle_lib.load()
    P = C.POINTER(C.c_double)
    xyz = np.ascontiguousarray(xyz, np.float64)
    ke = np.zeros(900)
    me = np.zeros(900)
    assert lib.orc_element_stiffness(10, xyz.ctypes.data_as(P), E, nu, 0.0, ke.ctypes.data_as(P)) == 0
    assert lib.orc_element_mass(10, xyz.ctypes.data_as(P), rho, 0.0, me.ctypes.data_as(P)) == 0
    return ke.reshape(30, 30), me.reshape(30, 30)


def tet10_nodes(corners):
    c = np.asarray(corners, float)
    mids = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
    return np.vstack([c] + [0.5 * (c[i] + c[j]) for i, j in mids])


def test_single_element(oracle_lib):
    xyz = tet10_nodes([[0.1, 0.0, 0.0], [1.2, 0.1, 0.0], [0.2, 0.9, 0.1], [0.0, 0.2, 1.1]])
    ke, me = element(oracle_lib, xyz, rho=7850.0)
    assert np.abs(ke - ke.T).max() <= 1e-12 * np.abs(ke).max()
    w = np.linalg.eigvalsh(ke)
    assert np.sum(np.abs(w) < 1e-9 * w.max()) == 6 and w[6] > 1e-6 * w.max()
    # consistent mass: total translational mass rho V per direction
    c = xyz[:4]
    vol = abs(np.linalg.det(np.stack([c[1] - c[0], c[2] - c[0], c[3] - c[0]]))) / 6
    for d in range(3):
        assert me[d::3, d::3].sum() == pytest.approx(7850.0 * vol, rel=1e-12)


def test_linear_patch(oracle_lib):
    """A linear field u = A x gives u^T K u = V eps^T C eps exactly."""
    xyz = tet10_nodes([[0, 0, 0], [1.0, 0.1, 0], [0.1, 1.0, 0.2], [0.2, 0.1, 0.9]])
    E, nu = 1e9, 0.25
    ke, _ = element(oracle_lib, xyz, E, nu)
    A = np.array([[1.0, 0.3, -0.2], [0.1, -0.5, 0.4], [0.2, 0.0, 0.7]]) * 1e-3
    u = (xyz @ A.T).ravel()
    eps = np.array([A[0, 0], A[1, 1], A[2, 2], A[0, 1] + A[1, 0], A[0, 2] + A[2, 0], A[1, 2] + A[2, 1]])
    la, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    Cm = np.zeros((6, 6))
    Cm[:3, :3] = la
    Cm[:3, :3] += 2 * mu * np.eye(3)
    Cm[3:, 3:] = mu * np.eye(3)
    c = xyz[:4]
    vol = abs(np.linalg.det(np.stack([c[1] - c[0], c[2] - c[0], c[3] - c[0]]))) / 6
    assert u @ ke @ u == pytest.approx(vol * eps @ Cm @ eps, rel=1e-12)


def bending_problem(mesh, kappa=1e-3):
    """u = -kappa x (z - z0), w = kappa x^2 / 2 prescribed on the boundary."""
    p = Problem(mesh, np.full(mesh.n_elems, 1e9), np.full(mesh.n_elems, 0.0), np.full(mesh.n_elems, 1.0))
    x, y, z = mesh.coords.T
    z0 = 0.5 * mesh.lz
    exact = np.stack([-kappa * x * (z - z0), np.zeros_like(x), 0.5 * kappa * x ** 2], axis=1)
    tol = 1e-9
    bnd = np.nonzero((x < tol) | (x > mesh.lx - tol) | (y < tol) | (y > mesh.ly - tol) | (z < tol)
                     | (z > mesh.lz - tol))[0]
    for nd in bnd:
        p.add_node_set(f"n{nd}", [int(nd)])
        for c in range(3):
            p.constraints.append(([(f"n{nd}", c + 1, 1.0)], float(exact[nd, c])))
    free = np.setdiff1d(np.arange(mesh.n_nodes), bnd)
    return p, exact, free


def test_quadratic_completeness(oracle_lib):
    mesh = block_tet10(3, 2, 2, 1.5, 1.0, 1.0)
    p, exact, free = bending_problem(mesh)
    assert len(free) == 45  # interior corner and mid-edge nodes
    o = oracle_lib.Oracle(p)
    # no applied load; orc_static_solve adds the penalty load sf C^T q itself
    u, rc, _ = o.solve(np.zeros(o.n_dof), precond=oracle_lib.PC_DIRECT)
    err = np.abs(u.reshape(-1, 3)[free] - exact[free]).max() / np.abs(exact).max()
    assert err < 1e-4, err
