"""Layered shell sections (ABD and section mass; element_properties.rs:75-222,
:581-646, :766-876, :1354-1408) on the CPU: the library's host routine
(asend_shell_section, no device needed) against the oracle's restatement
(1e-12 of the largest entry), closed forms of one isotropic layer, and the
reference's compositePlate known answers (examples/testCases/compositePlate/
notes.txt) through the oracle: a one-element 2 x 2 plate, t = 0.1,
E = 1e6, nu = 0, offset -1, clamped at x = -1 and pulled by F = 1 per xMax
node gives uz = 1.2e-3 at x = 1; the [+45 / -45] laminate (E11 = 1e7,
E22 = 1e6, G12 = 5e6) gives ux = 4.651452282161358e-6, uy =
2.6514522821613584e-6, uz = -1.79253112033e-4, thetax = -8.96265560167775e-5
at (1, 1).  The penalty supports leave 2e-6 relative in ux."""
import ctypes as C

import numpy as np
import pytest

from asend3d_gb300 import _lib
from asend3d_gb300.mesh import plate_quad4
from asend3d_gb300.solver import Problem

po = pytest.importorskip("oracle.pyoracle")


def lib_section(layers, z_offset):
    lib = _lib.load()
    lay = np.ascontiguousarray(layers, np.float64).reshape(-1, 7)
    abd, ms = np.zeros(81), np.zeros(36)
    p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    rc = lib.asend_shell_section(len(lay), p(lay), float(z_offset), p(abd), p(ms))
    return rc, abd, ms


def oracle_section(layers, z_offset):
    lib = po.load()
    lay = np.ascontiguousarray(layers, np.float64).reshape(-1, 7)
    abd, ms = np.zeros(81), np.zeros(36)
    assert lib.orc_shell_section(len(lay), po._p(lay), float(z_offset), po._p(abd), po._p(ms)) == 0
    return abd, ms


@pytest.mark.parametrize("z_offset", [-1.0, 0.0, 0.5, 1.0])
def test_library_section_matches_oracle(z_offset):
    rng = np.random.default_rng(11)
    for n in (1, 2, 3, 5):
        lay = np.column_stack([rng.uniform(1e9, 2e11, n), rng.uniform(1e9, 5e10, n), rng.uniform(0.0, 0.35, n),
                               rng.uniform(1e9, 3e10, n), rng.uniform(1000, 8000, n), rng.uniform(1e-4, 2e-3, n),
                               rng.uniform(-90, 90, n)])
        rc, abd, ms = lib_section(lay, z_offset)
        assert rc == 0
        oa, om = oracle_section(lay, z_offset)
        assert np.abs(abd - oa).max() <= 1e-12 * np.abs(oa).max()
        assert np.abs(ms - om).max() <= 1e-12 * np.abs(om).max()
        A = abd.reshape(9, 9)
        assert np.allclose(A, A.T, rtol=0, atol=1e-12 * np.abs(A).max())


def test_single_layer_closed_forms():
    E, nu, t, rho = 7e10, 0.3, 2e-3, 2700.0
    G = E / (2 * (1 + nu))
    q = E / (1 - nu * nu)
    Q = np.array([[q, nu * q, 0], [nu * q, q, 0], [0, 0, G]])
    for zoff, b in ((0.0, 0.0), (-1.0, 0.5 * t * t), (1.0, -0.5 * t * t)):
        rc, abd, ms = lib_section([[E, E, nu, G, rho, t, 30.0]], zoff)
        assert rc == 0
        A = abd.reshape(9, 9)
        np.testing.assert_allclose(A[:3, :3], t * Q, rtol=1e-12, atol=1e-9 * q * t)
        np.testing.assert_allclose(A[:3, 3:6], b * Q, rtol=1e-12, atol=1e-9 * q * t * t)
        assert A[6, 6] == A[7, 7] == A[8, 8] == A[2, 2]
        M = ms.reshape(6, 6)
        assert M[0, 0] == pytest.approx(rho * t) and M[0, 4] == pytest.approx(rho * b, abs=1e-18)
        assert M[1, 3] == pytest.approx(-rho * b, abs=1e-18)


def test_invalid_layers_rejected():
    assert lib_section([[0.0, 1e9, 0.3, 1e9, 1.0, 1e-3, 0.0]], 0.0)[0] == _lib.ASEND_EINVAL
    assert lib_section([[1e9, 1e9, 0.3, 1e9, 1.0, -1e-3, 0.0]], 0.0)[0] == _lib.ASEND_EINVAL
    assert lib_section([[1e9, 1e9, 2.0, 1e9, 1.0, 1e-3, 0.0]], 0.0)[0] == _lib.ASEND_EINVAL  # S not SPD


def composite_plate(layers, z_offset, supports):
    m = plate_quad4(1, 1, 2.0, 2.0)
    m.coords[:, :2] -= 1.0
    p = Problem(m, np.full(1, 1e6), np.full(1, 0.0), np.full(1, 1000.0), thickness=np.full(1, 0.1))
    p.shell_sections = [([0], layers, z_offset)]
    for name, xr, yr, comps in supports:
        p.add_node_set(name, m.nodes_in_range(xr=xr, yr=yr))
        p.fix_displacement(name, comps=comps)
    xmax = m.nodes_in_range(xr=(0.9, 1.1))
    p.add_node_set("xMax", xmax)
    p.add_nodal_force("xMax", [1.0, 0.0, 0.0])
    return p, m


HOMOG = ([[1e6, 1e6, 0.0, 5e5, 1000.0, 0.1, 0.0]], -1.0,
         [("xMin", (-1.1, -0.9), (-2, 2), (1, 2, 3, 4, 5, 6))])
TWOPLY = ([[1e7, 1e6, 0.0, 5e6, 1000.0, 0.05, 45.0], [1e7, 1e6, 0.0, 5e6, 1000.0, 0.05, -45.0]], 0.0,
          [("xyMin", (-1.1, -0.9), (-1.1, -0.9), (1, 2, 3, 4, 5, 6)),
           ("xMinyMax", (-1.1, -0.9), (0.9, 1.1), (1,))])


def test_composite_plate_known_answers_oracle():
    p, m = composite_plate(*HOMOG)
    o = po.Oracle(p)
    u, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=po.PC_DIRECT)
    tip = u.reshape(-1, 6)[m.nodes_in_range(xr=(0.9, 1.1))]
    np.testing.assert_allclose(tip[:, 2], 1.2e-3, rtol=1e-8)
    p, m = composite_plate(*TWOPLY)
    o = po.Oracle(p)
    u, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=po.PC_DIRECT)
    corner = u.reshape(-1, 6)[m.nodes_in_range(xr=(0.9, 1.1), yr=(0.9, 1.1))[0]]
    assert corner[0] == pytest.approx(4.651452282161358e-06, rel=1e-5)
    assert corner[1] == pytest.approx(2.6514522821613584e-06, rel=1e-8)
    assert corner[2] == pytest.approx(-1.79253112033e-04, rel=1e-8)
    assert corner[3] == pytest.approx(-8.96265560167775e-05, rel=1e-8)
