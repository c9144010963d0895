"""The oracle's strain-pair tensors (orc_adjoint_strain_pairs): contracted
with C_e / E_e they reproduce the isotropic modulus gradient of the same
adjoint (for brickIM through the condensed matrix, so the recovery of the
internal modes is exact), and for hex8, contracted with dC/dE_k, the
component gradient.  Tolerance 1e-10 relative to max |g|."""
import numpy as np
import pytest

from asend3d_gb300.mesh import block_hex8, block_tet10
from asend3d_gb300.solver import Problem


def iso_C(E, nu):
    la, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    C = np.zeros((6, 6))
    C[:3, :3] = la
    C[:3, :3] += 2 * mu * np.eye(3)
    C[3:, 3:] = mu * np.eye(3)
    return C


def beam(etype):
    m = block_tet10(4, 2, 2, 1.2, 0.3, 0.2) if etype == 10 else block_hex8(6, 2, 2, 1.2, 0.3, 0.2)
    if etype == 81:
        m.elem_type = 81
    rng = np.random.default_rng(8)
    p = Problem(m, rng.uniform(60e9, 80e9, m.n_elems), np.full(m.n_elems, 0.3), np.full(m.n_elems, 2700.0))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    tip = m.nodes_in_range(xr=(m.coords[:, 0].max() - 1e-9, 1e9))
    p.add_node_set("tip", tip)
    p.fix_displacement("xMin")
    p.add_nodal_force("tip", [0.0, 200.0, -1000.0])
    return p, tip


@pytest.mark.parametrize("etype", [8, 81, 10])
def test_pairs_reproduce_isotropic_gradient(oracle_lib, etype):
    p, tip = beam(etype)
    o = oracle_lib.Oracle(p)
    u, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    dLdu = np.zeros(o.n_dof)
    dLdu[3 * tip + 2] = 1.0 / len(tip)
    g, lam, _, _ = o.adjoint(u, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
    P = o.strain_pairs(u, lam)
    giso = np.array([-(iso_C(1.0, nu) * P[e]).sum() for e, nu in enumerate(p.nu)])
    assert np.abs(giso - g).max() <= 1e-10 * np.abs(g).max()


def test_pairs_reproduce_component_gradient(oracle_lib):
    p, tip = beam(8)
    o = oracle_lib.Oracle(p)
    u, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    dLdu = np.zeros(o.n_dof)
    dLdu[3 * tip + 2] = 1.0 / len(tip)
    _, lam, _, _ = o.adjoint(u, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
    P = o.strain_pairs(u, lam)
    for k in (1, 2, 3):
        ge = o.component_gradient(u, lam, k)
        gp = np.zeros(p.mesh.n_elems)
        for e in range(p.mesh.n_elems):
            E, nu = p.E[e], p.nu[e]
            C = iso_C(E, nu)
            dS = np.zeros((6, 6))
            dS[k - 1, k - 1] = -1.0 / E ** 2
            if k == 1:
                dS[0, 1] = dS[1, 0] = dS[0, 2] = dS[2, 0] = nu / E ** 2
            if k == 2:
                dS[1, 2] = dS[2, 1] = nu / E ** 2
            gp[e] = ((C @ dS @ C) * P[e]).sum()  # -(dC : P) with dC = -C dS C
        assert np.abs(gp - ge).max() <= 1e-10 * np.abs(ge).max()
