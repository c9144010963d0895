"""CPU tests pinning the FP64 oracle.

The reference ships no recorded solver outputs, so the oracle is pinned by:
  * the reference's analytic known answers (examples/testCases/hexBeam/notes.txt,
    singleHex scripts) -- stored in tests/golden/analytic_pins.json,
  * internal consistency (direct LDL^T vs PCG, block-LDL vs Jacobi),
  * central finite differences of the adjoint gradient (step 1e-6 E).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from asend3d_gb300 import configs
from asend3d_gb300.mesh import block_hex8, block_tet4
from asend3d_gb300.solver import Problem

GOLD = Path(__file__).resolve().parent / "golden"


def pins():
    return json.loads((GOLD / "analytic_pins.json").read_text())


def _axial_beam(po, nx=100, ny=10, nz=1):
    m = block_hex8(nx, ny, nz, 10.0, 1.0, 0.1)
    p = Problem(m, np.full(m.n_elems, 1e6), np.full(m.n_elems, 0.0), None)
    p.add_node_set("xMin", m.nodes_in_range(xr=(-0.1, 0.1)))
    p.fix_displacement("xMin")
    xmax = m.nodes_in_range(xr=(9.99, 10.01))
    p.add_node_set("xMax", xmax)
    p.add_nodal_force("xMax", [2.0 / len(xmax), 0, 0])
    return p, xmax


def test_single_hex_axial(oracle_lib):
    po = oracle_lib
    pin = pins()["singleHex_axial"]
    m = block_hex8(1, 1, 1, 1.0, 1.0, 1.0)
    p = Problem(m, np.full(1, 1e6), np.full(1, 0.0), np.full(1, 1000.0))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-0.1, 0.1)))
    p.fix_displacement("xMin")
    p.add_node_set("xMax", m.nodes_in_range(xr=(0.9, 1.1)))
    p.add_nodal_force("xMax", [0.25, 0, 0])
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    for pc in (po.PC_JACOBI, po.PC_BLOCK_LDL, po.PC_DIRECT):
        u, rc, st = o.solve(f, precond=pc, stop=po.STOP_REFERENCE, tol=1e-12)
        assert rc == 0
        ux = u[3 * p.node_sets["xMax"]]
        # penalty enforcement leaves a 1e-5 relative error (sf = 1e5 max|K|)
        np.testing.assert_allclose(ux, pin["value"], rtol=pin["rtol"])


def test_hexbeam_axial_and_strain_energy(oracle_lib):
    po = oracle_lib
    pk = pins()
    p, xmax = _axial_beam(po)
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    u, rc, st = o.solve(f, tol=1e-11)
    assert rc == 0 and st["rel_residual"] < 1e-10
    assert u[3 * xmax].mean() == pytest.approx(pk["hexBeam_axial_tip"]["value"], rel=pk["hexBeam_axial_tip"]["rtol"])
    se = 0.5 * f @ u
    assert se == pytest.approx(pk["hexBeam_axial_strain_energy"]["value"],
                               rel=pk["hexBeam_axial_strain_energy"]["rtol"])
    g, _, _, _ = o.adjoint(u, lam=u)
    dse = 0.5 * g.sum()  # scaling all element moduli = d/dE of the isotropic material
    assert dse == pytest.approx(pk["hexBeam_axial_dSEdE"]["value"], rel=pk["hexBeam_axial_dSEdE"]["rtol"])


def test_direct_vs_pcg_consistency(oracle_lib):
    po = oracle_lib
    p = configs.cantilever_small()
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    ud, rc, st = o.solve(f, precond=po.PC_DIRECT)
    assert rc == 0 and st["rel_residual"] < 1e-10
    for pc in (po.PC_JACOBI, po.PC_BLOCK_LDL):
        u, rc, st = o.solve(f, precond=pc, stop=po.STOP_RELATIVE, tol=1e-12)
        assert rc == 0
        assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e-9


def test_reference_stopping_rule_block_ldl(oracle_lib):
    """The reference PCG stops on the absolute g^T M^-1 g <= conv_tol (1e-12 by
    default, job.rs:78); with the block-LDL preconditioner it converges."""
    po = oracle_lib
    p = configs.cantilever_small()
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    u, rc, st = o.solve(f, precond=po.PC_BLOCK_LDL, stop=po.STOP_REFERENCE, tol=1e-12)
    assert rc == 0 and st["final_res"] <= 1e-12


def test_reorder_is_permutation(oracle_lib):
    po = oracle_lib
    p = configs.cantilever_small()
    o = po.Oracle(p)
    order = o.reorder()
    assert sorted(order.tolist()) == list(range(p.mesh.n_nodes))


def test_element_stiffness_properties(oracle_lib):
    po = oracle_lib
    rng = np.random.default_rng(0)
    m = block_hex8(1, 1, 1, 0.3, 0.2, 0.1)
    xyz = m.coords[m.conn[0]] + 0.01 * rng.standard_normal((8, 3))
    ke = po.element_stiffness(8, xyz, 2.0e11, 0.3)
    assert np.allclose(ke, ke.T, rtol=1e-12, atol=1e-12 * np.abs(ke).max())
    # rigid-body modes: 3 translations + 3 rotations in the null space
    modes = []
    for d in range(3):
        t = np.zeros((8, 3))
        t[:, d] = 1.0
        modes.append(t.ravel())
    for ax in range(3):
        w = np.zeros(3)
        w[ax] = 1.0
        modes.append(np.cross(w, xyz).ravel())
    for mvec in modes:
        assert np.linalg.norm(ke @ mvec) <= 1e-9 * np.abs(ke).max() * np.linalg.norm(mvec)
    ev = np.linalg.eigvalsh(ke)
    assert (ev[6:] > 0).all()


def test_tet4_constant_strain_patch(oracle_lib):
    """A linear displacement field is reproduced exactly (patch test)."""
    po = oracle_lib
    m = block_tet4(2, 2, 2, 1.0, 1.0, 1.0)
    p = Problem(m, np.full(m.n_elems, 1e6), np.full(m.n_elems, 0.25), None)
    o = po.Oracle(p)
    gradu = np.array([[1e-3, 2e-4, 0.0], [0.0, -3e-4, 1e-4], [5e-5, 0.0, 2e-4]])
    u = (m.coords @ gradu.T).ravel()
    r = o.apply(u)
    interior = m.nodes_in_range(xr=(0.4, 0.6), yr=(0.4, 0.6), zr=(0.4, 0.6))
    assert len(interior) == 1
    k = interior[0]
    assert np.abs(r[3 * k:3 * k + 3]).max() < 1e-9 * np.abs(r).max()


def test_surface_traction_total_force(oracle_lib):
    po = oracle_lib
    p = configs.block_large(nx=10, ny=4, nz=4)
    o = po.Oracle(p)
    f = o.loads()[0]
    area = 0.4 * 0.4
    assert f[2::3].sum() == pytest.approx(-1.0e6 * area, rel=1e-12)
    assert abs(f[0::3].sum()) < 1e-6 and abs(f[1::3].sum()) < 1e-6


def test_adjoint_central_difference_config1(oracle_lib):
    """dL/dE_e for L = tip u_z vs central FD with step 1e-6 E (config 1)."""
    po = oracle_lib
    p = configs.cantilever_small()
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    u, _, _ = o.solve(f, precond=po.PC_DIRECT)
    tip = p.node_sets["tip"][0]
    dldu = np.zeros(o.n_dof)
    dldu[3 * tip + 2] = 1.0
    g, _, rc, _ = o.adjoint(u, dLdu=dldu, precond=po.PC_DIRECT)
    assert rc == 0
    rng = np.random.default_rng(1)
    for e in rng.choice(p.mesh.n_elems, 6, replace=False):
        vals = []
        for s in (+1, -1):
            E2 = p.E.copy()
            E2[e] *= 1.0 + s * 1e-6
            p2 = Problem(p.mesh, E2, p.nu, p.rho, p.node_sets, p.elem_sets, p.constraints, p.loads, p.objective)
            o2 = po.Oracle(p2)
            # the penalty scale is held fixed, as the reference's adjoint does
            f2 = o2.loads()[0] + o2.penalty_rhs()
            u2, _, _ = o2.solve(f2, precond=po.PC_DIRECT)
            vals.append(u2[3 * tip + 2])
        fd = (vals[0] - vals[1]) / (2e-6 * p.E[e])
        assert g[e] == pytest.approx(fd, rel=2e-4, abs=1e-8 * np.abs(g).max())


def test_component_dv_sum_equals_isotropic(oracle_lib):
    """Reference-style 'modulus' DVs on E1..E3 (plus shear terms) sum to the
    isotropic modulus gradient; with nu = 0 the E_k parts alone cover the
    normal-strain energy."""
    po = oracle_lib
    p = configs.cantilever_small(nu=0.0)
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    u, _, _ = o.solve(f, precond=po.PC_DIRECT)
    g_iso, _, _, _ = o.adjoint(u, lam=u)
    gk = sum(o.component_gradient(u, u, k) for k in (1, 2, 3))
    # isotropic = E-part + G-part; the E-part is bounded by the total
    assert np.all(np.abs(gk) <= np.abs(g_iso) * (1 + 1e-9) + 1e-30)
    assert np.sum(gk) / np.sum(g_iso) > 0.5


def test_newmark_static_limit(oracle_lib):
    """A slowly ramped load gives the static displacement (Newmark, reference
    beta convention beta_ref = 0.25, gamma = 0.5)."""
    po = oracle_lib
    p = configs.cantilever_small(nx=8, ny=2, nz=2)
    dt = 2e-3
    o = po.Oracle(p, dynamic=True, dt=dt, beta=0.25, gamma=0.5)
    f = o.loads()[0]
    n = 400
    amp = np.clip(np.arange(n) / 300.0, 0.0, 1.0)
    tip = p.node_sets["tip"][0]
    hist, u, rc, its = o.newmark(n, dt, 0.25, 0.5, f, amp, 3 * tip + 2, precond=po.PC_DIRECT)
    assert rc == 0
    os_ = po.Oracle(p)
    us, _, _ = os_.solve(os_.loads()[0] + os_.penalty_rhs(), precond=po.PC_DIRECT)
    assert hist[-1] == pytest.approx(us[3 * tip + 2], rel=0.05)


def _shell_beam(F):
    from asend3d_gb300.mesh import plate_quad4
    m = plate_quad4(10, 1, 10.0, 1.0)
    p = Problem(m, np.full(m.n_elems, 1e6), np.full(m.n_elems, 0.0), np.full(m.n_elems, 1.0),
                thickness=np.full(m.n_elems, 0.1))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-0.1, 0.1)))
    p.add_node_set("xMax", m.nodes_in_range(xr=(9.9, 10.1)))
    p.fix_displacement("xMin", comps=(1, 2, 3, 4, 5, 6))
    p.add_nodal_force("xMax", F)
    return p


def test_shell_beam_pins(oracle_lib):
    """shell4 (type 41) cantilever of the reference's shellBeam case: tip
    deflection, dw/dE through the adjoint, axial stretch, and the first
    natural frequency (consistent shell mass) against notes.txt."""
    pins = json.loads((GOLD / "analytic_pins.json").read_text())
    p = _shell_beam([0.0, 0.0, 1.0])
    o = oracle_lib.Oracle(p)
    assert o.dpn == 6 and o.n_dof == 6 * 22
    u, rc, st = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    tip = p.node_sets["xMax"]
    w = u[6 * tip + 2]
    pin = pins["shellBeam_transverse_tip"]
    assert np.allclose(w, pin["value"], rtol=pin["rtol"])
    # L = 0.5 * sum of tip w (powerNorm, coefficient 0.5); sum_e dL/dE_e = dL/dE
    dLdu = np.zeros(o.n_dof)
    dLdu[6 * tip + 2] = 0.5
    g, lam, rc, st = o.adjoint(u, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
    assert g.sum() == pytest.approx(pin["dwdE"], rel=pin["rtol"])
    assert g.sum() == pytest.approx(-0.5 * w.sum() / 1e6, rel=1e-8)  # K is linear in E
    pa = _shell_beam([1.0, 0.0, 0.0])
    oa = oracle_lib.Oracle(pa)
    ua, rc, _ = oa.solve(oa.loads()[0] + oa.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    pin = pins["shellBeam_axial_tip"]
    assert np.allclose(ua[6 * tip], pin["value"], rtol=pin["rtol"])
    # first natural frequency: K x = w^2 M x with the fixed DOF eliminated (a
    # 1e10 penalty next to the ~1e-6 rotary inertias leaves the generalized
    # eigensolver no accuracy for the smallest eigenvalue)
    import scipy.linalg as sla
    od = oracle_lib.Oracle(p, dynamic=True, dt=1.0, beta=0.25, gamma=0.5)
    n = od.n_dof
    rp, col, val = od.csr(0)
    _, _, mval = od.csr(1)
    A = np.zeros((n, n))
    Mm = np.zeros((n, n))
    for r in range(n):
        A[r, col[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
        Mm[r, col[rp[r]:rp[r + 1]]] = mval[rp[r]:rp[r + 1]]
    cM = -1.0 / (1.0 * (0.25 - 0.5))  # the operator holds K + c_M M (Newmark, dt = 1)
    fixed = np.concatenate([6 * p.node_sets["xMin"] + c for c in range(6)])
    keep = np.setdiff1d(np.arange(n), fixed)
    K = (A - cM * Mm)[np.ix_(keep, keep)]
    lam_min = sla.eigh(K, Mm[np.ix_(keep, keep)], eigvals_only=True, subset_by_index=[0, 0])[0]
    f1 = np.sqrt(lam_min) / (2 * np.pi)
    pin = pins["shellBeam_first_frequency_hz"]
    assert f1 == pytest.approx(pin["value"], rel=pin["rtol"])


def test_shell_element_properties(oracle_lib):
    """Single shell4 element: symmetric, positive semi-definite with exactly
    six rigid-body modes; mass symmetric positive definite with total
    translational mass rho t A."""
    import ctypes as C
    lib = oracle_lib.load()
    xyz = np.array([[0, 0, 0], [1.2, 0.1, 0], [1.0, 0.9, 0], [-0.1, 1.1, 0]], float)
    ke = np.zeros(576)
    me = np.zeros(576)
    P = C.POINTER(C.c_double)
    assert lib.orc_element_stiffness(41, xyz.ctypes.data_as(P), 7e10, 0.33, 0.005, ke.ctypes.data_as(P)) == 0
    assert lib.orc_element_mass(41, xyz.ctypes.data_as(P), 2700.0, 0.005, me.ctypes.data_as(P)) == 0
    K, M = ke.reshape(24, 24), me.reshape(24, 24)
    assert np.abs(K - K.T).max() <= 1e-12 * np.abs(K).max()
    ev = np.linalg.eigvalsh(K)
    assert np.sum(ev < 1e-9 * ev[-1]) == 6 and ev[0] > -1e-9 * ev[-1]
    assert np.all(np.linalg.eigvalsh(M) > 0)
    area = 0.5 * abs(np.cross(xyz[2] - xyz[0], xyz[3] - xyz[1])[2])
    ones = np.zeros(24)
    ones[0::6] = 1.0
    assert ones @ M @ ones == pytest.approx(2700.0 * 0.005 * area, rel=1e-12)
    # a non-planar element is rejected
    xyz[2, 2] = 0.1
    assert lib.orc_element_stiffness(41, xyz.ctypes.data_as(P), 7e10, 0.33, 0.005, ke.ctypes.data_as(P)) != 0


def test_brickim_beam_bending_pin(oracle_lib):
    """brickIM (type 81, the reference's default hex element) on the hexBeam
    case: tip deflection F L^3 / 3EI = 8 and dw/dE = -8e-6
    (examples/testCases/hexBeam/notes.txt:10-13); plain hex8 locks in
    bending on the one-element-thick bar."""
    po = oracle_lib
    pin = pins()["hexBeam_transverse_tip"]
    out = {}
    for et in (8, 81):
        m = block_hex8(100, 10, 1, 10.0, 1.0, 0.1)
        m.elem_type = et
        p = Problem(m, np.full(m.n_elems, 1e6), np.full(m.n_elems, 0.0), None)
        p.add_node_set("xMin", m.nodes_in_range(xr=(-0.01, 0.01)))  # clamp at x = 0 only
        p.fix_displacement("xMin")
        xmax = m.nodes_in_range(xr=(9.99, 10.01))
        p.add_node_set("xMax", xmax)
        p.add_nodal_force("xMax", [0.0, 0.0, 2.0 / len(xmax)])
        o = po.Oracle(p)
        u, rc, st = o.solve(o.loads()[0] + o.penalty_rhs(), precond=po.PC_DIRECT)
        w = u[3 * xmax + 2].mean()
        out[et] = w
        if et == 81:
            assert w == pytest.approx(pin["value"], rel=pin["rtol"])
            dLdu = np.zeros(o.n_dof)
            dLdu[3 * xmax + 2] = 1.0 / len(xmax)
            g, _, _, _ = o.adjoint(u, dLdu=dLdu, precond=po.PC_DIRECT)
            assert g.sum() == pytest.approx(pin["dwdE"], rel=pin["rtol"])
            assert g.sum() == pytest.approx(-w / 1e6, rel=1e-8)
    assert out[8] < 0.8 * out[81]  # hex8 locks


def test_brickim_element_properties(oracle_lib):
    """Condensed brickIM stiffness: symmetric PSD with six rigid-body modes,
    softer in bending than hex8 on a distorted element; same mass as hex8."""
    import ctypes as C
    lib = oracle_lib.load()
    P = C.POINTER(C.c_double)
    rng = np.random.default_rng(4)
    xyz = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    xyz += rng.uniform(-0.1, 0.1, xyz.shape)
    k81, k8, m81, m8 = (np.zeros(576) for _ in range(4))
    assert lib.orc_element_stiffness(81, xyz.ctypes.data_as(P), 2e11, 0.3, 0.0, k81.ctypes.data_as(P)) == 0
    assert lib.orc_element_stiffness(8, xyz.ctypes.data_as(P), 2e11, 0.3, 0.0, k8.ctypes.data_as(P)) == 0
    assert lib.orc_element_mass(81, xyz.ctypes.data_as(P), 7850.0, 0.0, m81.ctypes.data_as(P)) == 0
    assert lib.orc_element_mass(8, xyz.ctypes.data_as(P), 7850.0, 0.0, m8.ctypes.data_as(P)) == 0
    K, K8 = k81.reshape(24, 24), k8.reshape(24, 24)
    assert np.abs(K - K.T).max() <= 1e-10 * np.abs(K).max()
    ev = np.linalg.eigvalsh(0.5 * (K + K.T))
    assert np.sum(ev < 1e-9 * ev[-1]) == 6 and ev[0] > -1e-9 * ev[-1]
    assert np.all(np.linalg.eigvalsh(K8 - K) > -1e-6 * ev[-1])  # condensation only softens
    np.testing.assert_array_equal(m81, m8)
