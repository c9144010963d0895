"""CPU tests pinning the oracle's beam2 element (type 2).

The reference's own beam2 cannot be run (its Rust toolchain is absent) and no
example of the reference uses it, so the element is pinned by beam theory:
  * the hexBeam / shellBeam known answers, restated for a 10 x 1 x 0.1 beam
    line (tip w = F L^3 / (3 E I) = 8, dw/dE = -8e-6, axial F L / (E A) = 2e-4,
    first frequency (0.56 / L^2) sqrt(E I / m)), stored in
    tests/golden/analytic_pins.json;
  * exact closed forms the element reproduces at any mesh: axial stretch,
    torsion T L / (G J), and the Timoshenko tip deflection
    F L^3 / (3 E I) + F L / (G A) within the element's O(1/n^2) error;
  * element invariants: symmetry, six rigid-body modes in the null space of
    K_e, total mass rho A L, frame invariance.
Tolerances are written per check; 1e-7 on quantities the element gets exactly
leaves room for the penalty clamp (scale 1e5 max|K|).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from asend3d_gb300.mesh import line_beam2
from asend3d_gb300.solver import Problem

GOLD = Path(__file__).resolve().parent / "golden"
L, B, H, E0 = 10.0, 1.0, 0.1, 1e6
A = B * H
IZZ = B * H**3 / 12.0   # int z^2 dA: bending in the x-z plane
IYY = H * B**3 / 12.0   # int y^2 dA
J = 2.8e-4              # any positive torsion constant


def section(v=(0.0, 1.0, 0.0), i1=0.0, i2=0.0, i5=0.0):
    return np.array([A, i1, i2, IZZ, IYY, i5, J, *v], np.float64)


def cantilever(n=100, F=(0.0, 0.0, 2.0, 0.0, 0.0, 0.0), direction=(1.0, 0.0, 0.0), v=(0.0, 1.0, 0.0), rho=None):
    m = line_beam2(n, L, direction)
    ne = m.n_elems
    p = Problem(m, np.full(ne, E0), np.full(ne, 0.0), None if rho is None else np.full(ne, rho))
    p.beam_sections = np.tile(section(v), (ne, 1))
    p.add_node_set("root", np.array([0], np.int32))
    p.add_node_set("tip", np.array([n], np.int32))
    p.fix_displacement("root", comps=(1, 2, 3, 4, 5, 6))
    p.add_nodal_force("tip", list(F))
    return p


def tip_solution(po, p):
    o = po.Oracle(p)
    f = o.loads()[0]
    u, rc, st = o.solve(f, precond=po.PC_DIRECT)
    assert rc == 0
    n = p.mesh.n_elems
    return u[6 * n:6 * n + 6], u, o


def pins():
    return json.loads((GOLD / "analytic_pins.json").read_text())


def test_element_invariants(oracle_lib):
    rng = np.random.default_rng(7)
    for _ in range(5):
        x0 = rng.uniform(-1, 1, 3)
        x1 = x0 + rng.uniform(-2, 2, 3)
        v = rng.normal(size=3)
        sec = np.array([0.3, 0.01, -0.02, 2e-3, 3e-3, 4e-4, 5e-3, *v])  # positive-definite C
        ke, me = oracle_lib.beam_element(np.stack([x0, x1]), 2e11, 0.3, 7800.0, sec)
        # symmetric to rounding
        assert np.abs(ke - ke.T).max() <= 1e-12 * np.abs(ke).max()
        assert np.abs(me - me.T).max() <= 1e-12 * np.abs(me).max()
        # six rigid-body modes: translations t and small rotations w about x0
        for k in range(6):
            u = np.zeros(12)
            for a, xa in enumerate((x0, x1)):
                if k < 3:
                    u[6 * a + k] = 1.0
                else:
                    w = np.eye(3)[k - 3]
                    u[6 * a:6 * a + 3] = np.cross(w, xa - x0)
                    u[6 * a + 3:6 * a + 6] = w
            assert np.abs(ke @ u).max() <= 1e-9 * np.abs(ke).max()
        # total translational mass rho A L in each direction
        Le = np.linalg.norm(x1 - x0)
        for k in range(3):
            t = np.zeros(12)
            t[k] = t[6 + k] = 1.0
            assert t @ me @ t == pytest.approx(7800.0 * 0.3 * Le, rel=1e-12)
        # exactly 6 zero eigenvalues
        ev = np.linalg.eigvalsh(0.5 * (ke + ke.T))
        assert (ev > 1e-9 * ev.max()).sum() == 6 and ev.min() > -1e-9 * ev.max()


def test_degenerate_frames_rejected(oracle_lib):
    with pytest.raises(ValueError):
        oracle_lib.beam_element(np.array([[0, 0, 0], [0, 0, 0]], float), 1e6, 0.0, 1.0, section())
    with pytest.raises(ValueError):
        oracle_lib.beam_element(np.array([[0, 0, 0], [1, 0, 0]], float), 1e6, 0.0, 1.0, section(v=(2.0, 0, 0)))


def test_transverse_tip_pin(oracle_lib):
    """hexBeam / shellBeam known answer on a beam line: w = 8 (rtol 1e-3, the
    pin's), and the element's own Timoshenko value within 3e-5 relative."""
    pin = pins()["hexBeam_transverse_tip"]
    t, _, _ = tip_solution(oracle_lib, cantilever())
    assert t[2] == pytest.approx(pin["value"], rel=pin["rtol"])
    timo = 2.0 * L**3 / (3 * E0 * IZZ) + 2.0 * L / (0.5 * E0 * A)
    assert t[2] == pytest.approx(timo, rel=3e-5)
    assert t[4] == pytest.approx(-2.0 * L**2 / (2 * E0 * IZZ), rel=1e-7)  # tip th2 = -F L^2 / (2 E I)
    assert abs(t[0]) + abs(t[1]) + abs(t[3]) + abs(t[5]) <= 1e-9


def test_convergence_order(oracle_lib):
    """Error of the tip deflection falls as 1/n^2 (one-point-shear Timoshenko)."""
    timo = 2.0 * L**3 / (3 * E0 * IZZ) + 2.0 * L / (0.5 * E0 * A)
    err = [abs(tip_solution(oracle_lib, cantilever(n))[0][2] - timo) for n in (10, 20, 40)]
    assert 3.6 < err[0] / err[1] < 4.4 and 3.6 < err[1] / err[2] < 4.4


def test_axial_and_torsion_exact(oracle_lib):
    pin = pins()["shellBeam_axial_tip"]
    t, _, _ = tip_solution(oracle_lib, cantilever(20, F=(2.0, 0, 0, 0, 0, 0)))
    assert t[0] == pytest.approx(pin["value"], rel=1e-6)
    T = 0.3
    t, _, _ = tip_solution(oracle_lib, cantilever(20, F=(0, 0, 0, T, 0, 0)))
    assert t[3] == pytest.approx(T * L / (0.5 * E0 * J), rel=1e-7)


def test_lateral_bending_uses_other_inertia(oracle_lib):
    t, _, _ = tip_solution(oracle_lib, cantilever(100, F=(0, 2.0, 0, 0, 0, 0)))
    timo = 2.0 * L**3 / (3 * E0 * IYY) + 2.0 * L / (0.5 * E0 * A)
    assert t[1] == pytest.approx(timo, rel=3e-5)
    assert t[5] == pytest.approx(2.0 * L**2 / (2 * E0 * IYY), rel=1e-7)  # th3 = +F L^2 / (2 E I)


def test_frame_invariance(oracle_lib):
    """A beam along d with v in the plane of d and the load: the deflection
    along e3 matches the beam along x."""
    d = np.array([1.0, 2.0, 2.0]) / 3.0
    v = np.array([0.0, 0.0, 1.0])
    e3 = np.cross(d, v)
    e3 /= np.linalg.norm(e3)
    F = np.zeros(6)
    F[:3] = 2.0 * e3
    t, _, _ = tip_solution(oracle_lib, cantilever(100, F=tuple(F), direction=d, v=v))
    t_x, _, _ = tip_solution(oracle_lib, cantilever(100))
    assert t[:3] @ e3 == pytest.approx(t_x[2], rel=1e-7)
    assert np.linalg.norm(t[:3] - (t[:3] @ e3) * e3) <= 1e-7 * abs(t_x[2])


def test_modulus_gradient(oracle_lib):
    """dw/dE = -8e-6 summed over the elements (the pin), and the per-element
    gradient against central differences of the oracle (step 1e-3 E: the
    penalised system's solve noise, ~1e-10 of w, swamps smaller steps;
    truncation error ~1e-6 relative)."""
    pin = pins()["hexBeam_transverse_tip"]
    p = cantilever(40)
    p.objective = ("displacement", "tip", 3, 1.0)
    t, u, o = tip_solution(oracle_lib, p)
    dldu = np.zeros(o.n_dof)
    dldu[6 * 40 + 2] = 1.0
    g, _, rc, _ = o.adjoint(u, dLdu=dldu, precond=oracle_lib.PC_DIRECT)
    assert rc == 0
    assert g.sum() * E0 == pytest.approx(pin["dwdE"] * E0, rel=2e-3)
    assert g.sum() == pytest.approx(-t[2] / E0, rel=1e-9)
    for e in (0, 17, 39):
        w = []
        for s in (1.0, -1.0):
            q = cantilever(40)
            q.E = q.E.copy()
            q.E[e] *= 1.0 + s * 1e-3
            w.append(tip_solution(oracle_lib, q)[0][2])
        fd = (w[0] - w[1]) / (2e-3 * E0)
        assert g[e] == pytest.approx(fd, rel=1e-4)


def test_first_frequency_pin(oracle_lib):
    pin = pins()["shellBeam_first_frequency_hz"]
    p = cantilever(100, F=(0, 0, 0, 0, 0, 0), rho=1.0)
    o = oracle_lib.Oracle(p, modal=True)
    _, fr, _, _ = o.eigen(2)
    f1 = min(fr)
    assert f1 == pytest.approx(pin["value"], rel=pin["rtol"])
    # beam theory: (1.8751^2 / (2 pi L^2)) sqrt(E I / (rho A)) (shear and rotary inertia: < 1e-4 here)
    assert f1 == pytest.approx(1.8751040687**2 / (2 * np.pi * L**2) * np.sqrt(E0 * IZZ / A), rel=2e-4)


def _tip_w(oracle_lib, E, nu, n=20):
    p = cantilever(n)
    p.E = np.full(n, E)
    p.nu = np.full(n, nu)
    return tip_solution(oracle_lib, p)[0][2]


def test_material_dv_pairs(oracle_lib):
    """Section-strain pairs of beam2 (bubbles recovered): the isotropic modulus
    gradient is -(C / E) : P per element (1e-10), and the reference's separate
    modulus (E with G held) and shearModulus (G with E held) DVs match central
    differences of the oracle (E and nu moved together to hold G or E; 1e-5)."""
    n = 20
    p = cantilever(n)
    t, u, o = tip_solution(oracle_lib, p)
    dldu = np.zeros(o.n_dof)
    dldu[6 * n + 2] = 1.0
    g, lam, rc, _ = o.adjoint(u, dLdu=dldu, precond=oracle_lib.PC_DIRECT)
    assert rc == 0
    P = o.strain_pairs(u, lam)
    sec = p.beam_sections[0]
    dE = oracle_lib.beam_section_dC(0, 1, sec)
    dG = sum(oracle_lib.beam_section_dC(1, k, sec) for k in (1, 2, 3))
    G0 = E0 / 2.0
    for e in range(n):
        assert -np.sum((dE * E0 + dG * G0) / E0 * P[e]) == pytest.approx(g[e], rel=1e-10)
    assert np.all(oracle_lib.beam_section_dC(2, 1, sec) == 0.0)
    g_E = -sum(np.sum(dE * P[e]) for e in range(n))
    g_G = -sum(np.sum(dG * P[e]) for e in range(n))
    h = 1e-3
    # E with G held: nu' = E' / (2 G) - 1
    wE = [_tip_w(oracle_lib, E0 * (1 + s * h), E0 * (1 + s * h) / (2 * G0) - 1.0) for s in (1, -1)]
    assert g_E == pytest.approx((wE[0] - wE[1]) / (2 * h * E0), rel=1e-5)
    # G with E held: nu' = E / (2 G') - 1
    wG = [_tip_w(oracle_lib, E0, E0 / (2 * G0 * (1 + s * h)) - 1.0) for s in (1, -1)]
    assert g_G == pytest.approx((wG[0] - wG[1]) / (2 * h * G0), rel=1e-5)


def _section_matrices(E, nu, rho, sec):
    """The computed section stiffness and mass (element_properties.rs:921-1010,
    :1440-1497) written out, for the given-matrix checks."""
    G = E / (2 * (1 + nu))
    A_, i1, i2, i3, i4, i5, J_ = sec[:7]
    C = np.zeros((6, 6))
    C[0, 0], C[0, 4], C[0, 5] = E * A_, E * i1, -E * i2
    C[1, 1], C[1, 3], C[2, 2], C[2, 3], C[3, 3] = G * A_, -G * i1, G * A_, G * i2, G * J_
    C[4, 4], C[4, 5], C[5, 5] = E * i3, -E * i5, E * i4
    M = np.zeros((6, 6))
    M[0, 0] = M[1, 1] = M[2, 2] = rho * A_
    M[0, 4], M[1, 3], M[0, 5], M[2, 3] = rho * i1, -rho * i1, -rho * i2, rho * i2
    M[3, 3], M[4, 4], M[4, 5], M[5, 5] = rho * J_, rho * i3, rho * i5, rho * i4
    return np.triu(C) + np.triu(C, 1).T, np.triu(M) + np.triu(M, 1).T


def test_given_section_matrices(oracle_lib):
    """beamProps stiffness / mass given as matrices: the computed ones given
    back reproduce the element (1e-14), a stiffer given bending entry acts as
    a larger moment of inertia (1e-9), and the modulus adjoint refuses them."""
    sec = np.array([0.3, 0.01, -0.02, 2e-3, 3e-3, 4e-4, 5e-3, 0.3, -1.0, 0.5])
    xyz = np.array([[0.1, 0.2, -0.3], [1.1, -0.4, 0.5]])
    C, M = _section_matrices(2e11, 0.3, 7800.0, sec)
    k0, m0 = oracle_lib.beam_element(xyz, 2e11, 0.3, 7800.0, sec)
    k1, m1 = oracle_lib.beam_element(xyz, 2e11, 0.3, 7800.0, sec, given=np.concatenate([C.ravel(), M.ravel()]))
    assert np.abs(k1 - k0).max() <= 1e-14 * np.abs(k0).max()
    assert np.abs(m1 - m0).max() <= 1e-14 * np.abs(m0).max()
    # given stiffness with E I3 doubled == a section with I3 doubled
    n = 20
    p = cantilever(n)
    Cg, _ = _section_matrices(E0, 0.0, 0.0, section())
    Cg[4, 4] *= 2.0
    p.beam_section_matrices = (Cg.ravel(), None)
    q = cantilever(n)
    q.beam_sections = q.beam_sections.copy()
    q.beam_sections[:, 3] *= 2.0
    t1, u1, o1 = tip_solution(oracle_lib, p)
    t2, _, _ = tip_solution(oracle_lib, q)
    assert t1[2] == pytest.approx(t2[2], rel=1e-9)
    _, _, rc, _ = o1.adjoint(u1, dLdu=np.ones(o1.n_dof), precond=oracle_lib.PC_DIRECT)
    assert rc == -2


def test_section_dvs_against_differences(oracle_lib):
    """The reference's beam section DVs (area, areaMoment, polarMoment) through
    the section-strain pairs, against central differences of the oracle on
    L = tip w + tip twist under a tip force and torque (step 1e-3; 1e-4: the
    penalty scale follows max|K|, which moves with A, a 1e-5 effect that the
    adjoint, like the reference's, leaves out)."""
    n = 20
    F = (0.0, 0.0, 2.0, 0.3, 0.0, 0.0)

    def objective(scale_col=None, h=0.0):
        p = cantilever(n, F=F)
        if scale_col is not None:
            p.beam_sections = p.beam_sections.copy()
            p.beam_sections[:, scale_col] *= 1.0 + h
        t, u, o = tip_solution(oracle_lib, p)
        return t[2] + t[3], u, o, p

    L0, u, o, p = objective()
    dldu = np.zeros(o.n_dof)
    dldu[6 * n + 2] = dldu[6 * n + 3] = 1.0
    lam, _, _ = o.solve(dldu, precond=oracle_lib.PC_DIRECT)
    P = o.strain_pairs(u, lam)
    sec = p.beam_sections[0]
    for cat, comp, col in ((3, 0, 0), (4, 3, 3), (5, 0, 6)):
        dC = oracle_lib.beam_section_dC(cat, comp, sec, E=E0, nu=0.0)
        g = -sum(np.sum(dC * P[e]) for e in range(n))
        h = 1e-3
        fd = (objective(col, h)[0] - objective(col, -h)[0]) / (2 * h * sec[col])
        assert g == pytest.approx(fd, rel=1e-4), (cat, comp)
