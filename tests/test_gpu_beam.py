"""GPU parity of the beam2 path (type 2) against the FP64 oracle.

Tolerances (written here, per quantity):
  * element stiffness / mass (FP64 both sides; the kernel works in the section
    frame and rotates blocks, the oracle builds global strain rows):
    1e-11 relative to max|K_e|, max|M_e|;
  * assembled operator: pattern bit-exact, values 1e-11 relative to max|K|;
  * displacements after an FP64 point-Jacobi solve: 1e-6 relative.  The
    slender penalty-clamped cantilever (L/h = 100) has an FP64 true-residual
    floor near 2e-9 under point Jacobi, so its solves stop at 1e-8; the short
    bent line (well conditioned) goes to 1e-11;
  * adjoint modulus gradients: 1e-5 relative (norm-wise), same reason;
  * Newmark probe history (steps solved to 1e-8): 1e-6 relative;
  * frequencies: 1e-6 relative to the dense spectrum of the oracle's K and
    diagonal mass (the oracle's own iterative pairs include unconverged ones).
The beam-theory pins (tip 8, dw/dE -8e-6, first frequency) are checked at the
known answers' own tolerances.
"""
import numpy as np
import pytest

from asend3d_gb300 import _lib
from asend3d_gb300.mesh import line_beam2
from asend3d_gb300.solver import AsendError, GpuSolver, Problem

from test_oracle_beam import A, E0, IZZ, L, cantilever, pins, section

pytestmark = pytest.mark.gpu

FP64 = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-11, max_iter=400000)
SLENDER = dict(FP64, rel_tol=1e-8)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def random_frame_problem(n=12, seed=5):
    """A bent line in 3D (every element its own frame), random E, nu, rho and
    sections with first moments and a product of inertia."""
    rng = np.random.default_rng(seed)
    m = line_beam2(n, 3.0)
    m.coords = np.cumsum(np.vstack([np.zeros(3), rng.uniform(0.1, 0.4, (n, 3)) * rng.choice([-1, 1], (n, 3))]), 0)
    ne = m.n_elems
    E, nu, rho = rng.uniform(5e10, 2e11, ne), rng.uniform(0.2, 0.35, ne), rng.uniform(2000, 8000, ne)
    sec = np.zeros((ne, 10))
    for e in range(ne):
        a = rng.uniform(0.01, 0.02)
        sec[e] = [a, 1e-4 * rng.normal(), 1e-4 * rng.normal(), rng.uniform(1e-5, 3e-5), rng.uniform(1e-5, 3e-5),
                  2e-7 * rng.normal(), rng.uniform(2e-5, 5e-5), *rng.normal(size=3)]
    p = Problem(m, E, nu, rho)
    p.beam_sections = sec
    return p


def test_beam_element_matrices_match_oracle(gpu_lib, oracle_lib):
    p = random_frame_problem()
    g = GpuSolver(p)
    ke, me = g.element_matrices()
    m = p.mesh
    for e in range(m.n_elems):
        ko, mo = oracle_lib.beam_element(m.coords[m.conn[e]], p.E[e], p.nu[e], p.rho[e], p.beam_sections[e])
        assert np.abs(ke[e] - ko).max() <= 1e-11 * np.abs(ko).max(), e
        assert np.abs(me[e] - mo).max() <= 1e-11 * np.abs(mo).max(), e
    g.close()


def test_beam_operator_and_static_solve(gpu_lib, oracle_lib):
    """Bent 3D line clamped at node 0, tip force and moment: operator, mass
    and the FP64 solve against the oracle's direct solve."""
    p = random_frame_problem()
    n = p.mesh.n_elems
    p.add_node_set("root", np.array([0], np.int32))
    p.add_node_set("tip", np.array([n], np.int32))
    p.fix_displacement("root", comps=(1, 2, 3, 4, 5, 6))
    p.add_nodal_force("tip", [1e3, -2e3, 5e2, 40.0, -10.0, 25.0])
    g = GpuSolver(p)
    o = oracle_lib.Oracle(p)
    g.assemble(precision=64)
    rp, col, val = g.csr(0)
    rpo, colo, valo = o.csr(2)
    np.testing.assert_array_equal(rp, rpo)
    np.testing.assert_array_equal(col, colo)
    assert np.abs(val - valo).max() <= 1e-11 * np.abs(valo).max()
    u, rc, st = g.static_solve(**FP64)
    assert rc == _lib.ASEND_OK, st
    uo, rco, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert rco == 0
    assert rel(u[0], uo) < 1e-6
    g.close()


def test_beam_cantilever_pins_and_adjoint(gpu_lib, oracle_lib):
    """The hexBeam / shellBeam cantilever as a beam line of 30 elements: tip
    w = 8 (pin rtol 1e-3; the element's discretisation error is 2.3e-4 here),
    dw/dE summed = -8e-6, per-element gradient against the oracle."""
    pin = pins()["hexBeam_transverse_tip"]
    n = 30
    p = cantilever(n)
    p.objective = ("displacement", "tip", 3, 1.0)
    g = GpuSolver(p)
    g.assemble(precision=64)
    u, rc, st = g.static_solve(**SLENDER)
    assert rc == _lib.ASEND_OK, st
    w = u[0][6 * n + 2]
    assert w == pytest.approx(pin["value"], rel=pin["rtol"])
    Lobj, gE, rc, st = g.adjoint_gradient(**SLENDER)
    assert rc == _lib.ASEND_OK
    assert gE.sum() == pytest.approx(pin["dwdE"], rel=2e-3)
    o = oracle_lib.Oracle(p)
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert w == pytest.approx(uo[6 * n + 2], rel=1e-6)
    dldu = np.zeros(o.n_dof)
    dldu[6 * n + 2] = 1.0
    go, _, _, _ = o.adjoint(uo, dLdu=dldu, precond=oracle_lib.PC_DIRECT)
    assert rel(gE, go) < 1e-5
    g.close()


def test_beam_newmark_matches_oracle(gpu_lib, oracle_lib):
    p = cantilever(20, rho=1.0)
    dt, beta, gamma, n = 0.05, 0.25, 0.5, 60
    amp = np.sin(np.linspace(0.0, np.pi, n))
    probe = 6 * 20 + 2
    g = GpuSolver(p)
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    hist, u, rc, st = g.newmark(amp, probe_dof=probe, method=_lib.METHOD_FP64, rel_tol=1e-8, max_iter=400000)
    assert rc == _lib.ASEND_OK
    o = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    href, uref, rc2, _ = o.newmark(n, dt, beta, gamma, o.loads()[0], amp, probe, precond=oracle_lib.PC_DIRECT)
    assert rc2 == 0
    assert rel(hist, href) < 1e-6
    assert rel(u, uref) < 1e-6
    assert hist.max() > 0
    g.close()


def test_beam_frequencies(gpu_lib, oracle_lib):
    from eigen_cases import dense_reference
    pin = pins()["shellBeam_first_frequency_hz"]
    p = cantilever(20, F=(0, 0, 0, 0, 0, 0), rho=1.0)
    o = oracle_lib.Oracle(p, modal=True)
    ref, _, Dref, _ = dense_reference(o, 6)
    g = GpuSolver(p)
    ev, fr, modes, D, rc, st = g.eigen(4, tol=1e-8, rel_tol=1e-9, max_iter=400000)
    assert rc == _lib.ASEND_OK, st
    np.testing.assert_allclose(D, Dref, rtol=1e-12)
    np.testing.assert_allclose(ev, ref[:4], rtol=1e-6)
    assert fr.min() == pytest.approx(pin["value"], rel=pin["rtol"])
    # the lowest mode is the first bending mode in the soft (x-z) plane; it
    # matches beam theory within the lumped mass's error (7e-4 at 20 elements)
    f1 = 1.8751040687**2 / (2 * np.pi * L**2) * np.sqrt(E0 * IZZ / A)
    assert fr.min() == pytest.approx(f1, rel=1e-3)
    g.close()


def test_beam_gravity_load(gpu_lib, oracle_lib):
    """Gravity on a centroidal section: rho A L / 2 per node, as the oracle's
    consistent-mass image."""
    p = cantilever(10, F=(0, 0, 0, 0, 0, 0), rho=2.5)
    p.add_elem_set("all", np.arange(10, dtype=np.int32))
    p.loads = []
    p.add_gravity("all", [0.0, 0.0, -9.81])
    g = GpuSolver(p)
    o = oracle_lib.Oracle(p)
    f = g.load_vector(0)
    fo = o.loads()[0]
    assert np.abs(f - fo).max() <= 1e-12 * np.abs(fo).max()
    assert f[2::6].sum() == pytest.approx(-9.81 * 2.5 * A * L, rel=1e-12)
    g.close()


def test_beam_input_checks(gpu_lib):
    m = line_beam2(4, 1.0)
    p = Problem(m, np.full(4, 1e9), np.full(4, 0.3))
    g = GpuSolver(p)
    with pytest.raises(AsendError, match="asend_set_beam_sections"):
        g.assemble(precision=64)
    g.close()
    p.beam_sections = section(v=(3.0, 0.0, 0.0))  # v along the element axis
    with pytest.raises(AsendError, match="along the element axis"):
        GpuSolver(p)
    p.beam_sections = section() * np.array([1, 1, 1, 1, 1, 1, 0, 1, 1, 1])  # J = 0
    with pytest.raises(AsendError, match="positive"):
        GpuSolver(p)
    m.coords[2] = m.coords[1]
    with pytest.raises(AsendError, match="zero length"):
        GpuSolver(Problem(m, np.full(4, 1e9), np.full(4, 0.3)))


def test_beam_material_dvs(gpu_lib, oracle_lib):
    """Section-strain pairs of the adjoint (bubbles recovered) against the
    oracle (1e-6 relative, the solves' floor), and the reference's separate
    material DVs on a beam: modulus component 1 (E in EA, EI), shearModulus
    components 1-3 (G in GA, GJ; GA; G I2), poissonRatio (absent from a beam
    section: zero), and the section DVs area, areaMoment and polarMoment."""
    n = 20
    p = cantilever(n)
    p.add_elem_set("all", np.arange(n, dtype=np.int32))
    p.objective = ("displacement", "tip", 3, 1.0)
    g = GpuSolver(p)
    g.assemble(precision=64)
    u, rc, _ = g.static_solve(**SLENDER)
    assert rc == _lib.ASEND_OK
    _, gE, rc, _ = g.adjoint_gradient(**SLENDER)
    assert rc == _lib.ASEND_OK
    P = g.strain_pairs()
    o = oracle_lib.Oracle(p)
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    dldu = np.zeros(o.n_dof)
    dldu[6 * n + 2] = 1.0
    go, lam, _, _ = o.adjoint(uo, dLdu=dldu, precond=oracle_lib.PC_DIRECT)
    Po = o.strain_pairs(uo, lam)
    assert rel(P, Po) < 1e-6
    sec = p.beam_sections[0]
    for cat, comp, name in ((0, 1, "modulus"), (1, 1, "shearModulus"), (1, 2, "shearModulus"),
                            (1, 3, "shearModulus"), (0, 2, "modulus"), (3, 0, "area"), (4, 3, "areaMoment"),
                            (4, 4, "areaMoment"), (5, 0, "polarMoment")):
        ref = -sum(np.sum(oracle_lib.beam_section_dC(cat, comp, sec, E=p.E[e], nu=p.nu[e]) * Po[e])
                   for e in range(n))
        got = g.material_dv_gradient(name, comp, "all")
        assert got == pytest.approx(ref, rel=1e-6, abs=1e-12 * abs(gE).max()), (name, comp)
    assert g.material_dv_gradient("poissonRatio", 1, "all") == 0.0
    # E and G together are the isotropic modulus gradient: dC/dE_iso = dC/dE1 + (G/E) sum_k dC/dG_k
    tot = g.material_dv_gradient("modulus", 1, "all") + 0.5 * sum(
        g.material_dv_gradient("shearModulus", k, "all") for k in (1, 2, 3))
    assert tot == pytest.approx(gE.sum(), rel=1e-9)
    g.close()


def test_beam_newmark_lumped_damped(gpu_lib, oracle_lib):
    """Newmark on a beam line with row-sum lumped mass and mass-proportional
    Rayleigh damping (the forms beam2 takes) against the oracle (1e-6)."""
    p = cantilever(20, rho=1.0)
    p.lump_mass = True
    p.damping = (0.3, 0.0, None)
    dt, beta, gamma, n = 0.05, 0.25, 0.5, 40
    amp = np.sin(np.linspace(0.0, np.pi, n))
    probe = 6 * 20 + 2
    g = GpuSolver(p)
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    hist, u, rc, st = g.newmark(amp, probe_dof=probe, method=_lib.METHOD_FP64, rel_tol=1e-8, max_iter=400000)
    assert rc == _lib.ASEND_OK
    o = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    href, uref, rc2, _ = o.newmark(n, dt, beta, gamma, o.loads()[0], amp, probe, precond=oracle_lib.PC_DIRECT)
    assert rc2 == 0
    assert rel(hist, href) < 1e-6
    assert rel(u, uref) < 1e-6
    g.close()


def test_beam_given_section_matrices(gpu_lib, oracle_lib):
    """beamProps stiffness / mass given as matrices on half of a bent line's
    elements (the other half computed): element matrices (1e-11), the static
    solve against the oracle (1e-6), the modulus adjoint refused, material DVs
    zero on the given-stiffness elements."""
    from test_oracle_beam import _section_matrices
    p = random_frame_problem(seed=9)
    ne = p.mesh.n_elems
    rng = np.random.default_rng(4)
    Cg, Mg = np.zeros((ne, 36)), np.zeros((ne, 36))
    for e in range(0, ne, 2):
        C, M = _section_matrices(p.E[e], p.nu[e], p.rho[e], p.beam_sections[e])
        S = np.diag(rng.uniform(0.8, 1.25, 6))  # a different, still positive-definite section
        Cg[e], Mg[e] = (S @ C @ S).ravel(), (S @ M @ S).ravel()
    p.beam_section_matrices = (Cg, Mg)
    p.add_node_set("root", np.array([0], np.int32))
    p.add_node_set("tip", np.array([ne], np.int32))
    p.add_elem_set("all", np.arange(ne, dtype=np.int32))
    p.fix_displacement("root", comps=(1, 2, 3, 4, 5, 6))
    p.add_nodal_force("tip", [1e3, -2e3, 5e2, 40.0, -10.0, 25.0])
    g = GpuSolver(p)
    ke, me = g.element_matrices()
    m = p.mesh
    for e in range(ne):
        given = np.concatenate([Cg[e], Mg[e]])
        ko, mo = oracle_lib.beam_element(m.coords[m.conn[e]], p.E[e], p.nu[e], p.rho[e], p.beam_sections[e], given)
        assert np.abs(ke[e] - ko).max() <= 1e-11 * np.abs(ko).max(), e
        assert np.abs(me[e] - mo).max() <= 1e-11 * np.abs(mo).max(), e
    g.assemble(precision=64)
    u, rc, st = g.static_solve(**FP64)
    assert rc == _lib.ASEND_OK, st
    o = oracle_lib.Oracle(p)
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert rel(u[0], uo) < 1e-6
    with pytest.raises(AsendError, match="isotropic"):
        g.adjoint_gradient(**FP64)
    g.adjoint_gradient(want_dLdE=False, **FP64)
    P = g.strain_pairs()
    mod = g.material_dv_gradient("modulus", 1, "all")
    ref = -sum(np.sum(oracle_lib.beam_section_dC(0, 1, p.beam_sections[e]) * P[e]) for e in range(1, ne, 2))
    assert mod == pytest.approx(ref, rel=1e-12)
    g.close()
