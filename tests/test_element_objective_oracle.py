"""The oracle's element-category objective terms (stress / strain /
strainEnergy at the element centroid with powerNorm, ks, volumeIntegral and
volumeAverage; objective_meth.rs:329-516, :592-720, :1051-1160,
:1372-1500) pinned on the CPU:

* a known answer: with constant-strain tet4 elements, twice the
  volume-integrated centroid strain energy equals the compliance f^T u (up to
  the penalty supports' share, 1e-6 here);
* dL/du against central differences of L along random directions (1e-6);
* the adjoint total dL/dE_e = explicit - lambda^T dR/dE_e against central
  differences of L over re-solved displacements (step 1e-4 E, 1e-5);
* the explicit material pairs Q against the explicit modulus term
  (dC/dE = C/E for isotropic elements)."""
import numpy as np
import pytest

from asend3d_gb300.mesh import block_hex8, block_tet4
from asend3d_gb300.solver import Problem

po = pytest.importorskip("oracle.pyoracle")

CASES = [("strainEnergy", 0, "volumeIntegral", 2.0, 1.0, ()),
         ("strainEnergy", 0, "powerNorm", 1.0, 2.0, ()),
         ("stress", 1, "powerNorm", 1e-6, 2.0, ()),
         ("strain", 4, "powerNorm", 1.0, 2.0, (1e-5,)),
         ("stress", 6, "ks", 1.0, 4.0, (2e5,)),
         ("strainEnergy", 0, "volumeAverage", 3.0, 2.0, (0.5,))]


def cantilever(kind):
    if kind == "tet4":
        m = block_tet4(4, 2, 2, 2.0, 0.4, 0.4)
    else:
        m = block_hex8(4, 2, 2, 2.0, 0.4, 0.4)
        m.coords[:, 2] += 0.02 * np.sin(2.0 * m.coords[:, 0]) * m.coords[:, 1]
        if kind == "brickIM":
            m.elem_type = 81
    E = 70e9 * (1.0 + 0.2 * np.sin(np.arange(m.n_elems)))
    p = Problem(m, E, np.full(m.n_elems, 0.3))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    p.add_node_set("tip", m.nodes_in_range(xr=(2.0 - 1e-9, 3.0)))
    p.add_nodal_force("tip", [0.0, 1e3, -2e3])
    return p


def solve(p):
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    u, _, _ = o.solve(f, precond=po.PC_DIRECT)
    return o, f, u


def test_tet4_strain_energy_is_half_the_compliance():
    p = cantilever("tet4")
    o, f, u = solve(p)
    L, _, _, _ = o.element_objective(u, np.arange(p.mesh.n_elems), "strainEnergy", 0, "volumeIntegral", 2.0, 1.0)
    assert L == pytest.approx(float(o.loads()[0] @ u), rel=1e-6)


@pytest.mark.parametrize("kind", ["hex8", "tet4", "brickIM"])
@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[2]}" for c in CASES])
def test_dLdu_matches_differences(kind, case):
    p = cantilever(kind)
    o, _, u = solve(p)
    cat, comp, op, coef, ex, tg = case
    els = np.arange(0, p.mesh.n_elems, 2) if op != "volumeAverage" else np.arange(p.mesh.n_elems)
    L, dLdu, _, _ = o.element_objective(u, els, cat, comp, op, coef, ex, tg)
    rng = np.random.default_rng(3)
    for _ in range(2):
        d = rng.standard_normal(len(u)) * np.abs(u).max()
        h = 1e-7
        lp = o.element_objective(u + h * d, els, cat, comp, op, coef, ex, tg)[0]
        lm = o.element_objective(u - h * d, els, cat, comp, op, coef, ex, tg)[0]
        fd = (lp - lm) / (2 * h)
        assert dLdu @ d == pytest.approx(fd, rel=1e-6, abs=1e-12 * abs(L))


@pytest.mark.parametrize("kind", ["hex8", "tet4"])
@pytest.mark.parametrize("case", [CASES[0], CASES[2], CASES[4]], ids=["se-vi", "s1-pn", "s6-ks"])
def test_adjoint_total_gradient_matches_differences(kind, case):
    p = cantilever(kind)
    o, f, u = solve(p)
    cat, comp, op, coef, ex, tg = case
    els = np.arange(p.mesh.n_elems)
    L, dLdu, Q, dLdE = o.element_objective(u, els, cat, comp, op, coef, ex, tg)
    gE, lam, rc, _ = o.adjoint(u, dLdu=dLdu, precond=po.PC_DIRECT)
    assert rc == 0
    total = dLdE + gE
    for e in (0, 5, p.mesh.n_elems - 1):
        vals = []
        for s in (+1, -1):
            q = cantilever(kind)
            q.E = q.E.copy()
            q.E[e] *= 1.0 + s * 1e-4
            oq, _, uq = solve(q)
            vals.append(oq.element_objective(uq, els, cat, comp, op, coef, ex, tg)[0])
        fd = (vals[0] - vals[1]) / (2e-4 * p.E[e])
        assert total[e] == pytest.approx(fd, rel=1e-5, abs=1e-6 * np.abs(total).max())


def test_explicit_pairs_match_modulus_term():
    p = cantilever("hex8")
    o, _, u = solve(p)
    _, _, Q, dLdE = o.element_objective(u, np.arange(p.mesh.n_elems), "strainEnergy", 0, "powerNorm", 1.0, 2.0)
    for e in range(p.mesh.n_elems):
        E, nu = p.E[e], p.nu[e]
        lam, mu = nu / ((1 + nu) * (1 - 2 * nu)), 1 / (2 * (1 + nu))
        C1 = np.zeros((6, 6))
        C1[:3, :3] = lam
        C1[[0, 1, 2], [0, 1, 2]] += 2 * mu
        C1[[3, 4, 5], [3, 4, 5]] = mu
        assert np.sum(C1 * Q[e]) == pytest.approx(dLdE[e], rel=1e-10, abs=1e-14 * np.abs(dLdE).max())
