"""Element-category objective terms on the GPU (centroid strain / stress /
strain energy with powerNorm, ks, volumeIntegral, volumeAverage; reference
objective_meth.rs:329-516, :665-720, :1051-1160, :1372-1500) against the
oracle's restatement, which tests/test_element_objective_oracle.py pins by
central differences and the tet4 compliance identity.

Tolerances: objective values 1e-9 relative (displacements from FP64 PCG to
1e-12 against the oracle's direct solve); total dL/dE 1e-7 relative
norm-wise (adjoint PCG to 1e-12); strain-pair tensors with the explicit
material term 1e-7 of their largest entry."""
import numpy as np
import pytest

from asend3d_gb300 import _lib
from asend3d_gb300.mesh import block_hex8, block_tet4
from asend3d_gb300.solver import AsendError, GpuSolver, Problem

pytestmark = pytest.mark.gpu

CASES = [("strainEnergy", 0, "volumeIntegral", 2.0, 1.0, ()),
         ("strainEnergy", 0, "powerNorm", 1.0, 2.0, ()),
         ("stress", 1, "powerNorm", 1e-6, 2.0, ()),
         ("strain", 4, "powerNorm", 1.0, 2.0, (1e-5,)),
         ("stress", 6, "ks", 1.0, 4.0, (2e5,)),
         ("strainEnergy", 0, "volumeAverage", 3.0, 2.0, (0.5,))]


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def cantilever(kind):
    if kind == "tet4":
        m = block_tet4(6, 2, 2, 2.0, 0.4, 0.4)
    else:
        m = block_hex8(8, 3, 3, 2.0, 0.4, 0.4)
        m.coords[:, 2] += 0.02 * np.sin(2.0 * m.coords[:, 0]) * m.coords[:, 1]
        if kind == "brickIM":
            m.elem_type = 81
    E = 70e9 * (1.0 + 0.2 * np.sin(np.arange(m.n_elems)))
    p = Problem(m, E, np.full(m.n_elems, 0.3))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    p.add_node_set("tip", m.nodes_in_range(xr=(2.0 - 1e-9, 3.0)))
    p.add_nodal_force("tip", [0.0, 1e3, -2e3])
    p.add_elem_set("all", np.arange(m.n_elems))
    return p


OPTS = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-12)


@pytest.mark.parametrize("kind", ["hex8", "tet4", "brickIM"])
def test_element_objective_matches_oracle(gpu_lib, oracle_lib, kind):
    p = cantilever(kind)
    g = GpuSolver(p)
    g.assemble(precision=64)
    u, rc, _ = g.static_solve(**OPTS)
    assert rc == 0
    o = oracle_lib.Oracle(p)
    ur, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    for cat, comp, op, coef, ex, tg in CASES:
        els = np.arange(0, p.mesh.n_elems, 2) if op in ("powerNorm", "ks") else np.arange(p.mesh.n_elems)
        L = g.set_element_objective(els, cat, comp, op, coef, ex, tg)
        Lo, dLdu, Q, dLdE = o.element_objective(ur, els, cat, comp, op, coef, ex, tg)
        assert L == pytest.approx(Lo, rel=1e-9), (cat, op)
        _, gE, rc, _ = g.adjoint_gradient(**OPTS)
        assert rc == 0
        go, _, rco, _ = o.adjoint(ur, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
        assert rco == 0
        assert rel(gE, dLdE + go) < 1e-7, (cat, op)


def test_element_objective_strain_pairs_include_explicit_term(gpu_lib, oracle_lib):
    p = cantilever("hex8")
    g = GpuSolver(p)
    g.assemble(precision=64)
    u, rc, _ = g.static_solve(**OPTS)
    assert rc == 0
    els = np.arange(p.mesh.n_elems)
    g.set_element_objective(els, "strainEnergy", 0, "powerNorm", 1.0, 2.0)
    _, _, rc, _ = g.adjoint_gradient(want_dLdE=False, **OPTS)
    assert rc == 0
    P = g.strain_pairs()
    o = oracle_lib.Oracle(p)
    ur, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    _, dLdu, Q, _ = o.element_objective(ur, els, "strainEnergy", 0, "powerNorm", 1.0, 2.0)
    _, lam, _, _ = o.adjoint(ur, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
    Po = o.strain_pairs(ur, lam) - Q
    assert np.abs(P - Po).max() <= 1e-7 * np.abs(Po).max()
    # a material DV over all elements: the total derivative by the contraction
    gm = g.material_dv_gradient("modulus", 1, "all")
    assert np.isfinite(gm) and gm != 0.0


def test_element_fields_volumes_and_guards(gpu_lib):
    p = cantilever("tet4")
    g = GpuSolver(p)
    g.assemble(precision=64)
    with pytest.raises(AsendError, match="solve"):
        g.element_fields()
    u, rc, _ = g.static_solve(**OPTS)
    eps, sig, vol = g.element_fields()
    assert vol.sum() == pytest.approx(2.0 * 0.4 * 0.4, rel=1e-12)
    # isotropic C: sigma = lambda tr(eps) I + mu * engineering shear
    nu = 0.3
    lam = p.E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = p.E / (2 * (1 + nu))
    tr = eps[:, :3].sum(1)
    assert np.allclose(sig[:, 0], lam * tr + 2 * mu * eps[:, 0], rtol=1e-12, atol=1e-9 * np.abs(sig).max())
    assert np.allclose(sig[:, 3], mu * eps[:, 3], rtol=1e-12, atol=1e-9 * np.abs(sig).max())
    with pytest.raises(ValueError):
        g.set_element_objective([0, 1], "stress", 7)
    with pytest.raises(NotImplementedError):
        g.set_element_objective([0, 1], "mises", 0)
    g.close()
