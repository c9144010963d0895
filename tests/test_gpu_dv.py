"""Material design-variable gradients from the adjoint strain-pair tensors
(asend_adjoint_strain_pairs, asend_material_dv_gradient) against the
oracle, exact identities, finite differences, and through a job file.

Tolerances (written here, per quantity):
  * pairs contracted with C_e / E_e vs the isotropic per-element gradient
    of the same adjoint: 1e-12 relative to max |g|;
  * modulus-component gradients vs the oracle's restatement
    (orc_adjoint_modulus_component_gradient, PCG to 1e-12 vs a direct
    solve): 1e-8;
  * isotropic identity sum_k dL/dE_k + sum_k dL/dG_k / (2 (1 + nu)) =
    sum_e dL/dE_e: 1e-10;
  * Poisson components vs a central difference of the oracle's objective
    in nu (step 1e-6, with G = E / (2 (1 + nu)) following): 1e-5; the
    difference also moves the penalty scale sf = 1e5 max|K| (which depends on
    nu), which the adjoint holds fixed as the reference does (3e-6 here).
"""
import numpy as np
import pytest

from asend3d_gb300 import _lib
from asend3d_gb300 import job as J
from asend3d_gb300.mesh import block_hex8, block_tet4
from asend3d_gb300.solver import AsendError, GpuSolver, Problem

from test_job import write_cantilever_job

pytestmark = pytest.mark.gpu
KW = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-12, max_iter=100000)


def beam(kind="hex8", nu=0.3):
    m = block_tet4(4, 2, 2, 1.0, 0.3, 0.2) if kind == "tet4" else block_hex8(6, 2, 2, 1.2, 0.3, 0.2)
    rng = np.random.default_rng(4)
    p = Problem(m, rng.uniform(60e9, 80e9, m.n_elems), np.full(m.n_elems, nu), np.full(m.n_elems, 2700.0))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    tip = m.nodes_in_range(xr=(m.coords[:, 0].max() - 1e-9, 1e9))
    p.add_node_set("tip", tip)
    p.fix_displacement("xMin")
    p.add_nodal_force("tip", [0.0, 200.0, -1000.0])
    p.objective = ("displacement", "tip", 3, 1.0 / len(tip))
    p.add_elem_set("all", np.arange(m.n_elems))
    p.add_elem_set("half", np.arange(m.n_elems // 2))
    return p


def iso_C(E, nu):
    la, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    C = np.zeros((6, 6))
    C[:3, :3] = la
    C[:3, :3] += 2 * mu * np.eye(3)
    C[3:, 3:] = mu * np.eye(3)
    return C


@pytest.mark.parametrize("kind", ["hex8", "tet4"])
def test_pairs_reproduce_isotropic_gradient(gpu_lib, kind):
    p = beam(kind)
    g = GpuSolver(p)
    g.assemble(precision=64)
    g.static_solve(**KW)
    L, gE, rc, st = g.adjoint_gradient(**KW)
    P = g.strain_pairs()
    giso = np.array([-(iso_C(1.0, nu) * P[e]).sum() for e, nu in enumerate(p.nu)])
    assert np.abs(giso - gE).max() <= 1e-12 * np.abs(gE).max()
    g.close()


def test_modulus_components_match_oracle(gpu_lib, oracle_lib):
    p = beam()
    g = GpuSolver(p)
    g.assemble(precision=64)
    g.static_solve(**KW)
    g.adjoint_gradient(**KW)
    o = oracle_lib.Oracle(p)
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    tip = p.node_sets["tip"]
    dLdu = np.zeros(o.n_dof)
    dLdu[3 * tip + 2] = 1.0 / len(tip)
    _, lam, _, _ = o.adjoint(uo, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
    coefs = np.linspace(0.5, 2.0, len(p.elem_sets["half"]))
    for k in (1, 2, 3):
        ge = o.component_gradient(uo, lam, k)
        assert g.material_dv_gradient("modulus", k, "all") == pytest.approx(ge.sum(), rel=1e-8)
        assert g.material_dv_gradient("modulus", k, "half", coefs) == pytest.approx(
            (coefs * ge[p.elem_sets["half"]]).sum(), rel=1e-8)
    g.close()


def test_isotropic_identity_and_poisson_fd(gpu_lib, oracle_lib):
    nu = 0.3
    p = beam(nu=nu)
    p.E[:] = 70e9  # uniform, so dG/dnu is one number
    g = GpuSolver(p)
    g.assemble(precision=64)
    g.static_solve(**KW)
    L, gE, rc, st = g.adjoint_gradient(**KW)
    gEk = [g.material_dv_gradient("modulus", k, "all") for k in (1, 2, 3)]
    gGk = [g.material_dv_gradient("shearModulus", k, "all") for k in (1, 2, 3)]
    gNk = [g.material_dv_gradient("poissonRatio", k, "all") for k in (1, 2, 3)]
    assert sum(gEk) + sum(gGk) / (2 * (1 + nu)) == pytest.approx(gE.sum(), rel=1e-10)
    # d L / d nu (isotropic, G following nu) by central differences of the oracle
    def objective(nu_v):
        q = beam(nu=nu_v)
        q.E[:] = 70e9
        o = oracle_lib.Oracle(q)
        u, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
        return u[3 * q.node_sets["tip"] + 2].mean()
    h = 1e-6
    fd = (objective(nu + h) - objective(nu - h)) / (2 * h)
    dG_dnu = -70e9 / (2 * (1 + nu) ** 2)
    assert sum(gNk) + dG_dnu * sum(gGk) == pytest.approx(fd, rel=1e-5)
    g.close()


def test_brickim_pairs_match_oracle(gpu_lib, oracle_lib):
    """brickIM: strain pairs with the condensed modes recovered against the
    oracle's (orc_adjoint_strain_pairs), 1e-8 of the largest entry; the
    pairs contracted with C_e / E_e reproduce the condensed per-element
    gradient (1e-10); material DV gradients equal -sum (dC/dD) : P_oracle."""
    p = beam()
    p.mesh.elem_type = 81
    g = GpuSolver(p)
    g.assemble(precision=64)
    g.static_solve(**KW)
    L, gE, rc, _ = g.adjoint_gradient(**KW)
    assert rc == 0
    P = g.strain_pairs()
    o = oracle_lib.Oracle(p)
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    tip = p.node_sets["tip"]
    dLdu = np.zeros(o.n_dof)
    dLdu[3 * tip + 2] = 1.0 / len(tip)
    _, lam, _, _ = o.adjoint(uo, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
    Po = o.strain_pairs(uo, lam)
    assert np.abs(P - Po).max() <= 1e-8 * np.abs(Po).max()
    giso = np.array([-(iso_C(1.0, nu) * P[e]).sum() for e, nu in enumerate(p.nu)])
    assert np.abs(giso - gE).max() <= 1e-10 * np.abs(gE).max()
    from test_gpu_job import compliance_dC
    for cat, k in (("modulus", 1), ("shearModulus", 3), ("poissonRatio", 2)):
        ref = -sum((compliance_dC(p.E[e], p.nu[e], p.E[e] / (2 * (1 + p.nu[e])), cat, k) * Po[e]).sum()
                   for e in range(p.mesh.n_elems))
        assert g.material_dv_gradient(cat, k, "all") == pytest.approx(ref, rel=1e-8)
    g.close()


@pytest.mark.parametrize("etype", ["brick8", "brickIM"])
def test_job_gradient_file(gpu_lib, oracle_lib, tmp_path, etype):
    """calcObjGradient through the job runner: the three DVs of the
    cantilever job against the oracle's strain pairs contracted with the
    compliance-form dC/dD (1e-7), brickIM with its condensed modes."""
    from test_gpu_job import compliance_dC
    m, xmin, xmax = write_cantilever_job(tmp_path, etype=etype, modal=False, dvs=True)
    r = J.JobRunner(tmp_path / "job.yaml").run()
    lines = (tmp_path / "obj_grad.csv").read_text().splitlines()
    assert lines[0] == "designVariable,objGrad" and len(lines) == 4
    grad = [float(ln.split(",")[1]) for ln in lines[1:]]
    if etype == "brickIM":
        m.elem_type = 81
    p = Problem(m, np.full(m.n_elems, 1e6), np.full(m.n_elems, 0.0), np.full(m.n_elems, 1.0))
    p.add_node_set("xMin", xmin)
    p.add_node_set("xMax", xmax)
    p.fix_displacement("xMin")
    p.add_nodal_force("xMax", [0.0, 0.0, -2.0 / len(xmax)])
    o = oracle_lib.Oracle(p)
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    dLdu = np.zeros(o.n_dof)
    dLdu[3 * xmax + 2] = 1.0 / len(xmax)
    _, lam, _, _ = o.adjoint(uo, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
    Po = o.strain_pairs(uo, lam)
    if etype == "brick8":
        assert grad[0] == pytest.approx(o.component_gradient(uo, lam, 1).sum(), rel=1e-7)
    dvs = [("modulus", 1, np.ones(m.n_elems)), ("shearModulus", 2, np.ones(m.n_elems)),
           ("poissonRatio", 3, np.array([2.0, 3.0, 4.0, 5.0]))]
    for k, (cat, comp, cf) in enumerate(dvs):
        dC = compliance_dC(1e6, 0.0, 5e5, cat, comp)
        ref = -np.sum(cf[:, None, None] * dC[None] * Po)
        assert grad[k] == pytest.approx(ref, rel=1e-7, abs=1e-9 * max(abs(g) for g in grad))
    # the bending beam's tip deflection falls as E1 grows
    assert grad[0] > 0  # w < 0, so dw/dE1 > 0
