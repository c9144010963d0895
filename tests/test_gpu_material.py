"""Orthotropic solids, damping and lumped mass on the GPU against the FP64
oracle (reference: get_solid_stiff element_properties.rs:648-764, get_rud
element_equations.rs:628-850, the dynamic combination :852-1062 with the
lumped-mass branch :950-971).

Tolerances:
  * assembled operator, mass and damping values: 2e-11 of the largest entry;
  * static displacements at rel_tol 1e-11: 1e-8 relative;
  * Newmark histories and final displacements (direct oracle solves, GPU
    PCG to 1e-12): 1e-8 relative;
  * orthotropic material DV gradients against central differences of the
    oracle's compliance (step 1e-5 of the constant): 1e-4 relative (the
    difference also moves the penalty scale).
"""
import numpy as np
import pytest

from asend3d_gb300 import _lib, configs
from asend3d_gb300.mesh import block_tet4
from asend3d_gb300.solver import GpuSolver, Problem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def ortho_props(n_el, seed=0):
    """Seeded orthotropic constants (a fibre-like material, varied per element)."""
    rng = np.random.default_rng(seed)
    s = np.exp(0.2 * rng.standard_normal(n_el))
    E = np.stack([140e9 * s, 10e9 * s, 10e9 * s], 1)
    nu = np.tile([0.3, 0.3, 0.4], (n_el, 1))
    G = np.stack([5e9 * s, 5e9 * s, 3.6e9 * s], 1)
    return np.concatenate([E, nu, G], 1)


def csr_close(g, o, which_gpu, which_orc):
    rp, col, val = g.csr(which=which_gpu)
    orp, ocol, oval = o.csr(which=which_orc)
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    assert np.abs(val - oval).max() <= 2e-11 * np.abs(oval).max()


@pytest.mark.parametrize("kind", ["hex8", "tet4"])
def test_orthotropic_operator_and_solve(gpu_lib, oracle_lib, kind):
    p = configs.cantilever_small(nx=8, ny=2, nz=2)
    if kind == "tet4":
        m = block_tet4(6, 2, 2, 2.0, 0.4, 0.4)
        q = Problem(m, np.full(m.n_elems, 200e9), np.full(m.n_elems, 0.3), np.full(m.n_elems, 7850.0))
        q.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
        q.fix_displacement("xMin")
        q.add_node_set("tip", [int(np.argmax(m.coords[:, 0] + m.coords[:, 2]))])
        q.add_nodal_force("tip", [0.0, 0.0, -1000.0])
        p = q
    p.ortho = ortho_props(p.mesh.n_elems)
    g = GpuSolver(p)
    g.assemble(precision=64)
    o = oracle_lib.Oracle(p)
    csr_close(g, o, 2, 0)
    u, rc, _ = g.static_solve(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-11)
    assert rc == 0
    ur, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    assert rel(u[0], ur) < 1e-8
    g.close()


def test_orthotropic_material_dv_gradient(gpu_lib, oracle_lib):
    p = configs.cantilever_small(nx=8, ny=2, nz=2)
    p.objective = ("compliance",)
    props = ortho_props(p.mesh.n_elems, seed=3)
    p.ortho = props
    g = GpuSolver(p)
    g.assemble(precision=64)
    g.static_solve(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-12)
    L, gE, rc, _ = g.adjoint_gradient(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-12, want_dLdE=False)
    assert rc == 0 and gE is None

    def compliance(pp):
        q = Problem(p.mesh, p.E, p.nu, p.rho, p.node_sets, p.elem_sets, p.constraints, p.loads, ("compliance",),
                    ortho=pp)
        o = oracle_lib.Oracle(q)
        f = o.loads()[0] + o.penalty_rhs()
        ur, _, _ = o.solve(f, precond=oracle_lib.PC_DIRECT)
        return f @ ur

    for cat, comp, col in [(_lib.DV_MODULUS, 1, 0), (_lib.DV_MODULUS, 2, 1), (_lib.DV_SHEAR_MODULUS, 1, 6),
                           (_lib.DV_POISSON_RATIO, 3, 5)]:
        d = g.material_dv_gradient(cat, comp, "all")
        h = 1e-5 * np.abs(props[:, col]).mean()
        pp, pm = props.copy(), props.copy()
        pp[:, col] += h
        pm[:, col] -= h
        fd = (compliance(pp) - compliance(pm)) / (2 * h)
        assert d == pytest.approx(fd, rel=1e-4), (cat, comp)
    g.close()


@pytest.mark.parametrize("case", ["rayleigh", "material", "lumped", "lumped_damped"])
def test_newmark_damping_and_lumped_mass(gpu_lib, oracle_lib, case):
    p = configs.cantilever_small(nx=10, ny=2, nz=2)
    ne = p.mesh.n_elems
    if case == "rayleigh":
        p.damping = (40.0, 2e-5, None)
    elif case == "material":
        D = np.zeros((ne, 36))
        for i in range(3):
            for j in range(3):
                D[:, 6 * i + j] = 4e5 if i == j else 1e5
        for i in range(3, 6):
            D[:, 7 * i] = 1.5e5
        p.damping = (0.0, 0.0, D)
    elif case == "lumped":
        p.lump_mass = True
    else:
        p.lump_mass = True
        p.damping = (40.0, 1e-5, None)
    dt, beta, gamma = 1e-4, 0.25, 0.5
    n = 60
    t = np.arange(n) * dt
    amp = np.exp(-0.5 * ((t - 2e-3) / 5e-4) ** 2)
    tip = int(p.node_sets["tip"][0])
    g = GpuSolver(p)
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    o = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    csr_close(g, o, 2, 0)
    csr_close(g, o, 1, 1)
    if p.damping is not None:
        csr_close(g, o, 3, 3)
    hist, u, rc, st = g.newmark(amp, probe_dof=3 * tip + 2, method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI,
                                rel_tol=1e-12)
    assert rc == 0
    href, uref, rc2, _ = o.newmark(n, dt, beta, gamma, o.loads()[0], amp, 3 * tip + 2, precond=oracle_lib.PC_DIRECT)
    assert rc2 == 0
    assert rel(hist, href) < 1e-8
    assert rel(u, uref) < 1e-8
    g.close()


def test_damping_reduces_the_response(gpu_lib):
    """Mass-proportional damping lowers the free vibration after the pulse."""
    p0 = configs.cantilever_small(nx=10, ny=2, nz=2)
    p1 = configs.cantilever_small(nx=10, ny=2, nz=2)
    p1.damping = (400.0, 0.0, None)
    dt = 1e-4
    amp = np.exp(-0.5 * ((np.arange(200) * dt - 2e-3) / 5e-4) ** 2)
    tip = int(p0.node_sets["tip"][0])
    late = []
    for p in (p0, p1):
        g = GpuSolver(p)
        g.assemble(dynamic=True, dt=dt, beta=0.25, gamma=0.5)
        hist, _, rc, _ = g.newmark(amp, probe_dof=3 * tip + 2, method=_lib.METHOD_FP64, rel_tol=1e-10)
        assert rc == 0
        late.append(np.abs(hist[120:]).max())
        g.close()
    assert late[1] < 0.7 * late[0]


def test_shell_rayleigh_mass_damping_and_lumped_mass(gpu_lib, oracle_lib):
    p = configs.shell_plate(n=8)
    p.damping = (200.0, 0.0, None)
    p.lump_mass = True
    dt, beta, gamma = 2e-5, 0.25, 0.5
    amp = configs.gaussian_pulse(40, dt, width=1e-4, t0=3e-4)
    probe = 6 * int(p.node_sets["centre"][0]) + 2
    g = GpuSolver(p)
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    hist, u, rc, _ = g.newmark(amp, probe_dof=probe, method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-12)
    assert rc == 0
    o = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    href, uref, rc2, _ = o.newmark(len(amp), dt, beta, gamma, o.loads()[0], amp, probe, precond=oracle_lib.PC_DIRECT)
    assert rc2 == 0
    assert rel(hist, href) < 1e-7
    assert rel(u, uref) < 1e-7
    g.close()
