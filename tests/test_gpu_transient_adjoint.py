"""Transient adjoint on the GPU (reverse Newmark sweep over the kept
displacement history) against the oracle's restatement of the reference's
sweep (model_analysis.rs:1544-1631, augmentd_ld_u :936-1063,
solve_for_adjoint :1065-1126), which is itself pinned by central differences
(tests/test_transient_adjoint_oracle.py).

Tolerances: the objective (a sum of step displacements) 1e-9 relative and
the per-element modulus gradient 1e-6 relative norm-wise for the solid beam
(GPU FP64 PCG to 1e-12 per step against the oracle's direct solves); 5e-7
and 1e-5 for the shell plate, whose step displacements agree to 1e-7 in the
forward Newmark comparison at the same residual; kept states equal the run's
probe history and final displacement exactly."""
import numpy as np
import pytest

from asend3d_gb300 import _lib, configs
from asend3d_gb300.mesh import block_hex8
from asend3d_gb300.solver import GpuSolver, Problem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def beam():
    m = block_hex8(6, 2, 2, 1.0, 0.25, 0.25)
    E = 70e9 * (1.0 + 0.1 * np.sin(np.arange(m.n_elems)))
    p = Problem(m, E, np.full(m.n_elems, 0.3), np.full(m.n_elems, 2700.0))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    tip = m.nodes_in_range(xr=(1.0 - 1e-9, 2.0))
    p.add_node_set("tip", tip)
    p.add_nodal_force("tip", [0.0, 0.0, -1000.0])
    return p, 3 * tip + 2


# (beta, gamma) in the reference's convention (beta_standard = gamma - beta,
# node_meth.rs:127-138): both pairs keep beta_standard >= gamma / 2, the
# unconditionally stable range; (0.25, 0.55) adds numerical damping.  (0.3,
# 0.55) has beta_standard = 0.25 < 0.275 and its response grows without bound
# on the plate's rotational modes.
PAIRS = [(0.25, 0.5), (0.25, 0.55)]


@pytest.mark.parametrize("beta,gamma", PAIRS)
def test_transient_adjoint_beam(gpu_lib, oracle_lib, beta, gamma):
    p, dof = beam()
    dt, N = 2e-4, 40
    amp = np.sin(np.linspace(0.0, 3.0, N))
    w = np.full(len(dof), 1.0 / len(dof))
    g = GpuSolver(p)
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    g.keep_history(1)
    kw = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-12)
    hist, u, rc, _ = g.newmark(amp, probe_dof=int(dof[0]), **kw)
    assert rc == 0
    assert np.array_equal(g.step_state(N)[0], u)
    assert all(g.step_state(s + 1)[0][dof[0]] == hist[s] for s in range(N))
    L, gE, rc, st = g.newmark_adjoint(dof, w, **kw)
    assert rc == 0 and st["n_rhs"] == N
    o = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    Lo, go = o.newmark_adjoint(N, dt, beta, gamma, o.loads()[0], amp, dof, w)
    assert L == pytest.approx(Lo, rel=1e-9)
    assert rel(gE, go) < 1e-6
    g.close()


@pytest.mark.parametrize("beta,gamma", PAIRS)
def test_transient_adjoint_shell_plate(gpu_lib, oracle_lib, beta, gamma):
    p = configs.shell_plate(n=20)
    dt, N = 2e-6, 150
    amp = configs.gaussian_pulse(N, dt, width=5e-5, t0=1e-4)
    centre = int(p.node_sets["centre"][0])
    dof = np.array([6 * centre + 2])
    w = np.array([1.0])
    g = GpuSolver(p)
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    g.keep_history(1)
    kw = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-12)
    _, _, rc, _ = g.newmark(amp, **kw)
    assert rc == 0
    L, gE, rc, _ = g.newmark_adjoint(dof, w, **kw)
    assert rc == 0
    o = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    Lo, go = o.newmark_adjoint(N, dt, beta, gamma, o.loads()[0], amp, dof, w)
    # the plate's penalty-supported, rotation-carrying operator leaves 1e-7
    # in each step's displacements at 1e-12 residual, as in the forward test
    assert L == pytest.approx(Lo, rel=5e-7)
    assert rel(gE, go) < 1e-5
    g.close()


def test_history_fields_and_adjoint_guards(gpu_lib):
    from asend3d_gb300.solver import AsendError

    p, dof = beam()
    g = GpuSolver(p)
    g.assemble(dynamic=True, dt=2e-4, beta=0.25, gamma=0.5)
    with pytest.raises(AsendError, match="history"):
        g.newmark_adjoint(dof, np.ones(len(dof)))
    g.keep_history(3)
    amp = np.ones(12)
    _, u, rc, _ = g.newmark(amp, method=_lib.METHOD_FP64, rel_tol=1e-12)
    assert rc == 0
    u1, v1, a1 = g.step_state(1, fields=3)
    u2, v2, a2 = g.step_state(2, fields=3)
    # the Newmark relations between consecutive stored states (trapezoidal rule)
    dt = 2e-4
    assert rel(v2, v1 + 0.5 * dt * (a1 + a2)) < 1e-9
    assert rel(u2, u1 + dt * v1 + 0.25 * dt * dt * (a1 + a2)) < 1e-9
    g.close()
