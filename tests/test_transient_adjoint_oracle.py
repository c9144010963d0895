"""The oracle's restatement of the reference's transient adjoint (reverse
Newmark sweep, model_analysis.rs:1544-1631, :936-1063, :1065-1126) against
central finite differences of its own Newmark run (step 1e-6 E_e).

Tolerance 2e-5 relative per element: the difference also moves the penalty
scale sf = 1e5 max|K + c_M M|, which the adjoint holds fixed as the
reference does (about 4e-6 here)."""
import numpy as np
import pytest

from asend3d_gb300.mesh import block_hex8
from asend3d_gb300.solver import Problem


def beam(E):
    m = block_hex8(4, 1, 1, 1.0, 0.25, 0.25)
    p = Problem(m, np.asarray(E, float).copy(), np.full(m.n_elems, 0.3), np.full(m.n_elems, 2700.0))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    tip = m.nodes_in_range(xr=(1.0 - 1e-9, 2.0))
    p.add_node_set("tip", tip)
    p.add_nodal_force("tip", [0.0, 0.0, -1000.0])
    return p, tip


@pytest.mark.parametrize("beta,gamma", [(0.25, 0.5), (0.3, 0.55)])
def test_transient_adjoint_matches_finite_differences(oracle_lib, beta, gamma):
    E0 = np.array([70e9, 72e9, 68e9, 71e9])
    dt, N = 2e-4, 40  # about one and a half periods of the first bending mode
    amp = np.sin(np.linspace(0.0, 3.0, N))
    p, tip = beam(E0)
    dof = 3 * tip + 2
    w = np.full(len(dof), 1.0 / len(dof))

    def run(E):
        q, _ = beam(E)
        o = oracle_lib.Oracle(q, dynamic=True, dt=dt, beta=beta, gamma=gamma)
        return o.newmark_adjoint(N, dt, beta, gamma, o.loads()[0], amp, dof, w)

    L, g = run(E0)
    # L is the sum over steps of the mean tip deflection (the Newmark history)
    o = oracle_lib.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
    hist, _, _, _ = o.newmark(N, dt, beta, gamma, o.loads()[0], amp, int(dof[0]), precond=oracle_lib.PC_DIRECT)
    assert L == pytest.approx(hist.sum(), rel=1e-10)  # the four tip nodes move together
    for e in range(4):
        h = 1e-6 * E0[e]
        Ep, Em = E0.copy(), E0.copy()
        Ep[e] += h
        Em[e] -= h
        fd = (run(Ep)[0] - run(Em)[0]) / (2 * h)
        assert g[e] == pytest.approx(fd, rel=2e-5), e
