"""GPU modal analysis (asend_eigen_solve) against the dense inverse-operator
reference and the oracle's restatement of the reference's frequency job
(model_analysis.rs:711-880, matrix_functions.rs:1099-1265).

Tolerances (written here, per quantity):
  * diagonal mass vs the oracle: 1e-10 relative (same row sums; the oracle's
    element Jacobians come from the reference's Givens-QR determinant);
  * eigenvalues vs the dense reference: 1e-8 relative (Ritz tol 1e-10, inner
    solves to 1e-12; shells to 1e-10: 1e-7);
  * eigenvalues vs the oracle: 1e-5 relative on the oracle pairs that are
    genuine eigenvalues (its power-iteration Ritz values stop at 1e-8 in the
    Rayleigh quotient; its Lanczos can report spurious pairs, see
    eigen_cases.genuine_pairs); 5e-5 on the 9,963-DOF block, whose 5 n_modes
    basis leaves its fourth and fifth pairs less converged;
  * mode shapes vs dense: 1 - |cos| <= 1e-7 for simple eigenvalues;
  * the library's Ritz residual (its stopping measure): <= the tol asked;
  * FP64 pencil residual ||K x - lambda D x|| / ||K x|| over the unconstrained
    rows: <= 1e-6, shells 1e-5 (the penalty rows, sf = 1e5 max|K|, amplify
    any error in the tiny constrained components and are left out);
  * multigrid vs Jacobi inner solves on the same model: 1e-8 relative.
"""
import numpy as np
import pytest

from asend3d_gb300 import _lib
from asend3d_gb300.mesh import block_hex8
from asend3d_gb300.solver import AsendError, GpuSolver, Problem

from eigen_cases import SMALL_MODELS, cantilever, dense_reference, genuine_pairs
from test_eigen_cpu import shell_beam, shell_beam_pin

pytestmark = pytest.mark.gpu

TIGHT = dict(tol=1e-10, rel_tol=1e-12, max_iter=200000)


@pytest.mark.parametrize("kind", list(SMALL_MODELS))
def test_eigen_small_models(gpu_lib, oracle_lib, kind):
    p = SMALL_MODELS[kind]()
    o = oracle_lib.Oracle(p, modal=True)
    ref, K, Dref, X = dense_reference(o, 8)
    evo, _, _, _ = o.eigen(4)
    g = GpuSolver(p)
    kw = dict(TIGHT)
    rtol, rres = 1e-8, 1e-6
    if kind == "shell4":
        kw.update(rel_tol=1e-10, precond=_lib.PC_BLOCK)
        rtol, rres = 1e-7, 1e-5
    ev, fr, modes, D, rc, st = g.eigen(4, **kw)
    assert rc == _lib.ASEND_OK, st
    assert st["n_converged"] == 4
    np.testing.assert_allclose(D, Dref, rtol=1e-10)
    np.testing.assert_allclose(ev, ref[:4], rtol=rtol)
    np.testing.assert_allclose(fr, np.sqrt(ev) / (2 * np.pi), rtol=1e-14)
    pairs = [(k, j) for k, j in genuine_pairs(evo, ref) if j < 4]
    assert len(pairs) >= 2
    for k, j in pairs:
        assert ev[j] == pytest.approx(evo[k], rel=1e-5)
    for k in range(4):
        assert np.linalg.norm(modes[k]) == pytest.approx(1.0, rel=1e-12)
        assert modes[k][np.argmax(np.abs(modes[k]))] > 0
        assert abs(modes[k] @ X[:, k]) >= 1 - 1e-7
    assert st["max_rel_residual"] <= kw["tol"]
    free = free_rows(p, o.n_dof)
    for k in range(4):
        kx = K @ modes[k]
        r = (kx - ev[k] * D * modes[k])[free]
        assert np.linalg.norm(r) <= rres * np.linalg.norm(kx[free])
    g.close()


def free_rows(p, n_dof):
    dpn = p.mesh.dpn
    fixed = np.zeros(n_dof, bool)
    for terms, _ in p.constraints:
        for set_name, comp, _ in terms:
            fixed[dpn * p.node_sets[set_name] + comp - 1] = True
    return ~fixed


def test_eigen_repeated_pair_and_block_sizes(gpu_lib, oracle_lib):
    """Square section: the two bending families share each eigenvalue.  Block
    Lanczos (b >= 2) returns both copies, as the dense reference does."""
    p = cantilever(10, 2, 2, 1.0, 0.2, 0.2, 81)
    o = oracle_lib.Oracle(p, modal=True)
    ref, _, _, _ = dense_reference(o, 4)
    assert ref[1] == pytest.approx(ref[0], rel=1e-9)
    g = GpuSolver(p)
    for b in (2, 4):
        ev, _, _, _, rc, st = g.eigen(4, block_size=b, **TIGHT)
        assert rc == _lib.ASEND_OK, (b, st)
        np.testing.assert_allclose(ev, ref, rtol=1e-8)
    g.close()


def test_eigen_shift(gpu_lib, oracle_lib):
    p = SMALL_MODELS["brickIM"]()
    o = oracle_lib.Oracle(p, modal=True)
    ref, _, _, _ = dense_reference(o, 3)
    g = GpuSolver(p)
    ev, _, _, _, rc, _ = g.eigen(3, shift=0.5 * ref[0], **TIGHT)
    assert rc == _lib.ASEND_OK
    np.testing.assert_allclose(ev, ref, rtol=1e-8)
    # the unshifted operator is back afterwards (bit-exact values)
    rp, col, val = g.csr(0)
    g2 = GpuSolver(p)
    g2.eigen(1, **TIGHT)
    np.testing.assert_array_equal(val, g2.csr(0)[2])
    ev0, _, _, _, rc, _ = g.eigen(3, **TIGHT)
    np.testing.assert_allclose(ev0, ref, rtol=1e-8)
    g2.close()
    g.close()


def test_eigen_multigrid_inner_solves(gpu_lib, oracle_lib):
    """Structured hex8 block: multigrid-preconditioned and Jacobi shift-invert
    solves give the same pairs; the oracle's direct-factor Lanczos agrees."""
    m = block_hex8(40, 8, 8, 2.0, 0.4, 0.3)
    p = Problem(m, np.full(m.n_elems, 70e9), np.full(m.n_elems, 0.33), np.full(m.n_elems, 2700.0))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    g = GpuSolver(p)
    ev_j, _, mj, _, rc, st_j = g.eigen(5, tol=1e-10, rel_tol=1e-11, max_iter=100000)
    assert rc == _lib.ASEND_OK, st_j
    ev_m, _, mm, _, rc, st_m = g.eigen(5, tol=1e-10, rel_tol=1e-11, precond=_lib.PC_MG)
    assert rc == _lib.ASEND_OK, st_m
    np.testing.assert_allclose(ev_m, ev_j, rtol=1e-8)
    for k in range(5):
        assert abs(mm[k] @ mj[k]) >= 1 - 1e-6
    assert st_m["inner_iterations"] < st_j["inner_iterations"] / 10
    o = oracle_lib.Oracle(p, modal=True)
    evo, _, _, _ = o.eigen(5)
    np.testing.assert_allclose(ev_m, evo, rtol=5e-5)
    g.close()


def test_eigen_large_block_properties(gpu_lib):
    """36,663-DOF brickIM cantilever (L/h = 10, square section) with multigrid
    shift-invert: D-orthogonal modes, small true residuals, the repeated
    bending pair, and the first frequency near Euler-Bernoulli (shear and
    rotary inertia lower it by about 1 %)."""
    L, b, E, rho = 2.0, 0.2, 70e9, 2700.0
    m = block_hex8(100, 10, 10, L, b, b)
    m.elem_type = 81
    p = Problem(m, np.full(m.n_elems, E), np.full(m.n_elems, 0.0), np.full(m.n_elems, rho))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    g = GpuSolver(p)
    ev, fr, modes, D, rc, st = g.eigen(6, tol=1e-9, rel_tol=1e-10, precond=_lib.PC_MG)
    assert rc == _lib.ASEND_OK, st
    assert st["max_rel_residual"] <= 1e-9
    assert np.all(np.diff(ev) >= -1e-9 * ev[-1])
    G = modes @ (D[:, None] * modes.T)
    off = G - np.diag(np.diag(G))
    assert np.abs(off).max() <= 1e-6 * np.abs(np.diag(G)).max()
    assert fr[1] == pytest.approx(fr[0], rel=1e-7)
    f1 = 1.875104069 ** 2 / (2 * np.pi * L ** 2) * np.sqrt(E * (b ** 4 / 12) / (rho * b * b))
    assert 0.95 * f1 <= fr[0] <= 1.005 * f1
    g.close()


def test_eigen_shell_beam_frequency_pin(gpu_lib, oracle_lib):
    """The reference's shellBeam known answer (first natural frequency)."""
    p = shell_beam()
    o = oracle_lib.Oracle(p, modal=True)
    ref, _, _, _ = dense_reference(o, 3)
    g = GpuSolver(p)
    ev, fr, _, _, rc, st = g.eigen(3, tol=1e-10, rel_tol=1e-10, precond=_lib.PC_BLOCK, max_iter=200000)
    assert rc == _lib.ASEND_OK, st
    np.testing.assert_allclose(ev, ref, rtol=1e-7)
    pin = shell_beam_pin()
    assert fr[0] == pytest.approx(pin["value"], rel=pin["rtol"])
    g.close()


def test_eigen_input_checks(gpu_lib):
    p = SMALL_MODELS["hex8"]()
    g = GpuSolver(p)
    with pytest.raises(AsendError, match="block_size"):
        g.eigen(2, block_size=5)
    with pytest.raises(AsendError, match="too few DOF"):
        g.eigen(10000)
    g.eigen(2, **TIGHT)
    with pytest.raises(AsendError, match="dynamic=1"):
        g.newmark(np.ones(3))
    g.close()
