"""Modal test models shared by the CPU and GPU eigen tests: small cantilevers
of each element type, a clamped shell strip, and the dense inverse-operator
reference eigensolve."""
import numpy as np

from asend3d_gb300.mesh import block_hex8, block_tet4, plate_quad4
from asend3d_gb300.solver import Problem


def cantilever(nx, ny, nz, L, b, h, etype=8, E=70e9, nu=0.33, rho=2700.0):
    m = block_tet4(nx, ny, nz, L, b, h) if etype == 4 else block_hex8(nx, ny, nz, L, b, h)
    if etype == 81:
        m.elem_type = 81
    p = Problem(m, np.full(m.n_elems, E), np.full(m.n_elems, nu), np.full(m.n_elems, rho))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    return p


def shell_strip(nx=6, ny=3):
    m = plate_quad4(nx, ny, 0.6, 0.3)
    p = Problem(m, np.full(m.n_elems, 70e9), np.full(m.n_elems, 0.33), np.full(m.n_elems, 2700.0),
                thickness=np.full(m.n_elems, 0.004))
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin", comps=(1, 2, 3, 4, 5, 6))
    return p


def dense_reference(o, n):
    """Lowest n eigenvalues (and D-normalised vectors) of K x = lambda D x from
    the dense inverse operator D^1/2 K^-1 D^1/2: accurate at the low end even
    where D spans many decades (shell rotations at the mass floor), unlike a
    Cholesky-based generalised solver whose error scales with lambda_max."""
    rp, col, val = o.csr(2)
    K = np.zeros((o.n_dof, o.n_dof))
    for r in range(o.n_dof):
        K[r, col[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
    _, _, _, D = o.eigen(1)
    s = np.sqrt(D)
    Op = s[:, None] * np.linalg.inv(K) * s[None, :]
    th, Y = np.linalg.eigh(0.5 * (Op + Op.T))
    th, Y = th[::-1][:n], Y[:, ::-1][:, :n]
    X = Y / s[:, None]
    return 1.0 / th, K, D, X / np.linalg.norm(X, axis=0)


SMALL_MODELS = {"hex8": lambda: cantilever(8, 2, 2, 0.8, 0.2, 0.1, 8),
                "brickIM": lambda: cantilever(8, 2, 2, 0.8, 0.2, 0.1, 81),
                "tet4": lambda: cantilever(6, 2, 2, 0.6, 0.2, 0.1, 4),
                "shell4": shell_strip}


def genuine_pairs(ev, ref, rtol=1e-5):
    """Indices k of reported eigenvalues ev[k] that equal some eigenvalue of
    the dense reference (ref, ascending, longer than ev) within rtol, with
    the index of that eigenvalue.  The reference's Lanczos orthogonalises
    against the previous two vectors only (matrix_functions.rs:1156-1176), so
    it can report spurious Ritz pairs; which ones depends on rounding (FMA
    contraction differs between hosts), hence matching by value."""
    out = []
    for k, v in enumerate(ev):
        j = int(np.argmin(np.abs(ref - v)))
        if abs(ref[j] - v) <= rtol * abs(ref[j]):
            out.append((k, j))
    return out
