"""Generate the committed golden fixtures from the FP64 oracle.

Run from the repository root:  python tests/golden/make_golden.py

cantilever_small.npz -- 20x4x4 hex8 cantilever (1575 DOF, E = 200 GPa,
nu = 0.3, x = 0 face fixed by penalty constraints, 1 kN downward at the free
end's top-centre node): displacement u (direct skyline LDL^T, the reference's
`direct` solver path), tip objective L = u_z(tip), per-element modulus
gradient dL/dE (adjoint), and the 80 column-group design-variable gradients.
tet_block.npz -- 4x2x2 tet4 block with a surface traction (u, operator
diagonal) for the tet4 path.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from asend3d_gb300 import configs  # noqa: E402
from asend3d_gb300.mesh import block_tet4  # noqa: E402
from asend3d_gb300.solver import Problem  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

OUT = Path(__file__).resolve().parent


def cantilever():
    p = configs.cantilever_small()
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    u, rc, st = o.solve(f, precond=po.PC_DIRECT)
    assert rc == 0
    tip = p.node_sets["tip"][0]
    dldu = np.zeros(o.n_dof)
    dldu[3 * tip + 2] = 1.0
    g, lam, rc, _ = o.adjoint(u, dLdu=dldu, precond=po.PC_DIRECT)
    assert rc == 0
    groups = np.array([g[p.elem_sets[name]].sum() for name, _ in p.design_vars])
    np.savez_compressed(OUT / "cantilever_small.npz", u=u, L=u[3 * tip + 2], dLdE=g, dLdD=groups, sf=o.sf)


def tet_block():
    m = block_tet4(4, 2, 2, 1.0, 0.5, 0.5)
    p = Problem(m, np.full(m.n_elems, 7.0e10), np.full(m.n_elems, 0.33), None)
    p.add_node_set("xMin", m.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")
    tets = np.arange(m.n_elems, dtype=np.int32)
    p.add_elem_set("all", tets)
    p.add_surface_traction("all", (1.0, 0.0, 0.0), (0.0, 0.0, -1.0e6))
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    u, rc, _ = o.solve(f, precond=po.PC_DIRECT)
    assert rc == 0
    np.savez_compressed(OUT / "tet_block.npz", u=u, f=o.loads()[0])


if __name__ == "__main__":
    cantilever()
    tet_block()
    print("wrote", sorted(x.name for x in OUT.glob("*.npz")))
