"""Structured meshes, node/element sets and seeded material fields.

The reference builds meshes in Python (asendUtils meshing, e.g.
``Mesh3D.createSweptMesh`` src/asendUtils/meshing/Mesh3D.py:45-289) and
selects node sets by coordinate ranges (``getNodeSetInXYZRange``
src/asendUtils/meshing/MeshTools.py:534-557).  These helpers generate the same
kind of structured hex8 blocks and coordinate-range sets directly as arrays.

Node numbering of a block is x-slowest, z-fastest: node(i, j, k) =
(i*(ny+1) + j)*(nz+1) + k, which keeps the matrix bandwidth of a long bar
(x the long axis) small.  Element corner order follows the reference's hex8
(element_soln_fields.rs:171-211: (-1,-1,-1), (1,-1,-1), (1,1,-1), (-1,1,-1),
then the same at +1).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class BlockMesh:
    nx: int
    ny: int
    nz: int
    lx: float
    ly: float
    lz: float
    coords: np.ndarray  # (n_nodes, 3) float64
    conn: np.ndarray    # (n_el, 8) int32
    elem_type: int = 8

    @property
    def n_nodes(self) -> int:
        return self.coords.shape[0]

    @property
    def n_elems(self) -> int:
        return self.conn.shape[0]

    @property
    def dpn(self) -> int:
        """DOF per node: 6 for shells and beams (u v w thx thy thz), else 3."""
        return 6 if self.elem_type in (41, 2) else 3

    @property
    def n_dof(self) -> int:
        return self.dpn * self.n_nodes

    def node_id(self, i, j, k):
        return (np.asarray(i) * (self.ny + 1) + np.asarray(j)) * (self.nz + 1) + np.asarray(k)

    def elem_id(self, i, j, k):
        return (np.asarray(i) * self.ny + np.asarray(j)) * self.nz + np.asarray(k)

    def centroids(self) -> np.ndarray:
        return self.coords[self.conn].mean(axis=1)

    def nodes_in_range(self, xr=None, yr=None, zr=None) -> np.ndarray:
        """Nodes with coordinates inside the closed ranges (getNodeSetInXYZRange)."""
        m = np.ones(self.n_nodes, dtype=bool)
        for ax, r in enumerate((xr, yr, zr)):
            if r is not None:
                m &= (self.coords[:, ax] >= r[0]) & (self.coords[:, ax] <= r[1])
        return np.nonzero(m)[0].astype(np.int32)

    def elems_in_range(self, xr=None, yr=None, zr=None) -> np.ndarray:
        c = self.centroids()
        m = np.ones(self.n_elems, dtype=bool)
        for ax, r in enumerate((xr, yr, zr)):
            if r is not None:
                m &= (c[:, ax] >= r[0]) & (c[:, ax] <= r[1])
        return np.nonzero(m)[0].astype(np.int32)


def block_hex8(nx: int, ny: int, nz: int, lx: float, ly: float, lz: float) -> BlockMesh:
    """nx*ny*nz hex8 elements on [0,lx]x[0,ly]x[0,lz]."""
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    zs = np.linspace(0.0, lz, nz + 1)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(np.float64)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()

    def nid(a, b, c):
        return (a * (ny + 1) + b) * (nz + 1) + c

    conn = np.stack([nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                     nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)],
                    axis=1).astype(np.int32)
    return BlockMesh(nx, ny, nz, lx, ly, lz, coords, conn)


def block_tet4(nx: int, ny: int, nz: int, lx: float, ly: float, lz: float) -> BlockMesh:
    """Each hex of a block split into 6 tets (type 4) sharing the main diagonal."""
    hexm = block_hex8(nx, ny, nz, lx, ly, lz)
    h = hexm.conn
    # Kuhn subdivision along the 0-6 diagonal; positive orientation for the
    # reference's tet4 shape functions (node 0 origin, nodes 1..3 axes)
    split = [(0, 1, 2, 6), (0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 4, 5, 6), (0, 5, 1, 6)]
    tets = np.concatenate([h[:, list(s)] for s in split], axis=0)
    # fix orientation so that det J > 0
    x = hexm.coords
    v1 = x[tets[:, 1]] - x[tets[:, 0]]
    v2 = x[tets[:, 2]] - x[tets[:, 0]]
    v3 = x[tets[:, 3]] - x[tets[:, 0]]
    det = np.einsum("ij,ij->i", v1, np.cross(v2, v3))
    neg = det < 0
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    return BlockMesh(nx, ny, nz, lx, ly, lz, hexm.coords, tets.astype(np.int32), elem_type=4)


def block_tet10(nx: int, ny: int, nz: int, lx: float, ly: float, lz: float) -> BlockMesh:
    """block_tet4 with a node added at the middle of every edge: quadratic
    tets (type 10) with the reference's node order, corners 0-3 then the
    edges 0-1, 1-2, 0-2, 0-3, 1-3, 2-3 (element_soln_fields.rs:229-298)."""
    t4 = block_tet4(nx, ny, nz, lx, ly, lz)
    coords = list(map(tuple, t4.coords))
    edge_node: dict = {}
    pairs = ((0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3))
    conn = []
    for tet in t4.conn:
        row = [int(v) for v in tet]
        for i, j in pairs:
            a, b = int(tet[i]), int(tet[j])
            key = (min(a, b), max(a, b))
            if key not in edge_node:
                edge_node[key] = len(coords)
                coords.append(tuple(0.5 * (t4.coords[a] + t4.coords[b])))
            row.append(edge_node[key])
        conn.append(row)
    return BlockMesh(nx, ny, nz, lx, ly, lz, np.array(coords, dtype=np.float64), np.array(conn, dtype=np.int32),
                     elem_type=10)


def ar1_field(shape, spacing, corr_len, rng: np.random.Generator) -> np.ndarray:
    """Standard Gaussian field on a grid with separable exponential correlation
    exp(-|dx|/l - |dy|/l - |dz|/l), generated exactly by AR(1) recursions along
    each axis (rho = exp(-h/l)) applied to white noise."""
    g = rng.standard_normal(shape)
    for ax, h in enumerate(spacing):
        rho = float(np.exp(-h / corr_len))
        s = float(np.sqrt(1.0 - rho * rho))
        g = np.moveaxis(g, ax, 0).copy()
        for t in range(1, g.shape[0]):
            g[t] = rho * g[t - 1] + s * g[t]
        g = np.moveaxis(g, 0, ax)
    return g


def lognormal_modulus(mesh: BlockMesh, median: float, sigma_log: float, corr_frac: float,
                      seed: int) -> np.ndarray:
    """Per-element modulus E = median * exp(sigma_log * g) with g a standard
    Gaussian field of correlation length corr_frac * lx (bar length)."""
    rng = np.random.default_rng(seed)
    h = (mesh.lx / mesh.nx, mesh.ly / mesh.ny, mesh.lz / mesh.nz)
    g = ar1_field((mesh.nx, mesh.ny, mesh.nz), h, corr_frac * mesh.lx, rng)
    e = median * np.exp(sigma_log * g.ravel())
    if mesh.elem_type == 4:
        e = np.tile(e, 6)
    return e.astype(np.float64)


def plate_quad4(nx: int, ny: int, lx: float, ly: float) -> BlockMesh:
    """Structured quad4 shell mesh of the rectangle [0, lx] x [0, ly] at z = 0
    (the reference's structured quad surface meshing with shell4 elements,
    Model.addMeshData quad -> shell4): node (i, j) = i*(ny+1) + j, element
    (i, j) = i*ny + j with corners (i,j), (i+1,j), (i+1,j+1), (i,j+1)
    (counter-clockwise, normal +z).  nz = 0, lz = 0."""
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    i, j = i.ravel(), j.ravel()

    def nid(a, b):
        return a * (ny + 1) + b

    conn = np.stack([nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)], axis=1).astype(np.int32)
    return BlockMesh(nx, ny, 0, lx, ly, 0.0, coords, conn, elem_type=41)


def line_beam2(n: int, length: float, direction=(1.0, 0.0, 0.0), origin=(0.0, 0.0, 0.0)) -> BlockMesh:
    """Straight line of n beam2 elements (type 2) of total length ``length``
    from ``origin`` along ``direction``: node i at origin + i/n * length * d,
    element i = (i, i+1).  ny = nz = 0."""
    d = np.asarray(direction, np.float64)
    d = d / np.linalg.norm(d)
    t = np.linspace(0.0, length, n + 1)
    coords = np.asarray(origin, np.float64)[None, :] + t[:, None] * d[None, :]
    conn = np.stack([np.arange(n), np.arange(1, n + 1)], axis=1).astype(np.int32)
    return BlockMesh(n, 0, 0, float(length), 0.0, 0.0, coords, conn, elem_type=2)
