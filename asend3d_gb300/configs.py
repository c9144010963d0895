"""Seeded synthetic workloads with the shapes of the five benchmark cases.

No public dataset is involved; every input is generated here from a seed.

  cantilever_small   20x4x4 hex8 bar 2.0 x 0.4 x 0.4 m, E = 200 GPa, nu = 0.3,
                     x = 0 face fixed, 1 kN downward load at the free end's
                     top-centre node, objective = tip u_z, modulus DVs
                     (80 column groups and 320 per-element).
  block_large        200x40x40 hex8 (1.01 M DOF), lognormal modulus (median
                     70 GPa, sigma_log 0.3, correlation 0.1 L), nu = 0.33,
                     fixed end + distributed end-face traction, compliance.
  batch_uq           64 blocks, nx in [20,120], ny = nz in [4,16], own field
                     each, 4 load cases (tip -z, tip +y, torsion couple,
                     uniform end traction).
  learned_grid       128x64x64 hex8 (1.6 M DOF), sigma_log 0.5, corr 0.05 L.
  learned_patch      training patch with learned_grid's element size.
  shell_plate        200x200 quad4 shell plate 1 x 1 m, t = 5 mm, aluminium,
                     simply supported, Gaussian central impulse (Newmark).
"""
from __future__ import annotations

import numpy as np

from .mesh import block_hex8, lognormal_modulus, plate_quad4
from .solver import Problem

BAR = (2.0, 0.4, 0.4)


def _fixed_end(p: Problem, mesh):
    p.add_node_set("xMin", mesh.nodes_in_range(xr=(-1e-9, 1e-9)))
    p.fix_displacement("xMin")


def cantilever_small(nx=20, ny=4, nz=4, E=200e9, nu=0.3, F=-1000.0) -> Problem:
    m = block_hex8(nx, ny, nz, *BAR)
    p = Problem(m, np.full(m.n_elems, E), np.full(m.n_elems, nu), np.full(m.n_elems, 7850.0))
    _fixed_end(p, m)
    tip = m.node_id(nx, ny // 2, nz)
    p.add_node_set("tip", [int(tip)])
    p.add_nodal_force("tip", [0.0, 0.0, F])
    p.objective = ("displacement", "tip", 3, 1.0)
    p.add_elem_set("all", np.arange(m.n_elems))
    # 80 DVs: one per (ix, iy) column of elements over iz; then 320 per element
    for i in range(nx):
        for j in range(ny):
            name = f"col_{i}_{j}"
            p.add_elem_set(name, m.elem_id(i, j, np.arange(nz)))
            p.design_vars.append((name, [1.0]))
    return p


def block_large(nx=200, ny=40, nz=40, median=70e9, sigma_log=0.3, corr=0.1, nu=0.33, seed=2024,
                traction=(0.0, 0.0, -1.0e6)) -> Problem:
    m = block_hex8(nx, ny, nz, *BAR)
    E = lognormal_modulus(m, median, sigma_log, corr, seed)
    p = Problem(m, E, np.full(m.n_elems, nu), np.full(m.n_elems, 2700.0))
    _fixed_end(p, m)
    p.add_elem_set("xMaxEls", m.elem_id(nx - 1, *np.meshgrid(np.arange(ny), np.arange(nz), indexing="ij")).ravel())
    p.add_surface_traction("xMaxEls", (1.0, 0.0, 0.0), traction)
    p.objective = ("compliance",)
    return p


def _batch_draw(k: int, seed: int):
    rng = np.random.default_rng([seed, k])
    nx = int(rng.integers(20, 121))
    ny = int(rng.integers(4, 17))
    return nx, ny, ny, int(rng.integers(1 << 30))


def batch_dims(k: int, seed: int = 7):
    """(nx, ny, nz) of instance k of the sweep, without building it."""
    return _batch_draw(k, seed)[:3]


def batch_instance(k: int, seed: int = 7, median=70e9, sigma_log=0.3, corr=0.1, nu=0.33) -> Problem:
    """Instance k of the 64-instance sweep with its 4 load cases."""
    nx, ny, nz, field_seed = _batch_draw(k, seed)
    m = block_hex8(nx, ny, nz, *BAR)
    E = lognormal_modulus(m, median, sigma_log, corr, field_seed)
    p = Problem(m, E, np.full(m.n_elems, nu), np.full(m.n_elems, 2700.0))
    _fixed_end(p, m)
    end = m.nodes_in_range(xr=(BAR[0] - 1e-9, BAR[0] + 1e-9))
    p.add_node_set("xMax", end)
    p.add_node_set("tip", [int(m.node_id(nx, ny // 2, nz))])
    p.add_nodal_force("tip", [0.0, 0.0, -1000.0], case=0)
    p.add_nodal_force("tip", [0.0, 1000.0, 0.0], case=1)
    # torsion couple about the bar axis on the end face: f = T * (-dz, dy) / sum r^2
    xyz = m.coords[end]
    dy, dz = xyz[:, 1] - BAR[1] / 2, xyz[:, 2] - BAR[2] / 2
    r2 = float(np.sum(dy * dy + dz * dz))
    f = np.zeros(m.n_dof)
    f[3 * end + 1] = -1000.0 * dz / r2
    f[3 * end + 2] = 1000.0 * dy / r2
    p.add_load_vector(f, case=2)
    p.add_elem_set("xMaxEls", m.elem_id(nx - 1, *np.meshgrid(np.arange(ny), np.arange(nz), indexing="ij")).ravel())
    p.add_surface_traction("xMaxEls", (1.0, 0.0, 0.0), (1.0e6, 0.0, 0.0), case=3)
    p.objective = ("compliance",)
    return p


def learned_grid(seed=11, nx=128, ny=64, nz=64, median=70e9, sigma_log=0.5, corr=0.05, nu=0.33) -> Problem:
    m = block_hex8(nx, ny, nz, *BAR)
    E = lognormal_modulus(m, median, sigma_log, corr, seed)
    p = Problem(m, E, np.full(m.n_elems, nu), np.full(m.n_elems, 2700.0))
    _fixed_end(p, m)
    p.add_elem_set("xMaxEls", m.elem_id(nx - 1, *np.meshgrid(np.arange(ny), np.arange(nz), indexing="ij")).ravel())
    p.add_surface_traction("xMaxEls", (1.0, 0.0, 0.0), (0.0, 0.0, -1.0e6))
    p.objective = ("compliance",)
    return p


def learned_patch(nx=32, ny=16, nz=16, full=(128, 64, 64), seed=0, median=70e9, sigma_log=0.5,
                  corr_abs=0.1, nu=0.33) -> Problem:
    """A smaller block with the element size of the ``full`` grid over the
    bar, the same supports and load type, and the same absolute correlation
    length (0.05 of the 2 m bar)."""
    lx, ly, lz = BAR[0] * nx / full[0], BAR[1] * ny / full[1], BAR[2] * nz / full[2]
    m = block_hex8(nx, ny, nz, lx, ly, lz)
    E = lognormal_modulus(m, median, sigma_log, corr_abs / lx, seed)
    p = Problem(m, E, np.full(m.n_elems, nu), np.full(m.n_elems, 2700.0))
    _fixed_end(p, m)
    p.add_elem_set("xMaxEls", m.elem_id(nx - 1, *np.meshgrid(np.arange(ny), np.arange(nz), indexing="ij")).ravel())
    p.add_surface_traction("xMaxEls", (1.0, 0.0, 0.0), (0.0, 0.0, -1.0e6))
    p.objective = ("compliance",)
    return p


def batch_uq(n_inst: int = 64, seed: int = 7, which=None):
    """The batched UQ / design sweep: n_inst uneven cantilevers, 4 load cases
    each, combined into one stacked problem (``which``: a subset of instance
    indices).  Returns (problem, node_ptr, elem_ptr, instances); the
    instances' structured blocks are ``[(p.mesh.nx, p.mesh.ny, p.mesh.nz)]``."""
    from .solver import combine

    ks = range(n_inst) if which is None else which
    inst = [batch_instance(k, seed=seed) for k in ks]
    prob, node_ptr, elem_ptr = combine(inst)
    return prob, node_ptr, elem_ptr, inst


def shell_plate(n=200, L=1.0, t=0.005, E=70e9, nu=0.33, rho=2700.0, peak=100.0) -> Problem:
    """Simply supported square plate of shell4 elements under a central point
    load (load case 0: peak newtons in -z at the centre node; the time history
    scales it).  Supports: w = 0 on the four edges; the in-plane rigid motions
    are removed by u = v = 0 at the corner (0, 0) and v = 0 at the corner
    (L, 0); rotations are free (simple support)."""
    m = plate_quad4(n, n, L, L)
    p = Problem(m, np.full(m.n_elems, E), np.full(m.n_elems, nu), np.full(m.n_elems, rho),
                thickness=np.full(m.n_elems, t))
    x, y = m.coords[:, 0], m.coords[:, 1]
    tol = 1e-9 * L
    edge = np.nonzero((x < tol) | (x > L - tol) | (y < tol) | (y > L - tol))[0]
    p.add_node_set("edges", edge)
    p.fix_displacement("edges", comps=(3,))
    p.add_node_set("c00", [int(np.nonzero((x < tol) & (y < tol))[0][0])])
    p.add_node_set("cL0", [int(np.nonzero((x > L - tol) & (y < tol))[0][0])])
    p.fix_displacement("c00", comps=(1, 2))
    p.fix_displacement("cL0", comps=(2,))
    centre = int(np.argmin((x - L / 2) ** 2 + (y - L / 2) ** 2))
    p.add_node_set("centre", [centre])
    p.add_nodal_force("centre", [0.0, 0.0, -peak])
    p.objective = ("displacement", "centre", 3, 1.0)
    return p


def gaussian_pulse(n_steps=2000, dt=2e-6, width=50e-6, t0=200e-6) -> np.ndarray:
    """Load amplitude at step i (time i*dt): exp(-(t - t0)^2 / (2 width^2))."""
    tt = np.arange(n_steps) * dt
    return np.exp(-0.5 * ((tt - t0) / width) ** 2)

