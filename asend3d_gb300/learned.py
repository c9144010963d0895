"""Training and evaluation driver for the learned nodal preconditioner blocks.

The network, its features, the loss and the Adam step all run on the GPU in
``libasend_gpu.so`` (asend_learned_*).  This module only chooses the data:
training fields are fresh seeded lognormal modulus fields on patch meshes with
the target grid's element size and correlation length; for every field the
plain point-Jacobi PCG generates the residual samples the loss is taken over,
and one or more Adam steps are taken.  The weights stay in the solver's
context, so they can be applied to another mesh (``set_learned_params``).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .configs import BAR, learned_patch
from .mesh import lognormal_modulus
from .solver import GpuSolver

# samples per field for the blocks used by PCG directly: two white-noise
# vectors (the SPAI-type Frobenius part of the loss) and Jacobi-PCG residuals
# after 4, 16 and 64 iterations
BLOCK_ITERS = (0, 0, 4, 16, 64)
# for the multigrid smoother: residuals after 4, 8, 12 and 16 stationary
# V-cycles (the modes the current smoother leaves)
MG_ITERS = (-4, -8, -12, -16)


@dataclass
class TrainLog:
    losses: list = field(default_factory=list)
    seconds: float = 0.0
    fields: int = 0
    samples: int = 0


def train_on_fresh_fields(solver: GpuSolver, n_fields: int, seed: int = 100, iters=None,
                          steps_per_field: int = 2, lr: float = 2e-3, lr_final: float = 2e-4,
                          sigma_log: float = 0.5, corr_abs: float = 0.1, median: float = 70e9,
                          init_seed: int | None = 0, objective: int = _lib.LEARN_MG) -> TrainLog:
    """Train the context's network on ``n_fields`` fresh modulus fields of the
    solver's (block) mesh.  The learning rate decays geometrically from lr to
    lr_final.  ``init_seed`` None keeps the current weights.  ``objective``:
    _lib.LEARN_MG trains the multigrid finest-level smoother (residual after
    one V-cycle), _lib.LEARN_BLOCK the blocks PCG uses directly."""
    m = solver.p.mesh
    if iters is None:
        iters = MG_ITERS if objective == _lib.LEARN_MG else BLOCK_ITERS
    if init_seed is not None:
        if objective == _lib.LEARN_MG:
            solver.set_learned_params(initial_weights(solver, init_seed))
        else:
            solver.learned_init(init_seed)
    solver.learned_set_objective(objective)
    log = TrainLog()
    t0 = time.perf_counter()
    for k in range(n_fields):
        E = lognormal_modulus(m, median, sigma_log, corr_abs / m.lx, seed + k)
        solver.set_modulus(E)
        solver.assemble(64)
        solver.learned_add_samples(iters, append=False, seed=seed + k)
        frac = k / max(1, n_fields - 1)
        rate = lr * (lr_final / lr) ** frac
        log.losses.append(solver.learned_train(steps_per_field, rate))
        log.samples += len(iters)
    log.seconds = time.perf_counter() - t0
    log.fields = n_fields
    return log


def initial_weights(solver: GpuSolver, init_seed: int = 0) -> np.ndarray:
    """The weights multigrid-smoother training starts from: the network's
    initialisation with the output bias set so that every block is the damped
    smoother 0.5 D^-1 (zero output would be the undamped block Jacobi, not a
    smoother on stiff grids).  The untrained network of a comparison."""
    solver.learned_init(init_seed)
    w = solver.learned_params()
    w[-8:-5] = 0.5 * np.log(0.5)
    return w


def timed_eval(solver: GpuSolver, seeds, runs, rel_tol=1e-8, sigma_log=0.5, corr_abs=0.1, median=70e9,
               max_iter=0) -> dict:
    """For each held-out field seed and each run (name, method, precond,
    weights or None): install the weights, re-assemble (FP64) and solve.
    Returns {name: [{iterations, ms_solve, ms_total, status, rel_residual}]};
    ms_solve is the library's device time of the iterations, ms_total the
    host wall time of assembly, preconditioner set-up (eigenvalue estimates
    or network inference) and solve together."""
    m = solver.p.mesh
    out = {r[0]: [] for r in runs}
    for s in seeds:
        solver.set_modulus(lognormal_modulus(m, median, sigma_log, corr_abs / m.lx, s))
        for name, method, pc, weights in runs:
            if weights is not None:
                solver.set_learned_params(weights)
            t0 = time.perf_counter()
            solver.assemble(64)
            rc, st = solver.static_solve_device(method=method, precond=pc, rel_tol=rel_tol, max_iter=max_iter,
                                                graph_iters=8)
            t1 = time.perf_counter()
            out[name].append({"iterations": int(st["iterations"]), "ms_solve": float(st["ms_solve"]),
                              "ms_total": 1e3 * (t1 - t0), "status": int(rc),
                              "rel_residual": float(st["rel_residual"])})
    return out


def patch_solver(nx=32, ny=16, nz=16, full=(128, 64, 64), device=0) -> GpuSolver:
    """A solver on a training patch with the element size of the ``full`` grid
    over the benchmark bar."""
    return GpuSolver(learned_patch(nx, ny, nz, full=full), device=device)


def evaluate(solver: GpuSolver, seeds, methods, rel_tol=1e-8, sigma_log=0.5, corr_abs=0.1, median=70e9,
             max_iter=0):
    """For each held-out field seed, assemble and solve with every
    (name, method, precond) in ``methods``; returns {name: [(iters, ms,
    status, rel_res), ...]}."""
    m = solver.p.mesh
    out = {name: [] for name, _, _ in methods}
    for s in seeds:
        solver.set_modulus(lognormal_modulus(m, median, sigma_log, corr_abs / m.lx, s))
        solver.assemble(64)
        for name, method, pc in methods:
            rc, st = solver.static_solve_device(method=method, precond=pc, rel_tol=rel_tol, max_iter=max_iter,
                                                graph_iters=8)
            out[name].append((st["iterations"], st["ms_solve"], rc, st["rel_residual"]))
    return out


PLAIN = ("jacobi", _lib.METHOD_FP64, _lib.PC_JACOBI)
BLOCK = ("block_jacobi", _lib.METHOD_FP64, _lib.PC_BLOCK)
LEARNED = ("learned", _lib.METHOD_FP64, _lib.PC_LEARNED)
MG = ("mg", _lib.METHOD_FP64, _lib.PC_MG)
MG_LEARNED = ("mg_learned", _lib.METHOD_FP64, _lib.PC_MG_LEARNED)
