"""Benchmark: DOF-solves/sec of the static + adjoint solve path on one GB300.

Workload (default): the 200x40x40 hex8 block (1,013,643 DOF) with a seeded
lognormal modulus field (median 70 GPa, sigma_log 0.3, correlation 0.1 L),
nu = 0.33, fixed end + distributed end-face traction, compliance objective.
One step = FP64 element integration + coloured CSR-block assembly + penalty,
multigrid-preconditioned CG (FP64 operator and recurrence, FP32 V-cycle) to
||f - A u|| / ||f|| <= 1e-8 (FP64 operator), and the
adjoint compliance gradient over all 320,000 element moduli.

value  = DOF-solves/s with inputs resident in HBM (device-event timed).
e2e    = the same through the C ABI with host buffers: per step the element
         moduli and the load go host->device and the displacement and the
         gradient come back, inside the timed region.
The plain FP64 point-Jacobi PCG on the same GPU is timed as well
(plain_fp64_*); the CPU baseline is the FP64 oracle's restatement of the
reference's block-LDL^T PCG on the host cores.

--impl reference times the reference's CPU algorithm (the oracle port:
block-LDL^T-preconditioned CG, reference stopping rule replaced by the same
1e-8 relative residual) on the host cores, one process per core.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# the headline metric, verbatim; each line's config.workload says what was run
# kernel of each shape of the split outer product (asend_set_product_variant)
PRODUCT_KERNEL = {1: "k_mg_spmv_dot_pair", 2: "k_mg_spmv_dot_staged<2,3>", 3: "k_mg_spmv_dot_staged<3,2>",
                  4: "k_mg_spmv_dot_staged<2,2>", 5: "k_mg_spmv_dot_staged<4,2>"}
METRIC = "DOF-solves/sec at 1e-8 rel. residual, learned+batched vs plain PCG, 1 GB300; HBM GB/s"
UNIT = "DOF-solves/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=200)
    ap.add_argument("--ny", type=int, default=40)
    ap.add_argument("--nz", type=int, default=40)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="omit the nested batch_uq block of the default line")
    ap.add_argument("--no-learned", action="store_true", help="omit the nested learned block of the default line")
    ap.add_argument("--cpu-sample-nx", type=int, default=40)
    ap.add_argument("--product", type=int, default=0,
                    help="--profile: shape of the split outer product (asend_set_product_variant; 0 = tune)")
    ap.add_argument("--no-size-series", action="store_true",
                    help="reference arm: skip the one-off 40/60/80-cell size series")
    ap.add_argument("--profile", action="store_true",
                    help="short run for ncu: one assembly, one multigrid solve, three FP32 SpMV launches")
    ap.add_argument("--workload", default="block_large",
                    choices=["block_large", "batch_uq", "shell_plate", "modal"],
                    help="block_large (default, the benchmark line), batch_uq (64 uneven instances x 4 cases) "
                         "shell_plate (200x200 shell4 plate, 2000 Newmark steps) or modal (10 lowest "
                         "eigenpairs of the 200x40x40 block)")
    return ap.parse_args()


def learned_measure(n_train: int = 2000, n_eval: int = 2) -> dict:
    """The learned preconditioner at its configuration's scale: the network
    (16 -> 64 -> 64 -> 8 per node, BF16 weights, FP32 accumulation) trained on
    the GPU by the library's own kernels on n_train fresh seeded lognormal
    fields (sigma_log 0.5, correlation 0.05 of the bar) of a 16x8x8 patch with
    the element size of the 128x64x64 grid, then evaluated on n_eval held-out
    fields of the 128x64x64 grid (1.6 M DOF) to 1e-8: plain FP64 point-Jacobi
    PCG, the multigrid CG with eigenvalue-damped finest smoothing, and the
    same multigrid CG with network-predicted finest smoother blocks, untrained
    and trained.  ms_total is assembly + preconditioner set-up + solve."""
    from asend3d_gb300 import _lib, configs
    from asend3d_gb300 import learned as LN
    from asend3d_gb300.solver import GpuSolver

    tr = GpuSolver(configs.learned_patch(16, 8, 8))
    w0 = LN.initial_weights(tr, 0)
    log = LN.train_on_fresh_fields(tr, n_fields=n_train, seed=1000)
    w = tr.learned_params()
    tr.close()
    ev = GpuSolver(configs.learned_patch(128, 64, 64))
    runs = [("plain_fp64_jacobi", _lib.METHOD_FP64, _lib.PC_JACOBI, None),
            ("mg_eigen_damped", _lib.METHOD_SPLIT, _lib.PC_MG, None),
            ("mg_learned_untrained", _lib.METHOD_SPLIT, _lib.PC_MG_LEARNED, w0),
            ("mg_learned", _lib.METHOD_SPLIT, _lib.PC_MG_LEARNED, w)]
    seeds = [95001 + k for k in range(n_eval)]
    ev.set_learned_params(w)
    LN.timed_eval(ev, seeds[:1], runs[1:])  # warm-up: hierarchy, graphs
    t = LN.timed_eval(ev, seeds, runs, max_iter=20000)
    n_dof = ev.n_dof
    ev.close()
    out = {"config": {"workload": "learned: 128x64x64 hex8 grid, lognormal E (median 70 GPa, sigma_log 0.5, "
                                  "correlation 0.05 of the bar), held-out fields, rel_tol 1e-8",
                      "n_dof": n_dof, "train_fields": n_train, "train_patch": "16x8x8 (same element size)",
                      "train_seconds": log.seconds, "eval_fields": n_eval}}
    for name, rows in t.items():
        out[name] = {"iterations": [r["iterations"] for r in rows], "ms_total": [r["ms_total"] for r in rows],
                     "ms_solve": [r["ms_solve"] for r in rows], "status": [r["status"] for r in rows],
                     "rel_residual": [r["rel_residual"] for r in rows]}
    mean = lambda k, f: float(np.mean(out[k][f]))
    out["gain_trained_vs_untrained"] = {"iterations": mean("mg_learned_untrained", "iterations") /
                                        mean("mg_learned", "iterations"),
                                        "wall": mean("mg_learned_untrained", "ms_total") / mean("mg_learned", "ms_total")}
    out["speedup_vs_plain_fp64_jacobi"] = mean("plain_fp64_jacobi", "ms_total") / mean("mg_learned", "ms_total")
    out["vs_eigen_damped"] = {"iterations": mean("mg_eigen_damped", "iterations") / mean("mg_learned", "iterations"),
                              "wall": mean("mg_eigen_damped", "ms_total") / mean("mg_learned", "ms_total")}
    return out


def batch_measure(steps: int, warmup: int, plain: bool = True, accuracy: bool = True) -> dict:
    """The batched sweep: 64 uneven cantilevers x 4 load cases (256
    right-hand sides) as one stacked operator.  One step = FP64 assembly of
    the stack + batched multigrid-preconditioned CG over every instance and
    load case (one V-cycle over all instances' hierarchies, captured in CUDA
    graphs) + the compliance gradient of every instance.  Compared with the
    plain FP64 point-Jacobi PCG run instance by instance and load case by
    load case on the same GPU."""
    import ctypes as C

    import torch

    from asend3d_gb300 import _lib, configs
    from asend3d_gb300.solver import GpuSolver

    prob, node_ptr, elem_ptr, inst = configs.batch_uq(64)
    dims = [(p.mesh.nx, p.mesh.ny, p.mesh.nz) for p in inst]
    g = GpuSolver(prob, instances=node_ptr, blocks=dims)
    stream = torch.cuda.ExternalStream(g.stream)
    n_real = sum(p.mesh.n_dof for p in inst)
    n_cases = len(prob.loads)
    best = dict(method=_lib.METHOD_SPLIT, precond=_lib.PC_MG, rel_tol=1e-8, graph_iters=8)
    o_adj = g.opts(**best)
    from asend3d_gb300 import autotune

    g.assemble(precision=48)
    shape, _ = autotune.tune_product(g)

    def step():
        g.assemble(precision=48)
        rc, st = g.static_solve_device(**best)
        Lc = C.c_double(0)
        s2 = _lib.SolveStats()
        rc2 = g.lib.asend_adjoint_gradient(g.ctx, C.byref(o_adj), C.byref(Lc), None, C.byref(s2))
        return rc, rc2, st

    for _ in range(warmup):
        rc, rc2, st = step()
        assert rc == 0 and rc2 == 0, st
    torch.cuda.synchronize()
    launches0 = g.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(steps):
            rc, rc2, st = step()
            assert rc == 0 and rc2 == 0, st
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    launches = (g.kernel_launches - launches0) // max(steps, 1)
    value = n_real * n_cases / (ms / 1e3)
    out = {"value": value, "unit": UNIT, "ms_per_step": ms, "steps": steps, "warmup": warmup,
           "dtype": "fp32-pair operator values and CG vectors (FP64-accurate), f64 x / reductions / true residual, f32 multigrid",
           "data": "synthetic (seeded lognormal fields)",
           "config": {"workload": "batch_uq: 64 uneven hex8 cantilevers nx in [20,120], ny=nz in [4,16], 4 load "
                                  "cases each (256 right-hand sides), batched multigrid CG + compliance gradients",
                      "n_dof_total": n_real, "rhs_per_step": 64 * n_cases, "rel_tol": 1e-8,
                      "method": "CG + per-instance geometric multigrid, one V-cycle over all instances",
                      "l2": "stack operator 1.2 GB FP64 + 0.6 GB FP32 > 129 MB L2"},
           "iterations_max": st["iterations"], "product_shape": PRODUCT_KERNEL[shape], "ms_breakdown": {"assemble": st["ms_assemble"], "solve": st["ms_solve"]},
           "gpu_launches_per_step": launches, "clocks": clk.summary()}
    if plain:
        # plain: FP64 point-Jacobi PCG, one instance and one load case at a time
        jac = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-8, graph_iters=32)
        t_plain = 0.0
        it_plain = 0
        for p in inst:
            for k in range(n_cases):
                q = type(p)(p.mesh, p.E, p.nu, p.rho, p.node_sets, p.elem_sets, p.constraints, [p.loads[k]],
                            ("compliance",))
                gi = GpuSolver(q)
                gi.assemble(precision=64)
                rc, sti = gi.static_solve_device(**jac)
                t_plain += sti["ms_solve"] + sti["ms_assemble"]
                it_plain = max(it_plain, sti["iterations"])
                gi.close()
        plain_value = n_real * n_cases / (t_plain / 1e3)
        out["plain_fp64_jacobi_sequential"] = {"value": plain_value, "ms_total": t_plain, "iterations_max": it_plain}
        out["speedup_vs_plain_fp64"] = value / plain_value
    if accuracy:
        acc = {}
        try:
            rel = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))
            g.assemble(precision=48)  # the benchmark's operator and solve
            u8, _, _ = g.static_solve(**best)
            L8, gE8, _, _ = g.adjoint_gradient(**best)
            g.assemble(precision=64)  # the FP64 reference
            tight = dict(best, method=_lib.METHOD_FP64, rel_tol=1e-11, max_iter=400)
            u11, rc11, st11 = g.static_solve(**tight)
            L11, gE11, _, _ = g.adjoint_gradient(**tight)
            acc["full_size_vs_fp64_1e-11"] = {"u_rel": rel(u8, u11), "compliance_rel": abs(L8 - L11) / abs(L11),
                                              "gradient_rel": rel(gE8, gE11), "rc_1e-11": rc11,
                                              "rel_residual_1e-11": st11["rel_residual"]}
            # the smallest instance of the stack against the FP64 oracle's direct LDL^T
            from oracle import pyoracle as po

            i = int(np.argmin([p.mesh.n_dof for p in inst]))
            p = inst[i]
            o = po.Oracle(p)
            F = np.stack([f + o.penalty_rhs() for f in o.loads()])
            U, _, _ = o.solve_cases(F, precond=po.PC_DIRECT)
            a0, e0_ = node_ptr[i], elem_ptr[i]
            ui = u8[:, 3 * a0:3 * a0 + p.mesh.n_dof]
            gref = sum(o.adjoint(U[k], lam=U[k])[0] for k in range(n_cases))
            acc["instance_vs_oracle"] = {"instance": i, "n_dof": p.mesh.n_dof,
                                         "u_rel": max(rel(ui[k], U[k]) for k in range(n_cases)),
                                         "gradient_rel": rel(gE8[e0_:e0_ + p.mesh.n_elems], gref)}
        except Exception as err:  # the measurement above stands on its own
            acc["error"] = repr(err)[:200]
        out["accuracy"] = acc
    g.close()
    return out


def run_batch(a):
    b = batch_measure(a.steps, a.warmup)
    out = {"metric": METRIC, "value": b["value"], "unit": UNIT, "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": b["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": b["dtype"], "data": b["data"], "config": b["config"],
           **{k: v for k, v in b.items() if k not in ("value", "unit", "ms_per_step", "steps", "warmup", "dtype",
                                                       "data", "config", "clocks", "gpu_launches_per_step")},
           "clocks": b["clocks"], "gpu_launches": b["gpu_launches_per_step"] * a.steps}
    print(json.dumps(out))


def run_shell(a):
    """Transient shell plate: 200x200 quad4 shell4 elements (242,406 DOF),
    simply supported, Gaussian central impulse (100 N peak, 50 us width),
    Newmark beta 0.25 / gamma 0.5, dt 2 us, 2000 steps.  One bench step = the
    whole 2000-step run: per time step the effective-load residual, a
    point-Jacobi PCG solve to 1e-8 started from the extrapolated increment,
    and the fused Newmark corrector/predictor.  Reported beside it: the plain
    FP64 Jacobi PCG run (started from the previous increment), the
    mixed-precision run, the centre-deflection history error against an FP64
    run at 1e-12 (all steps) and against the CPU oracle (first 40 steps)."""
    import torch

    from asend3d_gb300 import _lib, configs
    from asend3d_gb300.solver import GpuSolver
    from oracle import pyoracle as po

    p = configs.shell_plate(200)
    dt, beta, gamma, n_steps = 2e-6, 0.25, 0.5, 2000
    amp = configs.gaussian_pulse(n_steps, dt)
    probe = 6 * int(p.node_sets["centre"][0]) + 2
    g = GpuSolver(p)
    g.assemble(dynamic=True, dt=dt, beta=beta, gamma=gamma)
    stream = torch.cuda.ExternalStream(g.stream)
    # FP64 point-Jacobi: on this mass-dominated, L2-resident operator the FP64
    # recurrence beats the mixed method (its residual replacements cost more
    # than the FP32 products save); the mixed run is reported beside it
    ours = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-8, graph_iters=16, warm_start=2)

    def step(kw):
        hist, u, rc, st = g.newmark(amp, probe_dof=probe, **kw)
        assert rc == 0, st
        return hist, st

    for _ in range(a.warmup):
        hist, st = step(ours)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = g.kernel_launches
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(a.steps):
            hist, st = step(ours)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    launches = (g.kernel_launches - launches0) // a.steps
    n_dof = g.n_dof
    value = n_steps * n_dof / (ms / 1e3)
    def timed(kw):
        torch.cuda.synchronize()
        e0.record(stream)
        h, st_ = step(kw)
        e1.record(stream)
        torch.cuda.synchronize()
        return h, st_, e0.elapsed_time(e1)

    mixed = dict(method=_lib.METHOD_MIXED, precond=_lib.PC_JACOBI, rel_tol=1e-8, graph_iters=16, warm_start=2)
    h_mixed, st_mixed, ms_mixed = timed(mixed)
    # plain method: FP64 Jacobi PCG warm-started from the previous increment
    plain = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-8, graph_iters=16)
    h_plain, st_plain, ms_plain = timed(plain)
    h_ref, _ = step(dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-12, graph_iters=16))
    err_fp64 = float(np.linalg.norm(hist - h_ref) / np.linalg.norm(h_ref))
    spmv_ms, spmv_bytes = g.time_spmv(precision=32, n_launch=50)
    peak, kind = measured_peak()
    achieved = spmv_bytes / (spmv_ms / 1e3) / 1e9
    out = {"metric": METRIC, "value": value, "unit": UNIT,
           "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (uniform aluminium plate, Gaussian impulse)",
           "config": {"workload": "shell_plate 200x200 shell4, 2000 Newmark steps of 2 us (one bench step = "
                                  "the whole run)", "n_dof": n_dof, "time_steps": n_steps, "rel_tol": 1e-8,
                      "l2": "operator 105 MB FP64 + 53 MB FP32, mass 105 MB; per-step vectors stay in L2"},
           "pcg_iterations_total": st["iterations"], "gpu_launches": launches,
           "plain_fp64_jacobi": {"value": n_steps * n_dof / (ms_plain / 1e3), "ms_per_step": ms_plain,
                                 "iterations": st_plain["iterations"], "initial_guess": "previous increment"},
           "speedup_vs_plain_fp64": ms_plain / ms,
           "mixed_precision_jacobi": {"value": n_steps * n_dof / (ms_mixed / 1e3), "ms_per_step": ms_mixed,
                                      "iterations": st_mixed["iterations"]},
           "centre_history_rel_error": {"vs_gpu_fp64_1e-12_all_steps": err_fp64},
           "spmv_fp32_l2_resident": {"note": "the 60 MB FP32 operator fits in the 129 MB L2, so this is an "
                                             "L2-resident rate, not an HBM roofline fraction",
                                     "achieved_GBps": achieved, "bytes_per_launch": spmv_bytes,
                                     "ms_per_launch": spmv_ms},
           "clocks": clk.summary()}
    if not a.no_cpu_baseline:
        o = po.Oracle(p, dynamic=True, dt=dt, beta=beta, gamma=gamma)
        m = 40
        t0 = time.perf_counter()
        href, _, rc2, its = o.newmark(m, dt, beta, gamma, o.loads()[0], amp[:m], probe, precond=po.PC_JACOBI,
                                      stop=po.STOP_RELATIVE, tol=1e-12)
        t_cpu = time.perf_counter() - t0
        out["centre_history_rel_error"]["vs_cpu_oracle_first_40_steps"] = float(
            np.linalg.norm(hist[:m] - href) / np.linalg.norm(href))
        out["cpu_baseline"] = {"value": m * n_dof / t_cpu, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"first {m} Newmark steps of the same plate, FP64 Jacobi PCG to 1e-12 "
                                         f"({its} iterations, {t_cpu:.1f} s)"}
    print(json.dumps(out))
    g.close()


def run_modal(a):
    """Modal analysis of the 200x40x40 hex8 block (1,013,643 DOF, the lognormal
    modulus field of the static workload, rho 2700): the 10 lowest eigenpairs
    of (K + penalty) x = lambda D x, D the row-sum diagonal mass.  One bench
    step = modal assembly (K and M, FP64) + shift-invert block Lanczos (block
    2, full reorthogonalisation) with multigrid-preconditioned CG inner solves
    to 1e-10 (at most 300 iterations each), stopped at Ritz residual 1e-8.
    Reported beside it: the CPU oracle's restatement of the reference's
    frequency job (direct LDL^T + Lanczos, 5 n_modes vectors) on a 40x8x8
    sample of the same block.  Point-Jacobi inner solves are not timed here:
    to 1e-10 on this 1M-DOF lognormal block they stall at the FP64 floor."""
    import torch

    from asend3d_gb300 import _lib, configs
    from asend3d_gb300.solver import GpuSolver
    from oracle import pyoracle as po

    n_modes = 10
    p = configs.block_large()
    g = GpuSolver(p)
    stream = torch.cuda.ExternalStream(g.stream)
    ours = dict(block_size=2, tol=1e-8, method=_lib.METHOD_FP64, precond=_lib.PC_MG, rel_tol=1e-10, max_iter=300)

    def step(kw):
        g.assemble(precision=64, dynamic=2)
        ev, fr, _, _, rc, st = g.eigen(n_modes, modes=False, **kw)
        assert rc == 0, st
        print(f"modal step: {st['ms']:.1f} ms, basis {st['subspace']}, inner its {st['inner_iterations']}, "
              f"capped {st['inner_capped']}", file=sys.stderr, flush=True)
        return ev, fr, st

    for _ in range(a.warmup):
        ev, fr, st = step(ours)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = g.kernel_launches
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(a.steps):
            ev, fr, st = step(ours)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    launches = (g.kernel_launches - launches0) // a.steps
    n_dof = g.n_dof
    unit = "DOF-eigenpairs/s"
    out = {"metric": f"DOF-eigenpairs/sec ({n_modes} lowest modes, Ritz residual 1e-8), 1 GB300",
           "value": n_dof * n_modes / (ms / 1e3), "unit": unit, "n_gpus": 1, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64 Lanczos / operator / dots + f32 multigrid",
           "data": "synthetic (seeded lognormal modulus field)",
           "config": {"workload": f"modal: {n_modes} lowest eigenpairs of the 200x40x40 hex8 block",
                      "n_dof": n_dof, "block_size": 2, "inner": "MG-preconditioned CG to 1e-10"},
           "frequencies_hz": [float(f) for f in fr], "lanczos_basis": st["subspace"],
           "shift_invert_solves": st["n_solves"], "inner_iterations": st["inner_iterations"],
           "ritz_residual_max": st["max_rel_residual"], "inner_solves_at_cap": st["inner_capped"],
           "gpu_launches": launches, "clocks": clk.summary()}
    if not a.no_cpu_baseline:
        ps = configs.block_large(nx=40, ny=8, nz=8)
        o = po.Oracle(ps, modal=True)
        t0 = time.perf_counter()
        evo, _, _, _ = o.eigen(n_modes)
        t_cpu = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": o.n_dof * n_modes / t_cpu, "unit": unit, "cores": 1, "kind": "port",
                               "sample": f"40x8x8 block ({o.n_dof} DOF), {n_modes} modes, direct LDL^T + "
                                         f"Lanczos with {5 * n_modes} vectors ({t_cpu:.2f} s)"}
    print(json.dumps(out))
    g.close()


def run_profile(a):
    """The launch sequence the ncu summaries in profiles/ are taken from."""
    from asend3d_gb300 import _lib, configs
    from asend3d_gb300.solver import GpuSolver

    if a.workload == "shell_plate":  # 30 Newmark steps around the pulse peak
        p = configs.shell_plate(200)
        g = GpuSolver(p)
        g.assemble(dynamic=True, dt=2e-6, beta=0.25, gamma=0.5)
        amp = configs.gaussian_pulse(2000, 2e-6)[80:110]
        hist, u, rc, st = g.newmark(amp, probe_dof=6 * int(p.node_sets["centre"][0]) + 2,
                                    method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-8, graph_iters=16,
                                    warm_start=2)
        print(json.dumps({"rc": rc, "iterations": st["iterations"], "ms": st["ms_solve"],
                          "launches": g.kernel_launches}))
        g.close()
        return

    p = configs.block_large(nx=a.nx, ny=a.ny, nz=a.nz)
    g = GpuSolver(p)
    kw = dict(method=_lib.METHOD_SPLIT, precond=_lib.PC_MG, rel_tol=1e-8, graph_iters=8)
    g.assemble(precision=48)
    if a.product:
        g.set_product_variant(a.product)
    else:
        from asend3d_gb300 import autotune

        autotune.tune_product(g)
    # two benchmark steps (assembly + multigrid solve + compliance gradient):
    # the first warms the caches and graphs, the second is the one to read
    out = []
    for _ in range(2):
        n0 = g.kernel_launches
        g.assemble(precision=48)
        rc, st = g.static_solve_device(**kw)
        L, _, rc2, st2 = g.adjoint_gradient(want_dLdE=False, **kw)
        out.append({"rc": rc, "rc_adjoint": rc2, "iterations": st["iterations"], "ms_solve": st["ms_solve"],
                    "launches": g.kernel_launches - n0})
    print(json.dumps(out))
    g.close()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(ms: float, world: int) -> float:
    """Step time of the slowest replica (all_reduce MAX on the process group:
    NCCL with a CUDA tensor, gloo with a host tensor)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_value(units_per_rank: int, world: int, ms_max: float) -> float:
    """Whole-job throughput of `world` independent replicas: all ranks' units
    over the slowest rank's time."""
    return world * units_per_rank / (ms_max / 1000.0)


def measured_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


NCU_SUMMARY = {0: "mg_outer_split_block_large.md", 1: "vc_resid_block_large.md", 2: "vc_post_block_large.md"}


def ncu_traffic(kernel: int):
    """Per-launch DRAM traffic (read + write) of a multigrid-CG kernel at the
    full size, from the committed ncu summary of that kernel (None if absent)."""
    f = ROOT / "profiles" / NCU_SUMMARY[kernel]
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch_full_size:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


class ClockSampler:
    def __init__(self, gpu_index: int):
        self.proc = None
        # raw samples (the JSON line carries their summary); ASEND_CLOCK_DIR keeps them
        self.path = Path(os.environ.get("ASEND_CLOCK_DIR", tempfile.gettempdir())) / f"clocks_bench_{os.getpid()}.csv"
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
# CPU reference arm (the oracle's restatement of the reference algorithm)
# --------------------------------------------------------------------------
def _cpu_sample(args):
    nx, seed = args
    from asend3d_gb300 import configs
    from oracle import pyoracle as po

    p = configs.block_large(nx=nx, ny=nx // 5, nz=nx // 5, seed=seed)
    t0 = time.perf_counter()
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    u, rc, st = o.solve(f, precond=po.PC_BLOCK_LDL, stop=po.STOP_RELATIVE, tol=1e-8)
    g, _, _, _ = o.adjoint(u, lam=u)
    dt = time.perf_counter() - t0
    return o.n_dof, dt, st["iterations"], st["rel_residual"]


def cpu_baseline(nx: int, procs: int):
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_sample, [(nx, 100 + k) for k in range(procs)])
    wall = time.perf_counter() - t0
    ndof = sum(r[0] for r in res)
    per_proc = statistics.mean(r[1] for r in res)
    return {"value": ndof / wall, "unit": UNIT, "cores": procs, "kind": "port",
            "sample": f"{procs} x {nx}x{nx // 5}x{nx // 5} hex8 instances of the same workload "
                      f"({res[0][0]} DOF each), block-LDL^T PCG to 1e-8 + adjoint, one process per core; "
                      f"{per_proc:.2f} s per instance, {res[0][2]} iterations",
            "per_instance_s": per_proc}


def sample_accuracy(nx: int, kw: dict) -> dict:
    """The CPU-baseline sample (the first instance of the pool, seed 100)
    solved by this library with the benchmark's options and by the FP64
    oracle's direct LDL^T: relative errors of u, the compliance and its
    per-element gradient."""
    from asend3d_gb300 import configs
    from asend3d_gb300.solver import GpuSolver
    from oracle import pyoracle as po

    p = configs.block_large(nx=nx, ny=nx // 5, nz=nx // 5, seed=100)
    g = GpuSolver(p)
    g.assemble(precision=64)
    u, rc, _ = g.static_solve(**kw)
    L, gE, rc2, _ = g.adjoint_gradient(**kw)
    g.close()
    o = po.Oracle(p)
    f = o.loads()[0] + o.penalty_rhs()
    ur, _, _ = o.solve(f, precond=po.PC_DIRECT)
    gr, _, _, _ = o.adjoint(ur, lam=ur)
    rel = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))
    return {"sample": f"{nx}x{nx // 5}x{nx // 5} hex8, seed 100, oracle direct LDL^T", "rc": [rc, rc2],
            "u_rel": rel(u[0], ur), "compliance_rel": abs(L - f @ ur) / abs(f @ ur), "gradient_rel": rel(gE, gr)}


def size_series(nxs=(40, 60, 80), target_dof: int = 1_013_643) -> dict:
    """The CPU port on one core per block size (the sizes run concurrently,
    one process each), and a power-law fit rate = c * n_dof^k through them.
    The port's per-DOF rate falls with size (its LDL^T blocks grow with the
    cross-section and its PCG iteration count grows), so the fixed-size
    sample overstates what one core does on the 200x40x40 block; the fit's
    value there is an extrapolation, labelled as one."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    with ctx.Pool(len(nxs)) as pool:
        res = pool.map(_cpu_sample, [(nx, 100) for nx in nxs])
    pts = [{"cells": f"{nx}x{nx // 5}x{nx // 5}", "n_dof": r[0], "s": r[1], "iterations": r[2],
            "dof_solves_per_s_per_core": r[0] / r[1]} for nx, r in zip(nxs, res)]
    x = np.log([q["n_dof"] for q in pts])
    y = np.log([q["dof_solves_per_s_per_core"] for q in pts])
    k, c = np.polyfit(x, y, 1)
    return {"points": pts, "fit": f"rate = {np.exp(c):.4g} * n_dof^{k:.3f} per core",
            "exponent": float(k), "target_n_dof": target_dof,
            "extrapolated_dof_solves_per_s_per_core": float(np.exp(c) * target_dof ** k)}


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    vals = []
    for _ in range(a.warmup):
        cpu_baseline(a.cpu_sample_nx, procs)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        cb = cpu_baseline(a.cpu_sample_nx, procs)
        vals.append(cb["value"])
    wall = time.perf_counter() - t0
    v = statistics.mean(vals)
    series = None
    if not a.no_size_series:
        series = size_series(target_dof=3 * (a.nx + 1) * (a.ny + 1) * (a.nz + 1))
        series["extrapolated_dof_solves_per_s_all_cores"] = (series["extrapolated_dof_solves_per_s_per_core"]
                                                             * procs)
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": 1000 * wall / a.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"block_large sample {cb['sample']}"},
           "cpu_baseline": {**cb, "value": v},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "size_series": series}
    print(json.dumps(out))


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def run_ours(a):
    import torch

    from asend3d_gb300 import _lib, configs
    from asend3d_gb300.solver import GpuSolver

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    p = configs.block_large(nx=a.nx, ny=a.ny, nz=a.nz, seed=2024 + rank)
    g = GpuSolver(p, device=local)
    stream = torch.cuda.ExternalStream(g.stream, device=torch.device("cuda", local))
    n_dof = g.n_dof
    n_el = p.mesh.n_elems
    # headline method: FP64-accurate outer product on the FP32 pipes (hi + lo
    # value pairs), FP64 vectors / dots / residuals, FP32 multigrid V-cycle
    mixed = dict(method=_lib.METHOD_SPLIT, precond=_lib.PC_MG, rel_tol=1e-8, graph_iters=8)

    def step_device():
        g.assemble(precision=48)
        rc, st = g.static_solve_device(**mixed)
        L, rc2, st2 = adjoint_nocopy()
        return rc, st

    import ctypes as C

    o_adj = g.opts(**mixed)

    def adjoint_nocopy():
        Lc = C.c_double(0)
        st = _lib.SolveStats()
        rc = g.lib.asend_adjoint_gradient(g.ctx, C.byref(o_adj), C.byref(Lc), None, C.byref(st))
        return Lc.value, rc, st

    # ---- the split product's shape, tuned on this operator (bit-identical
    # results; the kernel alone is timed per shape)
    from asend3d_gb300 import autotune

    g.assemble(precision=48)
    shape, shape_ms = autotune.tune_product(g)

    # ---- warm-up
    for _ in range(a.warmup):
        rc, st = step_device()
        assert rc == 0, (rc, st)
    iters = st["iterations"]
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    launches0 = g.kernel_launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        stats = []
        for _ in range(a.steps):
            rc, st = step_device()
            assert rc == 0, (rc, st)
            stats.append(st)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = g.kernel_launches - launches0
    ms_step = max_over_ranks(ms / a.steps, world)
    value = replicas_value(n_dof, world, ms_step)

    # ---- e2e through the C ABI with pinned host buffers
    E_h = torch.from_numpy(p.E.copy()).pin_memory()
    u_h = torch.zeros(n_dof, dtype=torch.float64).pin_memory()
    gE_h = torch.zeros(n_el, dtype=torch.float64).pin_memory()
    f_np = g.load_vector(0)  # load (incl. penalty rhs after assembly)
    f_h = torch.from_numpy(f_np).pin_memory()
    P = C.POINTER(C.c_double)
    o_e2e = g.opts(**mixed)

    def step_e2e():
        g.lib.asend_set_modulus(g.ctx, C.cast(E_h.data_ptr(), P))
        g.lib.asend_clear_loads(g.ctx)
        g.lib.asend_add_load_vector(g.ctx, 0, C.cast(f_h.data_ptr(), P))
        g.lib.asend_assemble(g.ctx, 48, 0, 0.0, 0.25, 0.5)
        st = _lib.SolveStats()
        rc = g.lib.asend_static_solve(g.ctx, C.byref(o_e2e), C.cast(u_h.data_ptr(), P), C.byref(st))
        Lc = C.c_double(0)
        st2 = _lib.SolveStats()
        rc2 = g.lib.asend_adjoint_gradient(g.ctx, C.byref(o_e2e), C.byref(Lc), C.cast(gE_h.data_ptr(), P),
                                           C.byref(st2))
        return rc, rc2

    for _ in range(2):
        step_e2e()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.steps):
        rc, rc2 = step_e2e()
        assert rc == 0 and rc2 == 0
    e1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / a.steps
    wall_e2e = (time.perf_counter() - t0) * 1000 / a.steps
    ms_e2e = max(ms_e2e, wall_e2e)
    ms_e2e = max_over_ranks(ms_e2e, world)
    e2e_value = replicas_value(n_dof, world, ms_e2e)
    h2d = n_el * 8 + n_dof * 8
    d2h = n_dof * 8 + n_el * 8 + 8

    # restore the benchmark load for the remaining measurements
    g.set_loads()

    # ---- plain FP64 Jacobi PCG on the same GPU (the method the speed-up is measured against)
    plain = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-8, graph_iters=32)
    g.assemble(precision=64)
    g.static_solve_device(**plain)
    torch.cuda.synchronize()
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    n_plain = max(1, min(a.steps, 3))
    p0.record(stream)
    for _ in range(n_plain):
        g.assemble(precision=64)
        rc, st_plain = g.static_solve_device(**plain)
        adjoint_nocopy()
    p1.record(stream)
    torch.cuda.synchronize()
    ms_plain = p0.elapsed_time(p1) / n_plain
    ms_plain = max_over_ranks(ms_plain, world)
    plain_value = replicas_value(n_dof, world, ms_plain)

    # ---- roofline: the three kernels of every multigrid-CG iteration that
    # read a full finest-level operator (each launched once per iteration),
    # timed as they run in the step; the slowest is reported
    peak, peak_kind = measured_peak()
    kern = {}
    names = {0: f"{PRODUCT_KERNEL[shape]} (outer FP64-accurate product, FP32 hi+lo values, + p.Ap)",
             1: "k_vc_resid (finest-level V-cycle residual, FP32 SBELL SpMV)",
             2: "k_vc_post (finest-level post-smoothing, FP32 SBELL SpMV + block Jacobi)"}
    for k in (0, 1, 2):
        ms_k, by_k = g.time_mg_kernel(k, _lib.METHOD_SPLIT, 30)
        kern[k] = {"kernel": names[k], "ms_per_launch": ms_k, "algorithmic_bytes_per_launch": by_k,
                   "achieved_GBps": by_k / (ms_k * 1e-3) / 1e9}
    ms64, by64 = g.time_mg_kernel(0, _lib.METHOD_FP64, 20)
    top = max(kern, key=lambda k: kern[k]["ms_per_launch"])
    achieved = kern[top]["achieved_GBps"]
    roof = {"bound": "hbm", "kernel": kern[top]["kernel"], "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": f"of {peak_kind}", "traffic": ncu_traffic(top),
            "algorithmic_bytes_per_launch": kern[top]["algorithmic_bytes_per_launch"],
            "ms_per_launch": kern[top]["ms_per_launch"],
            "per_iteration_kernels": [dict(kern[k], frac=kern[k]["achieved_GBps"] / peak,
                                           traffic=ncu_traffic(k)) for k in (0, 1, 2)],
            "fp64_outer_product": {"kernel": "k_mg_spmv_dot<double,double> (native FP64 values)",
                                   "ms_per_launch": ms64, "achieved_GBps": by64 / (ms64 * 1e-3) / 1e9},
            "product_shapes_ms_per_launch": {PRODUCT_KERNEL[v]: t for v, t in shape_ms.items()}}

    # ---- accuracy at full size: the benchmark's 1e-8 solution and gradient
    # against the same library at 1e-11 (FP64 operator); never fatal
    accuracy = {"reference_parity": "unpinned at solver precision: the oracle restates the reference's "
                                    "algorithm in C++ and is tied to the reference by its analytic known answers "
                                    "(rtol 1e-3 to 2e-2; singleHex 2e-5), finite differences and self-consistency; "
                                    "the reference (Rust) cannot be built here"}
    if rank == 0:
        try:
            g.assemble(precision=48)  # the benchmark's operator and solve
            u8, _, _ = g.static_solve(**mixed)
            L8, gE8, _, _ = g.adjoint_gradient(**mixed)
            g.assemble(precision=64)  # the FP64 reference
            tight = dict(mixed, method=_lib.METHOD_FP64, rel_tol=1e-11, max_iter=400)
            u11, rc11, st11 = g.static_solve(**tight)
            L11, gE11, _, _ = g.adjoint_gradient(**tight)
            rel = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))
            accuracy["full_size_vs_fp64_1e-11"] = {"u_rel": rel(u8, u11), "compliance_rel": abs(L8 - L11) / abs(L11),
                                                    "gradient_rel": rel(gE8, gE11), "rc_1e-11": rc11,
                                                    "rel_residual_1e-11": st11["rel_residual"]}
        except Exception as err:  # the measurement above stands on its own
            accuracy["full_size_error"] = repr(err)[:200]

    out = None
    if rank == 0:
        cb = None
        if not a.no_cpu_baseline and world == 1:
            cb = cpu_baseline(a.cpu_sample_nx, 1)
            cb["kind"] = "port"
            try:
                accuracy["sample_vs_oracle"] = sample_accuracy(a.cpu_sample_nx, mixed)
            except Exception as err:
                accuracy["sample_vs_oracle_error"] = repr(err)[:200]
        clocks = clk.summary()
        batch = None
        if not a.no_batch and world == 1:
            try:
                batch = batch_measure(steps=3, warmup=2)
            except Exception as err:  # the headline measurement stands on its own
                batch = {"error": repr(err)[:300]}
        learned = None
        if not a.no_learned and world == 1:
            try:
                learned = learned_measure()
            except Exception as err:  # the headline measurement stands on its own
                learned = {"error": repr(err)[:300]}
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
               "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "fp32-pair operator values and CG vectors (FP64-accurate), f64 x / reductions / true residual, f32 multigrid",
               "data": "synthetic (seeded lognormal field)",
               "config": {"workload": f"block_large {a.nx}x{a.ny}x{a.nz} hex8 static + adjoint",
                          "n_dof": n_dof, "n_elems": n_el, "rhs_per_step": 1,
                          "method": "CG + geometric multigrid V-cycle (FP32 levels), FP64-accurate split operator",
                          "rel_tol": 1e-8, "l2": "operator 640 MB FP64 + 330 MB FP32 > 129 MB L2 (inputs larger than L2)",
                          "parallelism": f"replicas x{world}"},
               "iterations": iters, "ms_breakdown": {"assemble": stats[-1]["ms_assemble"],
                                                     "solve": stats[-1]["ms_solve"]},
               "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "ms_per_step": ms_e2e},
               "plain_fp64_jacobi": {"value": plain_value, "ms_per_step": ms_plain,
                                     "iterations": st_plain["iterations"]},
               "speedup_vs_plain_fp64": value / plain_value,
               "roofline": roof, "cpu_baseline": cb, "clocks": clocks, "gpu_launches": launches,
               "accuracy": accuracy, "batch_uq": batch, "learned": learned}
        print(json.dumps(out))
    g.close()
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return out


def main():
    a = parse()
    if a.profile:
        run_profile(a)
    elif a.workload == "batch_uq" and a.impl != "reference":
        run_batch(a)
    elif a.workload == "shell_plate" and a.impl != "reference":
        run_shell(a)
    elif a.workload == "modal" and a.impl != "reference":
        run_modal(a)
    elif a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
