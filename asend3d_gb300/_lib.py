"""ctypes binding of ``libasend_gpu.so`` (the C ABI in ``include/asend_gpu.h``).

The library is built in-tree by ``asend3d_gb300.build``.  Loading fails loudly
when it is missing: there is no CPU fallback for the solve path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libasend_gpu.so"

c_int = C.c_int32
c_dbl = C.c_double
P_int = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
P_dbl = C.POINTER(C.c_double)
P_flt = C.POINTER(C.c_float)

ASEND_OK, ASEND_MAX_ITER, ASEND_NONFINITE, ASEND_FALLBACK = 0, 1, 2, 3
ASEND_EINVAL, ASEND_ECUDA, ASEND_ESTATE = -1, -2, -3
METHOD_FP64, METHOD_MIXED, METHOD_SPLIT = 0, 1, 2
PC_JACOBI, PC_BLOCK, PC_LEARNED, PC_MG, PC_MG_LEARNED = 0, 1, 2, 3, 4
# shapes of the multigrid CG's split outer product (bit-identical results)
(PRODUCT_DEFAULT, PRODUCT_REGISTERS, PRODUCT_STAGED_2x3, PRODUCT_STAGED_3x2, PRODUCT_STAGED_2x2,
 PRODUCT_STAGED_4x2) = range(6)
PRODUCT_VARIANTS = (PRODUCT_REGISTERS, PRODUCT_STAGED_2x3, PRODUCT_STAGED_3x2, PRODUCT_STAGED_2x2, PRODUCT_STAGED_4x2)
OBJ_DISPLACEMENT, OBJ_COMPLIANCE, OBJ_ELEMENT = 0, 1, 2
LOAD_BODY_FORCE, LOAD_GRAVITY, LOAD_CENTRIFUGAL = 0, 1, 2
LEARN_BLOCK, LEARN_MG = 0, 1
DV_MODULUS, DV_SHEAR_MODULUS, DV_POISSON_RATIO = 0, 1, 2
DV_AREA, DV_AREA_MOMENT, DV_POLAR_MOMENT = 3, 4, 5  # beam2 sections


class SolveOpts(C.Structure):
    _fields_ = [("method", c_int), ("precond", c_int), ("rel_tol", c_dbl), ("max_iter", c_int),
                ("graph_iters", c_int), ("warm_start", c_int), ("replace_every", c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", c_int), ("status", c_int), ("replacements", c_int), ("n_rhs", c_int),
                ("rel_residual", c_dbl), ("ms_assemble", c_dbl), ("ms_solve", c_dbl),
                ("ms_adjoint", c_dbl), ("penalty_scale", c_dbl)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class EigenOpts(C.Structure):
    _fields_ = [("n_modes", c_int), ("block_size", c_int), ("max_subspace", c_int), ("reserved", c_int),
                ("shift", c_dbl), ("tol", c_dbl), ("inner", SolveOpts)]


class EigenStats(C.Structure):
    _fields_ = [("n_found", c_int), ("n_converged", c_int), ("subspace", c_int), ("n_solves", c_int),
                ("inner_iterations", C.c_int64), ("status", c_int), ("inner_capped", c_int),
                ("max_rel_residual", c_dbl), ("max_pencil_residual", c_dbl), ("ms", c_dbl)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# (name, restype, argtypes) for every symbol declared in include/asend_gpu.h
SIGNATURES = [
    ("asend_create", C.c_void_p, [c_int]),
    ("asend_destroy", None, [C.c_void_p]),
    ("asend_last_error", C.c_char_p, [C.c_void_p]),
    ("asend_version", C.c_char_p, []),
    ("asend_set_mesh", c_int, [C.c_void_p, c_int, c_int, P_dbl, c_int, P_int, P_dbl, P_dbl, P_dbl, P_dbl]),
    ("asend_set_modulus", c_int, [C.c_void_p, P_dbl]),
    ("asend_set_block_structure", c_int, [C.c_void_p, c_int, c_int, c_int]),
    ("asend_mg_levels", c_int, [C.c_void_p]),
    ("asend_mg_set_damping", c_int, [C.c_void_p, c_dbl]),
    ("asend_set_product_variant", c_int, [C.c_void_p, c_int]),
    ("asend_mg_set_fused_tail", c_int, [C.c_void_p, c_int]),
    ("asend_set_launch_overlap", c_int, [C.c_void_p, c_int]),
    ("asend_mg_level_info", c_int, [C.c_void_p, c_int, P_int, P_dbl, P_dbl, P_dbl]),
    ("asend_mg_vcycle", c_int, [C.c_void_p, P_flt, P_flt]),
    ("asend_set_instances", c_int, [C.c_void_p, c_int, P_int]),
    ("asend_set_instance_blocks", c_int, [C.c_void_p, c_int, P_int]),
    ("asend_add_node_set", c_int, [C.c_void_p, c_int, P_int]),
    ("asend_add_element_set", c_int, [C.c_void_p, c_int, P_int]),
    ("asend_add_constraint", c_int, [C.c_void_p, c_int, P_int, P_int, P_dbl, c_dbl]),
    ("asend_add_nodal_force", c_int, [C.c_void_p, c_int, c_int, P_dbl]),
    ("asend_add_surface_traction", c_int, [C.c_void_p, c_int, c_int, P_dbl, c_dbl, P_dbl]),
    ("asend_newmark_keep_history", c_int, [C.c_void_p, c_int]),
    ("asend_newmark_step_state", c_int, [C.c_void_p, c_int, P_dbl, P_dbl, P_dbl]),
    ("asend_newmark_adjoint", c_int, [C.c_void_p, C.c_void_p, c_int, P_int, P_dbl, P_dbl, P_dbl, C.c_void_p]),
    ("asend_add_surface_pressure", c_int, [C.c_void_p, c_int, c_int, P_dbl, c_dbl, c_dbl]),
    ("asend_add_body_load", c_int, [C.c_void_p, c_int, c_int, c_int, P_dbl, c_dbl, P_dbl, P_dbl]),
    ("asend_add_load_vector", c_int, [C.c_void_p, c_int, P_dbl]),
    ("asend_clear_loads", c_int, [C.c_void_p]),
    ("asend_n_dof", c_int, [C.c_void_p]),
    ("asend_n_load_cases", c_int, [C.c_void_p]),
    ("asend_get_load_vector", c_int, [C.c_void_p, c_int, P_dbl]),
    ("asend_assemble", c_int, [C.c_void_p, c_int, c_int, c_dbl, c_dbl, c_dbl]),
    ("asend_get_csr", c_int, [C.c_void_p, c_int, P_i64, P_i64, P_int, P_dbl]),
    ("asend_get_coloring", c_int, [C.c_void_p, P_int]),
    ("asend_static_solve", c_int, [C.c_void_p, C.POINTER(SolveOpts), P_dbl, C.POINTER(SolveStats)]),
    ("asend_static_solve_device", c_int, [C.c_void_p, C.POINTER(SolveOpts), C.POINTER(SolveStats)]),
    ("asend_get_solution", c_int, [C.c_void_p, c_int, P_dbl]),
    ("asend_set_objective", c_int, [C.c_void_p, c_int, c_int, c_int, c_dbl]),
    ("asend_adjoint_gradient", c_int, [C.c_void_p, C.POINTER(SolveOpts), P_dbl, P_dbl, C.POINTER(SolveStats)]),
    ("asend_element_fields", c_int, [C.c_void_p, c_int, P_dbl, P_dbl, P_dbl]),
    ("asend_shell_section", c_int, [c_int, P_dbl, c_dbl, P_dbl, P_dbl]),
    ("asend_set_shell_sections", c_int, [C.c_void_p, P_dbl, P_dbl]),
    ("asend_set_beam_sections", c_int, [C.c_void_p, P_dbl]),
    ("asend_set_beam_section_matrices", c_int, [C.c_void_p, P_dbl, P_dbl]),
    ("asend_set_element_objective", c_int, [C.c_void_p, P_dbl, P_dbl]),
    ("asend_add_modulus_design_var", c_int, [C.c_void_p, c_int, c_int, P_dbl]),
    ("asend_design_var_gradient", c_int, [C.c_void_p, P_dbl, P_dbl]),
    ("asend_newmark_run", c_int, [C.c_void_p, C.POINTER(SolveOpts), c_int, P_dbl, c_int, P_dbl, P_dbl,
                                  C.POINTER(SolveStats)]),
    ("asend_apply_operator", c_int, [C.c_void_p, c_int, P_dbl, P_dbl]),
    ("asend_time_spmv", c_int, [C.c_void_p, c_int, c_int, P_dbl, P_dbl]),
    ("asend_kernel_launches", C.c_int64, [C.c_void_p]),
    ("asend_stream", C.c_void_p, [C.c_void_p]),
    ("asend_element_matrices", c_int, [C.c_void_p, c_int, c_int, P_dbl, P_dbl]),
    ("asend_eigen_solve", c_int, [C.c_void_p, C.POINTER(EigenOpts), P_dbl, P_dbl, P_dbl, P_dbl,
                                  C.POINTER(EigenStats)]),
    ("asend_dense_sym_eigen", c_int, [c_int, P_dbl, P_dbl, P_dbl]),
    ("asend_adjoint_strain_pairs", c_int, [C.c_void_p, P_dbl]),
    ("asend_material_dv_gradient", c_int, [C.c_void_p, c_int, c_int, c_int, c_int, P_dbl, P_dbl]),
    ("asend_material_dC", c_int, [c_int, c_int, c_dbl, c_dbl, P_dbl]),
    ("asend_time_mg_kernel", c_int, [C.c_void_p, c_int, c_int, c_int, P_dbl, P_dbl]),
    ("asend_set_orthotropic", c_int, [C.c_void_p, P_dbl]),
    ("asend_orthotropic_cmat", c_int, [P_dbl, P_dbl]),
    ("asend_set_damping", c_int, [C.c_void_p, c_dbl, c_dbl, P_dbl]),
    ("asend_set_lumped_mass", c_int, [C.c_void_p, c_int]),
    ("asend_operator_energy_noalloc", c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("asend_learned_n_params", c_int, []),
    ("asend_learned_init", c_int, [C.c_void_p, C.c_uint64]),
    ("asend_learned_set_params", c_int, [C.c_void_p, P_flt]),
    ("asend_learned_get_params", c_int, [C.c_void_p, P_flt]),
    ("asend_learned_add_samples", c_int, [C.c_void_p, c_int, P_int, c_int, C.c_uint64]),
    ("asend_learned_set_objective", c_int, [C.c_void_p, c_int]),
    ("asend_learned_set_samples", c_int, [C.c_void_p, c_int, P_flt]),
    ("asend_learned_train", c_int, [C.c_void_p, c_int, C.c_float, P_dbl]),
    ("asend_learned_loss_grad", c_int, [C.c_void_p, P_dbl, P_flt]),
    ("asend_learned_features", c_int, [C.c_void_p, P_flt, P_flt, P_flt]),
    ("asend_learned_blocks", c_int, [C.c_void_p, c_int, P_flt]),
    ("asend_learned_forward", c_int, [C.c_void_p, c_int, P_flt, P_flt]),
    ("asend_learned_backward", c_int, [C.c_void_p, c_int, P_flt, P_flt, P_flt]),
]

_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                           "(the solve path has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
