"""Host-side mirror of the reference's model / load / DV / objective interface,
driving the CUDA library through its C ABI.

The reference's user interface (asendUtils, Python) describes a model as
node/element sets, 'displacement' constraints built from (nodeSet, dof,
coefficient) terms (src/asendUtils/model/Constraint.py), nodal forces and
surface tractions (Model.addNodalForce / addSurfaceTraction,
src/asendUtils/model/Model.py:306-354), design variables over element sets
(src/asendUtils/variables/DesignVariables.py:13-30) and objective terms
(src/asendUtils/objective/Objective.py:14-39), then runs the Rust solver.
``Problem`` holds the same description; ``GpuSolver`` hands it to
``libasend_gpu.so`` (the GB300 replacement of the Rust solver core).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import SolveOpts, SolveStats
from .mesh import BlockMesh


class AsendError(RuntimeError):
    pass


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


@dataclass
class Problem:
    mesh: BlockMesh
    E: np.ndarray
    nu: np.ndarray
    rho: np.ndarray | None = None
    node_sets: dict = field(default_factory=dict)
    elem_sets: dict = field(default_factory=dict)
    # constraints: (terms=[(node_set, comp(1-based), coef), ...], rhs)
    constraints: list = field(default_factory=list)
    # loads[case] = list of ("nodalForce", set, load6) | ("surfaceTraction", elset, normDir, normTol, t3)
    #               | ("surfacePressure", elset, normDir, normTol, p) | ("bodyForce" | "gravitational", elset, v3)
    #               | ("centrifugal", elset, omega, center3, axis3) | ("vector", f)
    loads: list = field(default_factory=list)
    objective: tuple = ("compliance",)
    # design variables: (elem_set, coefficients)
    design_vars: list = field(default_factory=list)
    thickness: np.ndarray | None = None  # per element (shell sections)
    # orthotropic constants per element [n_el][9] = E1 E2 E3 nu12 nu13 nu23 G12 G13 G23
    # (solids; replaces E, nu in the stiffness)
    ortho: np.ndarray | None = None
    # damping of Newmark runs: (rayleigh_cm, rayleigh_ck, material damping [n_el][36] or None)
    damping: tuple | None = None
    lump_mass: bool = False  # row-sum lumped mass in Newmark runs
    # layered shell4 sections: [(element indices, layers [n, 7] = E1 E2 nu12
    # G12 density thickness angle[deg], z offset)]; other elements keep E, nu, t
    shell_sections: list | None = None
    # beam2 sections [n_el][10] (or one row for every element): area, I1..I5
    # (int z, int y, int z^2, int y^2, int yz dA in the section axes), polar
    # moment J, and the vector v fixing the section's xy plane
    beam_sections: np.ndarray | None = None
    # given beam section matrices (stiffness [n_el][36] or None, mass [n_el][36]
    # or None); an element whose [0] entry is <= 0 keeps the computed one
    beam_section_matrices: tuple | None = None

    def add_node_set(self, name, nodes):
        self.node_sets[name] = np.asarray(nodes, dtype=np.int32)

    def add_elem_set(self, name, elems):
        self.elem_sets[name] = np.asarray(elems, dtype=np.int32)

    def fix_displacement(self, set_name, comps=(1, 2, 3), rhs=0.0):
        for c in comps:
            self.constraints.append(([(set_name, c, 1.0)], rhs))

    def _case(self, case):
        while len(self.loads) <= case:
            self.loads.append([])
        return self.loads[case]

    def add_nodal_force(self, set_name, F, case=0):
        load = np.zeros(6)
        load[: len(F)] = F
        self._case(case).append(("nodalForce", set_name, load))

    def add_surface_traction(self, elem_set, normal_dir, traction, norm_tol=1.0, case=0):
        self._case(case).append(("surfaceTraction", elem_set, np.asarray(normal_dir, float), float(norm_tol),
                                 np.asarray(traction, float)))

    def add_surface_pressure(self, elem_set, normal_dir, pressure, norm_tol=1.0, case=0):
        self._case(case).append(("surfacePressure", elem_set, np.asarray(normal_dir, float), float(norm_tol),
                                 float(pressure)))

    def add_body_force(self, elem_set, f, case=0):
        """Force per unit volume (the reference's 'bodyForce')."""
        self._case(case).append(("bodyForce", elem_set, np.asarray(f, float)))

    def add_gravity(self, elem_set, g, case=0):
        self._case(case).append(("gravitational", elem_set, np.asarray(g, float)))

    def add_centrifugal(self, elem_set, omega, center, axis, case=0):
        self._case(case).append(("centrifugal", elem_set, float(omega), np.asarray(center, float),
                                 np.asarray(axis, float)))

    def add_load_vector(self, f, case=0):
        self._case(case).append(("vector", np.asarray(f, float)))


class GpuSolver:
    """One library context (one CUDA stream) holding one problem."""

    def __init__(self, problem: Problem, device: int = 0, instances=None, blocks=None):
        self.lib = _lib.load()
        self.ctx = self.lib.asend_create(device)
        if not self.ctx:
            raise AsendError("asend_create failed (no CUDA device?)")
        self.p = problem
        self.set_ids = {}
        self.elset_ids = {}
        self.instances = None if instances is None else np.ascontiguousarray(instances, dtype=np.int32)
        # structured block (nx, ny, nz) of every instance: enables multigrid on the stack
        self.blocks = None if blocks is None else np.ascontiguousarray(blocks, dtype=np.int32).reshape(-1, 3)
        self._setup()

    # -- helpers -----------------------------------------------------------
    def _check(self, rc, what):
        if rc < 0:
            msg = self.lib.asend_last_error(self.ctx).decode()
            raise AsendError(f"{what} failed ({rc}): {msg}")
        return rc

    def close(self):
        if self.ctx:
            self.lib.asend_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _setup(self):
        p, m = self.p, self.p.mesh
        coords = np.ascontiguousarray(m.coords, dtype=np.float64)
        conn = np.ascontiguousarray(m.conn, dtype=np.int32)
        E = np.ascontiguousarray(p.E, dtype=np.float64)
        nu = np.ascontiguousarray(np.broadcast_to(p.nu, E.shape), dtype=np.float64)
        rho = None if p.rho is None else np.ascontiguousarray(np.broadcast_to(p.rho, E.shape), dtype=np.float64)
        thk = None if p.thickness is None else np.ascontiguousarray(np.broadcast_to(p.thickness, E.shape),
                                                                    dtype=np.float64)
        self._keep = (coords, conn, E, nu, rho, thk)
        self._check(self.lib.asend_set_mesh(self.ctx, m.elem_type, m.n_nodes, _ptr(coords, C.c_double), m.n_elems,
                                            _ptr(conn, C.c_int32), _ptr(E, C.c_double), _ptr(nu, C.c_double),
                                            None if rho is None else _ptr(rho, C.c_double),
                                            None if thk is None else _ptr(thk, C.c_double)), "set_mesh")
        if p.ortho is not None:
            self._ortho = np.ascontiguousarray(p.ortho, dtype=np.float64).reshape(-1, 9)
            self._check(self.lib.asend_set_orthotropic(self.ctx, _ptr(self._ortho, C.c_double)), "set_orthotropic")
        if p.damping is not None:
            cm, ck, dm = p.damping
            self._dmat = None if dm is None else np.ascontiguousarray(dm, dtype=np.float64).reshape(-1, 36)
            self._check(self.lib.asend_set_damping(self.ctx, float(cm), float(ck),
                                                   None if self._dmat is None else _ptr(self._dmat, C.c_double)),
                        "set_damping")
        if p.lump_mass:
            self._check(self.lib.asend_set_lumped_mass(self.ctx, 1), "set_lumped_mass")
        if p.shell_sections:
            self._set_shell_sections(p, E, nu, rho, thk)
        if p.beam_sections is not None:
            self._bsec = np.ascontiguousarray(np.broadcast_to(np.asarray(p.beam_sections, np.float64),
                                                              (m.n_elems, 10)))
            self._check(self.lib.asend_set_beam_sections(self.ctx, _ptr(self._bsec, C.c_double)),
                        "set_beam_sections")
            if p.beam_section_matrices is not None:
                cs, ms = (None if x is None else np.ascontiguousarray(np.broadcast_to(np.asarray(x, np.float64),
                                                                                      (m.n_elems, 36)))
                          for x in p.beam_section_matrices)
                self._bcm = (cs, ms)
                self._check(self.lib.asend_set_beam_section_matrices(
                    self.ctx, None if cs is None else _ptr(cs, C.c_double),
                    None if ms is None else _ptr(ms, C.c_double)), "set_beam_section_matrices")
        if m.elem_type in (8, 81) and m.conn.shape[0] == m.nx * m.ny * m.nz:
            self._check(self.lib.asend_set_block_structure(self.ctx, m.nx, m.ny, m.nz), "set_block_structure")
        for name, nodes in p.node_sets.items():
            arr = np.ascontiguousarray(nodes, dtype=np.int32)
            self.set_ids[name] = self._check(self.lib.asend_add_node_set(self.ctx, len(arr), _ptr(arr, C.c_int32)),
                                             "add_node_set")
        for name, els in p.elem_sets.items():
            arr = np.ascontiguousarray(els, dtype=np.int32)
            self.elset_ids[name] = self._check(
                self.lib.asend_add_element_set(self.ctx, len(arr), _ptr(arr, C.c_int32)), "add_element_set")
        for terms, rhs in p.constraints:
            sets = np.array([self.set_ids[t[0]] for t in terms], dtype=np.int32)
            comps = np.array([t[1] for t in terms], dtype=np.int32)
            coefs = np.array([t[2] for t in terms], dtype=np.float64)
            self._check(self.lib.asend_add_constraint(self.ctx, len(terms), _ptr(sets, C.c_int32),
                                                      _ptr(comps, C.c_int32), _ptr(coefs, C.c_double), rhs),
                        "add_constraint")
        if self.instances is not None:  # validated against elements and constraints
            self._check(self.lib.asend_set_instances(self.ctx, len(self.instances) - 1,
                                                     _ptr(self.instances, C.c_int32)), "set_instances")
            if self.blocks is not None:
                self._check(self.lib.asend_set_instance_blocks(self.ctx, len(self.blocks),
                                                               _ptr(self.blocks, C.c_int32)), "set_instance_blocks")
        self.set_loads()
        obj = p.objective
        if obj[0] == "compliance":
            self._check(self.lib.asend_set_objective(self.ctx, _lib.OBJ_COMPLIANCE, -1, 0, 1.0), "set_objective")
        else:
            _, set_name, comp, coef = obj
            self._check(self.lib.asend_set_objective(self.ctx, _lib.OBJ_DISPLACEMENT, self.set_ids[set_name],
                                                     comp, coef), "set_objective")
        for elset, coefs in p.design_vars:
            cf = np.ascontiguousarray(np.atleast_1d(coefs), dtype=np.float64)
            self._check(self.lib.asend_add_modulus_design_var(self.ctx, self.elset_ids[elset], len(cf),
                                                              _ptr(cf, C.c_double)), "add_design_var")

    def set_loads(self):
        self._check(self.lib.asend_clear_loads(self.ctx), "clear_loads")
        for case, items in enumerate(self.p.loads):
            for it in items:
                if it[0] == "nodalForce":
                    load = np.ascontiguousarray(it[2], dtype=np.float64)
                    self._check(self.lib.asend_add_nodal_force(self.ctx, case, self.set_ids[it[1]],
                                                               _ptr(load, C.c_double)), "add_nodal_force")
                elif it[0] == "surfaceTraction":
                    nd = np.ascontiguousarray(it[2], dtype=np.float64)
                    t = np.ascontiguousarray(it[4], dtype=np.float64)
                    self._check(self.lib.asend_add_surface_traction(self.ctx, case, self.elset_ids[it[1]],
                                                                    _ptr(nd, C.c_double), it[3],
                                                                    _ptr(t, C.c_double)), "add_surface_traction")
                elif it[0] == "surfacePressure":
                    nd = np.ascontiguousarray(it[2], dtype=np.float64)
                    self._check(self.lib.asend_add_surface_pressure(self.ctx, case, self.elset_ids[it[1]],
                                                                    _ptr(nd, C.c_double), it[3], float(it[4])),
                                "add_surface_pressure")
                elif it[0] in ("bodyForce", "gravitational", "centrifugal"):
                    kind = {"bodyForce": _lib.LOAD_BODY_FORCE, "gravitational": _lib.LOAD_GRAVITY,
                            "centrifugal": _lib.LOAD_CENTRIFUGAL}[it[0]]
                    if kind == _lib.LOAD_CENTRIFUGAL:
                        cen = np.ascontiguousarray(it[3], dtype=np.float64)
                        ax = np.ascontiguousarray(it[4], dtype=np.float64)
                        rc = self.lib.asend_add_body_load(self.ctx, case, self.elset_ids[it[1]], kind, None,
                                                          float(it[2]), _ptr(cen, C.c_double), _ptr(ax, C.c_double))
                    else:
                        v = np.ascontiguousarray(it[2], dtype=np.float64)
                        rc = self.lib.asend_add_body_load(self.ctx, case, self.elset_ids[it[1]], kind,
                                                          _ptr(v, C.c_double), 0.0, None, None)
                    self._check(rc, "add_body_load")
                else:
                    f = np.ascontiguousarray(it[1], dtype=np.float64)
                    self._check(self.lib.asend_add_load_vector(self.ctx, case, _ptr(f, C.c_double)),
                                "add_load_vector")

    # -- API ---------------------------------------------------------------
    @property
    def n_dof(self) -> int:
        return self.lib.asend_n_dof(self.ctx)

    @property
    def n_cases(self) -> int:
        return self.lib.asend_n_load_cases(self.ctx)

    def set_modulus(self, E):
        E = np.ascontiguousarray(E, dtype=np.float64)
        self._keep_E = E
        self._check(self.lib.asend_set_modulus(self.ctx, _ptr(E, C.c_double)), "set_modulus")

    def assemble(self, precision=64, dynamic=False, dt=0.0, beta=0.25, gamma=0.5):
        self._check(self.lib.asend_assemble(self.ctx, precision, int(dynamic), dt, beta, gamma), "assemble")

    def load_vector(self, case=0) -> np.ndarray:
        f = np.zeros(self.n_dof)
        self._check(self.lib.asend_get_load_vector(self.ctx, case, _ptr(f, C.c_double)), "get_load_vector")
        return f

    def opts(self, method=_lib.METHOD_MIXED, precond=_lib.PC_JACOBI, rel_tol=1e-8, max_iter=0, graph_iters=16,
             warm_start=0, replace_every=0, product=None) -> SolveOpts:
        """Solve options; `product` (an autotuned _lib.PRODUCT_* shape of the
        split outer product) is a context setting and is installed here."""
        if product is not None:
            self.set_product_variant(product)
        return SolveOpts(method, precond, rel_tol, max_iter, graph_iters, warm_start, replace_every)

    def static_solve(self, u0=None, **kw):
        o = self.opts(warm_start=int(u0 is not None), **kw)
        nc = max(1, self.n_cases)
        u = np.zeros(nc * self.n_dof) if u0 is None else np.ascontiguousarray(u0, dtype=np.float64).ravel().copy()
        st = SolveStats()
        rc = self._check(self.lib.asend_static_solve(self.ctx, C.byref(o), _ptr(u, C.c_double), C.byref(st)),
                         "static_solve")
        return u.reshape(nc, self.n_dof), rc, st.as_dict()

    def static_solve_device(self, **kw):
        o = self.opts(**kw)
        st = SolveStats()
        rc = self._check(self.lib.asend_static_solve_device(self.ctx, C.byref(o), C.byref(st)), "static_solve")
        return rc, st.as_dict()

    def solution(self, case=0) -> np.ndarray:
        u = np.zeros(self.n_dof)
        self._check(self.lib.asend_get_solution(self.ctx, case, _ptr(u, C.c_double)), "get_solution")
        return u

    def adjoint_gradient(self, want_dLdE=True, **kw):
        """(L, dL/dE per element or None, status, stats).  want_dLdE=False
        skips the per-element modulus gradient (orthotropic elements: material
        DV gradients come from material_dv_gradient)."""
        o = self.opts(**kw)
        L = C.c_double(0.0)
        g = np.zeros(self.p.mesh.n_elems) if want_dLdE else None
        st = SolveStats()
        rc = self._check(self.lib.asend_adjoint_gradient(self.ctx, C.byref(o), C.byref(L),
                                                         _ptr(g, C.c_double) if want_dLdE else None,
                                                         C.byref(st)), "adjoint_gradient")
        return L.value, g, rc, st.as_dict()

    def set_objective(self, objective):
        """("compliance",) or ("displacement", node_set, component, coefficient)."""
        if objective[0] == "compliance":
            rc = self.lib.asend_set_objective(self.ctx, _lib.OBJ_COMPLIANCE, -1, 0, 1.0)
        else:
            _, set_name, comp, coef = objective
            rc = self.lib.asend_set_objective(self.ctx, _lib.OBJ_DISPLACEMENT, self.set_ids[set_name], comp, coef)
        self._check(rc, "set_objective")

    def shell_section(self, layers, z_offset=0.0):
        """(ABD [81], section mass [36]) of a layered shell section; layers
        [n, 7] = E1, E2, nu12, G12, density, thickness, angle [deg]."""
        lay = np.ascontiguousarray(layers, dtype=np.float64).reshape(-1, 7)
        abd, ms = np.zeros(81), np.zeros(36)
        rc = self.lib.asend_shell_section(len(lay), _ptr(lay, C.c_double), float(z_offset), _ptr(abd, C.c_double),
                                          _ptr(ms, C.c_double))
        if rc != 0:
            raise AsendError("asend_shell_section: invalid layers")
        return abd, ms

    def _set_shell_sections(self, p, E, nu, rho, thk):
        ne = p.mesh.n_elems
        abd, ms = np.zeros((ne, 81)), np.zeros((ne, 36))
        r = np.zeros(ne) if rho is None else rho
        for e in range(ne):  # elements outside the sections: one isotropic layer
            abd[e], ms[e] = self.shell_section([[E[e], E[e], nu[e], E[e] / (2 * (1 + nu[e])), r[e], thk[e], 0.0]])
        for els, layers, zoff in p.shell_sections:
            a, mm = self.shell_section(layers, zoff)
            abd[np.asarray(els)] = a
            ms[np.asarray(els)] = mm
        self._sec = (np.ascontiguousarray(abd), np.ascontiguousarray(ms))
        self._check(self.lib.asend_set_shell_sections(self.ctx, _ptr(self._sec[0], C.c_double),
                                                      _ptr(self._sec[1], C.c_double)), "set_shell_sections")

    def element_fields(self, rhs=0):
        """Centroid strain and stress [n_el, 6] of load case rhs of the last
        solve and the element volumes [n_el] (solid meshes)."""
        n = self.p.mesh.n_elems
        eps, sig, vol = np.zeros((n, 6)), np.zeros((n, 6)), np.zeros(n)
        self._check(self.lib.asend_element_fields(self.ctx, rhs, _ptr(eps, C.c_double), _ptr(sig, C.c_double),
                                                  _ptr(vol, C.c_double)), "element_fields")
        return eps, sig, vol

    def set_element_objective(self, elems, category, component=0, operator="powerNorm", coef=1.0, exponent=1.0,
                              targets=None) -> float:
        """Evaluate an element-category term ('stress', 'strain',
        'strainEnergy' with powerNorm / ks / volumeIntegral / volumeAverage)
        on the last solution and select it for the next adjoint_gradient.
        Returns its value."""
        from .objective import element_term
        eps, sig, vol = self.element_fields(0)
        L, wa, wb = element_term(eps, sig, vol, elems, category, component, operator, coef, exponent, targets)
        wa = np.ascontiguousarray(wa)
        wb = np.ascontiguousarray(wb)
        self._check(self.lib.asend_set_element_objective(self.ctx, _ptr(wa, C.c_double), _ptr(wb, C.c_double)),
                    "set_element_objective")
        return L

    def strain_pairs(self) -> np.ndarray:
        """[n_el, 6, 6] strain-pair tensors of the last adjoint gradient."""
        P = np.zeros((self.p.mesh.n_elems, 6, 6))
        self._check(self.lib.asend_adjoint_strain_pairs(self.ctx, _ptr(P, C.c_double)), "adjoint_strain_pairs")
        return P

    def material_dv_gradient(self, category, component, elem_set, coefs=()) -> float:
        """dL/dD of a single-component material DV ('modulus', 'shearModulus',
        'poissonRatio' or the _lib.DV_* code) over an element set, from the
        last adjoint gradient."""
        cat = {"modulus": _lib.DV_MODULUS, "shearModulus": _lib.DV_SHEAR_MODULUS,
               "poissonRatio": _lib.DV_POISSON_RATIO, "area": _lib.DV_AREA, "areaMoment": _lib.DV_AREA_MOMENT,
               "polarMoment": _lib.DV_POLAR_MOMENT}.get(category, category)
        cf = np.ascontiguousarray(np.atleast_1d(coefs), dtype=np.float64)
        out = C.c_double(0.0)
        self._check(self.lib.asend_material_dv_gradient(self.ctx, cat, component, self.elset_ids[elem_set], len(cf),
                                                        _ptr(cf, C.c_double) if len(cf) else None, C.byref(out)),
                    "material_dv_gradient")
        return out.value

    def design_var_gradient(self, dLdE) -> np.ndarray:
        dLdE = np.ascontiguousarray(dLdE, dtype=np.float64)
        out = np.zeros(max(1, len(self.p.design_vars)))
        n = self._check(self.lib.asend_design_var_gradient(self.ctx, _ptr(dLdE, C.c_double), _ptr(out, C.c_double)),
                        "design_var_gradient")
        return out[:n]

    def newmark(self, amp, probe_dof=-1, **kw):
        o = self.opts(**kw)
        amp = np.ascontiguousarray(amp, dtype=np.float64)
        hist = np.zeros(len(amp))
        u = np.zeros(self.n_dof)
        st = SolveStats()
        rc = self._check(self.lib.asend_newmark_run(self.ctx, C.byref(o), len(amp), _ptr(amp, C.c_double), probe_dof,
                                                    _ptr(hist, C.c_double), _ptr(u, C.c_double), C.byref(st)),
                         "newmark_run")
        return hist, u, rc, st.as_dict()

    def keep_history(self, fields=1):
        """Keep the next Newmark run's per-step states on the device (1: u; 3: u, v, a)."""
        self._check(self.lib.asend_newmark_keep_history(self.ctx, fields), "newmark_keep_history")

    def step_state(self, step, fields=1):
        """(u, v, a) after step `step` (1-based) of the last run (v, a: None unless fields == 3)."""
        n = self.n_dof
        u = np.zeros(n)
        v = np.zeros(n) if fields == 3 else None
        a = np.zeros(n) if fields == 3 else None
        self._check(self.lib.asend_newmark_step_state(self.ctx, step, _ptr(u, C.c_double),
                                                      None if v is None else _ptr(v, C.c_double),
                                                      None if a is None else _ptr(a, C.c_double)), "step_state")
        return u, v, a

    def newmark_adjoint(self, obj_dof, obj_w, **kw):
        """(L, dL/dE, status, stats) of L = sum over the last run's steps of
        sum_k w_k u[dof_k]."""
        o = self.opts(**kw)
        dofs = np.ascontiguousarray(obj_dof, dtype=np.int32)
        w = np.ascontiguousarray(obj_w, dtype=np.float64)
        L = C.c_double(0.0)
        g = np.zeros(self.p.mesh.n_elems)
        st = SolveStats()
        rc = self._check(self.lib.asend_newmark_adjoint(self.ctx, C.byref(o), len(dofs), _ptr(dofs, C.c_int32),
                                                        _ptr(w, C.c_double), C.byref(L), _ptr(g, C.c_double),
                                                        C.byref(st)), "newmark_adjoint")
        return L.value, g, rc, st.as_dict()

    def eigen(self, n_modes, shift=0.0, block_size=2, tol=1e-8, max_subspace=0, modes=True, **inner):
        """Frequency job: the n_modes eigenpairs of (K + penalty) x = lambda D x
        nearest to ``shift`` (lowest first), D the row-sum diagonal mass.
        ``inner`` are the shift-invert solve options (default FP64 Jacobi PCG
        to 1e-10).  Returns (eigenvalues, frequencies [Hz], modes [n, n_dof]
        or None, diagonal mass, rc, stats)."""
        kw = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=1e-10)
        kw.update(inner)
        eo = _lib.EigenOpts(n_modes, block_size, max_subspace, 0, shift, tol, self.opts(**kw))
        ev = np.zeros(n_modes)
        fr = np.zeros(n_modes)
        vecs = np.zeros((n_modes, self.n_dof)) if modes else None
        dm = np.zeros(self.n_dof)
        st = _lib.EigenStats()
        rc = self._check(self.lib.asend_eigen_solve(self.ctx, C.byref(eo), _ptr(ev, C.c_double), _ptr(fr, C.c_double),
                                                    None if vecs is None else _ptr(vecs, C.c_double),
                                                    _ptr(dm, C.c_double), C.byref(st)), "eigen_solve")
        k = st.n_found
        return ev[:k], fr[:k], None if vecs is None else vecs[:k], dm, rc, st.as_dict()

    def csr(self, which=0):
        nnz = C.c_int64(0)
        self._check(self.lib.asend_get_csr(self.ctx, which, C.byref(nnz), None, None, None), "get_csr")
        rp = np.zeros(self.n_dof + 1, dtype=np.int64)
        col = np.zeros(nnz.value, dtype=np.int32)
        val = np.zeros(nnz.value, dtype=np.float64)
        self._check(self.lib.asend_get_csr(self.ctx, which, C.byref(nnz), _ptr(rp, C.c_int64), _ptr(col, C.c_int32),
                                           _ptr(val, C.c_double)), "get_csr")
        return rp, col, val

    def coloring(self):
        col = np.zeros(self.p.mesh.n_elems, dtype=np.int32)
        n = self._check(self.lib.asend_get_coloring(self.ctx, _ptr(col, C.c_int32)), "get_coloring")
        return col, n

    def apply(self, x, precision=64):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self._check(self.lib.asend_apply_operator(self.ctx, precision, _ptr(x, C.c_double), _ptr(y, C.c_double)),
                    "apply_operator")
        return y

    def time_spmv(self, precision=32, n_launch=50):
        ms = C.c_double(0)
        by = C.c_double(0)
        self._check(self.lib.asend_time_spmv(self.ctx, precision, n_launch, C.byref(ms), C.byref(by)), "time_spmv")
        return ms.value, by.value

    def time_mg_kernel(self, kernel, method=_lib.METHOD_SPLIT, n_launch=20):
        """(ms per launch, algorithmic bytes per launch) of a multigrid-CG
        kernel: 0 outer product, 1 level-0 V-cycle residual, 2 post-smoothing."""
        ms = C.c_double(0)
        by = C.c_double(0)
        self._check(self.lib.asend_time_mg_kernel(self.ctx, kernel, method, n_launch, C.byref(ms), C.byref(by)),
                    "time_mg_kernel")
        return ms.value, by.value

    def element_matrices(self, first=0, count=None, mass=True):
        """shell4 / brickIM element stiffness (and mass) matrices [count][24][24]
        ([count][12][12] for beam2)."""
        n = self.p.mesh.n_elems - first if count is None else count
        d = 12 if self.p.mesh.elem_type == 2 else 24
        ke = np.zeros((n, d, d))
        me = np.zeros((n, d, d)) if mass else None
        self._check(self.lib.asend_element_matrices(self.ctx, first, n, _ptr(ke, C.c_double),
                                                    None if me is None else _ptr(me, C.c_double)), "element_matrices")
        return ke, me

    @property
    def stream(self) -> int:
        return int(self.lib.asend_stream(self.ctx) or 0)

    def mg_set_damping(self, factor):
        """Multigrid smoother omega = factor / lambda_max(D^-1 A) (default 1.5)."""
        self._check(self.lib.asend_mg_set_damping(self.ctx, factor), "mg_set_damping")

    def set_product_variant(self, variant):
        """Shape of the multigrid CG's split outer product (_lib.PRODUCT_*):
        register-fed or staged through shared memory; results are identical."""
        self._check(self.lib.asend_set_product_variant(self.ctx, int(variant)), "set_product_variant")

    def mg_set_fused_tail(self, enable=True):
        """Multigrid: the smallest levels as one fused launch (default) or one
        launch per level and step; same arithmetic."""
        self._check(self.lib.asend_mg_set_fused_tail(self.ctx, int(bool(enable))), "mg_set_fused_tail")

    def set_launch_overlap(self, enable=True):
        """Programmatic dependent launch between the multigrid CG's kernels
        (default on); same results either way."""
        self._check(self.lib.asend_set_launch_overlap(self.ctx, int(bool(enable))), "set_launch_overlap")

    @property
    def mg_levels(self) -> int:
        return int(self.lib.asend_mg_levels(self.ctx))

    def mg_level_info(self, level):
        dims = np.zeros(3, dtype=np.int32)
        est, bound, om = C.c_double(0), C.c_double(0), C.c_double(0)
        self._check(self.lib.asend_mg_level_info(self.ctx, level, _ptr(dims, C.c_int32), C.byref(est),
                                                 C.byref(bound), C.byref(om)), "mg_level_info")
        return {"dims": tuple(int(d) for d in dims), "lambda_est": est.value, "lambda_bound": bound.value,
                "omega": om.value}

    def mg_vcycle(self, b) -> np.ndarray:
        b = np.ascontiguousarray(b, dtype=np.float32)
        z = np.zeros_like(b)
        self._check(self.lib.asend_mg_vcycle(self.ctx, _ptr(b, C.c_float), _ptr(z, C.c_float)), "mg_vcycle")
        return z

    # -- learned nodal preconditioner blocks -------------------------------
    @property
    def n_learned_params(self) -> int:
        return int(self.lib.asend_learned_n_params())

    def learned_init(self, seed=0):
        self._check(self.lib.asend_learned_init(self.ctx, seed), "learned_init")

    def learned_params(self) -> np.ndarray:
        w = np.zeros(self.n_learned_params, dtype=np.float32)
        self._check(self.lib.asend_learned_get_params(self.ctx, _ptr(w, C.c_float)), "learned_get_params")
        return w

    def set_learned_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        if w.shape != (self.n_learned_params,):
            raise ValueError(f"expected {self.n_learned_params} parameters")
        self._check(self.lib.asend_learned_set_params(self.ctx, _ptr(w, C.c_float)), "learned_set_params")

    def learned_add_samples(self, iters, append=False, seed=0):
        it = np.ascontiguousarray(np.atleast_1d(iters), dtype=np.int32)
        self._check(self.lib.asend_learned_add_samples(self.ctx, len(it), _ptr(it, C.c_int32), int(append), seed),
                    "learned_add_samples")

    def learned_set_objective(self, kind):
        """kind: _lib.LEARN_BLOCK (blocks for PCG) or _lib.LEARN_MG (multigrid smoother)."""
        self._check(self.lib.asend_learned_set_objective(self.ctx, kind), "learned_set_objective")

    def learned_set_samples(self, samples):
        a = np.ascontiguousarray(np.atleast_2d(samples), dtype=np.float32)
        self._check(self.lib.asend_learned_set_samples(self.ctx, a.shape[0], _ptr(a, C.c_float)),
                    "learned_set_samples")

    def learned_train(self, n_steps=1, lr=1e-3) -> float:
        loss = C.c_double(0)
        rc = self._check(self.lib.asend_learned_train(self.ctx, n_steps, lr, C.byref(loss)), "learned_train")
        if rc != _lib.ASEND_OK:
            raise AsendError(f"learned_train returned status {rc} (loss {loss.value})")
        return loss.value

    def learned_loss_grad(self):
        loss = C.c_double(0)
        g = np.zeros(self.n_learned_params, dtype=np.float32)
        self._check(self.lib.asend_learned_loss_grad(self.ctx, C.byref(loss), _ptr(g, C.c_float)),
                    "learned_loss_grad")
        return loss.value, g

    def learned_features(self, outputs=True):
        n = self.p.mesh.n_nodes
        f = np.zeros((n, 16), dtype=np.float32)
        ch = np.zeros((n, 6), dtype=np.float32)
        y = np.zeros((n, 8), dtype=np.float32) if outputs else None
        self._check(self.lib.asend_learned_features(self.ctx, _ptr(f, C.c_float), _ptr(ch, C.c_float),
                                                    None if y is None else _ptr(y, C.c_float)), "learned_features")
        return f, ch, y

    def learned_blocks(self, use_net=True) -> np.ndarray:
        b = np.zeros((self.p.mesh.n_nodes, 3, 3), dtype=np.float32)
        self._check(self.lib.asend_learned_blocks(self.ctx, int(use_net), _ptr(b, C.c_float)), "learned_blocks")
        return b

    def learned_forward(self, feat) -> np.ndarray:
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        y = np.zeros((feat.shape[0], 8), dtype=np.float32)
        self._check(self.lib.asend_learned_forward(self.ctx, feat.shape[0], _ptr(feat, C.c_float),
                                                   _ptr(y, C.c_float)), "learned_forward")
        return y

    def learned_backward(self, feat, dy) -> np.ndarray:
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        dy = np.ascontiguousarray(dy, dtype=np.float32)
        g = np.zeros(self.n_learned_params, dtype=np.float32)
        self._check(self.lib.asend_learned_backward(self.ctx, feat.shape[0], _ptr(feat, C.c_float),
                                                    _ptr(dy, C.c_float), _ptr(g, C.c_float)), "learned_backward")
        return g

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.asend_kernel_launches(self.ctx))


def combine(problems, align: int = 128):
    """Stack independent problems into one (disconnected) problem for a batched
    solve.  Instance i's nodes start at node_ptr[i], a multiple of ``align``
    (padding nodes carry no element and stay zero); node/element set names get
    the suffix ``@i``; load case k of the result holds every instance's case k.
    Returns (problem, node_ptr, elem_ptr)."""
    node_ptr, elem_ptr = [0], [0]
    for p in problems:
        n = p.mesh.n_nodes
        node_ptr.append(node_ptr[-1] + ((n + align - 1) // align) * align)
        elem_ptr.append(elem_ptr[-1] + p.mesh.n_elems)
    node_ptr[-1] = node_ptr[-2] + problems[-1].mesh.n_nodes  # no padding after the last instance
    n_nodes = node_ptr[-1]
    coords = np.zeros((n_nodes, 3))
    conn = np.zeros((elem_ptr[-1], problems[0].mesh.conn.shape[1]), dtype=np.int32)
    E = np.zeros(elem_ptr[-1])
    nu = np.zeros(elem_ptr[-1])
    rho = np.zeros(elem_ptr[-1])
    out_sets, out_elsets, cons = {}, {}, []
    n_cases = max(len(p.loads) for p in problems)
    loads = [[] for _ in range(n_cases)]
    for i, p in enumerate(problems):
        m, o, eo = p.mesh, node_ptr[i], elem_ptr[i]
        coords[o:o + m.n_nodes] = m.coords
        conn[eo:eo + m.n_elems] = m.conn + o
        E[eo:eo + m.n_elems] = p.E
        nu[eo:eo + m.n_elems] = np.broadcast_to(p.nu, p.E.shape)
        rho[eo:eo + m.n_elems] = 0.0 if p.rho is None else np.broadcast_to(p.rho, p.E.shape)
        for name, s in p.node_sets.items():
            out_sets[f"{name}@{i}"] = np.asarray(s, dtype=np.int32) + o
        for name, s in p.elem_sets.items():
            out_elsets[f"{name}@{i}"] = np.asarray(s, dtype=np.int32) + eo
        for terms, q in p.constraints:
            cons.append(([(f"{t[0]}@{i}", t[1], t[2]) for t in terms], q))
        for k, items in enumerate(p.loads):
            for it in items:
                if it[0] == "nodalForce":
                    loads[k].append(("nodalForce", f"{it[1]}@{i}", it[2]))
                elif it[0] == "surfaceTraction":
                    loads[k].append(("surfaceTraction", f"{it[1]}@{i}", it[2], it[3], it[4]))
                else:
                    f = np.zeros(3 * n_nodes)
                    f[3 * o:3 * o + 3 * m.n_nodes] = it[1]
                    loads[k].append(("vector", f))
    mesh = BlockMesh(0, 0, 0, 0.0, 0.0, 0.0, coords, conn, elem_type=problems[0].mesh.elem_type)
    prob = Problem(mesh, E, nu, rho, out_sets, out_elsets, cons, loads, ("compliance",))
    return prob, np.array(node_ptr, dtype=np.int32), np.array(elem_ptr, dtype=np.int32)
