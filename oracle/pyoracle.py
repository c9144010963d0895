"""ctypes front end of the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, as the checker.  It takes the same ``Problem`` description as the
GPU solver and restates, in Python, the reference's constraint-row building
(const_meth.rs:30-90) and nodal-force load building (model_analysis.rs:37-46);
the numerics live in ``liboracle.so`` (asend_oracle.cpp).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"

PC_NONE, PC_JACOBI, PC_BLOCK_LDL, PC_DIRECT = 0, 1, 2, 3
STOP_REFERENCE, STOP_RELATIVE = 0, 1

P_d = C.POINTER(C.c_double)
P_i = C.POINTER(C.c_int32)
P_l = C.POINTER(C.c_int64)


class Stats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("status", C.c_int32), ("final_res", C.c_double),
                ("rel_residual", C.c_double), ("seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            from oracle import build as _b
            _b.build()
        lib = C.CDLL(str(LIB))
        sig = {
            "orc_create": (C.c_void_p, [C.c_int32, C.c_int32, P_d, C.c_int32, P_i, P_d, P_d, P_d, P_d]),
            "orc_destroy": (None, [C.c_void_p]),
            "orc_n_dof": (C.c_int32, [C.c_void_p]),
            "orc_set_constraints": (C.c_int, [C.c_void_p, C.c_int32, P_i, P_i, P_d, P_d]),
            "orc_assemble": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double]),
            "orc_nnz": (C.c_int64, [C.c_void_p]),
            "orc_get_csr": (C.c_int, [C.c_void_p, C.c_int32, P_l, P_i, P_d]),
            "orc_penalty_scale": (C.c_double, [C.c_void_p]),
            "orc_element_stiffness": (C.c_int, [C.c_int32, P_d, C.c_double, C.c_double, C.c_double, P_d]),
            "orc_element_mass": (C.c_int, [C.c_int32, P_d, C.c_double, C.c_double, P_d]),
            "orc_surface_traction": (C.c_int, [C.c_void_p, C.c_int32, P_i, P_d, C.c_double, P_d, P_d]),
            "orc_static_solve": (C.c_int, [C.c_void_p, P_d, P_d, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                           C.c_int32, C.POINTER(Stats)]),
            "orc_static_solve_multi": (C.c_int, [C.c_void_p, C.c_int32, P_d, P_d, C.c_int32, C.c_int32, C.c_double,
                                                 C.c_int32, C.c_int32, C.POINTER(Stats)]),
            "orc_apply_operator": (C.c_int, [C.c_void_p, P_d, P_d]),
            "orc_set_cmat": (C.c_int, [C.c_void_p, P_d]),
            "orc_surface_pressure": (C.c_int, [C.c_void_p, C.c_int32, P_i, P_d, C.c_double, C.c_double, P_d]),
            "orc_body_load": (C.c_int, [C.c_void_p, C.c_int32, P_i, C.c_int32, P_d, C.c_double, P_d, P_d, P_d]),
            "orc_set_damping": (C.c_int, [C.c_void_p, C.c_double, C.c_double, P_d]),
            "orc_set_lumped_mass": (C.c_int, [C.c_void_p, C.c_int32]),
            "orc_orthotropic_cmat": (C.c_int, [P_d, P_d, P_d, P_d]),
            "orc_adjoint_modulus_gradient": (C.c_int, [C.c_void_p, P_d, P_d, P_d, P_d, P_d, C.c_int32, C.c_int32,
                                                       C.c_double, C.c_int32, C.POINTER(Stats)]),
            "orc_adjoint_modulus_component_gradient": (C.c_int, [C.c_void_p, P_d, P_d, C.c_int32, P_d]),
            "orc_newmark_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double, P_d, P_d,
                                          C.c_int32, P_d, C.c_int32, C.c_int32, C.c_double, C.c_int32, P_d, P_i]),
            "orc_reorder_nodes": (C.c_int, [C.c_void_p, C.c_int32, P_i]),
            "orc_eigen_solve": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, P_d, P_d, P_d, P_d]),
            "orc_adjoint_strain_pairs": (C.c_int, [C.c_void_p, P_d, P_d, P_d]),
            "orc_newmark_adjoint": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double, P_d, P_d,
                                              C.c_int32, P_i, P_d, P_d, P_d]),
            "orc_shell_section": (C.c_int, [C.c_int32, P_d, C.c_double, P_d, P_d]),
            "orc_set_shell_sections": (C.c_int, [C.c_void_p, P_d, P_d]),
            "orc_set_beam_sections": (C.c_int, [C.c_void_p, P_d]),
            "orc_beam_element": (C.c_int, [P_d, C.c_double, C.c_double, C.c_double, P_d, P_d, P_d]),
            "orc_beam_section_dC": (C.c_int, [C.c_int32, C.c_int32, C.c_double, C.c_double, P_d, P_d]),
            "orc_beam_element_given": (C.c_int, [P_d, C.c_double, C.c_double, C.c_double, P_d, P_d, P_d, P_d]),
            "orc_set_beam_section_matrices": (C.c_int, [C.c_void_p, P_d, P_d]),
            "orc_element_objective": (C.c_int, [C.c_void_p, P_d, C.c_int32, P_i, C.c_int32, C.c_int32, C.c_int32,
                                                C.c_double, C.c_double, C.c_int32, P_d, P_d, P_d, P_d, P_d]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def constraint_rows(problem, dpn=3):
    """Constraint::build_mat (const_meth.rs:30-90): rows = largest term-set
    size; a one-node term contributes to every row, an n-node term its k-th
    node to row k."""
    ptr, dof, coef, rhs = [0], [], [], []
    for terms, q in problem.constraints:
        rows = max(len(problem.node_sets[t[0]]) for t in terms)
        for r in range(rows):
            for set_name, comp, cf in terms:
                s = problem.node_sets[set_name]
                nd = s[0] if len(s) == 1 else s[r]
                dof.append(int(nd) * dpn + comp - 1)
                coef.append(cf)
            ptr.append(len(dof))
            rhs.append(q)
    return (np.array(ptr, np.int32), np.array(dof, np.int32), np.array(coef, np.float64), np.array(rhs, np.float64))


class Oracle:
    def __init__(self, problem, dynamic=False, dt=0.0, beta=0.25, gamma=0.5, modal=False):
        self.lib = load()
        self.p = problem
        m = problem.mesh
        self._coords = np.ascontiguousarray(m.coords, np.float64)
        self._conn = np.ascontiguousarray(m.conn, np.int32)
        self._E = np.ascontiguousarray(problem.E, np.float64)
        self._nu = np.ascontiguousarray(np.broadcast_to(problem.nu, self._E.shape), np.float64)
        rho = problem.rho if problem.rho is not None else np.zeros_like(self._E)
        self._rho = np.ascontiguousarray(np.broadcast_to(rho, self._E.shape), np.float64)
        thk = getattr(problem, "thickness", None)
        self._thk = None if thk is None else np.ascontiguousarray(np.broadcast_to(thk, self._E.shape), np.float64)
        self.m = self.lib.orc_create(m.elem_type, m.n_nodes, _p(self._coords), m.n_elems, _p(self._conn, C.c_int32),
                                     _p(self._E), _p(self._nu), _p(self._rho),
                                     None if self._thk is None else _p(self._thk))
        if not self.m:
            raise RuntimeError("orc_create failed")
        self.n_dof = self.lib.orc_n_dof(self.m)
        self.dpn = 6 if m.elem_type in (41, 2) else 3
        ptr, dof, coef, rhs = constraint_rows(problem, self.dpn)
        self._c = (ptr, dof, coef, rhs)
        if len(rhs):
            rc = self.lib.orc_set_constraints(self.m, len(rhs), _p(ptr, C.c_int32), _p(dof, C.c_int32), _p(coef),
                                              _p(rhs))
            assert rc == 0
        ortho = getattr(problem, "ortho", None)
        if ortho is not None:
            self._cmat = np.stack([self.orthotropic_cmat(row) for row in np.asarray(ortho, np.float64).reshape(-1, 9)])
            assert self.lib.orc_set_cmat(self.m, _p(np.ascontiguousarray(self._cmat))) == 0
        damping = getattr(problem, "damping", None)
        if damping is not None:
            cm, ck, dm = damping
            self._dmat = None if dm is None else np.ascontiguousarray(dm, np.float64).reshape(-1, 36)
            self.lib.orc_set_damping(self.m, float(cm), float(ck), None if self._dmat is None else _p(self._dmat))
        if getattr(problem, "lump_mass", False):
            self.lib.orc_set_lumped_mass(self.m, 1)
        bsec = getattr(problem, "beam_sections", None)
        if bsec is not None:
            self._bsec = np.ascontiguousarray(np.broadcast_to(np.asarray(bsec, np.float64), (m.n_elems, 10)))
            assert self.lib.orc_set_beam_sections(self.m, _p(self._bsec)) == 0
            given = getattr(problem, "beam_section_matrices", None)
            if given is not None:
                self._bcm = [None if x is None else np.ascontiguousarray(
                    np.broadcast_to(np.asarray(x, np.float64), (m.n_elems, 36))) for x in given]
                assert self.lib.orc_set_beam_section_matrices(
                    self.m, None if self._bcm[0] is None else _p(self._bcm[0]),
                    None if self._bcm[1] is None else _p(self._bcm[1])) == 0
        secs = getattr(problem, "shell_sections", None)
        if secs:
            # layered sections: (element indices, layer table [n, 7], z offset);
            # other elements keep their single isotropic layer
            ne = m.n_elems
            abd, ms = np.zeros((ne, 81)), np.zeros((ne, 36))
            for e in range(ne):
                G = self._E[e] / (2.0 * (1.0 + self._nu[e]))
                row = [self._E[e], self._E[e], self._nu[e], G, self._rho[e], self._thk[e], 0.0]
                abd[e], ms[e] = self.shell_section([row], 0.0)
            for els, props, zoff in secs:
                a, mm = self.shell_section(props, zoff)
                abd[np.asarray(els)] = a
                ms[np.asarray(els)] = mm
            self._abd, self._msec = np.ascontiguousarray(abd), np.ascontiguousarray(ms)
            assert self.lib.orc_set_shell_sections(self.m, _p(self._abd), _p(self._msec)) == 0
        rc = self.lib.orc_assemble(self.m, 2 if modal else int(dynamic), dt, beta, gamma)
        if rc != 0:
            raise RuntimeError(f"orc_assemble failed ({rc})")
        self.sf = self.lib.orc_penalty_scale(self.m)

    def __del__(self):
        try:
            if self.m:
                self.lib.orc_destroy(self.m)
        except Exception:
            pass

    def loads(self):
        """Load cases in natural numbering (without the penalty rhs)."""
        out = []
        for items in self.p.loads:
            f = np.zeros(self.n_dof)
            for it in items:
                if it[0] == "nodalForce":
                    d = self.dpn
                    for nd in self.p.node_sets[it[1]]:
                        f[d * nd:d * nd + d] += it[2][:d]
                elif it[0] == "surfaceTraction":
                    els = np.ascontiguousarray(self.p.elem_sets[it[1]], np.int32)
                    nd = np.ascontiguousarray(it[2], np.float64)
                    t = np.ascontiguousarray(it[4], np.float64)
                    self.lib.orc_surface_traction(self.m, len(els), _p(els, C.c_int32), _p(nd), it[3], _p(t), _p(f))
                elif it[0] == "surfacePressure":
                    els = np.ascontiguousarray(self.p.elem_sets[it[1]], np.int32)
                    nd = np.ascontiguousarray(it[2], np.float64)
                    self.lib.orc_surface_pressure(self.m, len(els), _p(els, C.c_int32), _p(nd), it[3], float(it[4]),
                                                  _p(f))
                elif it[0] in ("bodyForce", "gravitational", "centrifugal"):
                    els = np.ascontiguousarray(self.p.elem_sets[it[1]], np.int32)
                    kind = ("bodyForce", "gravitational", "centrifugal").index(it[0])
                    if kind == 2:
                        cen = np.ascontiguousarray(it[3], np.float64)
                        ax = np.ascontiguousarray(it[4], np.float64)
                        self.lib.orc_body_load(self.m, len(els), _p(els, C.c_int32), 2, None, float(it[2]), _p(cen),
                                               _p(ax), _p(f))
                    else:
                        v = np.ascontiguousarray(it[2], np.float64)
                        self.lib.orc_body_load(self.m, len(els), _p(els, C.c_int32), kind, _p(v), 0.0, None, None,
                                               _p(f))
                else:
                    f += it[1]
            out.append(f)
        return out

    def penalty_rhs(self):
        ptr, dof, coef, rhs = self._c
        b = np.zeros(self.n_dof)
        for r in range(len(rhs)):
            for k in range(ptr[r], ptr[r + 1]):
                b[dof[k]] += coef[k] * self.sf * rhs[r]
        return b

    def csr(self, which=0):
        nnz = self.lib.orc_nnz(self.m)
        rp = np.zeros(self.n_dof + 1, np.int64)
        col = np.zeros(nnz, np.int32)
        val = np.zeros(nnz)
        rc = self.lib.orc_get_csr(self.m, which, _p(rp, C.c_int64), _p(col, C.c_int32), _p(val))
        assert rc == 0, rc
        return rp, col, val

    def apply(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self.lib.orc_apply_operator(self.m, _p(x), _p(y))
        return y

    def solve(self, f, precond=PC_JACOBI, stop=STOP_RELATIVE, tol=1e-8, max_it=0, block_dim=0):
        f = np.ascontiguousarray(f, np.float64)
        u = np.zeros(self.n_dof)
        st = Stats()
        rc = self.lib.orc_static_solve(self.m, _p(f), _p(u), precond, stop, tol, max_it, block_dim, C.byref(st))
        return u, rc, st.as_dict()

    def orthotropic_cmat(self, props):
        """6x6 C of the constants E1 E2 E3 nu12 nu13 nu23 G12 G13 G23."""
        p = np.ascontiguousarray(props, np.float64)
        Cm = np.zeros(36)
        self.lib.orc_orthotropic_cmat(_p(p[0:3].copy()), _p(p[3:6].copy()), _p(p[6:9].copy()), _p(Cm))
        return Cm

    def solve_cases(self, F, precond=PC_DIRECT, stop=STOP_RELATIVE, tol=1e-12, max_it=0, block_dim=0):
        """Every row of F[n_rhs][n_dof] against one preconditioner set-up."""
        F = np.ascontiguousarray(F, np.float64)
        U = np.zeros_like(F)
        st = Stats()
        rc = self.lib.orc_static_solve_multi(self.m, F.shape[0], _p(F), _p(U), precond, stop, tol, max_it,
                                             block_dim, C.byref(st))
        return U, rc, st.as_dict()

    def adjoint(self, u, dLdu=None, lam=None, precond=PC_JACOBI, stop=STOP_RELATIVE, tol=1e-10, max_it=0):
        u = np.ascontiguousarray(u, np.float64)
        g = np.zeros(self.p.mesh.n_elems)
        lam_out = np.zeros(self.n_dof)
        st = Stats()
        d = None if dLdu is None else np.ascontiguousarray(dLdu, np.float64)
        li = None if lam is None else np.ascontiguousarray(lam, np.float64)
        rc = self.lib.orc_adjoint_modulus_gradient(self.m, _p(u), None if d is None else _p(d),
                                                   None if li is None else _p(li), _p(lam_out), _p(g), precond, stop,
                                                   tol, max_it, C.byref(st))
        return g, lam_out, rc, st.as_dict()

    def component_gradient(self, u, lam, component):
        g = np.zeros(self.p.mesh.n_elems)
        u = np.ascontiguousarray(u, np.float64)
        lam = np.ascontiguousarray(lam, np.float64)
        rc = self.lib.orc_adjoint_modulus_component_gradient(self.m, _p(u), _p(lam), component, _p(g))
        assert rc == 0
        return g

    def newmark(self, n_steps, dt, beta, gamma, f_shape, amp, probe_dof, precond=PC_JACOBI, stop=STOP_RELATIVE,
                tol=1e-10, max_it=0):
        f_shape = np.ascontiguousarray(f_shape, np.float64)
        amp = np.ascontiguousarray(amp, np.float64)
        hist = np.zeros(n_steps)
        u = np.zeros(self.n_dof)
        its = C.c_int32(0)
        rc = self.lib.orc_newmark_run(self.m, n_steps, dt, beta, gamma, _p(f_shape), _p(amp), probe_dof, _p(hist),
                                      precond, stop, tol, max_it, _p(u), C.byref(its))
        return hist, u, rc, its.value

    def eigen(self, n_modes, shift=0.0):
        """Frequency job (construct with modal=True): eigenvalues, frequencies
        [Hz], unit-norm mode shapes [n_found, n_dof] and the diagonal mass."""
        ev = np.zeros(n_modes)
        fr = np.zeros(n_modes)
        vecs = np.zeros((n_modes, self.n_dof))
        dm = np.zeros(self.n_dof)
        k = self.lib.orc_eigen_solve(self.m, n_modes, shift, _p(ev), _p(fr), _p(vecs), _p(dm))
        if k < 0:
            raise RuntimeError(f"orc_eigen_solve failed ({k})")
        return ev[:k], fr[:k], vecs[:k], dm

    def strain_pairs(self, u, lam):
        """[n_el, 6, 6] strain-pair tensors of (u, lambda) (solid elements)."""
        u = np.ascontiguousarray(u, np.float64)
        lam = np.ascontiguousarray(lam, np.float64)
        P = np.zeros((self.p.mesh.n_elems, 6, 6))
        rc = self.lib.orc_adjoint_strain_pairs(self.m, _p(u), _p(lam), _p(P))
        if rc != 0:
            raise RuntimeError(f"orc_adjoint_strain_pairs failed ({rc})")
        return P

    def shell_section(self, props, z_offset):
        """Layered shell section: (ABD [81], section mass [36]) of layers
        props [n, 7] = E1, E2, nu12, G12, density, thickness, angle [deg]."""
        pr = np.ascontiguousarray(props, np.float64).reshape(-1, 7)
        abd, ms = np.zeros(81), np.zeros(36)
        assert self.lib.orc_shell_section(len(pr), _p(pr), float(z_offset), _p(abd), _p(ms)) == 0
        return abd, ms

    ELEM_CATEGORIES = {"stress": 0, "strain": 1, "strainEnergy": 2}
    ELEM_OPERATORS = {"powerNorm": 0, "ks": 1, "volumeIntegral": 2, "volumeAverage": 3}

    def element_objective(self, u, elems, category, component=0, operator="powerNorm", coef=1.0, exponent=1.0,
                          targets=()):
        """Element-category objective term at the centroids: returns L,
        dL/du [n_dof], the explicit material pairs Q [n_el, 6, 6] and the
        explicit isotropic-modulus term dL/dE [n_el]."""
        u = np.ascontiguousarray(u, np.float64)
        el = np.ascontiguousarray(elems, np.int32)
        tg = np.ascontiguousarray(targets if len(targets) else [0.0], np.float64)
        L = C.c_double(0.0)
        dLdu = np.zeros(self.n_dof)
        Q = np.zeros((self.p.mesh.n_elems, 6, 6))
        dLdE = np.zeros(self.p.mesh.n_elems)
        rc = self.lib.orc_element_objective(self.m, _p(u), len(el), _p(el, C.c_int32), self.ELEM_CATEGORIES[category],
                                            component, self.ELEM_OPERATORS[operator], coef, exponent, len(targets),
                                            _p(tg), C.byref(L), _p(dLdu), _p(Q), _p(dLdE))
        if rc != 0:
            raise RuntimeError(f"orc_element_objective failed ({rc})")
        return L.value, dLdu, Q, dLdE

    def newmark_adjoint(self, n_steps, dt, beta, gamma, f_shape, amp, obj_dof, obj_w):
        """Transient adjoint (construct with dynamic=True): L = sum over steps of
        sum_k w_k u_n[dof_k] and dL/dE per element."""
        f_shape = np.ascontiguousarray(f_shape, np.float64)
        amp = np.ascontiguousarray(amp, np.float64)
        dof = np.ascontiguousarray(obj_dof, np.int32)
        w = np.ascontiguousarray(obj_w, np.float64)
        L = C.c_double(0.0)
        g = np.zeros(self.p.mesh.n_elems)
        rc = self.lib.orc_newmark_adjoint(self.m, n_steps, dt, beta, gamma, _p(f_shape), _p(amp), len(dof),
                                          _p(dof, C.c_int32), _p(w), C.byref(L), _p(g))
        if rc != 0:
            raise RuntimeError(f"orc_newmark_adjoint failed ({rc})")
        return L.value, g

    def reorder(self, block_dim=0):
        out = np.zeros(self.n_dof // 3, np.int32)
        self.lib.orc_reorder_nodes(self.m, block_dim, _p(out, C.c_int32))
        return out


def element_stiffness(elem_type, xyz, E, nu):
    lib = load()
    xyz = np.ascontiguousarray(xyz, np.float64).ravel()
    n = xyz.size
    ke = np.zeros(n * n)
    rc = lib.orc_element_stiffness(elem_type, _p(xyz), E, nu, 0.0, _p(ke))
    assert rc == 0
    return ke.reshape(n, n)


def beam_element(xyz, E, nu, rho, sec, given=None):
    """beam2 element stiffness and mass [12][12] (global DOF 6 a + c);
    ``given`` [72]: section stiffness then mass matrices (each used when its
    [0] entry is positive)."""
    lib = load()
    xyz = np.ascontiguousarray(xyz, np.float64).ravel()
    sec = np.ascontiguousarray(sec, np.float64)
    ke, me = np.zeros(144), np.zeros(144)
    if given is None:
        rc = lib.orc_beam_element(_p(xyz), float(E), float(nu), float(rho), _p(sec), _p(ke), _p(me))
    else:
        gv = np.ascontiguousarray(given, np.float64)
        rc = lib.orc_beam_element_given(_p(xyz), float(E), float(nu), float(rho), _p(sec), _p(gv), _p(ke), _p(me))
    if rc != 0:
        raise ValueError(f"orc_beam_element failed ({rc})")
    return ke.reshape(12, 12), me.reshape(12, 12)


def beam_section_dC(category, component, sec, E=1.0, nu=0.0):
    """dC[6][6] of the beam section stiffness per unit change of a DV
    (0 modulus, 1 shearModulus, 2 poissonRatio, 3 area, 4 areaMoment,
    5 polarMoment; the last three at the element's E and nu)."""
    lib = load()
    sec = np.ascontiguousarray(sec, np.float64)
    dC = np.zeros(36)
    assert lib.orc_beam_section_dC(int(category), int(component), float(E), float(nu), _p(sec), _p(dC)) == 0
    return dC.reshape(6, 6)
