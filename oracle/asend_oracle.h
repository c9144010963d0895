/*
 * asend_oracle.h -- FP64 CPU oracle for the ASenD3D linear-elastic solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke test and bench.py's CPU-baseline leg may call it; the product
 * (libasend_gpu.so) never links or calls it.
 *
 * It restates, in plain single-threaded C++ and FP64 (as the reference runs),
 * the reference's CPU algorithms for:
 *   - element integration (hex8 type 8, brickIM 81, tet4 4, tet10 10,
 *     shell4 41, beam2 2),
 *   - row-list sparse assembly, penalty constraints,
 *   - the block-LDL^T preconditioned CG and the direct skyline LDL^T,
 *   - the spatial node reordering that defines the preconditioner blocks,
 *   - the static adjoint gradient, and the Newmark time loop.
 * Each function in asend_oracle.cpp cites the reference file:line it follows
 * (paths relative to solverSrc/asend_run_job/src/ of MSDOToolz/ASenD3D).
 *
 * Parity pinning: the reference ships no recorded solver outputs and its Rust
 * toolchain is absent, so the oracle is pinned by the reference's analytic
 * known answers (the notes.txt files under examples/testCases) and by central
 * finite differences and self-consistency (tests/golden holds the fixtures).
 */
#ifndef ASEND_ORACLE_H
#define ASEND_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_model orc_model;

typedef struct orc_stats {
    int32_t iterations;     /* CG iterations (summed over restarts)            */
    int32_t status;         /* 0 converged, 1 max-iter, 2 non-finite           */
    double  final_res;      /* reference stopping quantity g^T M^-1 g at exit  */
    double  rel_residual;   /* ||f - K u||_2 / ||f||_2 with the FP64 operator  */
    double  seconds;        /* wall time of the solve only                     */
} orc_stats;

/* preconditioners */
enum { ORC_PC_NONE = 0, ORC_PC_JACOBI = 1, ORC_PC_BLOCK_LDL = 2, ORC_PC_DIRECT = 3 };
/* stopping rules */
enum { ORC_STOP_REFERENCE = 0, ORC_STOP_RELATIVE = 1 };

/* Mesh of one element type (8 hex8, 81 brickIM, 4 tet4, 10 tet10, 41 shell4,
 * 2 beam2).  coords[n_nodes*3], conn[n_elems*nodes_per_elem] (0-based),
 * per-element isotropic E, nu, rho.  For shell4, thickness[n_elems] gives the
 * section thickness (else NULL); beam2 takes orc_set_beam_sections. */
orc_model* orc_create(int32_t elem_type, int32_t n_nodes, const double* coords,
                      int32_t n_elems, const int32_t* conn, const double* E,
                      const double* nu, const double* rho, const double* thickness);
void orc_destroy(orc_model* m);
int32_t orc_dof_per_node(const orc_model* m);
int32_t orc_n_dof(const orc_model* m);

/* Linear constraint rows C u = q in natural DOF numbering (node*dpn + comp). */
int orc_set_constraints(orc_model* m, int32_t n_rows, const int32_t* row_ptr,
                        const int32_t* dof, const double* coef, const double* rhs);

/* Assemble K (and M when dynamic != 0) in natural numbering, element order.
 * Sets the penalty scale sf = 1e5 * max|K_ij|. */
/* dynamic: 0 static, 1 Newmark operator K + cM M (M kept), 2 modal (K and M kept apart). */
int orc_assemble(orc_model* m, int32_t dynamic, double dt, double beta, double gamma);
/* Per-element 6x6 solid stiffness C[n_el][36] (Voigt 11,22,33,12,13,23,
 * engineering shear) in place of the isotropic one; NULL restores it. */
int orc_set_cmat(orc_model* m, const double* C);
/* Damping for Newmark assemblies: Rayleigh coefficients (mass, stiffness) and
 * per-element material damping matrices D[n_el][36] (may be NULL). */
int orc_set_damping(orc_model* m, double ray_cm, double ray_ck, const double* D);
/* Row-sum lumped mass in Newmark assemblies (the reference's lumpMass). */
int orc_set_lumped_mass(orc_model* m, int32_t on);
/* 6x6 stiffness from engineering constants (E1 E2 E3), (nu12 nu13 nu23),
 * (G12 G13 G23) by inverting the compliance (element_properties.rs:648-764). */
int orc_orthotropic_cmat(const double* e3, const double* nu3, const double* g3, double* C);
int64_t orc_nnz(const orc_model* m);
/* which: 0 = K, 1 = M, 2 = operator (K [+ c_M M] + sf C^T C), 3 = damping D */
int orc_get_csr(const orc_model* m, int32_t which, int64_t* row_ptr, int32_t* col, double* val);
double orc_penalty_scale(const orc_model* m);

/* Single element stiffness (natural element DOF order node*dpn+comp). */
int orc_element_stiffness(int32_t elem_type, const double* xyz, double E, double nu,
                          double thickness, double* ke);
int orc_element_mass(int32_t elem_type, const double* xyz, double rho, double thickness,
                     double* me);

/* Load builders (reference load types). */
int orc_surface_traction(const orc_model* m, int32_t n_set, const int32_t* elem_set,
                         const double* norm_dir, double norm_tol_deg, const double* traction,
                         double* f);
/* surfacePressure: traction -pressure * n on each loaded face. */
int orc_surface_pressure(const orc_model* m, int32_t n_set, const int32_t* elem_set, const double* norm_dir,
                         double norm_tol_deg, double pressure, double* f);
/* bodyForce (kind 0), gravitational (1), centrifugal (2) element loads added to f. */
int orc_body_load(const orc_model* m, int32_t n_set, const int32_t* elem_set, int32_t kind, const double* vec,
                  double omega, const double* center, const double* axis, double* f);

/* Static linear solve: (K + sf C^T C) u = f + sf C^T q, x0 = 0. */
int orc_static_solve(orc_model* m, const double* f, double* u, int32_t precond,
                     int32_t stop_rule, double tol, int32_t max_it, int32_t block_dim,
                     orc_stats* st);
/* All n_rhs load cases f[n_rhs][n_dof] against one preconditioner set-up
 * (one factorization with ORC_PC_DIRECT); u[n_rhs][n_dof]. */
int orc_static_solve_multi(orc_model* m, int32_t n_rhs, const double* f, double* u, int32_t precond,
                           int32_t stop_rule, double tol, int32_t max_it, int32_t block_dim, orc_stats* st);

/* Apply the solve operator (natural numbering): y = A x. */
int orc_apply_operator(const orc_model* m, const double* x, double* y);

/* Static adjoint: lambda = A^-1 dLdu, then per-element isotropic-modulus
 * sensitivity gE[e] = -lambda_e^T (dK_e/dE_e) u_e.  lambda may be supplied
 * (self-adjoint objectives) by passing dLdu == NULL and lambda_in != NULL. */
int orc_adjoint_modulus_gradient(orc_model* m, const double* u, const double* dLdu,
                                 const double* lambda_in, double* lambda_out, double* gE,
                                 int32_t precond, int32_t stop_rule, double tol,
                                 int32_t max_it, orc_stats* st);

/* Reference-style orthotropic "modulus" DV (component 1..3) on every element
 * of the mesh, one DV per element: gD[e] = -lambda_e^T dK_e/dE_k u_e. */
int orc_adjoint_modulus_component_gradient(orc_model* m, const double* u, const double* lambda,
                                           int32_t component, double* gD);

/* Newmark (reference convention) linear transient run.  The load at step i
 * (time = i*dt) is amp[i] * f_shape.  Records u[probe_dof] after each step.
 * Initial u, v, a are zero.  orc_assemble(m, 1, dt, beta, gamma) first. */
int orc_newmark_run(orc_model* m, int32_t n_steps, double dt, double beta, double gamma,
                    const double* f_shape, const double* amp, int32_t probe_dof,
                    double* probe_hist, int32_t precond, int32_t stop_rule, double tol,
                    int32_t max_it, double* u_final, int32_t* total_iters);

/* Reference node reordering (spatial BFS blocks); perm[new] = old node. */
/* Frequency job: eigen pairs of (K + penalty - shift D) x = (lambda - shift) D x
 * with D the row-sum diagonal mass, by the reference's shift-invert Lanczos.
 * Needs orc_assemble(m, 2, ...).  Returns the number of pairs found. */
int orc_eigen_solve(orc_model* m, int32_t n_modes, double shift, double* eig, double* freq, double* modes,
                    double* diag_mass);

/* Transient adjoint of L = sum over the N steps of sum_k w_k u_n[dof_k] with
 * respect to the per-element moduli (direct solves; the reference's reverse
 * sweep).  Needs orc_assemble(m, 1, dt, beta, gamma). */
int orc_newmark_adjoint(orc_model* m, int32_t n_steps, double dt, double beta, double gamma,
                        const double* f_shape, const double* amp, int32_t n_obj, const int32_t* obj_dof,
                        const double* obj_w, double* L_out, double* gE);

/* Strain-pair tensors P[n_el][36] = sum_gp w detJ eps(lambda_e) eps(u_e)^T of
 * solid elements (brickIM with its condensed modes recovered) and of beam2
 * section strains (bubbles recovered). */
int orc_adjoint_strain_pairs(const orc_model* m, const double* u, const double* lam, double* P);

int orc_reorder_nodes(const orc_model* m, int32_t block_dim, int32_t* order_out);

/* Layered shell section: layer k props[7k..] = E1, E2, nu12, G12, density,
 * thickness, angle [deg]; z_offset -1 / 0 / 1 = reference plane on the lower
 * surface / mid-plane / upper surface.  abd[81] (9x9), msec[36] (6x6). */
int orc_shell_section(int32_t n_layers, const double* props, double z_offset, double* abd, double* msec);
/* Per-element sections of a shell4 model (NULL abd: back to E, nu, t). */
int orc_set_shell_sections(orc_model* m, const double* abd, const double* msec);

/* beam2 (type 2) sections, sec[n_el][10] = area, I1..I5 (int z, int y,
 * int z^2, int y^2, int yz over the section), polar moment J, and the
 * direction v (3) that fixes the section's xy plane (the element axis is x).
 * Required before orc_assemble of a beam2 model. */
int orc_set_beam_sections(orc_model* m, const double* sec);
/* One beam2 element: xyz[2][3], ke[12][12] (internal DOF condensed), me
 * [12][12] (may be NULL), global DOF 6 a + c.  -2: zero length or v along
 * the axis. */
int orc_beam_element(const double* xyz, double E, double nu, double rho, const double* sec, double* ke,
                     double* me);
/* As orc_beam_element with given section matrices given[72] (stiffness then
 * mass, each used when its [0] entry is positive; may be NULL). */
int orc_beam_element_given(const double* xyz, double E, double nu, double rho, const double* sec,
                           const double* given, double* ke, double* me);
/* Given beam section matrices of a beam2 model, stiffness[n_el][36] and
 * mass[n_el][36] (either may be NULL; both NULL clears them). */
int orc_set_beam_section_matrices(orc_model* m, const double* stiffness, const double* mass);
/* dC[36] of the beam section stiffness per unit change of a DV (category 0
 * modulus, 1 shearModulus, 2 poissonRatio: component 1-3; 3 area, 4
 * areaMoment component 1-5, 5 polarMoment, with the element's E and nu). */
int orc_beam_section_dC(int32_t category, int32_t component, double E, double nu, const double* sec, double* dC);

/* Element-category objective term at the element centroids (category 0
 * stress, 1 strain, 2 strainEnergy; component 1-6 for 0/1; optr 0 powerNorm,
 * 1 ks, 2 volumeIntegral, 3 volumeAverage).  n_tgt 0, 1 or n_set targets.
 * Outputs L, dLdu[n_dof], Q[n_el][36] (explicit material term: dL/dD =
 * sum (dC/dD) : Q_e) and dLdE[n_el] (explicit isotropic-modulus term);
 * any output may be NULL. */
int orc_element_objective(const orc_model* m, const double* u, int32_t n_set, const int32_t* elem_set,
                          int32_t category, int32_t component, int32_t optr, double coef, double expnt,
                          int32_t n_tgt, const double* tgt, double* L_out, double* dLdu, double* Q,
                          double* dLdE);

#ifdef __cplusplus
}
#endif
#endif
