/*
 * asend_gpu.h -- C ABI of the GB300 (sm_103a) linear-elastic solve library.
 *
 * Drop-in boundary for ASenD3D's static / Newmark / adjoint solve path.  The
 * reference drives this path in-process through Rust methods on `Model`
 * (paths relative to solverSrc/asend_run_job/src/):
 *   Model::read_model_input / read_constraint_input / read_load_input /
 *       read_des_var_input / read_objective_input   model_input.rs:312-1375
 *   Model::analysis_prep                           model_prep.rs:881-952
 *   Model::solve                                   model_analysis.rs:560-673
 *   Model::solve_step (elastic branch)             model_analysis.rs:450-534
 *   conj_grad_sparse                               matrix_functions.rs:285-362
 *   Model::solve_for_adjoint                       model_analysis.rs:1065-1231
 *   Model::get_obj_gradient                        model_analysis.rs:1544-1706
 * Each entry point below names the reference interface it replaces.
 *
 * Conventions
 *   - Plain pointers and sizes; no C++ or torch types cross the boundary.
 *   - Host buffers are caller-owned; device memory is library-owned.
 *   - Return codes: 0 ok, 1 iteration cap reached, 2 non-finite values,
 *     3 preconditioner fallback used, negative = input / CUDA error
 *     (asend_last_error() gives the message).  Nothing aborts the process.
 *   - One context per host thread; a context owns one CUDA stream.
 *   - DOF numbering is natural: dof = node * dof_per_node + component
 *     (component 0-based).  Element types use the reference codes:
 *     8 = hex8 (brick8), 81 = brickIM (hex8 + 9 condensed incompatible
 *     modes, the reference's default hex), 4 = tet4, 41 = shell4 (quad shell).
 */
#ifndef ASEND_GPU_H
#define ASEND_GPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct asend_ctx asend_ctx;

/* status codes */
#define ASEND_OK 0
#define ASEND_MAX_ITER 1
#define ASEND_NONFINITE 2
#define ASEND_FALLBACK 3
#define ASEND_EINVAL (-1)
#define ASEND_ECUDA (-2)
#define ASEND_ESTATE (-3)

/* solver methods */
#define ASEND_METHOD_FP64 0   /* plain FP64 PCG (values, SpMV, vectors all FP64)           */
#define ASEND_METHOD_MIXED 1  /* FP32 SpMV + FP64 vectors/dots + FP64 residual replacement */
#define ASEND_METHOD_SPLIT 2  /* FP64-accurate SpMV on the FP32 pipes: each FP64 value and
                                 direction entry held as an FP32 hi + lo pair (same bytes as
                                 FP64), products in compensated FP32 arithmetic; FP64
                                 vectors, dots and residuals                               */

/* preconditioners */
#define ASEND_PC_JACOBI 0     /* point Jacobi                                             */
#define ASEND_PC_BLOCK 1      /* nodal block Jacobi (dof_per_node x dof_per_node blocks)  */
#define ASEND_PC_LEARNED 2    /* MLP-predicted nodal blocks, Jacobi fallback              */
#define ASEND_PC_MG 3         /* geometric multigrid V-cycle (structured hex8 blocks)     */
#define ASEND_PC_MG_LEARNED 4 /* multigrid with learned finest-level smoother blocks      */

/* training objectives of the learned blocks */
#define ASEND_LEARN_BLOCK 0   /* mean ||r - A M r||^2: blocks used directly by PCG        */
#define ASEND_LEARN_MG 1      /* mean ||b - A V(b)||^2, V = V-cycle with the blocks as the
                                 finest-level smoother (needs the block structure)       */

/* objective kinds (reference objective categories, objective_meth.rs:592-942) */
#define ASEND_OBJ_DISPLACEMENT 0 /* 'displacement' + 'powerNorm' on a node set            */
#define ASEND_OBJ_COMPLIANCE 1   /* f^T u summed over load cases (self-adjoint)           */
#define ASEND_OBJ_ELEMENT 2      /* element-category term ('stress', 'strain',
                                    'strainEnergy' at the centroid) given as
                                    per-element weights (asend_set_element_objective) */

typedef struct asend_solve_opts {
    int32_t method;       /* ASEND_METHOD_*                                          */
    int32_t precond;      /* ASEND_PC_*                                              */
    double rel_tol;       /* target ||f - A u||_2 / ||f||_2 with the FP64 operator   */
    int32_t max_iter;     /* iteration cap (0 = n_dof, as model_prep.rs:236-244)      */
    int32_t graph_iters;  /* PCG iterations per captured CUDA graph (0 = 16)         */
    int32_t warm_start;   /* 1: use u_io on entry as the initial guess               */
    int32_t replace_every;/* mixed: force a true-residual replacement after this many
                             iterations without one (0 = only on residual drops)     */
} asend_solve_opts;

typedef struct asend_solve_stats {
    int32_t iterations;     /* PCG iterations (max over right-hand sides)           */
    int32_t status;         /* ASEND_OK / ASEND_MAX_ITER / ...                      */
    int32_t replacements;   /* FP64 true-residual replacements (mixed method)       */
    int32_t n_rhs;
    double rel_residual;    /* final ||f - A u|| / ||f|| (FP64 operator), max over RHS */
    double ms_assemble;     /* device time of the last assembly                     */
    double ms_solve;        /* device time of the solve (event-timed on the stream) */
    double ms_adjoint;      /* device time of the adjoint contraction               */
    double penalty_scale;   /* sf = 1e5 * max|K_ij| (model_analysis.rs:255-259)     */
} asend_solve_stats;

/* ---- context -------------------------------------------------------------- */
asend_ctx* asend_create(int32_t device);
void asend_destroy(asend_ctx* ctx);
const char* asend_last_error(const asend_ctx* ctx);
/* Version / build string (sm arch, compile flags). */
const char* asend_version(void);

/* ---- model input (replaces model_input.rs:312-860 read_model_input) --------
 * One element type per mesh.  coords[n_nodes*3]; conn[n_elems*nodes_per_elem];
 * per-element isotropic material E, nu, rho (rho may be NULL for statics);
 * thickness per element for shells (else NULL).  shell4 (41): 4 nodes per
 * element, 6 DOF per node (u v w thx thy thz), one isotropic layer centred
 * on the element plane; elements must be flat in a plane z = const (their
 * frame is then the global one).  beam2 (2): 2 nodes per element, 6 DOF per
 * node, sections from asend_set_beam_sections (thickness may be NULL).
 * Shell and beam meshes take nodal forces/moments, constraints and objectives
 * on all 6 components; surface tractions, multigrid and batched instances
 * take solid meshes. */
int asend_set_mesh(asend_ctx* ctx, int32_t elem_type, int32_t n_nodes, const double* coords,
                   int32_t n_elems, const int32_t* conn, const double* E, const double* nu,
                   const double* rho, const double* thickness);
/* Replace the per-element moduli (a new design / UQ sample) without
 * rebuilding the pattern.  Replaces the DV-perturbed property path of
 * element_properties.rs:648-764 for the isotropic-modulus case. */
int asend_set_modulus(asend_ctx* ctx, const double* E);

/* Declare the hex8 mesh a structured nx*ny*nz block in the numbering of the
 * reference's swept meshing (node (i,j,k) = (i*(ny+1)+j)*(nz+1)+k, element
 * (i,j,k) = (i*ny+j)*nz+k, hex8 corner order).  Enables ASEND_PC_MG, which
 * replaces the reference's block-LDL^T preconditioner
 * (lower_tri_mat_meth.rs:15-241).  Validated against the connectivity. */
int asend_set_block_structure(asend_ctx* ctx, int32_t nx, int32_t ny, int32_t nz);
/* Number of multigrid levels built so far (0 before the first MG solve). */
int asend_mg_levels(const asend_ctx* ctx);
/* Smoother damping of the multigrid levels: omega = factor / lambda, lambda a
 * power-iteration estimate of the largest eigenvalue of D^-1 A on each level
 * (D = nodal diagonal blocks).  Default 1.5; factor in (0, 2). */
int asend_mg_set_damping(asend_ctx* ctx, double factor);
/* Shape of the multigrid CG's outer split product (ASEND_METHOD_SPLIT), a
 * kernel variant picked at run time (e.g. by an autotuner): the values and
 * column indices are fed through registers, or staged through shared memory
 * by bulk copies with G block-column groups per stage and S stages per warp.
 * Every shape gives bit-identical results.  No counterpart in the reference
 * (it has no GPU kernels): it tunes the kernel that replaces the products of
 * SparseMat::vector_multiply (list_ent_meth.rs:64-79) inside
 * conj_grad_sparse (matrix_functions.rs:285-362). */
#define ASEND_PRODUCT_DEFAULT 0
#define ASEND_PRODUCT_REGISTERS 1
#define ASEND_PRODUCT_STAGED_2x3 2
#define ASEND_PRODUCT_STAGED_3x2 3
#define ASEND_PRODUCT_STAGED_2x2 4
#define ASEND_PRODUCT_STAGED_4x2 5
int asend_set_product_variant(asend_ctx* ctx, int32_t variant);
/* Multigrid V-cycle: run the deepest levels whose every block has at most
 * 512 nodes (one block per instance), the coarsest dense solve included, as
 * one fused launch with one CTA per block (enable = 1, the default), or as
 * one launch per level and step (enable = 0).  Same arithmetic either way.
 * No counterpart in the reference (it has no multigrid); a tuning and
 * diagnostic switch of the preconditioner that replaces the reference's
 * block-LDL^T (lower_tri_mat_meth.rs:15-241). */
int asend_mg_set_fused_tail(asend_ctx* ctx, int32_t enable);
/* Multigrid CG: launch each V-cycle and CG kernel with programmatic
 * dependent launch (enable = 1), so that its launch and CTA set-up overlap
 * the end of the kernel before it; every such kernel waits for its
 * predecessor before reading or writing anything, so results do not change.
 * enable = 0 (the default) serialises the launches: on GB300 the overlapped
 * solve measured slower.  No counterpart in the reference (no GPU code). */
int asend_set_launch_overlap(asend_ctx* ctx, int32_t enable);
/* Level diagnostics after a multigrid solve: dims[3] = (nx, ny, nz) of the
 * level's cells, the power-iteration estimate and the guaranteed bound
 * ||D^-1 A||_inf of lambda_max(D^-1 A), and the smoother damping in use (the
 * coarsest level, solved directly, reports zeros).  Any pointer may be NULL.
 * The damping switches to factor / bound on every level after a multigrid
 * solve turned non-finite (the solve is then repeated from zero). */
int asend_mg_level_info(asend_ctx* ctx, int32_t level, int32_t* dims, double* lambda_est,
                        double* lambda_bound, double* omega);
/* z = V(b): one V-cycle with the current smoothers (FP32 host vectors of
 * n_dof entries); builds the hierarchy if needed. */
int asend_mg_vcycle(asend_ctx* ctx, const float* b, float* z);

/* Batched solves (no counterpart in the single-model reference; it replaces
 * running the reference's Model::solve once per UQ / design sample): the
 * mesh is a stack of n_inst independent sub-systems, instance i owning nodes
 * [node_ptr[i], node_ptr[i+1]).  Each instance must start at a multiple of
 * 128 nodes (pad with unused nodes, which get a unit diagonal and stay 0)
 * and no element or constraint may span two instances.  Every PCG kernel
 * then runs over all instances at once while step lengths, convergence and
 * stopping are kept per instance and load case. */
int asend_set_instances(asend_ctx* ctx, int32_t n_inst, const int32_t* node_ptr);
/* Declares each instance of the stack (after asend_set_instances) a
 * structured hex8 / brickIM block dims[3i..3i+2] = (nx, ny, nz) in the
 * numbering of asend_set_block_structure relative to the instance's first
 * node; instance i's elements are the next nx*ny*nz elements.  Enables
 * ASEND_PC_MG on the stack: every instance gets its own multigrid hierarchy
 * and one V-cycle serves all of them, in place of the reference's per-model
 * block-LDL^T preconditioner (lower_tri_mat_meth.rs:15-241).  Validated
 * against the connectivity. */
int asend_set_instance_blocks(asend_ctx* ctx, int32_t n_inst, const int32_t* dims);

/* Node / element sets (model_input.rs:720-860 'sets' blocks).  Returns the
 * set id (>= 0) or a negative error code. */
int asend_add_node_set(asend_ctx* ctx, int32_t n, const int32_t* nodes);
int asend_add_element_set(asend_ctx* ctx, int32_t n, const int32_t* elems);

/* 'displacement' constraint (read_constraint_input model_input.rs:872-969;
 * matrix rows per const_meth.rs:30-90): sum_t coef_t * u[node_t, comp_t] = rhs
 * for every row, where a term over an n-node set contributes its k-th node to
 * row k and a term over a 1-node set contributes to every row.  comp is the
 * reference's 1-based DOF component. */
int asend_add_constraint(asend_ctx* ctx, int32_t n_terms, const int32_t* node_set,
                         const int32_t* comp, const double* coef, double rhs);

/* ---- loads (read_load_input model_input.rs:981-1123;
 *      build_elastic_app_load model_analysis.rs:21-75) ----------------------
 * Loads accumulate into load case `rhs` (0-based; cases are created on use). */
int asend_add_nodal_force(asend_ctx* ctx, int32_t rhs, int32_t node_set, const double* load6);
int asend_add_surface_traction(asend_ctx* ctx, int32_t rhs, int32_t elem_set,
                               const double* norm_dir, double norm_tol_deg,
                               const double* traction);
/* Surface pressure: each loaded face (selected like asend_add_surface_traction)
 * carries the traction -pressure * n, n its outward unit normal
 * (get_app_load_dfd0 'surfacePressure', element_equations.rs:1970-1996). */
int asend_add_surface_pressure(asend_ctx* ctx, int32_t rhs, int32_t elem_set, const double* norm_dir,
                               double norm_tol_deg, double pressure);
/* Element loads of a uniform acceleration field (get_app_load_dfd0,
 * element_equations.rs:1875-1968; the reference's 'bodyForce',
 * 'gravitational' and 'centrifugal' load types): for each element of the set,
 * M_e acc on its translational DOF, with
 *   ASEND_LOAD_BODY_FORCE: acc = vec (force per unit volume, unit density);
 *   ASEND_LOAD_GRAVITY:    acc = vec, the element's density;
 *   ASEND_LOAD_CENTRIFUGAL: acc = omega^2 (r - (r . a) a), r = element
 *     centroid - center, a = axis normalised; the element's density.
 * vec is unused by centrifugal loads; omega, center, axis only by them. */
#define ASEND_LOAD_BODY_FORCE 0
#define ASEND_LOAD_GRAVITY 1
#define ASEND_LOAD_CENTRIFUGAL 2
int asend_add_body_load(asend_ctx* ctx, int32_t rhs, int32_t elem_set, int32_t kind, const double* vec,
                        double omega, const double* center, const double* axis);
/* Raw load vector in natural DOF numbering (adds to load case `rhs`). */
int asend_add_load_vector(asend_ctx* ctx, int32_t rhs, const double* f);
int asend_clear_loads(asend_ctx* ctx);
int asend_n_dof(const asend_ctx* ctx);
int asend_n_load_cases(const asend_ctx* ctx);
/* Copy load case `rhs` (with the penalty right-hand side folded in once the
 * operator is assembled) to the host. */
int asend_get_load_vector(asend_ctx* ctx, int32_t rhs, double* f_out);

/* ---- assembly (analysis_prep + prep_matrix_factorizations,
 *      model_prep.rs:556-618, 881-952; element loop model_analysis.rs:179-201;
 *      element kernels element_equations.rs:206-418 / 852-1062) ------------
 * precision: 64 = FP64 element integration (FP32 copy made by rounding),
 *            32 = FP32 element integration (FP64 copy made by widening),
 *            48 = FP64-accurate values as FP32 hi + lo pairs only, summed in
 *                 FP32-pair arithmetic (static hex8 / brickIM meshes on the
 *                 geometry-class gather; otherwise as 64): the operator for
 *                 ASEND_METHOD_SPLIT solves.  The FP64 copy is rebuilt from
 *                 the pairs by the first call that needs it.
 * dynamic = 1 assembles K + c_M M with c_M = -1/(dt^2 (beta - gamma)) and
 * keeps M (Newmark, element_equations.rs:977-988); dynamic = 2 assembles K
 * and keeps M apart (modal analysis; dt, beta, gamma unused). */
int asend_assemble(asend_ctx* ctx, int32_t precision, int32_t dynamic, double dt, double beta,
                   double gamma);
/* Assembled matrices as scalar CSR in natural DOF numbering with sorted
 * columns: which 0 = operator (K [+ c_M M] [+ c_D D] + sf C^T C), 1 = mass,
 * 2 = operator without the penalty terms, 3 = damping.  Pass NULL to query
 * sizes: *nnz_out. */
int asend_get_csr(asend_ctx* ctx, int32_t which, int64_t* nnz_out, int64_t* row_ptr,
                  int32_t* col, double* val);
/* Element colouring used by the scatter assembly (no two elements of one
 * colour share a node).  colour[n_elems]; returns the number of colours. */
int asend_get_coloring(asend_ctx* ctx, int32_t* colour_out);

/* ---- static solve (Model::solve / solve_step, model_analysis.rs:450-673;
 *      conj_grad_sparse matrix_functions.rs:285-362) -----------------------
 * Solves A u_r = f_r + sf C^T q for every load case r.  u_io[n_rhs*n_dof]
 * (natural numbering, case-major); used as the initial guess when
 * opts->warm_start, overwritten with the solution. */
int asend_static_solve(asend_ctx* ctx, const asend_solve_opts* opts, double* u_io,
                       asend_solve_stats* stats);
/* Device-resident variant: the solution stays on the device (for chained
 * solve -> adjoint calls without host copies). */
int asend_static_solve_device(asend_ctx* ctx, const asend_solve_opts* opts,
                              asend_solve_stats* stats);
int asend_get_solution(asend_ctx* ctx, int32_t rhs, double* u_out);

/* ---- objective + adjoint gradient (read_objective_input
 *      model_input.rs:1298-1375; Model::get_obj_gradient static branch
 *      model_analysis.rs:1632-1704; solve_for_adjoint :1065-1126;
 *      d_relasticd_d :1379-1457) --------------------------------------------
 * kind ASEND_OBJ_DISPLACEMENT: L = coef * sum_{n in set} u[n, comp]
 *   ('powerNorm' with exponent 1, objective_meth.rs:329-337), comp 1-based.
 * kind ASEND_OBJ_COMPLIANCE: L = sum_r f_r^T u_r.
 * Gradient w.r.t. the per-element isotropic modulus: dLdE[n_elems].
 * The solution of the preceding asend_static_solve* call is used. */
int asend_set_objective(asend_ctx* ctx, int32_t kind, int32_t node_set, int32_t comp,
                        double coef);
int asend_adjoint_gradient(asend_ctx* ctx, const asend_solve_opts* opts, double* L_out,
                           double* dLdE_out, asend_solve_stats* stats);

/* Element-category objective terms (ObjectiveTerm::get_obj_val
 * objective_meth.rs:665-720, getd_ld_u :1051-1160, getd_ld_d :1372-1500) on
 * solid meshes (hex8, brickIM, tet4).
 *   asend_element_fields: centroid strain eps[n_el][6] and stress
 *     sig[n_el][6] (Voigt 11,22,33,12,13,23, engineering shear; s_cent of
 *     get_stress_strain_dfd0, element_soln_fields.rs:1463-1576) of load case
 *     rhs of the last solve, and the element volumes vol[n_el] (sum_ip w detJ,
 *     get_volume_dfd0 :1118-1155).  Any output may be NULL.
 *   asend_set_element_objective: selects ASEND_OBJ_ELEMENT with the weights
 *     w_stress[e] = dL/dsigma_e and w_strain[e] = dL/deps_e ([n_el][6] each,
 *     NULL = zeros) that the caller derives from its operator (powerNorm, ks,
 *     volumeIntegral, volumeAverage) on the fields above.  The next
 *     asend_adjoint_gradient then solves K lambda = sum_e B_c^T (w_strain_e +
 *     C_e w_stress_e) for a single load case and returns dLdE = explicit
 *     w_stress . sigma / E - lambda^T dR/dE (isotropic elements); its L_out
 *     is 0 (the caller evaluates the operator).  The strain pairs of
 *     asend_adjoint_strain_pairs then include the explicit material term,
 *     P_e - w_stress_e eps_e^T, so that asend_material_dv_gradient returns
 *     the total derivative. */
int asend_element_fields(asend_ctx* ctx, int32_t rhs, double* eps_out, double* sig_out, double* vol_out);
int asend_set_element_objective(asend_ctx* ctx, const double* w_stress, const double* w_strain);
/* Design variables over element sets with per-element coefficients
 * (read_des_var_input model_input.rs:1218-1296; element coefficient lists
 * model_prep.rs:414-442): dL/dD_i = sum_e coef_ie dL/dE_e. */
int asend_add_modulus_design_var(asend_ctx* ctx, int32_t elem_set, int32_t n_coef,
                                 const double* coefs);
int asend_design_var_gradient(asend_ctx* ctx, const double* dLdE, double* dLdD_out);

/* Material design variables of single components (the reference's
 * 'modulus', 'shearModulus', 'poissonRatio' categories with component 1-3,
 * DesignVariable design_var.rs:8-40 applied by get_solid_stiff,
 * element_properties.rs:648-764).  After asend_adjoint_gradient:
 *   asend_adjoint_strain_pairs fills pairs_out[n_el][6][6] with
 *     P_e = sum_gp w detJ eps(lambda) eps(u)^T (Voigt 11,22,33,12,13,23,
 *     engineering shear), so that lambda^T dR_e/dD = sum_ij (dC/dD)_ij P_e;
 *   asend_material_dv_gradient returns dL/dD for one DV over an element set
 *     (coefficients as asend_add_modulus_design_var), with C = S^-1 from the
 *     reference's compliance form at the element's isotropic E, nu.
 * hex8, tet4 and brickIM meshes: brickIM strains include the condensed
 * modes recovered per element (alpha = -Kii^-1 Kie f_e for both fields,
 * update_internal element_equations.rs:19-194); elements with orthotropic
 * constants (asend_set_orthotropic) use their own S.  beam2 meshes: the pairs
 * are of the section strains (axial, two shears, twist, two curvatures) with
 * the bubbles recovered, and the DVs act on the section stiffness as the
 * reference's get_beam_stiff_dfd0 does: modulus component 1 scales the E
 * entries, shearModulus components 1 / 2 / 3 the G entries of the first
 * shear and twist / the second shear / the I2 coupling, the other
 * components and poissonRatio give zero. */
#define ASEND_DV_MODULUS 0
#define ASEND_DV_SHEAR_MODULUS 1
#define ASEND_DV_POISSON_RATIO 2
/* beam2 section DVs (get_beam_stiff_dfd0's area, areaMoment and polarMoment
 * categories): area (component ignored), areaMoment component 1-5 (I1..I5),
 * polarMoment (component ignored); dC/dD with the element's E and
 * G = E / (2 (1 + nu)). */
#define ASEND_DV_AREA 3
#define ASEND_DV_AREA_MOMENT 4
#define ASEND_DV_POLAR_MOMENT 5
int asend_adjoint_strain_pairs(asend_ctx* ctx, double* pairs_out);
int asend_material_dv_gradient(asend_ctx* ctx, int32_t category, int32_t component, int32_t elem_set,
                               int32_t n_coef, const double* coefs, double* grad_out);
/* ---- material model and damping (solids) ----------------------------------
 * Orthotropic elements (the reference's material 'modulus', 'poissonRatio'
 * and 'shearModulus' lists, element_properties.rs:648-764): props[n_el][9] =
 * E1 E2 E3 nu12 nu13 nu23 G12 G13 G23 per element, C = S^-1 from the
 * compliance form; NULL restores the isotropic E, nu.  hex8 / tet4 meshes.
 * With orthotropic elements asend_adjoint_gradient takes dLdE_out = NULL and
 * material DV gradients come from asend_material_dv_gradient. */
int asend_set_orthotropic(asend_ctx* ctx, const double* props);
/* The 6 x 6 C (row-major, Voigt 11,22,33,12,13,23, engineering shear) of one
 * set of constants props[9]; host only. */
int asend_orthotropic_cmat(const double* props, double* C_out);
/* Damping of Newmark assemblies (get_rud_dfd0, element_equations.rs:628-850):
 * D = rayleigh_cm M + rayleigh_ck K + sum_gp B^T D_e B w detJ with the
 * material damping matrices D[n_el][36] (the reference's material 'damping'
 * entries, element_properties.rs:1537-1575; may be NULL).  The Newmark
 * operator gains c_D D with c_D = dt gamma c_M (element_equations.rs:995-1005)
 * and the step residual D v.  rayleigh_ck and D take hex8 / tet4 meshes. */
int asend_set_damping(asend_ctx* ctx, double rayleigh_cm, double rayleigh_ck, const double* D);
/* Layered shell4 sections (the reference's shell section 'layup': layers of
 * orthotropic material, thickness and angle, and zOffset).
 *   asend_shell_section (host only): the 9 x 9 ABD of the section
 *     (get_layer_thk_z element_properties.rs:75-136, get_layer_q :138-222,
 *     transform_q :581-646, get_abd :766-876: A, B, D from the rotated
 *     plane-stress layer stiffnesses, transverse shear and drilling = A66)
 *     and its 6 x 6 section mass (get_shell_mass :1354-1408).  Layer k:
 *     layers[7k..7k+6] = E1, E2, nu12, G12, density, thickness, angle [deg];
 *     z_offset -1 / 0 / 1 puts the reference plane on the lower surface /
 *     mid-plane / upper surface.
 *   asend_set_shell_sections: per-element abd[n_el][81] and msec[n_el][36]
 *     replacing the isotropic E, nu, t section of a shell4 mesh (NULL abd:
 *     back to E, nu, t).  Layered sections have no per-element modulus
 *     gradient (asend_adjoint_gradient takes dLdE_out = NULL) and no body
 *     loads. */
int asend_shell_section(int32_t n_layers, const double* layers, double z_offset, double* abd_out,
                        double* msec_out);
int asend_set_shell_sections(asend_ctx* ctx, const double* abd, const double* msec);
/* beam2 sections (the reference's beam section: area, areaMoment[5],
 * polarMoment, orientation; Section in section_meth.rs, stiffness
 * get_beam_stiff_dfd0 element_properties.rs:878-1017, mass
 * get_beam_mass_dfd0 :1410-1500), required before assembling a beam2 mesh.
 * sections[n_el][10] = area A, I1 = int z dA, I2 = int y dA, I3 = int z^2 dA,
 * I4 = int y^2 dA, I5 = int yz dA, polar moment J, and a direction v (3)
 * fixing the section's xy plane.  Element frame: e1 along the element
 * (node 1 -> node 2; the reference takes x from the section orientation and
 * needs it along the element), e3 = e1 x v / |e1 x v|, e2 = e3 x e1.
 * Section stiffness with the element's E and G = E / (2 (1 + nu)):
 * EA, GA, GA, GJ, E I3, E I4 on the diagonal of (axial strain, the two
 * transverse shears, twist, the two curvatures), couplings E I1, -E I2, -G I1,
 * G I2, -E I5; section mass rho (A, A, A, J, I3, I4) with couplings rho I1,
 * -rho I1, -rho I2, rho I2, rho I5, as the reference writes them.  A, I3, I4,
 * J > 0 and v off the element axis are required (EINVAL otherwise).  K_e is
 * proportional to E_e, so asend_adjoint_gradient gives per-element modulus
 * gradients; body loads need I1 = I2 = 0; damping takes rayleigh_cm only. */
int asend_set_beam_sections(asend_ctx* ctx, const double* sections);
/* Given beam section matrices (the reference's beamProps stiffness / mass
 * entries, section_meth.rs:61-71, used in place of the area and moments when
 * their [0] entry is positive, element_properties.rs:896-920, :1430-1440):
 * stiffness[n_el][36] and mass[n_el][36] in the section axes and the section
 * deformation order, symmetric (the upper triangle is read); an element whose
 * [0] entry is <= 0 keeps the computed matrix; either pointer may be NULL,
 * both NULL clears them.  After asend_set_beam_sections.  A given stiffness is
 * not proportional to E: asend_adjoint_gradient then takes dLdE_out = NULL and
 * material DVs give zero on those elements; a given mass takes no body loads. */
int asend_set_beam_section_matrices(asend_ctx* ctx, const double* stiffness, const double* mass);
/* Row-sum lumped mass in Newmark assemblies (the reference's 'lumpMass: yes',
 * element_equations.rs:950-971): the mass is diag(row sums of M). */
int asend_set_lumped_mass(asend_ctx* ctx, int32_t on);

/* dC/dD (row-major 6 x 6, Voigt order) of an isotropic element (E, nu,
 * G = E / (2 (1 + nu))) for a DV of the given category on one component;
 * host only, used by asend_material_dv_gradient. */
int asend_material_dC(int32_t category, int32_t component, double E, double nu, double* dC_out);

/* ---- Newmark transient (Model::solve dynamic loop model_analysis.rs:591-624;
 *      Node::update_vel_acc node_meth.rs:127-138, advance_disp :158-165) -----
 * Load at step i (time i*dt) = amp[i] * (load case 0).  Records
 * u[probe_dof] after each step in probe_hist[n_steps] (may be NULL) and the
 * final displacement in u_final[n_dof] (may be NULL).  Requires
 * asend_assemble(..., dynamic=1, dt, beta, gamma).  Each step's PCG is
 * warm-started from the previous step's increment, or with
 * opts->warm_start == 2 from 2 du_{n-1} - du_{n-2} (linear extrapolation). */
int asend_newmark_run(asend_ctx* ctx, const asend_solve_opts* opts, int32_t n_steps,
                      const double* amp, int32_t probe_dof, double* probe_hist,
                      double* u_final, asend_solve_stats* stats);

/* Solution history of the next asend_newmark_run, kept on the device:
 * fields 1 = displacements, 3 = displacements, velocities and accelerations
 * after every step (the solnTStep fields, write_time_step_soln
 * model_output.rs:14-82), 0 = none.  n_steps x fields x n_dof doubles. */
int asend_newmark_keep_history(asend_ctx* ctx, int32_t fields);
/* State after step `step` (1-based) of the last run; pointers may be NULL
 * (v_out, a_out need fields = 3). */
int asend_newmark_step_state(asend_ctx* ctx, int32_t step, double* u_out, double* v_out, double* a_out);
/* Transient adjoint (Model::get_obj_gradient's time-stepping branch,
 * model_analysis.rs:1544-1631, augmentd_ld_u :936-1063, solve_for_adjoint
 * :1065-1126): L = sum over the run's steps of sum_k obj_w[k] u[obj_dof[k]],
 * and dL/dE per element by the reverse Newmark sweep over the kept
 * displacement history (one operator solve per step).  Undamped,
 * consistent-mass, isotropic models; needs asend_newmark_keep_history(>= 1)
 * before the run. */
int asend_newmark_adjoint(asend_ctx* ctx, const asend_solve_opts* opts, int32_t n_obj, const int32_t* obj_dof,
                          const double* obj_w, double* L_out, double* dLdE_out, asend_solve_stats* stats);

/* ---- kernel-level entry points (measurement / tests) ----------------------
 * y = A x with the assembled operator at the given value precision (32 =
 * FP32 values, 64 = FP64, 48 = the split FP32 hi + lo product of
 * ASEND_METHOD_SPLIT), host buffers.  Equivalent of SparseMat::vector_multiply
 * (list_ent_meth.rs:64-79) plus the penalty product (const_meth.rs:92-103). */
int asend_apply_operator(asend_ctx* ctx, int32_t precision, const double* x, double* y);
/* Time n_launch back-to-back operator applications on the library stream with
 * CUDA events; returns the mean ms per launch and the algorithmic bytes per
 * launch. */
int asend_time_spmv(asend_ctx* ctx, int32_t precision, int32_t n_launch, double* ms_per_launch,
                    double* bytes_per_launch);
/* Time n_launch back-to-back launches of one kernel of the multigrid-
 * preconditioned CG on the assembled operator (building the hierarchy if
 * needed): kernel 0 = the outer product with its p.Ap reduction in the given
 * method's value format, 1 = the finest level's V-cycle residual, 2 = its
 * post-smoothing sweep.  Returns the mean ms per launch and the algorithmic
 * bytes per launch (values, column indices, gathered and streamed vectors
 * counted once).  No reference counterpart (measurement). */
int asend_time_mg_kernel(asend_ctx* ctx, int32_t kernel, int32_t method, int32_t n_launch, double* ms_per_launch,
                         double* bytes_per_launch);
/* Number of kernels this library launched since the context was created. */
int64_t asend_kernel_launches(const asend_ctx* ctx);
/* The context's CUDA stream (cudaStream_t as void*), so a caller can record
 * its own CUDA events around library calls. */
void* asend_stream(const asend_ctx* ctx);

/* ---- modal analysis (frequency job: Model::eigen_solve model_analysis.rs:711-880,
 *      eigen_sparse_direct matrix_functions.rs:1099-1265) -------------------
 * The n_modes eigenpairs of (K + sf C^T C) x = lambda D x nearest to the
 * shift (the reference's tgtEval), lowest first.  D is the row-sum diagonal
 * mass (model_analysis.rs:748-766) with entries below 1e-6 mean|D| raised to
 * it (:768-779).  Shift-invert block Lanczos on D^1/2 (A - shift D)^-1 D^1/2
 * with full reorthogonalisation; the inner solves use `inner` (any method /
 * preconditioner of asend_static_solve; A - shift D must be positive
 * definite).  Assembles K and M itself (FP64, c_M = 0) unless the last
 * assembly was asend_assemble(..., dynamic = 2).  Outputs (each may be NULL):
 * eig_out[n_modes], freq_out[n_modes] = sqrt(lambda) / (2 pi) (-1 for
 * lambda < 0, :874-879), modes_out[n_modes][n_dof] at unit 2-norm with the
 * largest-magnitude component positive, diag_mass_out[n_dof].  Returns
 * ASEND_OK when every wanted pair met tol, else ASEND_MAX_ITER (results
 * still written). */
typedef struct asend_eigen_opts {
    int32_t n_modes;        /* eigenpairs wanted                                       */
    int32_t block_size;     /* right-hand sides per shift-invert solve, 1..4 (0 = 2)   */
    int32_t max_subspace;   /* basis size cap (0 = max(5 n_modes, n_modes + 20)
                               x max(1, block_size / 2))                               */
    int32_t reserved;
    double shift;           /* tgtEval; eigenvalues are returned unshifted              */
    double tol;             /* Ritz residual ||Op y - theta y|| <= tol theta (0 = 1e-8)   */
    asend_solve_opts inner; /* options of the shift-invert solves                      */
} asend_eigen_opts;

typedef struct asend_eigen_stats {
    int32_t n_found;        /* pairs written                                           */
    int32_t n_converged;    /* pairs within tol                                         */
    int32_t subspace;       /* Lanczos basis size at exit                               */
    int32_t n_solves;       /* shift-invert right-hand sides solved                     */
    int64_t inner_iterations;
    int32_t status;
    int32_t inner_capped;   /* shift-invert solves that stopped at their iteration cap  */
    double max_rel_residual;/* max_k Ritz residual ||Op y_k - theta_k y_k|| / theta_k,
                               Op = D^1/2 (A - shift D)^-1 D^1/2 (the stopping measure) */
    double max_pencil_residual; /* max_k ||A x_k - lambda_k D x_k|| / ||A x_k|| (FP64);
                               the penalty rows (sf = 1e5 max|K|) dominate it          */
    double ms;              /* device time                                              */
} asend_eigen_stats;

int asend_eigen_solve(asend_ctx* ctx, const asend_eigen_opts* opts, double* eig_out, double* freq_out,
                      double* modes_out, double* diag_mass_out, asend_eigen_stats* stats);

/* Dense symmetric eigenproblem of a row-major m x m matrix (host routine of
 * the Lanczos projection; no device needed): eigenvalues ascending in
 * vals[m], vecs[k*m + i] = component i of eigenvector k (may be NULL). */
int asend_dense_sym_eigen(int32_t m, const double* a, double* vals, double* vecs);

/* shell4 / brickIM / beam2 element matrices of elements [first, first +
 * count): ke (and me when not NULL) [count][24][24] ([count][12][12] for
 * beam2) in node-major DOF order (shell4, beam2: u v w thx thy thz per node;
 * brickIM: u v w per node), stiffness after condensing the internal DOF
 * (element_equations.rs:19-57: 8 for shell4, 9 for brickIM, 2 for beam2),
 * consistent mass over the node DOF (:420-626). */
int asend_element_matrices(asend_ctx* ctx, int32_t first, int32_t count, double* ke, double* me);

/* y = A x and *energy = x^T A x with the assembled FP64 operator, on DEVICE
 * buffers (x, y: n_dof doubles; energy: one double; the three must not
 * overlap, else ASEND_EINVAL), without allocating any device memory.  No counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc -- applications that give all device memory to their
 * own pool allocator or run under a fixed HBM budget, and optimisation loops
 * that evaluate the energy many times where an allocation could fail or stall.
 * Its reduction scratch is a fixed 256 KiB array compiled into the library,
 * which every GPU that loads the library holds until the process exits.
 * Limit: 4,194,304 node rows (12,582,912 DOF), 3 DOF per node; larger
 * operators are rejected with ASEND_EINVAL and a message.  The first call on a
 * device looks up the array's device address (a one-time set-up), so make
 * that first call before any stream capture.  With CUDA's lazy module
 * loading (the default) that first call also loads this part of the library
 * onto the device, which reserves device memory for the array and its kernel
 * code; a caller whose pool will take all HBM makes the first call before
 * the pool does, or sets CUDA_MODULE_LOADING=EAGER.  Later calls allocate
 * nothing.  The work is enqueued on the
 * context's stream and not synchronised.  All calls share the scratch array:
 * calls that overlap on the GPU (other streams or contexts on the same
 * device) race and must be serialised by the caller. */
int asend_operator_energy_noalloc(asend_ctx* ctx, const double* d_x, double* d_y, double* d_energy);

/* ---- learned nodal preconditioner blocks (no reference counterpart; the
 *      reference preconditions CG with block LDL^T factors,
 *      lower_tri_mat_meth.rs:15-241) -------------------------------------------
 * A 3-layer MLP (16 -> 64 -> 64 -> 8, ReLU; BF16 weights and activations, FP32
 * accumulation) maps per-node features to a lower-triangular correction U of
 * the block-Jacobi inverse: M_n = C_n U_n U_n^T C_n^T with C_n C_n^T = D_n^-1,
 * so every block is SPD and a zero output is plain block Jacobi.
 * Features (16 per node, 12 used): the node's diagonal 3x3 block divided by
 * its mean diagonal (6 entries), 0.1 * (log mean diagonal - mesh mean), mean,
 * standard deviation and range of log E - mean log E over the adjacent
 * elements, adjacent-element count / 8, and a flag for penalty-dominated
 * nodes.  Parameters, FP32, in the order W1[64][16] b1[64] W2[64][64] b2[64]
 * W3[8][64] b3[8] (row-major [out][in]).
 * The weights belong to the context and survive asend_set_mesh and
 * asend_set_modulus, so a model trained on small meshes is applied to a large
 * one in the same context (or moved with get/set_params).
 * ASEND_PC_LEARNED solves with the blocks; a non-finite or non-converged
 * solve is rerun with point-Jacobi PCG (status ASEND_FALLBACK when that
 * converges), and with no weights the solve is the Jacobi one with status
 * ASEND_FALLBACK.  ASEND_PC_MG_LEARNED uses the blocks as the multigrid
 * finest-level smoother and needs weights. */
int32_t asend_learned_n_params(void);
/* Random initial weights (last layer ~1e-3, i.e. block Jacobi); resets Adam. */
int asend_learned_init(asend_ctx* ctx, uint64_t seed);
int asend_learned_set_params(asend_ctx* ctx, const float* params);
int asend_learned_get_params(asend_ctx* ctx, float* params);
/* Training samples from the assembled operator and load case 0: sample s is
 * the residual of plain point-Jacobi PCG after iters[s] > 0 iterations; for
 * iters[s] == 0 a standard normal vector from the seed; for iters[s] < 0 the
 * residual after -iters[s] stationary multigrid V-cycle iterations from such
 * a vector (the modes the V-cycle reduces slowest; needs the block
 * structure).  Each is normalised.  append = 0 replaces the stored samples. */
int asend_learned_add_samples(asend_ctx* ctx, int32_t n_samples, const int32_t* iters, int32_t append,
                              uint64_t seed);
/* Caller-supplied samples [n_samples][n_dof] (each scaled to unit norm),
 * replacing the stored ones. */
int asend_learned_set_samples(asend_ctx* ctx, int32_t n_samples, const float* samples);
/* Selects the training loss (ASEND_LEARN_*; default ASEND_LEARN_BLOCK). */
int asend_learned_set_objective(asend_ctx* ctx, int32_t kind);
/* Loss = the selected objective's mean over the samples (FP32 operator).  train:
 * n_steps Adam steps (beta 0.9/0.999) at learning rate lr on the stored
 * samples, on the GPU; *loss_out = the loss before the last step (n_steps = 0:
 * the current loss, no step). */
int asend_learned_train(asend_ctx* ctx, int32_t n_steps, float lr, double* loss_out);
/* Current loss and its gradient with respect to the parameters (no step). */
int asend_learned_loss_grad(asend_ctx* ctx, double* loss_out, float* grad_out);
/* Per-node features [n_nodes][16] (the BF16 values), Cholesky factors of
 * D_n^-1 [n_nodes][6] (l00 l10 l11 l20 l21 l22) and network outputs
 * [n_nodes][8]; any pointer may be NULL (outputs need weights). */
int asend_learned_features(asend_ctx* ctx, float* feat, float* chol, float* outputs);
/* The nodal blocks M_n [n_nodes][9] (use_net = 0: block-Jacobi inverse). */
int asend_learned_blocks(asend_ctx* ctx, int32_t use_net, float* blocks_out);
/* Kernel checks: network outputs [n][8] for features [n][16] (rounded to
 * BF16), and the parameter gradient of sum(outputs * dy) over the n rows. */
int asend_learned_forward(asend_ctx* ctx, int32_t n, const float* feat, float* outputs);
int asend_learned_backward(asend_ctx* ctx, int32_t n, const float* feat, const float* dy, float* grad_out);

#ifdef __cplusplus
}
#endif
#endif
