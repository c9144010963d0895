// common.cuh -- shared device helpers and the library context.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "../../include/asend_gpu.h"

#define ASEND_CUDA(call)                                                        \
    do {                                                                        \
        cudaError_t e__ = (call);                                               \
        if (e__ != cudaSuccess) {                                               \
            throw asend::CudaError(std::string(#call) + ": " + cudaGetErrorString(e__)); \
        }                                                                       \
    } while (0)

namespace asend {

struct CudaError {
    std::string msg;
    explicit CudaError(std::string m) : msg(std::move(m)) {}
};
struct InputError {
    std::string msg;
    explicit InputError(std::string m) : msg(std::move(m)) {}
};

// Device array owned by the context.
template <typename T>
struct DArr {
    T* p = nullptr;
    size_t n = 0;
    DArr() = default;
    DArr(const DArr&) = delete;
    DArr& operator=(const DArr&) = delete;
    ~DArr() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        if (count == n && p) return;
        release();
        if (count == 0) return;
        ASEND_CUDA(cudaMalloc(&p, count * sizeof(T)));
        n = count;
    }
    void upload(const T* h, size_t count, cudaStream_t s) {
        alloc(count);
        if (count) ASEND_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T>& h, cudaStream_t s) { upload(h.data(), h.size(), s); }
    void zero(cudaStream_t s) {
        if (n) ASEND_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

constexpr int kSlice = 32;  // rows per slice of the sliced block-ELL matrix

// Sliced block-ELL ("SBELL") matrix over node rows with b x b blocks.
// Block column group g = slice_off[row/32] + j holds, for the 32 rows of the
// slice, column node col[g*32 + lane] and values
// vals[(g*b*b + v)*32 + lane], v = a*b + c (row component a, column comp c).
// Rows shorter than the slice width are padded (never read: row_len).
struct Sbell {
    int b = 3, n_rows = 0, n_slices = 0;
    int64_t n_groups = 0;  // total block-column groups (slots = 32 * n_groups)
    std::vector<int64_t> h_slice_off;
    std::vector<int32_t> h_col;
    std::vector<uint8_t> h_row_len, h_diag;
    DArr<int64_t> slice_off;
    DArr<int32_t> col;
    DArr<uint8_t> row_len, diag;
    DArr<double> v64, m64;  // operator values (K [+cM M] [+cD D] + penalty), mass values
    DArr<double> d64;       // damping values (Newmark with damping)
    DArr<float> v32;        // FP32 values: float(v64), the high part of each value
    DArr<float> v32lo;      // low parts float(v64 - v32): v64 = v32 + v32lo to 2^-48 relative
    int64_t nnz_scalar() const {  // stored scalar entries excluding padding
        int64_t s = 0;
        for (int r = 0; r < n_rows; ++r) s += (int64_t)h_row_len[r];
        return s * b * b;
    }
    int64_t slot(int row, int j) const {
        return (h_slice_off[row / kSlice] + j) * kSlice + (row % kSlice);
    }
};

struct PcgScalars {
    double rz, rz_new, pAp, rr, bb, alpha, beta, target_rr, rr_last_true;
    int32_t iter, done, status, since_replace;
    uint32_t ticket_a, ticket_b, ticket_c, pad;
};

struct MgHierarchy;
struct LearnedState;

// Quadratic tetrahedron (type 10) at s: corners 0..3, mid-edge nodes 4 (0-1),
// 5 (1-2), 6 (0-2), 7 (0-3), 8 (1-3), 9 (2-3) (element_soln_fields.rs:229-298).
__host__ __device__ inline void tet10_shape(const double* s, double* n, double (*dn)[3]) {
    const double p1 = 1.0 - s[0] - s[1] - s[2];
    n[0] = p1 * (2.0 * p1 - 1.0);
    for (int j = 0; j < 3; ++j) dn[0][j] = 1.0 - 4.0 * p1;
    for (int k = 0; k < 3; ++k) {
        n[1 + k] = s[k] * (2.0 * s[k] - 1.0);
        for (int j = 0; j < 3; ++j) dn[1 + k][j] = (j == k) ? 4.0 * s[k] - 1.0 : 0.0;
    }
    const int edge0[3] = {4, 6, 7};  // edges (0, k+1): 4 s_k p1
    for (int k = 0; k < 3; ++k) {
        const int a = edge0[k];
        n[a] = 4.0 * s[k] * p1;
        for (int j = 0; j < 3; ++j) dn[a][j] = (j == k) ? 4.0 * (p1 - s[k]) : -4.0 * s[k];
    }
    const int edge[3][3] = {{5, 0, 1}, {8, 0, 2}, {9, 1, 2}};  // edges between corners 1..3: 4 s_i s_j
    for (int q = 0; q < 3; ++q) {
        const int a = edge[q][0], i = edge[q][1], k = edge[q][2];
        n[a] = 4.0 * s[i] * s[k];
        for (int j = 0; j < 3; ++j) dn[a][j] = (j == i) ? 4.0 * s[k] : (j == k ? 4.0 * s[i] : 0.0);
    }
}

// The tet10 rule: four points with R_TET1 ~ (5 - sqrt 5) / 20 on every axis
// but one, which takes R_TET2 ~ (5 + 3 sqrt 5) / 20, weights 1/24
// (element_meth.rs:228-262).  The values are the reference's own 16-digit
// constants (constants.rs:10-11), 2e-14 from the exact roots, so that the
// element matrices agree with the reference's to rounding.
constexpr double kRTet1 = 0.1381966011250071;
constexpr double kRTet2 = 0.585410196624929;
__host__ __device__ inline void tet10_point(int gp, double* s) {
    s[0] = s[1] = s[2] = kRTet1;
    if (gp > 0) s[gp - 1] = kRTet2;
}

struct Ctx {
    int device = 0;
    // structured-block metadata (multigrid) and its hierarchy
    int bx = 0, by = 0, bz = 0;
    std::shared_ptr<MgHierarchy> mg;
    float mg_damping = 1.5f;  // smoother omega = mg_damping / lambda_max(D^-1 A)
    int product_variant = 0;  // split outer product: ASEND_PRODUCT_* (0 = the default shape)
    bool mg_tail = true;      // multigrid: fuse the V-cycle's smallest levels into one launch
    bool time_solves = true;  // record CUDA events around each PCG solve (off inside Newmark runs)
    int64_t dinv_epoch = -1;  // assembly whose point-Jacobi diagonal d_dinv holds
    bool pdl = false;         // multigrid CG: programmatic dependent launch between its kernels
                              // (off: measured slower on GB300, 12.3 vs 11.3 ms per solve)
    std::shared_ptr<LearnedState> learned;  // learned nodal preconditioner blocks
    int64_t assembly_epoch = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t launches = 0;

    // ---- mesh (host).  The solver works on nodes of dpn = 3 DOF; a shell4
    // node (6 DOF) is two of them (translations, rotations), so n_nodes counts
    // those internal nodes while n_unodes / udpn are the caller's.
    int type = 0, nn = 0, dpn = 3, nip = 0;
    int n_nodes = 0, n_el = 0, n_dof = 0;
    int n_unodes = 0, udpn = 3;
    std::vector<double> xyz, E, nu, rho, thk;
    std::vector<int32_t> conn;
    std::vector<std::vector<int32_t>> node_sets, elem_sets;
    // constraint rows (natural DOF numbering)
    std::vector<int32_t> c_ptr{0}, c_dof;
    std::vector<double> c_coef, c_rhs;
    // load cases (FP64 host, natural numbering, without penalty rhs)
    std::vector<std::vector<double>> loads;
    int64_t loads_version = 0, rhs_version = -1;  // device copy valid when equal
    double rhs_sf = -1.0;
    // objective + design variables
    int obj_kind = ASEND_OBJ_COMPLIANCE, obj_set = -1, obj_comp = 1;
    double obj_coef = 1.0;
    std::vector<int32_t> dv_ptr{0}, dv_el;
    std::vector<double> dv_coef;

    // ---- device mesh
    DArr<double> d_xyz, d_E, d_nu, d_rho, d_thk;
    DArr<int32_t> d_conn;
    DArr<int32_t> d_shell_conn;  // shell4 / beam2: physical nodes per element (4 / 2)
    DArr<double> d_shell_xyz;    // shell4 / beam2: physical node coordinates
    // beam2 sections [n_el][10]: area, I1..I5, polar moment J, xy-plane direction;
    // optional given section stiffness and mass matrices [n_el][72] (C then M,
    // entry [0] <= 0: computed); the device table joins both per element
    std::vector<double> beam_sec, beam_cm;
    DArr<double> d_beam_sec;
    bool beam_given_stiffness() const {
        for (size_t e = 0; e < beam_cm.size() / 72; ++e)
            if (beam_cm[e * 72] > 0.0) return true;
        return false;
    }
    // shell4 layered sections: per-element ABD [n_el][81] and section mass
    // [n_el][36] replacing the isotropic E, nu, t section
    bool shell_layered = false;
    DArr<double> d_shell_abd, d_shell_msec;
    bool pattern_ready = false, assembled = false, dynamic = false;
    bool modal = false;  // K and M assembled apart (c_M = 0) for the frequency job
    double dt = 0, beta = 0.25, gamma = 0.5, cM = 0;
    double cD = 0;                  // damping coefficient of the Newmark operator (dt gamma cM)
    // material model beyond isotropic E, nu (solids without internal DOF):
    // engineering constants per element [n_el][9] = E1 E2 E3 nu12 nu13 nu23
    // G12 G13 G23 and the 6x6 stiffness from them
    std::vector<double> ortho;
    DArr<double> d_cmat;
    // damping: Rayleigh coefficients and material damping matrices [n_el][36]
    double ray_cm = 0, ray_ck = 0;
    std::vector<double> dmat;
    DArr<double> d_dmat;
    bool lump = false;              // row-sum lumped mass in Newmark assemblies
    double sf = 0;
    int assembled_precision = 64;
    // A split-only assembly (precision 48) writes the operator's FP32 hi / lo
    // values and leaves the FP64 copy stale until ensure_v64() rebuilds it.
    bool v64_valid = true;
    float last_assemble_ms = 0.f;

    // ---- pattern / assembly
    Sbell A;
    // geometry classes: elements whose matrices at unit modulus (and unit
    // density) coincide share one reference matrix; K_e = E_e * Khat_class
    int cls_type = 0, n_cls = 0;
    std::vector<int32_t> h_cls_of;
    DArr<int32_t> d_cls_of;          // class of each element
    DArr<double> cls_ke, cls_me;     // [n_cls][(3 nn)^2] stiffness, [n_cls][nn nn] mass (FP64)
    DArr<float> cls_ke32;            // FP32 copy of cls_ke (multigrid coarsening)
    DArr<float2> cls_ke2;            // cls_ke as FP32 pairs (split-only assembly)
    DArr<float2> d_E2;               // element moduli as FP32 pairs (split-only assembly)
    DArr<int32_t> d_gat_ptr, d_gat;  // per value slot: contributing (element, a, b) entries
    bool cls_ready = false;
    DArr<int32_t> d_slot_map;  // [n_el * nn * nn] slot of block (a, b)
    std::vector<int32_t> colour_of, colour_ptr, colour_elems;
    DArr<int32_t> d_colour_elems;
    DArr<int64_t> d_pen_idx;   // value indices receiving penalty terms
    DArr<double> d_pen_coef;   // coef_i * coef_j per penalty entry
    DArr<double> d_max_partial;

    // ---- solver state (nrhs * n_dof each)
    int nrhs = 0;
    DArr<double> d_f, d_x, d_r;        // rhs incl. penalty, solution, residual
    DArr<float> d_p32, d_ap32;         // mixed: padded direction, A p
    DArr<double> d_p64, d_ap64;        // fp64: padded direction, A p
    DArr<float4> d_xpair;              // split multigrid CG: correction of x as node-padded FP32 pairs
    DArr<float4> d_xtrip;              // split multigrid CG on a split-only operator: x as 3 FP32 parts
    DArr<double> d_dinv;               // point Jacobi inverse diagonal (n_dof)
    DArr<float> d_binv;                // nodal block inverse (n_nodes * b*b)
    DArr<double> d_partials;           // block partial sums
    DArr<PcgScalars> d_sc;
    PcgScalars* h_sc = nullptr;        // pinned mirror
    bool solved = false;
    int last_method = ASEND_METHOD_MIXED;

    // adjoint
    DArr<double> d_lam, d_gE;
    DArr<double> d_adj_b;          // second field of the last adjoint contraction (displacement objective)
    // element-category objective: per-element weights dL/dsigma, dL/deps at
    // the centroid [n_el][6] each (ASEND_OBJ_ELEMENT)
    DArr<double> d_obj_wa, d_obj_wb;
    int adj_kind = -1;             // objective of the last adjoint gradient (-1: none)
    int64_t adj_serial = 0, pairs_serial = -1;
    std::vector<double> h_pairs;   // strain-pair tensors of the last adjoint [n_el][36]

    // Newmark solution history (kept when hist_fields > 0): per step the
    // displacement (fields = 1) or displacement, velocity and acceleration
    // (fields = 3), [steps][fields][n_dof]
    int hist_fields = 0, hist_steps = 0;
    double hist_dt = 0.0;
    DArr<double> d_hist;

    // timing
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    // independent instances stacked in one operator (batched solves)
    int n_inst = 0;
    std::vector<int32_t> inst_node_ptr;
    std::vector<int32_t> inst_dims;          // structured block (nx, ny, nz) per instance (multigrid)
    DArr<int32_t> d_cta_inst, d_inst_cta0, d_inst_ncta;
    DArr<int64_t> d_unit_idx;  // diagonal entries of nodes without elements (set to 1)
    std::vector<double> sf_inst;             // penalty scale per instance
    std::vector<int32_t> pen_dof;            // DOF of each penalty entry (host)
    std::vector<double> pen_coef_host;       // coef_i * coef_j of each penalty entry (host)
    DArr<double> d_pen_val;                  // per-entry penalty values (batched)
    size_t h_sc_bytes = 0;

    // graphs
    // cached PCG iteration graph and the launch arguments it was captured
    // with (reused while they are identical, e.g. every Newmark step), and
    // the persistent scalar / control / ticket buffers it points at
    cudaGraphExec_t graph = nullptr;
    std::vector<uint8_t> graph_key;
    DArr<uint8_t> pcg_sc, pcg_ctl, pcg_tk;
};

// ---- device reductions -----------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum of K values per thread (K small); result valid in thread 0.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* smem /* [32*K] */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) smem[warp * K + k] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double t = (lane < nw) ? smem[lane * K + k] : 0.0;
            v[k] = warp_sum(t);
        }
    }
}

// host-side helpers implemented in the .cu files
void assemble_operator(Ctx& c, int precision);
// Rebuild the FP64 operator values from the hi / lo pairs after a split-only
// assembly (no-op otherwise); every path that reads A.v64 calls it first.
void ensure_v64(Ctx& c);
cudaError_t ensure_v64_rc(Ctx& c);  // the same, returning the launch status instead of throwing
void build_classes(Ctx& c, const std::vector<int32_t>& slot_map);
void build_pattern(Ctx& c);
void apply_operator_device(Ctx& c, int precision, const double* d_x, double* d_y);
double time_spmv(Ctx& c, int precision, int n_launch, double* bytes);
int pcg_solve(Ctx& c, const asend_solve_opts& o, asend_solve_stats* st, bool warm, const double* d_f,
              double* d_x, int nrhs);
void device_dot(Ctx& c, size_t n, const double* a, const double* b, double* d_out, double* d_part);
void device_axpy(Ctx& c, size_t n, double alpha, const double* x, double* y);
void adjoint_contract(Ctx& c, const double* d_a, const double* d_b, double* d_g, bool accumulate);
void adjoint_pairs(Ctx& c, const double* d_a, const double* d_b, double* d_P, bool accumulate);
int eigen_solve(Ctx& c, const asend_eigen_opts& eo, double* eig_out, double* freq_out, double* modes_out,
                double* diag_mass_out, asend_eigen_stats* st);
int sym_eigen_dense(int m, const double* a, double* vals, double* vecs);
int newmark_run(Ctx& c, const asend_solve_opts& o, int n_steps, const double* amp, int probe,
                double* probe_hist, double* u_final, asend_solve_stats* st);
void upload_rhs(Ctx& c);
int newmark_adjoint(Ctx& c, const asend_solve_opts& o, int n_obj, const int32_t* obj_dof, const double* obj_w,
                    double* L_out, double* gE_out, asend_solve_stats* st);
void ensure_pinned_scalars(Ctx& c, size_t bytes);
int instance_of_node(const Ctx& c, int node);
bool orthotropic_cmat(const double* props9, double* C36);
double row_penalty_scale(const Ctx& c, int row);
// multigrid (k_mg.cu)
void mg_prepare(Ctx& c, bool learned = false);  // learned: the finest smoother comes from the learned model
void mg_invalidate_values(Ctx& c);
void mg_level_info(Ctx& c, int level, int32_t* dims, double* lam_est, double* lam_bound, double* omega);
void mg_vcycle_host(Ctx& c, const float* b, float* z);
void mg_select_smoother(Ctx& c, bool learned);
void mg_stationary_residual(Ctx& c, float* r_host, int k, bool learned_smoother);
void mg_learned_loss_grad(Ctx& c, const float* samples, int n_samples, float* gblk, double* d_loss);
void mg_apply(Ctx& c, const float* d_b, float* d_z4);
int mg_levels(const Ctx& c);
double mg_time_kernel(Ctx& c, int kernel, int method, int n_launch, double* bytes);
int pcg_solve_mg(Ctx& c, const asend_solve_opts& o, asend_solve_stats* st, bool warm, const double* d_f, double* d_x,
                 int nrhs);
// element-category objectives (k_objective.cu)
void element_fields(Ctx& c, const double* d_u, double* d_eps, double* d_sig, double* d_vol);
void element_objective_rhs(Ctx& c, double* d_rhs);
void element_objective_explicit(Ctx& c, const double* d_u, double* d_gE, double* d_P);
// shell4 elements (k_shell.cu)
void shell_assemble(Ctx& c, double* vals, double* mvals);
void shell_adjoint(Ctx& c, const double* d_u, const double* d_lam, double* d_g, bool accumulate);
void shell_element_matrices(Ctx& c, int e0, int n, double* ke_host, double* me_host);
// beam2 elements (k_beam.cu)
void beam_assemble(Ctx& c, double* vals, double* mvals);
void beam_adjoint(Ctx& c, const double* d_u, const double* d_lam, double* d_g, bool accumulate);
void beam_element_matrices(Ctx& c, int e0, int n, double* ke_host, double* me_host);
void beam_pairs(Ctx& c, const double* d_a, const double* d_b, double* d_P, bool accumulate);
std::vector<double> beam_device_table(const Ctx& c);
// dC[36] of the beam section stiffness per unit change of a material DV
void beam_section_dC(int category, int component, const double* sec, double E, double nu, double* dC);
// brickIM elements (k_brickim.cu)
void brickim_assemble(Ctx& c, double* vals, double* mvals);
void brickim_adjoint(Ctx& c, const double* d_u, const double* d_lam, double* d_g, bool accumulate);
void brickim_element_matrices(Ctx& c, int e0, int n, double* ke_host, double* me_host);
void brickim_pairs(Ctx& c, const double* d_a, const double* d_b, double* d_P, bool accumulate);
void brickim_element_ke32(Ctx& c, float* d_ke);
// learned nodal preconditioner blocks (k_learned.cu)
bool learned_ready(const Ctx& c);
void learned_mesh_changed(Ctx& c);
void learned_init(Ctx& c, uint64_t seed);
void learned_set_objective(Ctx& c, int kind);
void learned_set_params(Ctx& c, const float* params);
void learned_get_params(Ctx& c, float* params);
int learned_n_params();
int learned_n_features();
int learned_n_outputs();
void learned_blocks(Ctx& c, float* d_binv, bool use_net);
void learned_add_samples(Ctx& c, int n_samples, const int32_t* iters, bool append, uint64_t seed);
void learned_set_samples(Ctx& c, int n_samples, const float* samples);
double learned_loss_grad(Ctx& c, bool grad);
double learned_train(Ctx& c, int n_steps, float lr);
void learned_get_grad(Ctx& c, float* out);
void learned_get_features(Ctx& c, float* feat, float* cfac, float* y);
void learned_forward_host(Ctx& c, int n, const float* feat, float* y_out);
void learned_backward_host(Ctx& c, int n, const float* feat, const float* dy, float* grad_out);

}  // namespace asend
