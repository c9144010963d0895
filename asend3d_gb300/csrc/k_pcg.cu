// k_pcg.cu -- K3: preconditioned CG on the sliced block-ELL operator.
//
// Reference: conj_grad_sparse, solverSrc/asend_run_job/src/matrix_functions.rs:285-362
// (x0 = 0, g = A x - b, alpha = res / h^T A h, beta = r_next / res,
// SparseMat::vector_multiply list_ent_meth.rs:64-79 plus the penalty product
// ConstraintList::get_total_vec_mult const_meth.rs:161-168, folded into the
// assembled operator here).  Stopping: the reference stops on the absolute
// g^T M^-1 g <= conv_tol; this solver stops on ||b - A x||_2 <= tol ||b||_2
// evaluated with the FP64 operator (the residual is re-formed in FP64 before
// convergence is accepted).
//
// GB300 design.
//  * One thread per node row (3 DOFs) of the sliced block-ELL matrix: each
//    warp reads its 9 block values per column group as 9 coalesced 128-byte
//    loads, and gathers the search direction as one 16-byte vector per
//    neighbour node (direction stored node-padded to 4 components).
//  * METHOD_MIXED: FP32 values, FP32 direction p and A p, FP32 FMAs in the
//    SpMV; FP64 x, r, all inner products and the scalar recurrence.  A true
//    FP64 residual b - A64 x replaces the recurrence residual when the latter
//    converges or drops by 1e4 since the last replacement (reliable updates),
//    which keeps the FP32 operator error out of the final answer.
//  * METHOD_FP64: every value, vector and FMA in FP64 (the plain method).
//  * Inner products: warp shuffles -> shared memory -> one partial per CTA ->
//    the last CTA (atomic ticket) sums the partials in a fixed order, so the
//    reductions are deterministic and need no extra launch.
//  * Three kernels per iteration (SpMV+dot, x/r update+dots, p update),
//    captured G iterations at a time in a CUDA graph; every kernel returns
//    at once when all right-hand sides have converged, so a graph may
//    overrun convergence harmlessly.  Up to 4 right-hand sides share one
//    matrix read (block SpMM).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "pcg_common.cuh"

namespace asend {
namespace {
using namespace pcg;

// K_a: Ap = A p, pAp; alpha = rz / pAp.
template <typename TV, typename TP, int NR>
__global__ void __launch_bounds__(kThreads) k_spmv_dot(PcgArgs A) {
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (cta_done<NR>(A, S)) return;
    if constexpr (std::is_same<TP, float>::value) {
        // Mixed: once the FP32-operator recurrence has dropped 1e4 below the
        // last true residual, stop this graph chunk at an iteration boundary
        // (p is consistent) so the host replaces the residual before the two
        // drift apart.  Every CTA decides from scalars no kernel of this
        // iteration has changed; the instance's first CTA records it.
        const int b0 = A.cta_inst ? A.inst_cta0[cta_instance(A)] : 0;
        bool skip_all = true;
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            const bool drop = !S[k].done && S[k].rr < 1e-4 * S[k].rr_last_true;
            skip_all &= S[k].done || drop;
            if (drop && blockIdx.x == b0 && threadIdx.x == 0) S[k].done = 1;
        }
        if (skip_all) return;
    }
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    double d[NR][1];
#pragma unroll
    for (int k = 0; k < NR; ++k) d[k][0] = 0.0;
    if (row < A.n_rows) {
        typename ApOf<TP>::T y[NR][3];
        const TV* vals;
        if constexpr (sizeof(TV) == 4) vals = A.v32; else vals = A.v64;
        spmv_row<TV, TP, NR>(row, A, vals, A.p, y);
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            typename ApOf<TP>::T pv[3];
            PadVec<TP>::load(A.p, (size_t)k * A.n_rows + row, pv);
            typename ApOf<TP>::T* ap = reinterpret_cast<typename ApOf<TP>::T*>(A.ap) + (size_t)k * A.n_dof + 3 * (size_t)row;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                ap[a] = y[k][a];
                d[k][0] += (double)pv[a] * (double)y[k][a];
            }
        }
    }
    double tot[NR][1];
    if (last_block_reduce<NR, 1>(A, d, 0, tot) && threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            RhsScalars& s = S[k];
            if (s.done) continue;
            s.pAp = tot[k][0];
            s.alpha = s.rz / s.pAp;
        }
    }
}

// K_b: x += alpha p; r -= alpha Ap; z = M r; dots (r,z), (r,r); beta.
template <typename TP, int NR, int PC>
__global__ void __launch_bounds__(kThreads) k_update_xr(PcgArgs A) {
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (cta_done<NR>(A, S)) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    double d[NR][2];
#pragma unroll
    for (int k = 0; k < NR; ++k) d[k][0] = d[k][1] = 0.0;
    if (row < A.n_rows) {
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            if (S[k].done) continue;
            const double alpha = S[k].alpha;
            typename ApOf<TP>::T pv[3];
            PadVec<TP>::load(A.p, (size_t)k * A.n_rows + row, pv);
            const size_t o = (size_t)k * A.n_dof + 3 * (size_t)row;
            const typename ApOf<TP>::T* ap = reinterpret_cast<const typename ApOf<TP>::T*>(A.ap) + o;
            double rv[3], z[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                A.x[o + a] += alpha * (double)pv[a];
                rv[a] = A.r[o + a] - alpha * (double)ap[a];
                A.r[o + a] = rv[a];
            }
            precond<PC>(A, row, rv, z);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                d[k][0] += rv[a] * z[a];
                d[k][1] += rv[a] * rv[a];
            }
        }
    }
    double tot[NR][2];
    if (last_block_reduce<NR, 2>(A, d, 1, tot) && threadIdx.x == 0) {
        int all = 1;
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            RhsScalars& s = S[k];
            if (!s.done) {
                s.rz_new = tot[k][0];
                s.rr = tot[k][1];
                s.beta = s.rz_new / s.rz;
                s.rz = s.rz_new;
                s.iter += 1;
                if (!isfinite(s.rr) || !isfinite(s.rz)) {
                    s.nonfinite = 1;
                    s.done = 1;
                } else if (s.rr <= s.target) {
                    s.done = 1;  // recurrence converged: the host verifies in FP64
                    s.restart = 1;
                }
            }
            all &= s.done;
        }
        if (all && !A.cta_inst) A.ctl->all_done = 1;
    }
}

// K_c: p = M r + beta p (node-padded store).
template <typename TP, int NR, int PC>
__global__ void __launch_bounds__(kThreads) k_update_p(PcgArgs A) {
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (cta_done<NR>(A, S)) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= A.n_rows) return;
#pragma unroll
    for (int k = 0; k < NR; ++k) {
        if (S[k].done) continue;
        const double beta = S[k].beta;
        const size_t o = (size_t)k * A.n_dof + 3 * (size_t)row;
        double rv[3] = {A.r[o], A.r[o + 1], A.r[o + 2]}, z[3];
        precond<PC>(A, row, rv, z);
        typename ApOf<TP>::T pv[3];
        PadVec<TP>::load(A.p, (size_t)k * A.n_rows + row, pv);
        double pn[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) pn[a] = z[a] + beta * (double)pv[a];
        PadVec<TP>::store(A.p, (size_t)k * A.n_rows + row, pn);
    }
}

// True FP64 residual r = b - A64 x (x in natural layout), z = M r, dots.
// mode 0 = initialise (p = z, bb, target), mode 1 = replace for RHS with
// sc.replace set (p kept).
template <typename TP, int NR, int PC>
__global__ void __launch_bounds__(kThreads) k_residual(PcgArgs A, int mode, double tol2) {
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (mode == 1) {  // nothing to replace in this instance (the same answer in all its CTAs)
        bool any = false;
#pragma unroll
        for (int k = 0; k < NR; ++k) any |= (S[k].replace != 0);
        if (!any) return;
    }
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = row & 31;
    double d[NR][3];
#pragma unroll
    for (int k = 0; k < NR; ++k) d[k][0] = d[k][1] = d[k][2] = 0.0;
    if (row < A.n_rows) {
        double y[NR][3];
#pragma unroll
        for (int k = 0; k < NR; ++k) y[k][0] = y[k][1] = y[k][2] = 0.0;
        const int64_t g0 = A.slice_off[row >> 5];
        const int len = A.row_len[row];
        for (int j = 0; j < len; ++j) {
            const int64_t g = g0 + j;
            const int c = A.col[g * 32 + lane];
            const double* v = A.v64 + (g * 9) * 32 + lane;
            double m[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) m[q] = v[q * 32];
#pragma unroll
            for (int k = 0; k < NR; ++k) {
                const double* xk = A.x + (size_t)k * A.n_dof + 3 * (size_t)c;
                const double x0 = xk[0], x1 = xk[1], x2 = xk[2];
#pragma unroll
                for (int a = 0; a < 3; ++a) y[k][a] = fma(m[a * 3], x0, fma(m[a * 3 + 1], x1, fma(m[a * 3 + 2], x2, y[k][a])));
            }
        }
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            if (mode == 1 && !S[k].replace) continue;
            const size_t o = (size_t)k * A.n_dof + 3 * (size_t)row;
            double rv[3], z[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                rv[a] = A.f[o + a] - y[k][a];
                A.r[o + a] = rv[a];
            }
            precond<PC>(A, row, rv, z);
            // initial residual, or a replacement after the recurrence converged
            // (the last p update was skipped): restart the direction p = z
            if (mode == 0 || S[k].restart) PadVec<TP>::store(A.p, (size_t)k * A.n_rows + row, z);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                d[k][0] += rv[a] * z[a];
                d[k][1] += rv[a] * rv[a];
                d[k][2] += A.f[o + a] * A.f[o + a];
            }
        }
    }
    double tot[NR][3];
    if (last_block_reduce<NR, 3>(A, d, 2, tot) && threadIdx.x == 0) {
        int all = 1;
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            RhsScalars& s = S[k];
            if (mode == 0 || s.replace) {
                s.rz = tot[k][0];
                s.rr = tot[k][1];
                s.rr_last_true = tot[k][1];
                if (mode == 0) {
                    s.bb = tot[k][2];
                    s.target = tol2 * s.bb;
                    s.iter = 0;
                    s.beta = 0.0;
                }
                s.replace = 0;
                s.restart = 0;
                s.nonfinite = (!isfinite(s.rr) || !isfinite(s.rz)) ? 1 : 0;
                s.finished = (s.rr <= s.target) || s.nonfinite;
                s.done = s.finished;
            }
            all &= s.done;
        }
        if (!A.cta_inst) A.ctl->all_done = all;
    }
}

// Device-side replacement request, captured at the end of each graph chunk:
// every right-hand side whose recurrence converged (or, mixed method, dropped
// far below its last true residual: both set done) but that is not finished
// gets its true residual formed by the k_residual(mode 1) that follows, with
// no host round trip.
__global__ void k_mark_replace(RhsScalars* sc, int n_slots, int nr) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_slots || q % kMaxRhs >= nr) return;
    RhsScalars& s = sc[q];
    if (s.done && !s.finished && !s.nonfinite) {
        s.replace = 1;
        s.n_repl += 1;
    }
}

// apply helpers (tests / timing)
template <typename TP>
__global__ void k_pack(int n_rows, const double* __restrict__ x, void* p) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    double v[3] = {x[3 * (size_t)row], x[3 * (size_t)row + 1], x[3 * (size_t)row + 2]};
    PadVec<TP>::store(p, row, v);
}
template <typename TV, typename TP>
__global__ void __launch_bounds__(kThreads) k_spmv_plain(PcgArgs A, double* __restrict__ y) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= A.n_rows) return;
    typename ApOf<TP>::T acc[1][3];
    const TV* vals;
    if constexpr (sizeof(TV) == 4) vals = A.v32; else vals = A.v64;
    spmv_row<TV, TP, 1>(row, A, vals, A.p, acc);
    typename ApOf<TP>::T* out = reinterpret_cast<typename ApOf<TP>::T*>(A.ap) + 3 * (size_t)row;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        out[a] = acc[0][a];
        if (y) y[3 * (size_t)row + a] = (double)acc[0][a];
    }
}

__global__ void k_jacobi(int n_rows, const int64_t* __restrict__ slice_off, const uint8_t* __restrict__ diag,
                         const double* __restrict__ v64, double* __restrict__ dinv) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    const int64_t g = slice_off[row >> 5] + diag[row];
    const int lane = row & 31;
#pragma unroll
    for (int a = 0; a < 3; ++a) dinv[3 * (size_t)row + a] = 1.0 / v64[(g * 9 + a * 4) * 32 + lane];
}

__global__ void k_block_inv(int n_rows, const int64_t* __restrict__ slice_off, const uint8_t* __restrict__ diag,
                            const double* __restrict__ v64, float* __restrict__ binv) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    const int64_t g = slice_off[row >> 5] + diag[row];
    const int lane = row & 31;
    double m[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) m[q] = v64[(g * 9 + q) * 32 + lane];
    // symmetric positive definite 3x3 block: inverse by cofactors
    const double c00 = m[4] * m[8] - m[5] * m[7];
    const double c01 = m[5] * m[6] - m[3] * m[8];
    const double c02 = m[3] * m[7] - m[4] * m[6];
    const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    const double id = 1.0 / det;
    double inv[9];
    inv[0] = c00 * id;
    inv[1] = (m[2] * m[7] - m[1] * m[8]) * id;
    inv[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    inv[3] = c01 * id;
    inv[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    inv[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    inv[6] = c02 * id;
    inv[7] = (m[1] * m[6] - m[0] * m[7]) * id;
    inv[8] = (m[0] * m[4] - m[1] * m[3]) * id;
#pragma unroll
    for (int q = 0; q < 9; ++q) binv[9 * (size_t)row + q] = (float)inv[q];
}

int grid_rows(int n_rows) { return (n_rows + kThreads - 1) / kThreads; }

struct Launcher {
    Ctx& c;
    PcgArgs a;
    int method, pc, nr;
    template <typename TP, int NR, int PC>
    void iter_t() {
        const int g = grid_rows(a.n_rows);
        if constexpr (std::is_same<TP, float>::value) k_spmv_dot<float, float, NR><<<g, kThreads, 0, c.stream>>>(a);
        else if constexpr (std::is_same<TP, SplitP>::value)
            k_spmv_dot<float, SplitP, NR><<<g, kThreads, 0, c.stream>>>(a);
        else k_spmv_dot<double, double, NR><<<g, kThreads, 0, c.stream>>>(a);
        k_update_xr<TP, NR, PC><<<g, kThreads, 0, c.stream>>>(a);
        k_update_p<TP, NR, PC><<<g, kThreads, 0, c.stream>>>(a);
    }
    template <typename TP, int NR, int PC>
    void resid_t(int mode, double tol2) {
        k_residual<TP, NR, PC><<<grid_rows(a.n_rows), kThreads, 0, c.stream>>>(a, mode, tol2);
    }
    template <typename TP, int NR>
    void dispatch_pc(bool iter, int mode, double tol2) {
        if (pc == ASEND_PC_JACOBI) {
            if (iter) iter_t<TP, NR, ASEND_PC_JACOBI>(); else resid_t<TP, NR, ASEND_PC_JACOBI>(mode, tol2);
        } else {
            if (iter) iter_t<TP, NR, ASEND_PC_BLOCK>(); else resid_t<TP, NR, ASEND_PC_BLOCK>(mode, tol2);
        }
    }
    template <typename TP>
    void dispatch_nr(bool iter, int mode, double tol2) {
        switch (nr) {
            case 1: dispatch_pc<TP, 1>(iter, mode, tol2); break;
            case 2: dispatch_pc<TP, 2>(iter, mode, tol2); break;
            case 3: dispatch_pc<TP, 3>(iter, mode, tol2); break;
            default: dispatch_pc<TP, 4>(iter, mode, tol2); break;
        }
    }
    void iteration() {  // launches are counted per graph launch
        if (method == ASEND_METHOD_MIXED) dispatch_nr<float>(true, 0, 0.0);
        else if (method == ASEND_METHOD_SPLIT) dispatch_nr<SplitP>(true, 0, 0.0);
        else dispatch_nr<double>(true, 0, 0.0);
    }
    void residual(int mode, double tol2) {
        if (method == ASEND_METHOD_MIXED) dispatch_nr<float>(false, mode, tol2);
        else if (method == ASEND_METHOD_SPLIT) dispatch_nr<SplitP>(false, mode, tol2);
        else dispatch_nr<double>(false, mode, tol2);
        c.launches += 1;
    }
    // end of a graph chunk: replacement requests and the true residuals they ask for
    void chunk_tail(int n_slots) {
        k_mark_replace<<<(n_slots + 127) / 128, 128, 0, c.stream>>>(a.sc, n_slots, nr);
        residual(1, 0.0);
    }
};

}  // namespace

// Device-side y = A x (natural layout), value precision 32, 64 or 48 (the
// split FP32 hi + lo product, FP64-accurate).
void apply_operator_device(Ctx& c, int precision, const double* d_x, double* d_y) {
    ensure_v64(c);
    PcgArgs a{};
    a.n_rows = c.A.n_rows;
    a.nrhs = 1;
    a.n_dof = c.n_dof;
    a.slice_off = c.A.slice_off.p;
    a.row_len = c.A.row_len.p;
    a.col = c.A.col.p;
    a.v32 = c.A.v32.p;
    a.v32lo = c.A.v32lo.p;
    a.v64 = c.A.v64.p;
    const int g = grid_rows(a.n_rows);
    if (precision == 48) {
        DArr<double> p, ap;
        p.alloc((size_t)4 * a.n_rows);
        ap.alloc(c.n_dof);
        a.p = p.p;
        a.ap = ap.p;
        k_pack<SplitP><<<g, kThreads, 0, c.stream>>>(a.n_rows, d_x, p.p);
        k_spmv_plain<float, SplitP><<<g, kThreads, 0, c.stream>>>(a, d_y);
        ASEND_CUDA(cudaGetLastError());
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
    } else if (precision == 32) {
        DArr<float> p, ap;
        p.alloc((size_t)4 * a.n_rows);
        ap.alloc(c.n_dof);
        a.p = p.p;
        a.ap = ap.p;
        k_pack<float><<<g, kThreads, 0, c.stream>>>(a.n_rows, d_x, p.p);
        k_spmv_plain<float, float><<<g, kThreads, 0, c.stream>>>(a, d_y);
        ASEND_CUDA(cudaGetLastError());
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
    } else {
        DArr<double> p, ap;
        p.alloc((size_t)4 * a.n_rows);
        ap.alloc(c.n_dof);
        a.p = p.p;
        a.ap = ap.p;
        k_pack<double><<<g, kThreads, 0, c.stream>>>(a.n_rows, d_x, p.p);
        k_spmv_plain<double, double><<<g, kThreads, 0, c.stream>>>(a, d_y);
        ASEND_CUDA(cudaGetLastError());
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
    }
    c.launches += 2;
}

// Mean time of n_launch SpMV launches (the PCG's dominant kernel) and its
// algorithmic bytes: values + column indices + one read of the direction +
// one write of A p.
double time_spmv(Ctx& c, int precision, int n_launch, double* bytes) {
    ensure_v64(c);
    const int n = c.A.n_rows;
    PcgArgs a{};
    a.n_rows = n;
    a.nrhs = 1;
    a.n_dof = c.n_dof;
    a.slice_off = c.A.slice_off.p;
    a.row_len = c.A.row_len.p;
    a.col = c.A.col.p;
    a.v32 = c.A.v32.p;
    a.v32lo = c.A.v32lo.p;
    a.v64 = c.A.v64.p;
    const int g = grid_rows(n);
    const int64_t blocks = c.A.nnz_scalar() / 9;
    const size_t vsz = (precision == 32) ? 4 : 8;  // split: hi + lo, 8 bytes per value
    *bytes = (double)blocks * (9.0 * vsz + 4.0) + (double)n * (4.0 * vsz) + (double)c.n_dof * vsz;
    std::vector<double> ones(c.n_dof, 1.0);
    DArr<double> x;
    x.upload(ones, c.stream);
    DArr<char> p, ap;
    p.alloc((size_t)4 * n * vsz);
    ap.alloc((size_t)c.n_dof * vsz);
    a.p = p.p;
    a.ap = ap.p;
    if (precision == 32) k_pack<float><<<g, kThreads, 0, c.stream>>>(n, x.p, p.p);
    else if (precision == 48) k_pack<SplitP><<<g, kThreads, 0, c.stream>>>(n, x.p, p.p);
    else k_pack<double><<<g, kThreads, 0, c.stream>>>(n, x.p, p.p);
    auto launch = [&]() {
        if (precision == 32) k_spmv_plain<float, float><<<g, kThreads, 0, c.stream>>>(a, nullptr);
        else if (precision == 48) k_spmv_plain<float, SplitP><<<g, kThreads, 0, c.stream>>>(a, nullptr);
        else k_spmv_plain<double, double><<<g, kThreads, 0, c.stream>>>(a, nullptr);
    };
    for (int w = 0; w < 3; ++w) launch();
    ASEND_CUDA(cudaEventRecord(c.ev0, c.stream));
    for (int i = 0; i < n_launch; ++i) launch();
    ASEND_CUDA(cudaEventRecord(c.ev1, c.stream));
    ASEND_CUDA(cudaEventSynchronize(c.ev1));
    ASEND_CUDA(cudaGetLastError());
    float ms = 0.f;
    ASEND_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.launches += n_launch + 4;
    return ms / n_launch;
}

// Batched PCG over all load cases (chunks of up to 4 sharing one matrix read).
int pcg_solve(Ctx& c, const asend_solve_opts& o, asend_solve_stats* st, bool warm, const double* d_f,
              double* d_x, int nrhs_all) {
    if (o.method != ASEND_METHOD_FP64 && o.method != ASEND_METHOD_MIXED && o.method != ASEND_METHOD_SPLIT)
        throw InputError("unknown method");
    if (!(o.rel_tol > 0.0)) throw InputError("rel_tol must be positive");
    if (o.precond == ASEND_PC_MG || o.precond == ASEND_PC_MG_LEARNED) {
        if (o.precond == ASEND_PC_MG_LEARNED && !learned_ready(c)) throw InputError("no learned weights");
        return pcg_solve_mg(c, o, st, warm, d_f, d_x, nrhs_all);  // keeps a split-only operator as pairs
    }
    ensure_v64(c);
    int pc = o.precond;
    bool use_learned = false;
    if (pc == ASEND_PC_LEARNED) {
        if (learned_ready(c)) {
            // learned nodal blocks through the block-Jacobi kernels; on a
            // non-finite or non-converged solve the plain Jacobi PCG is rerun
            // from zero and judges convergence
            use_learned = true;
            pc = ASEND_PC_BLOCK;
        } else {
            asend_solve_opts oj = o;
            oj.precond = ASEND_PC_JACOBI;
            const int rc = pcg_solve(c, oj, st, warm, d_f, d_x, nrhs_all);
            if (rc == ASEND_OK) {
                if (st) st->status = ASEND_FALLBACK;
                return ASEND_FALLBACK;
            }
            return rc;
        }
    }
    if (pc != ASEND_PC_JACOBI && pc != ASEND_PC_BLOCK) throw InputError("unknown preconditioner");
    if (!(o.rel_tol > 0.0)) throw InputError("rel_tol must be positive");
    const int n = c.A.n_rows, nd = c.n_dof;
    const int max_it = o.max_iter > 0 ? o.max_iter : nd;
    const int G = o.graph_iters > 0 ? o.graph_iters : 16;
    const size_t tot = (size_t)nrhs_all * nd;
    if (!warm) ASEND_CUDA(cudaMemsetAsync(d_x, 0, tot * sizeof(double), c.stream));
    c.d_r.alloc(std::max(c.d_r.n, tot));
    const int grid = grid_rows(n);
    c.d_partials.alloc((size_t)grid * kMaxRhs * 3);
    // preconditioner
    if (pc == ASEND_PC_JACOBI) {
        if (c.dinv_epoch != c.assembly_epoch || c.d_dinv.n != (size_t)nd) {  // once per assembly
            c.d_dinv.alloc(nd);
            k_jacobi<<<grid, kThreads, 0, c.stream>>>(n, c.A.slice_off.p, c.A.diag.p, c.A.v64.p, c.d_dinv.p);
            ++c.launches;
            c.dinv_epoch = c.assembly_epoch;
        }
    } else {
        c.d_binv.alloc((size_t)9 * n);
        if (use_learned) {
            learned_blocks(c, c.d_binv.p, true);
        } else {
            k_block_inv<<<grid, kThreads, 0, c.stream>>>(n, c.A.slice_off.p, c.A.diag.p, c.A.v64.p, c.d_binv.p);
            ++c.launches;
        }
    }
    const bool mixed = o.method == ASEND_METHOD_MIXED;
    if (mixed) {
        c.d_p32.alloc((size_t)kMaxRhs * 4 * n);
        c.d_ap32.alloc((size_t)kMaxRhs * nd);
    } else {  // FP64: 2 x double2 per node; split: hi + lo float4 per node (same bytes)
        c.d_p64.alloc((size_t)kMaxRhs * 4 * n);
        c.d_ap64.alloc((size_t)kMaxRhs * nd);
    }
    // independent instances: one scalar set per (instance, load case)
    const int NI = c.n_inst > 1 ? c.n_inst : 1;
    // persistent scalar buffers (grow only), so repeated solves with the same
    // vectors reuse the captured iteration graph
    const size_t sc_need = sizeof(RhsScalars) * NI * kMaxRhs, tk_need = sizeof(uint32_t) * NI * 4;
    if (c.pcg_sc.n < sc_need) c.pcg_sc.alloc(sc_need);
    if (c.pcg_ctl.n < sizeof(Control)) c.pcg_ctl.alloc(sizeof(Control));
    if (NI > 1 && c.pcg_tk.n < tk_need) c.pcg_tk.alloc(tk_need);
    RhsScalars* d_sc_p = reinterpret_cast<RhsScalars*>(c.pcg_sc.p);
    Control* d_ctl_p = reinterpret_cast<Control*>(c.pcg_ctl.p);
    uint32_t* d_tk_p = reinterpret_cast<uint32_t*>(c.pcg_tk.p);
    ensure_pinned_scalars(c, sizeof(RhsScalars) * NI * kMaxRhs);
    RhsScalars* h_sc = reinterpret_cast<RhsScalars*>(c.h_sc);
    const size_t sc_bytes = sizeof(RhsScalars) * NI * kMaxRhs;
    int iters_max = 0, repl_total = 0, status = 0;
    double relres_max = 0.0;
    if (c.time_solves) ASEND_CUDA(cudaEventRecord(c.ev0, c.stream));
    for (int r0 = 0; r0 < nrhs_all; r0 += kMaxRhs) {
        const int nr = std::min(kMaxRhs, nrhs_all - r0);
        Launcher L{c, PcgArgs{}, o.method, pc, nr};
        PcgArgs& a = L.a;
        std::memset(&a, 0, sizeof(PcgArgs));  // padding too: the bytes key the cached graph
        a.n_rows = n;
        a.nrhs = nr;
        a.n_dof = nd;
        a.slice_off = c.A.slice_off.p;
        a.row_len = c.A.row_len.p;
        a.col = c.A.col.p;
        a.v32 = c.A.v32.p;
        a.v32lo = c.A.v32lo.p;
        a.v64 = c.A.v64.p;
        a.f = d_f + (size_t)r0 * nd;
        a.x = d_x + (size_t)r0 * nd;
        a.r = c.d_r.p + (size_t)r0 * nd;
        a.p = mixed ? (void*)c.d_p32.p : (void*)c.d_p64.p;
        a.ap = mixed ? (void*)c.d_ap32.p : (void*)c.d_ap64.p;
        a.dinv = c.d_dinv.p;
        a.binv = c.d_binv.p;
        a.partials = c.d_partials.p;
        a.sc = d_sc_p;
        a.ctl = d_ctl_p;
        if (NI > 1) {
            a.cta_inst = c.d_cta_inst.p;
            a.inst_cta0 = c.d_inst_cta0.p;
            a.inst_ncta = c.d_inst_ncta.p;
            a.tickets = d_tk_p;
            ASEND_CUDA(cudaMemsetAsync(d_tk_p, 0, tk_need, c.stream));
        }
        ASEND_CUDA(cudaMemsetAsync(d_sc_p, 0, sc_need, c.stream));
        ASEND_CUDA(cudaMemsetAsync(d_ctl_p, 0, sizeof(Control), c.stream));
        L.residual(0, o.rel_tol * o.rel_tol);
        ASEND_CUDA(cudaGetLastError());
        // G iterations as one graph; the executable is kept and reused while
        // the launch arguments are the same (they fully define the graph)
        std::vector<uint8_t> key(sizeof(PcgArgs) + 4 * sizeof(int));
        std::memcpy(key.data(), &a, sizeof(PcgArgs));
        const int extra[4] = {o.method, pc, nr, G};
        std::memcpy(key.data() + sizeof(PcgArgs), extra, sizeof(extra));
        if (!c.graph || key != c.graph_key) {
            if (c.graph) ASEND_CUDA(cudaGraphExecDestroy(c.graph));
            c.graph = nullptr;
            cudaGraph_t graph;
            ASEND_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            for (int i = 0; i < G; ++i) L.iteration();
            L.chunk_tail(NI * kMaxRhs);
            ASEND_CUDA(cudaStreamEndCapture(c.stream, &graph));
            ASEND_CUDA(cudaGraphInstantiate(&c.graph, graph, 0));
            ASEND_CUDA(cudaGraphDestroy(graph));
            c.graph_key = key;
        }
        cudaGraphExec_t exec = c.graph;
        // One host check per graph chunk: the chunk ends with the device-side
        // replacement of converged recurrences, so a typical solve (or a
        // Newmark step) is the initial residual, one chunk and one check.
        int since_repl = 0;
        bool chunk = true;
        for (;;) {
            if (chunk) {
                ASEND_CUDA(cudaGraphLaunch(exec, c.stream));
                c.launches += 3 * G + 2;
                since_repl += G;
            }
            chunk = true;
            ASEND_CUDA(cudaMemcpyAsync(h_sc, d_sc_p, sc_bytes, cudaMemcpyDeviceToHost, c.stream));
            ASEND_CUDA(cudaStreamSynchronize(c.stream));
            bool all_finished = true, any_replace = false, any_nonfinite = false;
            int it_now = 0;
            for (int q = 0; q < NI * kMaxRhs; ++q) {
                if (q % kMaxRhs >= nr) continue;
                RhsScalars& s = h_sc[q];
                it_now = std::max(it_now, (int)s.iter);
                if (s.nonfinite) { any_nonfinite = true; continue; }
                if (s.finished) continue;
                all_finished = false;
                if (o.replace_every > 0 && since_repl >= o.replace_every) {  // periodic, on request
                    s.replace = 1;
                    any_replace = true;
                }
            }
            if (any_nonfinite) { status = ASEND_NONFINITE; break; }
            if (all_finished) break;
            if (it_now >= max_it) { status = std::max(status, (int)ASEND_MAX_ITER); break; }
            if (any_replace) {
                ASEND_CUDA(cudaMemcpyAsync(d_sc_p, h_sc, sc_bytes, cudaMemcpyHostToDevice, c.stream));
                L.residual(1, 0.0);
                ++repl_total;
                since_repl = 0;
                chunk = false;  // re-check (a replaced RHS may now be finished)
            }
        }
        // h_sc holds the scalars read at the loop's last check
        for (int q = 0; q < NI * kMaxRhs; ++q) {
            if (q % kMaxRhs >= nr) continue;
            const RhsScalars& s = h_sc[q];
            iters_max = std::max(iters_max, (int)s.iter);
            repl_total += s.n_repl;
            if (s.bb == 0.0) continue;  // empty load case of this instance
            relres_max = std::max(relres_max, std::sqrt(s.rr_last_true / s.bb));
            if (s.nonfinite) status = ASEND_NONFINITE;
            else if (!s.finished) status = std::max(status, (int)ASEND_MAX_ITER);
        }
    }
    float ms = 0.f;
    if (c.time_solves) {  // (a Newmark run times its whole loop instead)
        ASEND_CUDA(cudaEventRecord(c.ev1, c.stream));
        ASEND_CUDA(cudaEventSynchronize(c.ev1));
        ASEND_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    }
    ASEND_CUDA(cudaGetLastError());
    c.last_method = o.method;
    if (st) {
        st->iterations = iters_max;
        st->status = status;
        st->replacements = repl_total;
        st->n_rhs = nrhs_all;
        st->rel_residual = relres_max;
        st->ms_solve = ms;
        st->ms_assemble = c.last_assemble_ms;
        st->penalty_scale = c.sf;
    }
    if (use_learned && (status == ASEND_NONFINITE || status == ASEND_MAX_ITER)) {
        asend_solve_opts oj = o;
        oj.precond = ASEND_PC_JACOBI;
        const int rc = pcg_solve(c, oj, st, false, d_f, d_x, nrhs_all);
        status = rc == ASEND_OK ? ASEND_FALLBACK : rc;
    }
    if (st) st->status = status;
    return status;
}

}  // namespace asend
