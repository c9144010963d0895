// k_newmark.cu -- K5: Newmark transient loop (fused predictor/corrector).
//
// Reference (solverSrc/asend_run_job/src/):
//   Model::solve dynamic loop, model_analysis.rs:591-624: for time = 0, dt, ...
//     solve_step(time) -> load = f(time) - R(u, v, a) + penalty load
//     (R = K u + M a + D v, element_equations.rs:852-1062), solve
//     K_eff du = load, u += du, update_vel_acc (corrector);
//     then advance_disp (prev := current) and update_vel_acc (predictor).
//   Node::update_vel_acc node_meth.rs:127-138:
//     a = c1 (u_prev - u + dt v_prev + c2 a_prev), c1 = 1/(dt^2 (beta - gamma)),
//     c2 = dt^2 (0.5 + beta - gamma); v = v_prev + dt ((1 - gamma) a_prev + gamma a).
//   With the operator A = K + c_M M + c_D D + sf C^T C (c_M = -c1, c_D =
//   dt gamma c_M, element_equations.rs:977-1005), the step load is
//     b(t) - A u - M (a - c_M u) - D (v - c_D u),  b(t) = amp(t) f0 + sf C^T q.
//
// GB300 design: the step right-hand side is one fused FP64 pass over the
// operator and mass values (same slots, one column-index read); the
// corrector, history shift and next predictor are one streaming FP64 kernel
// over (u, v, a, u_prev, v_prev, a_prev); each step's PCG starts from the
// previous step's increment, or (opts.warm_start == 2) from the linear
// extrapolation of the two previous increments.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace asend {
namespace {

__global__ void __launch_bounds__(128)
k_dyn_residual(int n_rows, int n_dof, const int64_t* __restrict__ slice_off, const uint8_t* __restrict__ row_len,
               const int32_t* __restrict__ col, const double* __restrict__ v64, const double* __restrict__ m64,
               double cM, double amp, const double* __restrict__ f0, const double* __restrict__ pen,
               const double* __restrict__ u, const double* __restrict__ a, double* __restrict__ out,
               const double* __restrict__ d64, const double* __restrict__ v, double cD) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    const int lane = row & 31;
    const int64_t g0 = slice_off[row >> 5];
    const int len = row_len[row];
    double y[3] = {0, 0, 0};
    for (int j = 0; j < len; ++j) {
        const int64_t g = g0 + j;
        const int c = col[g * 32 + lane];
        const double u0 = u[3 * (size_t)c], u1 = u[3 * (size_t)c + 1], u2 = u[3 * (size_t)c + 2];
        const double w0 = a[3 * (size_t)c] - cM * u0, w1 = a[3 * (size_t)c + 1] - cM * u1,
                     w2 = a[3 * (size_t)c + 2] - cM * u2;
        const double* kv = v64 + (g * 9) * 32 + lane;
        const double* mv = m64 + (g * 9) * 32 + lane;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            y[r] += kv[(3 * r) * 32] * u0 + kv[(3 * r + 1) * 32] * u1 + kv[(3 * r + 2) * 32] * u2;
            y[r] += mv[(3 * r) * 32] * w0 + mv[(3 * r + 1) * 32] * w1 + mv[(3 * r + 2) * 32] * w2;
        }
        if (d64) {  // + D (v - cD u): the damping force D v without its operator share
            const double z0 = v[3 * (size_t)c] - cD * u0, z1 = v[3 * (size_t)c + 1] - cD * u1,
                         z2 = v[3 * (size_t)c + 2] - cD * u2;
            const double* dv = d64 + (g * 9) * 32 + lane;
#pragma unroll
            for (int r = 0; r < 3; ++r) y[r] += dv[(3 * r) * 32] * z0 + dv[(3 * r + 1) * 32] * z1 + dv[(3 * r + 2) * 32] * z2;
        }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const size_t i = 3 * (size_t)row + r;
        out[i] = amp * f0[i] + pen[i] - y[r];
    }
}

// Corrector (u += du; a, v from update_vel_acc), history shift (advance_disp)
// and the next step's predictor (update_vel_acc with u = u_prev).
__global__ void k_newmark_update(int n, double dt, double gamma, double c1, double c2,
                                 const double* __restrict__ du, double* __restrict__ u, double* __restrict__ v,
                                 double* __restrict__ a, double* __restrict__ up, double* __restrict__ vp,
                                 double* __restrict__ ap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double un = u[i] + du[i];
    const double upi = up[i], vpi = vp[i], api = ap[i];
    const double an = c1 * (upi - un + dt * vpi + c2 * api);
    const double vn = vpi + dt * ((1.0 - gamma) * api + gamma * an);
    // advance: prev := current
    up[i] = un;
    vp[i] = vn;
    ap[i] = an;
    // predictor with u == u_prev
    const double a2 = c1 * (dt * vn + c2 * an);
    u[i] = un;
    a[i] = a2;
    v[i] = vn + dt * ((1.0 - gamma) * an + gamma * a2);
}

// Initial guess of the step's increment by linear extrapolation of the two
// previous increments: du := 2 du - du_prev, du_prev := the old du.
__global__ void k_extrapolate(int n, double* __restrict__ du, double* __restrict__ du_prev) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = du[i];
    du[i] = 2.0 * d - du_prev[i];
    du_prev[i] = d;
}

// y = A x for an FP64 SBELL value array (the mass in the adjoint sweep)
__global__ void __launch_bounds__(128) k_sbell_apply64(int n_rows, const int64_t* __restrict__ slice_off,
                                                       const uint8_t* __restrict__ row_len,
                                                       const int32_t* __restrict__ col, const double* __restrict__ vals,
                                                       const double* __restrict__ x, double* __restrict__ y) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    const int lane = row & 31;
    const int64_t g0 = slice_off[row >> 5];
    const int len = row_len[row];
    double acc[3] = {0, 0, 0};
    for (int j = 0; j < len; ++j) {
        const int64_t g = g0 + j;
        const int cn = col[g * 32 + lane];
        const double x0 = x[3 * (size_t)cn], x1 = x[3 * (size_t)cn + 1], x2 = x[3 * (size_t)cn + 2];
        const double* v = vals + (g * 9) * 32 + lane;
#pragma unroll
        for (int r = 0; r < 3; ++r) acc[r] += v[(3 * r) * 32] * x0 + v[(3 * r + 1) * 32] * x1 + v[(3 * r + 2) * 32] * x2;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) y[3 * (size_t)row + r] = acc[r];
}

// One step of the reverse Newmark sweep (the adjoint of update_vel_acc and
// of the coupling to the next step, augmentd_ld_u model_analysis.rs:936-1063
// and solve_for_adjoint :1065-1126): from the next step's adjoints (mu =
// M u_adj) form dL/du, dL/dv, dL/da, then v_adj = dL/dv, a_adj = dL/da +
// dt gamma v_adj and the right-hand side dL/du - d_ad_up a_adj of this step's
// operator solve.  w: the step's objective weights (dense).
__global__ void k_adjoint_step(int n, int first, double d_ad_up, double d_ad_vp, double d_ad_ap, double c3, double c4,
                               double dt_gamma, const double* __restrict__ mu, const double* __restrict__ w,
                               double* __restrict__ v_adj, double* __restrict__ a_adj, double* __restrict__ rhs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double du = w[i], dv = 0.0, da = 0.0;
    if (!first) {
        const double m = mu[i], aa = a_adj[i], vv = v_adj[i];
        du += -d_ad_up * m + d_ad_up * aa;
        da = -d_ad_ap * m + d_ad_ap * aa + c3 * vv;
        dv = -d_ad_vp * m + c4 * aa + vv;
    }
    const double vn = dv, an = da + dt_gamma * vn;
    v_adj[i] = vn;
    a_adj[i] = an;
    rhs[i] = du - d_ad_up * an;
}

__global__ void k_probe(const double* __restrict__ u, int dof, double* __restrict__ hist, int step) {
    if (threadIdx.x == 0 && blockIdx.x == 0) hist[step] = u[dof];
}

}  // namespace

int newmark_run(Ctx& c, const asend_solve_opts& o, int n_steps, const double* amp, int probe, double* probe_hist,
                double* u_final, asend_solve_stats* st) {
    ensure_v64(c);
    const int n = c.n_dof;
    const double dt = c.dt, beta = c.beta, gamma = c.gamma;
    const double c1 = 1.0 / (dt * dt * (beta - gamma));
    const double c2 = dt * dt * (0.5 + beta - gamma);
    upload_rhs(c);  // case 0 = f0 (+ penalty rhs); pen part isolated below
    std::vector<double> pen(n, 0.0);
    {
        const int nrow_c = (int)c.c_rhs.size();
        for (int q = 0; q < nrow_c; ++q)
            for (int k = c.c_ptr[q]; k < c.c_ptr[q + 1]; ++k)
                pen[c.c_dof[k]] += c.c_coef[k] * row_penalty_scale(c, q) * c.c_rhs[q];
    }
    DArr<double> d_f0, d_pen, u, v, a, up, vp, ap, du, du_prev, rhs, hist;
    d_f0.upload(c.loads.empty() ? std::vector<double>(n, 0.0) : c.loads[0], c.stream);
    d_pen.upload(pen, c.stream);
    for (DArr<double>* z : {&u, &v, &a, &up, &vp, &ap, &du, &du_prev, &rhs}) {
        z->alloc(n);
        z->zero(c.stream);
    }
    hist.alloc(std::max(1, n_steps));
    c.hist_steps = 0;
    if (c.hist_fields > 0) {
        c.d_hist.alloc((size_t)n_steps * c.hist_fields * n);
        c.hist_steps = n_steps;
        c.hist_dt = dt;
    }
    hist.zero(c.stream);
    // prep predictor (model_prep.rs:584-590): all zero initial state -> zeros
    const int rows = c.A.n_rows;
    const int g_rows = (rows + 127) / 128, g_dof = (n + 255) / 256;
    asend_solve_opts so = o;
    int iters_total = 0, status = 0;
    double relmax = 0.0;
    ASEND_CUDA(cudaEventRecord(c.ev0, c.stream));
    cudaEvent_t e0, e1;
    ASEND_CUDA(cudaEventCreate(&e0));
    ASEND_CUDA(cudaEventCreate(&e1));
    ASEND_CUDA(cudaEventRecord(e0, c.stream));
    struct TimeSolves {  // per-solve event timing off for the run (restored on every exit)
        Ctx& c;
        bool saved;
        ~TimeSolves() { c.time_solves = saved; }
    } time_guard{c, c.time_solves};
    c.time_solves = false;
    for (int s = 0; s < n_steps; ++s) {
        k_dyn_residual<<<g_rows, 128, 0, c.stream>>>(rows, n, c.A.slice_off.p, c.A.row_len.p, c.A.col.p, c.A.v64.p,
                                                      c.A.m64.p, c.cM, amp[s], d_f0.p, d_pen.p, u.p, a.p, rhs.p,
                                                      c.A.d64.n ? c.A.d64.p : nullptr, v.p, c.cD);
        ASEND_CUDA(cudaGetLastError());
        ++c.launches;
        if (s >= 1 && o.warm_start == 2) {  // extrapolated start (the previous increment at step 1)
            if (s >= 2) {
                k_extrapolate<<<g_dof, 256, 0, c.stream>>>(n, du.p, du_prev.p);
            } else {
                ASEND_CUDA(cudaMemcpyAsync(du_prev.p, du.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
            }
            ++c.launches;
        }
        asend_solve_stats ps{};
        const int rc = pcg_solve(c, so, &ps, s > 0, rhs.p, du.p, 1);
        iters_total += ps.iterations;
        relmax = std::max(relmax, ps.rel_residual);
        if (rc == ASEND_NONFINITE) { status = rc; break; }
        if (rc == ASEND_MAX_ITER) status = rc;
        k_newmark_update<<<g_dof, 256, 0, c.stream>>>(n, dt, gamma, c1, c2, du.p, u.p, v.p, a.p, up.p, vp.p, ap.p);
        ++c.launches;
        if (c.hist_fields > 0) {  // the corrected state of step s + 1 (the solnTStep fields)
            double* h = c.d_hist.p + (size_t)s * c.hist_fields * n;
            ASEND_CUDA(cudaMemcpyAsync(h, up.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
            if (c.hist_fields == 3) {
                ASEND_CUDA(cudaMemcpyAsync(h + n, vp.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
                ASEND_CUDA(cudaMemcpyAsync(h + 2 * (size_t)n, ap.p, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                           c.stream));
            }
        }
        if (probe >= 0) {
            k_probe<<<1, 32, 0, c.stream>>>(u.p, probe, hist.p, s);
            ++c.launches;
        }
    }
    ASEND_CUDA(cudaEventRecord(e1, c.stream));
    ASEND_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    ASEND_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (probe_hist && probe >= 0)
        ASEND_CUDA(cudaMemcpy(probe_hist, hist.p, sizeof(double) * n_steps, cudaMemcpyDeviceToHost));
    if (u_final) ASEND_CUDA(cudaMemcpy(u_final, u.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (st) {
        st->iterations = iters_total;
        st->status = status;
        st->rel_residual = relmax;
        st->ms_solve = ms;
        st->n_rhs = 1;
        st->penalty_scale = c.sf;
    }
    return status;
}

// Reverse Newmark sweep for L = sum_{steps s} sum_k w_k u_s[dof_k] and its
// per-element modulus gradient (Model::get_obj_gradient's transient branch,
// model_analysis.rs:1544-1631, with augmentd_ld_u :936-1063): per step from
// the last, the fused adjoint update, one solve with the step operator
// (warm-started from the later step's adjoint) and the contraction
// dL/dE_e -= u_adj_e^T (K_e / E_e) u_s,e with the stored displacement.  Needs
// the displacement history of the preceding asend_newmark_run.  Undamped,
// consistent-mass, isotropic models (the oracle's restatement covers these).
int newmark_adjoint(Ctx& c, const asend_solve_opts& o, int n_obj, const int32_t* obj_dof, const double* obj_w,
                    double* L_out, double* gE_out, asend_solve_stats* st) {
    const int n = c.n_dof, N = c.hist_steps, F = c.hist_fields;
    const double dt = c.hist_dt, beta = c.beta, gamma = c.gamma;
    const double d_ad_up = 1.0 / (dt * dt * (beta - gamma));
    const double d_ad_vp = d_ad_up * dt;
    const double d_ad_ap = d_ad_up * dt * dt * (0.5 + beta - gamma);
    const double c3 = dt * (1.0 - gamma), c4 = 1.0 / (dt * (beta - gamma));
    std::vector<double> w(n, 0.0);
    double L = 0.0;
    {
        std::vector<double> us(n);
        for (int k = 0; k < n_obj; ++k) w[obj_dof[k]] += obj_w[k];
        // L from the stored displacements at the objective DOFs
        for (int s = 0; s < N; ++s)
            for (int k = 0; k < n_obj; ++k) {
                double v = 0.0;
                ASEND_CUDA(cudaMemcpyAsync(&v, c.d_hist.p + (size_t)s * F * n + obj_dof[k], sizeof(double),
                                           cudaMemcpyDeviceToHost, c.stream));
                ASEND_CUDA(cudaStreamSynchronize(c.stream));
                L += obj_w[k] * v;
            }
    }
    DArr<double> d_w, mu, v_adj, a_adj, rhs, u_adj, gE;
    d_w.upload(w, c.stream);
    for (DArr<double>* z : {&mu, &v_adj, &a_adj, &rhs, &u_adj}) {
        z->alloc(n);
        z->zero(c.stream);
    }
    gE.alloc(c.n_el);
    gE.zero(c.stream);
    const int rows = c.A.n_rows, g_rows = (rows + 127) / 128, g_dof = (n + 255) / 256;
    int iters = 0, status = 0;
    double relmax = 0.0;
    ASEND_CUDA(cudaEventRecord(c.ev0, c.stream));
    struct TimeSolves {  // per-solve event timing off for the sweep (restored on every exit)
        Ctx& c;
        bool saved;
        ~TimeSolves() { c.time_solves = saved; }
    } time_guard{c, c.time_solves};
    c.time_solves = false;
    for (int s = N - 1; s >= 0; --s) {
        const bool first = (s == N - 1);
        if (!first) {
            k_sbell_apply64<<<g_rows, 128, 0, c.stream>>>(rows, c.A.slice_off.p, c.A.row_len.p, c.A.col.p, c.A.m64.p,
                                                          u_adj.p, mu.p);
            ++c.launches;
        }
        k_adjoint_step<<<g_dof, 256, 0, c.stream>>>(n, first ? 1 : 0, d_ad_up, d_ad_vp, d_ad_ap, c3, c4, dt * gamma,
                                                    mu.p, d_w.p, v_adj.p, a_adj.p, rhs.p);
        ++c.launches;
        asend_solve_stats ps{};
        const int rc = pcg_solve(c, o, &ps, !first, rhs.p, u_adj.p, 1);
        iters += ps.iterations;
        relmax = std::max(relmax, ps.rel_residual);
        if (rc == ASEND_NONFINITE) { status = rc; break; }
        if (rc == ASEND_MAX_ITER) status = rc;
        adjoint_contract(c, u_adj.p, c.d_hist.p + (size_t)s * F * n, gE.p, true);
    }
    ASEND_CUDA(cudaEventRecord(c.ev1, c.stream));
    ASEND_CUDA(cudaEventSynchronize(c.ev1));
    float ms = 0.f;
    ASEND_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    if (gE_out) ASEND_CUDA(cudaMemcpy(gE_out, gE.p, sizeof(double) * c.n_el, cudaMemcpyDeviceToHost));
    if (L_out) *L_out = L;
    if (st) {
        std::memset(st, 0, sizeof(*st));
        st->iterations = iters;
        st->status = status;
        st->rel_residual = relmax;
        st->ms_solve = ms;
        st->n_rhs = N;
        st->penalty_scale = c.sf;
    }
    return status;
}

}  // namespace asend
