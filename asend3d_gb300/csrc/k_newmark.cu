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

__global__ void k_probe(const double* __restrict__ u, int dof, double* __restrict__ hist, int step) {
    if (threadIdx.x == 0 && blockIdx.x == 0) hist[step] = u[dof];
}

}  // namespace

int newmark_run(Ctx& c, const asend_solve_opts& o, int n_steps, const double* amp, int probe, double* probe_hist,
                double* u_final, asend_solve_stats* st) {
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

}  // namespace asend
