// k_brickim.cu -- brickIM (type 81) element kernels: hex8 with 9 incompatible
// modes, condensed; consistent mass; coloured scatter; adjoint contraction.
//
// Reference formulation (solverSrc/asend_run_job/src/):
//   element_meth.rs:157-201       type 81: 8 nodes, 2x2x2 points, 9 internal DOF
//                                 (bubble k = 1 - s_k^2 on each displacement component)
//   element_soln_fields.rs:171-227  shape functions; :424-461 the bubbles'
//                                 derivatives at a point use the centroid Jacobian
//   element_soln_fields.rs:1345-1461 small strain, Voigt 11,22,33,12,13,23
//   element_equations.rs:206-418    K = sum B^T C B detJ w (33x33); :19-57 condensation
//   element_equations.rs:583-609    consistent mass over the node DOF only
//
// GB300 mapping: one 64-thread CTA per element, FP64 in shared memory, the
// condensed 24x24 matrix scattered as 8x8 node blocks through the hex slot
// map, one colour at a time (no atomics).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace asend {
namespace {

constexpr int kBT = 64;
constexpr double kG = 0.57735026918962576451;  // 1/sqrt(3)
constexpr int kTot = 33, kNd = 24;

__constant__ int c_sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                               {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};

struct BrickSmem {
    double xyz[8][3];
    double C[6][6];
    double ji[9][9];        // inverse Jacobian per point (8 = centroid)
    double det[8];
    double n[8][8];         // N_a at each point
    double dx[8][11][3];    // dN/dx per point: 8 nodal functions, 3 bubbles
    double B[6][kTot];
    double CB[6][kTot];
    double K[kTot][kTot];
    double Kii[9][9];
    double X[9][kNd];
    double K24[kNd][kNd];
    double rho;
};

__device__ void inv3(const double (&J)[9], double* Ji, double& det) {
    const double c00 = J[4] * J[8] - J[5] * J[7], c01 = J[5] * J[6] - J[3] * J[8], c02 = J[3] * J[7] - J[4] * J[6];
    det = J[0] * c00 + J[1] * c01 + J[2] * c02;
    const double id = 1.0 / det;
    Ji[0] = c00 * id;
    Ji[1] = (J[2] * J[7] - J[1] * J[8]) * id;
    Ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
    Ji[3] = c01 * id;
    Ji[4] = (J[0] * J[8] - J[2] * J[6]) * id;
    Ji[5] = (J[2] * J[3] - J[0] * J[5]) * id;
    Ji[6] = c02 * id;
    Ji[7] = (J[1] * J[6] - J[0] * J[7]) * id;
    Ji[8] = (J[0] * J[4] - J[1] * J[3]) * id;
}

__device__ void brick_element(BrickSmem& S, int e, const int32_t* __restrict__ conn, const double* __restrict__ xyz,
                              const double* __restrict__ Ev, const double* __restrict__ nuv,
                              const double* __restrict__ rhov) {
    const int t = threadIdx.x;
    if (t < 24) S.xyz[t / 3][t % 3] = xyz[3 * (size_t)conn[8 * (size_t)e + t / 3] + t % 3];
    if (t == 24) {
        const double E = Ev[e], nu = nuv[e];
        const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = E / (2.0 * (1.0 + nu));
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) S.C[i][j] = 0.0;
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) S.C[i][j] = lam;
            S.C[i][i] = lam + 2.0 * mu;
            S.C[i + 3][i + 3] = mu;
        }
        S.rho = rhov ? rhov[e] : 0.0;
    }
    __syncthreads();
    if (t < 9) {  // Gauss points (s0 fastest, element_meth.rs:176-189) and the centroid
        double s[3] = {0.0, 0.0, 0.0};
        if (t < 8) {
            s[0] = (t & 1) ? kG : -kG;
            s[1] = (t & 2) ? kG : -kG;
            s[2] = (t & 4) ? kG : -kG;
        }
        double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int a = 0; a < 8; ++a) {
            const double f0 = 1 + c_sg[a][0] * s[0], f1 = 1 + c_sg[a][1] * s[1], f2 = 1 + c_sg[a][2] * s[2];
            const double d0 = 0.125 * c_sg[a][0] * f1 * f2, d1 = 0.125 * c_sg[a][1] * f0 * f2,
                         d2 = 0.125 * c_sg[a][2] * f0 * f1;
            if (t < 8) S.n[t][a] = 0.125 * f0 * f1 * f2;
            for (int i = 0; i < 3; ++i) {
                J[3 * i] += S.xyz[a][i] * d0;
                J[3 * i + 1] += S.xyz[a][i] * d1;
                J[3 * i + 2] += S.xyz[a][i] * d2;
            }
        }
        double det;
        inv3(J, S.ji[t], det);
        if (t < 8) S.det[t] = det;
    }
    for (int q = t; q < kTot * kTot; q += kBT) S.K[q / kTot][q % kTot] = 0.0;
    __syncthreads();
    // dN/dx: nodal functions with the point's Jacobian, bubbles (d/ds_k = -2 s_k)
    // with the centroid's
    for (int q = t; q < 8 * 11; q += kBT) {
        const int ip = q / 11, f = q % 11;
        const double s[3] = {(ip & 1) ? kG : -kG, (ip & 2) ? kG : -kG, (ip & 4) ? kG : -kG};
        double ds[3];
        const double* Ji;
        if (f < 8) {
            const double f0 = 1 + c_sg[f][0] * s[0], f1 = 1 + c_sg[f][1] * s[1], f2 = 1 + c_sg[f][2] * s[2];
            ds[0] = 0.125 * c_sg[f][0] * f1 * f2;
            ds[1] = 0.125 * c_sg[f][1] * f0 * f2;
            ds[2] = 0.125 * c_sg[f][2] * f0 * f1;
            Ji = S.ji[ip];
        } else {
            const int k = f - 8;
            ds[0] = ds[1] = ds[2] = 0.0;
            ds[k] = -2.0 * s[k];
            Ji = S.ji[8];
        }
        for (int j = 0; j < 3; ++j) S.dx[ip][f][j] = ds[0] * Ji[j] + ds[1] * Ji[3 + j] + ds[2] * Ji[6 + j];
    }
    __syncthreads();
    for (int ip = 0; ip < 8; ++ip) {
        if (t < kTot) {  // column t: node t/3 (t < 24) or bubble (t-24)/3, component t%3
            const int f = (t < kNd) ? t / 3 : 8 + (t - kNd) / 3, d = t % 3;
            const double g0 = S.dx[ip][f][0], g1 = S.dx[ip][f][1], g2 = S.dx[ip][f][2];
            double col[6] = {0, 0, 0, 0, 0, 0};
            if (d == 0) { col[0] = g0; col[3] = g1; col[4] = g2; }
            if (d == 1) { col[1] = g1; col[3] = g0; col[5] = g2; }
            if (d == 2) { col[2] = g2; col[4] = g0; col[5] = g1; }
            for (int k = 0; k < 6; ++k) S.B[k][t] = col[k];
        }
        __syncthreads();
        for (int q = t; q < 6 * kTot; q += kBT) {
            const int i = q / kTot, c = q % kTot;
            double acc = 0.0;
            for (int k = 0; k < 6; ++k) acc += S.C[i][k] * S.B[k][c];
            S.CB[i][c] = acc * S.det[ip];
        }
        __syncthreads();
        for (int q = t; q < kTot * kTot; q += kBT) {
            const int r = q / kTot, c = q % kTot;
            double acc = 0.0;
            for (int k = 0; k < 6; ++k) acc += S.B[k][r] * S.CB[k][c];
            S.K[r][c] += acc;
        }
        __syncthreads();
    }
    // condensation of the 9 internal DOF
    for (int q = t; q < 81; q += kBT) S.Kii[q / 9][q % 9] = S.K[kNd + q / 9][kNd + q % 9];
    __syncthreads();
    if (t == 0) {  // in-place Gauss-Jordan inverse of the SPD 9x9 block
        for (int p = 0; p < 9; ++p) {
            const double piv = 1.0 / S.Kii[p][p];
            S.Kii[p][p] = 1.0;
            for (int j = 0; j < 9; ++j) S.Kii[p][j] *= piv;
            for (int i = 0; i < 9; ++i) {
                if (i == p) continue;
                const double f = S.Kii[i][p];
                S.Kii[i][p] = 0.0;
                for (int j = 0; j < 9; ++j) S.Kii[i][j] -= f * S.Kii[p][j];
            }
        }
    }
    __syncthreads();
    for (int q = t; q < 9 * kNd; q += kBT) {
        const int i = q / kNd, c = q % kNd;
        double acc = 0.0;
        for (int k = 0; k < 9; ++k) acc += S.Kii[i][k] * S.K[kNd + k][c];
        S.X[i][c] = acc;
    }
    __syncthreads();
    for (int q = t; q < kNd * kNd; q += kBT) {
        const int r = q / kNd, c = q % kNd;
        double acc = 0.0;
        for (int k = 0; k < 9; ++k) acc += S.K[r][kNd + k] * S.X[k][c];
        S.K24[r][c] = S.K[r][c] - acc;
    }
    __syncthreads();
}

__device__ __forceinline__ double brick_mass(const BrickSmem& S, int a, int b) {
    double acc = 0.0;
    for (int ip = 0; ip < 8; ++ip) acc += S.n[ip][a] * S.n[ip][b] * S.det[ip];
    return S.rho * acc;
}

__global__ void __launch_bounds__(kBT)
k_brick_assemble(const int32_t* __restrict__ elems, const int32_t* __restrict__ conn, const double* __restrict__ xyz,
                 const double* __restrict__ E, const double* __restrict__ nu, const double* __restrict__ rho,
                 const int32_t* __restrict__ slot_map, double* __restrict__ vals, double* __restrict__ mvals,
                 double cM) {
    __shared__ BrickSmem S;
    const int e = elems[blockIdx.x];
    brick_element(S, e, conn, xyz, E, nu, mvals ? rho : nullptr);
    const int pr = threadIdx.x, a = pr >> 3, b = pr & 7;
    const int32_t slot = slot_map[(size_t)e * 64 + pr];
    const int64_t g = slot >> 5, lane = slot & 31;
    double* vb = vals + (g * 9) * 32 + lane;
    double* mb = mvals ? mvals + (g * 9) * 32 + lane : nullptr;
    const double m = mb ? brick_mass(S, a, b) : 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double k = S.K24[3 * a + i][3 * b + j];
            if (mb && i == j) {
                mb[(i * 3 + j) * 32] += m;
                k += cM * m;
            }
            vb[(i * 3 + j) * 32] += k;
        }
}

// g_e = -(lambda_e^T K_e u_e) / E_e
__global__ void __launch_bounds__(kBT)
k_brick_adjoint(const int32_t* __restrict__ conn, const double* __restrict__ xyz, const double* __restrict__ E,
                const double* __restrict__ nu, const double* __restrict__ u, const double* __restrict__ lam,
                double* __restrict__ gout, int accumulate) {
    __shared__ BrickSmem S;
    __shared__ double red[kBT];
    const int e = blockIdx.x;
    brick_element(S, e, conn, xyz, E, nu, nullptr);
    double acc = 0.0;
    for (int q = threadIdx.x; q < kNd * kNd; q += kBT) {
        const int r = q / kNd, c = q % kNd;
        const size_t dr = 3 * (size_t)conn[8 * (size_t)e + r / 3] + r % 3;
        const size_t dc = 3 * (size_t)conn[8 * (size_t)e + c / 3] + c % 3;
        acc += lam[dr] * S.K24[r][c] * u[dc];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kBT / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double v = -red[0] / E[e];
        gout[e] = accumulate ? gout[e] + v : v;
    }
}

// Strain-pair tensors with the condensed modes recovered (update_internal,
// element_equations.rs:19-194): each field's internal DOF are
// alpha = -Kii^-1 Kie f_e (the element's X), so the full 33-DOF strains give
// P_e[i][j] = sum_gp w detJ eps_i(a) eps_j(b), the tensor whose contraction
// with dC/dD is a^T dK~_e/dD b of the condensed matrix K~ = Kee - Kei X
// (d K~ = [I, -X^T] dK [I; -X]).
__global__ void __launch_bounds__(kBT)
k_brick_pairs(const int32_t* __restrict__ conn, const double* __restrict__ xyz, const double* __restrict__ E,
              const double* __restrict__ nu, const double* __restrict__ av, const double* __restrict__ bv,
              double* __restrict__ P, int accumulate) {
    __shared__ BrickSmem S;
    __shared__ double f[2][kTot];
    __shared__ double eps[2][8][6];
    const int e = blockIdx.x, t = threadIdx.x;
    brick_element(S, e, conn, xyz, E, nu, nullptr);
    if (t < 2 * kNd) {
        const int fld = t / kNd, c = t % kNd;
        const size_t g = 3 * (size_t)conn[8 * (size_t)e + c / 3] + c % 3;
        f[fld][c] = fld ? bv[g] : av[g];
    }
    __syncthreads();
    if (t < 18) {
        const int fld = t / 9, i = t % 9;
        double acc = 0.0;
        for (int c = 0; c < kNd; ++c) acc += S.X[i][c] * f[fld][c];
        f[fld][kNd + i] = -acc;
    }
    __syncthreads();
    if (t < 16) {  // strains of both fields at the 8 points
        const int fld = t / 8, ip = t % 8;
        double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int fn = 0; fn < 11; ++fn)
            for (int i = 0; i < 3; ++i) {
                const double v = (fn < 8) ? f[fld][3 * fn + i] : f[fld][kNd + 3 * (fn - 8) + i];
                for (int j = 0; j < 3; ++j) H[i][j] += v * S.dx[ip][fn][j];
            }
        double* ep = eps[fld][ip];
        ep[0] = H[0][0];
        ep[1] = H[1][1];
        ep[2] = H[2][2];
        ep[3] = H[0][1] + H[1][0];
        ep[4] = H[0][2] + H[2][0];
        ep[5] = H[1][2] + H[2][1];
    }
    __syncthreads();
    if (t < 36) {
        const int i = t / 6, j = t % 6;
        double acc = 0.0;
        for (int ip = 0; ip < 8; ++ip) acc += eps[0][ip][i] * eps[1][ip][j] * S.det[ip];
        double* out = P + (size_t)e * 36 + t;
        *out = accumulate ? *out + acc : acc;
    }
}

__global__ void __launch_bounds__(kBT)
k_brick_export(int e0, const int32_t* __restrict__ conn, const double* __restrict__ xyz, const double* __restrict__ E,
               const double* __restrict__ nu, const double* __restrict__ rho, double* __restrict__ ke,
               double* __restrict__ me) {
    __shared__ BrickSmem S;
    const int e = e0 + blockIdx.x;
    brick_element(S, e, conn, xyz, E, nu, rho);
    for (int q = threadIdx.x; q < kNd * kNd; q += kBT) {
        const int r = q / kNd, c = q % kNd;
        ke[(size_t)blockIdx.x * kNd * kNd + q] = S.K24[r][c];
        if (me) me[(size_t)blockIdx.x * kNd * kNd + q] = (r % 3 == c % 3) ? brick_mass(S, r / 3, c / 3) : 0.0;
    }
}

// all condensed element stiffness matrices, FP32 [n_el][24][24] (the fine
// level's input to Galerkin multigrid coarsening)
__global__ void __launch_bounds__(kBT)
k_brick_ke32(const int32_t* __restrict__ conn, const double* __restrict__ xyz, const double* __restrict__ E,
             const double* __restrict__ nu, float* __restrict__ ke) {
    __shared__ BrickSmem S;
    const int e = blockIdx.x;
    brick_element(S, e, conn, xyz, E, nu, nullptr);
    for (int q = threadIdx.x; q < kNd * kNd; q += kBT) ke[(size_t)e * kNd * kNd + q] = (float)S.K24[q / kNd][q % kNd];
}

}  // namespace

void brickim_element_ke32(Ctx& c, float* d_ke) {
    k_brick_ke32<<<c.n_el, kBT, 0, c.stream>>>(c.d_conn.p, c.d_xyz.p, c.d_E.p, c.d_nu.p, d_ke);
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

void brickim_assemble(Ctx& c, double* vals, double* mvals) {
    const int n_col = (int)c.colour_ptr.size() - 1;
    for (int k = 0; k < n_col; ++k) {
        const int n = c.colour_ptr[k + 1] - c.colour_ptr[k];
        if (n == 0) continue;
        k_brick_assemble<<<n, kBT, 0, c.stream>>>(c.d_colour_elems.p + c.colour_ptr[k], c.d_conn.p, c.d_xyz.p,
                                                 c.d_E.p, c.d_nu.p, c.d_rho.p, c.d_slot_map.p, vals, mvals, c.cM);
        ASEND_CUDA(cudaGetLastError());
        ++c.launches;
    }
}

void brickim_adjoint(Ctx& c, const double* d_u, const double* d_lam, double* d_g, bool accumulate) {
    k_brick_adjoint<<<c.n_el, kBT, 0, c.stream>>>(c.d_conn.p, c.d_xyz.p, c.d_E.p, c.d_nu.p, d_u, d_lam, d_g,
                                                 accumulate ? 1 : 0);
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

void brickim_pairs(Ctx& c, const double* d_a, const double* d_b, double* d_P, bool accumulate) {
    k_brick_pairs<<<c.n_el, kBT, 0, c.stream>>>(c.d_conn.p, c.d_xyz.p, c.d_E.p, c.d_nu.p, d_a, d_b, d_P,
                                               accumulate ? 1 : 0);
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

void brickim_element_matrices(Ctx& c, int e0, int n, double* ke_host, double* me_host) {
    DArr<double> ke, me;
    ke.alloc((size_t)n * 576);
    if (me_host) me.alloc((size_t)n * 576);
    k_brick_export<<<n, kBT, 0, c.stream>>>(e0, c.d_conn.p, c.d_xyz.p, c.d_E.p, c.d_nu.p, c.d_rho.p, ke.p,
                                            me_host ? me.p : nullptr);
    ++c.launches;
    ASEND_CUDA(cudaGetLastError());
    ASEND_CUDA(cudaMemcpyAsync(ke_host, ke.p, sizeof(double) * n * 576, cudaMemcpyDeviceToHost, c.stream));
    if (me_host)
        ASEND_CUDA(cudaMemcpyAsync(me_host, me.p, sizeof(double) * n * 576, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace asend
