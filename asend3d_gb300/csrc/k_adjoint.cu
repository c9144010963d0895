// k_adjoint.cu -- K4: per-element adjoint modulus-sensitivity contraction.
//
// Reference: Model::get_obj_gradient static branch
// (solverSrc/asend_run_job/src/model_analysis.rs:1632-1704): for every design
// variable i, d_relasticd_d(i) (:1379-1457) re-integrates the elements that
// depend on D_i with forward-mode dual numbers and the gradient gets
// dL/dD_i -= sum_dof lambda * dR/dD_i (:1692-1700).  That loop is
// O(n_dv * (n_dof + n_el)).  For a modulus DV on element e only that element's
// internal force R_e = K_e u_e depends on it, and with C linear in E at fixed
// nu, dR_e/dE_e = (K_e / E_e) u_e, so all n_el sensitivities come from one
// O(n_el) pass:
//     g_e = -(1/E_e) sum_gp w detJ  eps(a_e)^T C eps(b_e)
// with (a, b) = (lambda, u).  Strains use the reference's Voigt order and
// engineering shear (element_soln_fields.rs:1345-1461).
//
// GB300 design: one thread per element, 8 Gauss points unrolled, node data
// gathered once into registers; displacements are made element-relative in
// FP64 (rigid translation removed) before forming gradients.
#include <algorithm>

#include "common.cuh"

namespace asend {
namespace {

// Element-relative node data of element e: coordinates and the two
// displacement fields with node 0's translation removed.
template <int NN>
__device__ __forceinline__ void gather_element(int e, const int32_t* __restrict__ conn, const double* __restrict__ xyz,
                                               const double* __restrict__ av, const double* __restrict__ bv,
                                               double (&x)[NN][3], double (&ua)[NN][3], double (&ub)[NN][3]) {
    int nd[NN];
#pragma unroll
    for (int a = 0; a < NN; ++a) nd[a] = conn[(size_t)e * NN + a];
#pragma unroll
    for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            x[a][j] = xyz[3 * (size_t)nd[a] + j] - xyz[3 * (size_t)nd[0] + j];
            ua[a][j] = av[3 * (size_t)nd[a] + j];
            ub[a][j] = bv[3 * (size_t)nd[a] + j];
        }
#pragma unroll
    for (int a = NN - 1; a >= 0; --a)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            ua[a][j] -= ua[0][j];
            ub[a][j] -= ub[0][j];
        }
}

// Voigt strains (11,22,33,12,13,23, engineering shear) of both fields at
// Gauss point gp, and its weight w detJ.
template <int NN>
__device__ __forceinline__ double point_strains(int gp, const double (&x)[NN][3], const double (&ua)[NN][3],
                                                const double (&ub)[NN][3], double (&ea)[6], double (&eb)[6]) {
    const double gq = 0.5773502691896257;
    double dn[NN][3];
    double wt;
    if constexpr (NN == 8) {
        const double s0 = (gp & 1) ? gq : -gq, s1 = (gp & 2) ? gq : -gq, s2 = (gp & 4) ? gq : -gq;
        const double sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                 {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const double f0 = 1 + sg[a][0] * s0, f1 = 1 + sg[a][1] * s1, f2 = 1 + sg[a][2] * s2;
            dn[a][0] = 0.125 * sg[a][0] * f1 * f2;
            dn[a][1] = 0.125 * sg[a][1] * f0 * f2;
            dn[a][2] = 0.125 * sg[a][2] * f0 * f1;
        }
        wt = 1.0;
    } else if constexpr (NN == 10) {
        double sp[3], nv[10];
        tet10_point(gp, sp);
        tet10_shape(sp, nv, dn);
        wt = 1.0 / 24.0;
    } else {
        const double d[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) dn[a][j] = d[a][j];
        wt = 1.0 / 6.0;
    }
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) J[i][j] += x[a][i] * dn[a][j];
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    const double id = 1.0 / det;
    double Ji[3][3];
    Ji[0][0] = c00 * id;
    Ji[1][0] = c01 * id;
    Ji[2][0] = c02 * id;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    // displacement gradients H[i][j] = du_i/dx_j
    double Ha[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, Hb[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int a = 1; a < NN; ++a) {
        double gx[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) gx[j] = dn[a][0] * Ji[0][j] + dn[a][1] * Ji[1][j] + dn[a][2] * Ji[2][j];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                Ha[i][j] += ua[a][i] * gx[j];
                Hb[i][j] += ub[a][i] * gx[j];
            }
    }
    ea[0] = Ha[0][0]; ea[1] = Ha[1][1]; ea[2] = Ha[2][2];
    ea[3] = Ha[0][1] + Ha[1][0]; ea[4] = Ha[0][2] + Ha[2][0]; ea[5] = Ha[1][2] + Ha[2][1];
    eb[0] = Hb[0][0]; eb[1] = Hb[1][1]; eb[2] = Hb[2][2];
    eb[3] = Hb[0][1] + Hb[1][0]; eb[4] = Hb[0][2] + Hb[2][0]; eb[5] = Hb[1][2] + Hb[2][1];
    return det * wt;
}

template <int NN>
__global__ void __launch_bounds__(128)
k_adjoint_modulus(int n_el, const int32_t* __restrict__ conn, const double* __restrict__ xyz,
                  const double* __restrict__ nu, const double* __restrict__ av, const double* __restrict__ bv,
                  double* __restrict__ g, int accumulate) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    double x[NN][3], ua[NN][3], ub[NN][3];
    gather_element<NN>(e, conn, xyz, av, bv, x, ua, ub);
    const double ne = nu[e];
    const double lam = ne / ((1.0 + ne) * (1.0 - 2.0 * ne));  // C / E
    const double mu = 1.0 / (2.0 * (1.0 + ne));
    constexpr int NIP = (NN == 8) ? 8 : (NN == 10 ? 4 : 1);
    double acc = 0.0;
#pragma unroll
    for (int gp = 0; gp < NIP; ++gp) {
        double ea[6], eb[6];
        const double wd = point_strains<NN>(gp, x, ua, ub, ea, eb);
        const double trb = eb[0] + eb[1] + eb[2];
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < 3; ++i) s += ea[i] * (lam * trb + 2.0 * mu * eb[i]);
#pragma unroll
        for (int i = 3; i < 6; ++i) s += ea[i] * (mu * eb[i]);
        acc += s * wd;
    }
    const double v = -acc;  // -(1/E) eps(a)^T C eps(b), C / E folded into lam, mu
    if (accumulate) g[e] += v;
    else g[e] = v;
}

// Strain-pair tensors P_e[i][j] = sum_gp w detJ eps_i(a) eps_j(b): any
// material derivative of the element's internal force then contracts as
// a^T dR_e/dD = sum_ij (dC/dD)_ij P_e[i][j] (C constant over the element).
template <int NN>
__global__ void __launch_bounds__(128)
k_adjoint_pairs(int n_el, const int32_t* __restrict__ conn, const double* __restrict__ xyz,
                const double* __restrict__ av, const double* __restrict__ bv, double* __restrict__ P, int accumulate) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    double x[NN][3], ua[NN][3], ub[NN][3];
    gather_element<NN>(e, conn, xyz, av, bv, x, ua, ub);
    constexpr int NIP = (NN == 8) ? 8 : (NN == 10 ? 4 : 1);
    double acc[36];
#pragma unroll
    for (int k = 0; k < 36; ++k) acc[k] = 0.0;
#pragma unroll 1
    for (int gp = 0; gp < NIP; ++gp) {
        double ea[6], eb[6];
        const double wd = point_strains<NN>(gp, x, ua, ub, ea, eb);
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
            for (int j = 0; j < 6; ++j) acc[6 * i + j] += ea[i] * eb[j] * wd;
    }
    double* out = P + (size_t)e * 36;
#pragma unroll
    for (int k = 0; k < 36; ++k) out[k] = accumulate ? out[k] + acc[k] : acc[k];
}

// The same contraction for hex8 meshes kept as geometry classes (K_e = E_e K^):
// g_e = -a_e^T K^_cls b_e, one thread per element, 576 FP64 FMA against the
// class matrix (read through L1; a structured block has one class, so a warp
// reads each entry once) in place of the Gauss-point integration.
__global__ void __launch_bounds__(128)
k_adjoint_cls(int n_el, const int32_t* __restrict__ conn, const int32_t* __restrict__ cls_of,
              const double* __restrict__ cls_ke, const double* __restrict__ av, const double* __restrict__ bv,
              double* __restrict__ g, int accumulate) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    int nd[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) nd[a] = conn[(size_t)e * 8 + a];
    double ua[24], ub[24];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            ua[3 * a + j] = av[3 * (size_t)nd[a] + j];
            ub[3 * a + j] = bv[3 * (size_t)nd[a] + j];
        }
    // element-relative: K^ annihilates a rigid translation
#pragma unroll
    for (int a = 7; a >= 0; --a)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            ua[3 * a + j] -= ua[j];
            ub[3 * a + j] -= ub[j];
        }
    const double* K = cls_ke + (size_t)cls_of[e] * 576;
    double acc = 0.0;
#pragma unroll
    for (int r = 3; r < 24; ++r) {
        double s = 0.0;
#pragma unroll
        for (int q = 3; q < 24; ++q) s = fma(__ldg(K + r * 24 + q), ub[q], s);
        acc = fma(ua[r], s, acc);
    }
    g[e] = accumulate ? g[e] - acc : -acc;
}

__global__ void k_dot_partial(size_t n, const double* __restrict__ a, const double* __restrict__ b,
                              double* __restrict__ part) {
    __shared__ double sm[32];
    double v[1] = {0.0};
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        v[0] += a[i] * b[i];
    block_sum<1>(v, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}
__global__ void k_dot_final(int nb, const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sm[32];
    double v[1] = {0.0};
    for (int i = threadIdx.x; i < nb; i += blockDim.x) v[0] += part[i];
    block_sum<1>(v, sm);
    if (threadIdx.x == 0) *out = v[0];
}
__global__ void k_axpy(size_t n, double alpha, const double* __restrict__ x, double* __restrict__ y) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        y[i] += alpha * x[i];
}

}  // namespace

// Deterministic FP64 dot product (fixed two-stage order) into *d_out.
void device_dot(Ctx& c, size_t n, const double* a, const double* b, double* d_out, double* d_part) {
    constexpr int nb = 256;
    k_dot_partial<<<nb, 256, 0, c.stream>>>(n, a, b, d_part);
    k_dot_final<<<1, 256, 0, c.stream>>>(nb, d_part, d_out);
    ASEND_CUDA(cudaGetLastError());
    c.launches += 2;
}
void device_axpy(Ctx& c, size_t n, double alpha, const double* x, double* y) {
    k_axpy<<<(int)std::min<size_t>((n + 255) / 256, 2432), 256, 0, c.stream>>>(n, alpha, x, y);
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

void adjoint_contract(Ctx& c, const double* d_a, const double* d_b, double* d_g, bool accumulate) {
    if (c.type == 41) {
        shell_adjoint(c, d_b, d_a, d_g, accumulate);
        return;
    }
    if (c.type == 2) {
        beam_adjoint(c, d_b, d_a, d_g, accumulate);
        return;
    }
    if (c.type == 81) {
        brickim_adjoint(c, d_b, d_a, d_g, accumulate);
        return;
    }
    const int blocks = (c.n_el + 127) / 128;
    if (c.type == 8 && c.cls_ready && c.cls_type == 8 && c.ortho.empty())
        k_adjoint_cls<<<blocks, 128, 0, c.stream>>>(c.n_el, c.d_conn.p, c.d_cls_of.p, c.cls_ke.p, d_a, d_b, d_g,
                                                    accumulate ? 1 : 0);
    else if (c.nn == 8)
        k_adjoint_modulus<8><<<blocks, 128, 0, c.stream>>>(c.n_el, c.d_conn.p, c.d_xyz.p, c.d_nu.p, d_a, d_b, d_g,
                                                            accumulate ? 1 : 0);
    else if (c.nn == 10)
        k_adjoint_modulus<10><<<blocks, 128, 0, c.stream>>>(c.n_el, c.d_conn.p, c.d_xyz.p, c.d_nu.p, d_a, d_b, d_g,
                                                             accumulate ? 1 : 0);
    else
        k_adjoint_modulus<4><<<blocks, 128, 0, c.stream>>>(c.n_el, c.d_conn.p, c.d_xyz.p, c.d_nu.p, d_a, d_b, d_g,
                                                            accumulate ? 1 : 0);
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

void adjoint_pairs(Ctx& c, const double* d_a, const double* d_b, double* d_P, bool accumulate) {
    if (c.type == 2) {
        beam_pairs(c, d_a, d_b, d_P, accumulate);
        return;
    }
    if (c.type == 81) {
        brickim_pairs(c, d_a, d_b, d_P, accumulate);
        return;
    }
    if (c.type != 8 && c.type != 4 && c.type != 10)
        throw InputError("strain-pair tensors are built for hex8, brickIM, tet4, tet10 and beam2 meshes");
    const int blocks = (c.n_el + 127) / 128;
    if (c.nn == 8)
        k_adjoint_pairs<8><<<blocks, 128, 0, c.stream>>>(c.n_el, c.d_conn.p, c.d_xyz.p, d_a, d_b, d_P, accumulate ? 1 : 0);
    else if (c.nn == 10)
        k_adjoint_pairs<10><<<blocks, 128, 0, c.stream>>>(c.n_el, c.d_conn.p, c.d_xyz.p, d_a, d_b, d_P,
                                                           accumulate ? 1 : 0);
    else
        k_adjoint_pairs<4><<<blocks, 128, 0, c.stream>>>(c.n_el, c.d_conn.p, c.d_xyz.p, d_a, d_b, d_P, accumulate ? 1 : 0);
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

}  // namespace asend
