// k_objective.cu -- element-category objective terms at the element centroid.
//
// Reference: ObjectiveTerm::get_obj_val (objective_meth.rs:665-720) takes
// stress, strain or strain energy of each element of a set at the element's
// centroid s_cent (get_stress_strain_dfd0, element_soln_fields.rs:1463-1576)
// and its volume sum_ip w detJ (get_volume_dfd0 :1118-1155).  getd_ld_u
// (objective_meth.rs:1051-1160) differentiates the term with respect to the
// element DOF and getd_ld_d (:1372-1500) with respect to the material at
// fixed u.  Here the operator (powerNorm, ks, volumeIntegral, volumeAverage)
// stays on the host, which hands each element two 6-vectors of weights,
//     a_e = dL/dsigma_e,   b_e = dL/deps_e   (Voigt 11,22,33,12,13,23),
// so that dL/du = sum_e B_c^T (b_e + C_e a_e) and the explicit material term
// is dL/dD = sum_e a_e^T (dC_e/dD) eps_e.  B_c is the strain-displacement
// matrix at the centroid: s = 0 for hex8 and brickIM (whose incompatible
// modes 1 - s_i^2 have zero slope there, element_soln_fields.rs:212-227),
// the constant tet4 gradients, and s = (1/4, 1/4, 1/4) for tet10
// (element_meth.rs:257-259).
//
// GB300 design: one thread per element; node data gathered once and made
// element-relative in FP64; the adjoint right-hand side is scattered with
// FP64 atomics (at most 8 elements meet at a node of a block mesh).
#include <algorithm>
#include <type_traits>

#include "common.cuh"

namespace asend {
namespace {

// Centroid shape-function gradients dN_a/dx and (optionally) the volume.
template <int NN>
__device__ __forceinline__ void centroid_gradients(int e, const int32_t* __restrict__ conn,
                                                   const double* __restrict__ xyz, int (&nd)[NN],
                                                   double (&g)[NN][3], double* vol) {
#pragma unroll
    for (int a = 0; a < NN; ++a) nd[a] = conn[(size_t)e * NN + a];
    double x[NN][3];
#pragma unroll
    for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j) x[a][j] = xyz[3 * (size_t)nd[a] + j] - xyz[3 * (size_t)nd[0] + j];
    double dn[NN][3];
    if constexpr (NN == 8) {
        const double sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                 {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) dn[a][j] = 0.125 * sg[a][j];
    } else if constexpr (NN == 10) {
        const double sc[3] = {0.25, 0.25, 0.25};  // s_cent of tet10 (element_meth.rs:257-259)
        double nv[10];
        tet10_shape(sc, nv, dn);
    } else {
        const double d[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) dn[a][j] = d[a][j];
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
#pragma unroll
    for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j) g[a][j] = dn[a][0] * Ji[0][j] + dn[a][1] * Ji[1][j] + dn[a][2] * Ji[2][j];
    if (!vol) return;
    if constexpr (NN == 8) {
        // sum over the 2x2x2 Gauss points of detJ (weights 1)
        const double gq = 0.5773502691896257;
        const double sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                 {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
        double v = 0.0;
#pragma unroll 1
        for (int gp = 0; gp < 8; ++gp) {
            const double s0 = (gp & 1) ? gq : -gq, s1 = (gp & 2) ? gq : -gq, s2 = (gp & 4) ? gq : -gq;
            double Jp[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                const double f0 = 1 + sg[a][0] * s0, f1 = 1 + sg[a][1] * s1, f2 = 1 + sg[a][2] * s2;
                const double d0 = 0.125 * sg[a][0] * f1 * f2, d1 = 0.125 * sg[a][1] * f0 * f2,
                             d2 = 0.125 * sg[a][2] * f0 * f1;
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    Jp[i][0] += x[a][i] * d0;
                    Jp[i][1] += x[a][i] * d1;
                    Jp[i][2] += x[a][i] * d2;
                }
            }
            v += Jp[0][0] * (Jp[1][1] * Jp[2][2] - Jp[1][2] * Jp[2][1]) +
                 Jp[0][1] * (Jp[1][2] * Jp[2][0] - Jp[1][0] * Jp[2][2]) +
                 Jp[0][2] * (Jp[1][0] * Jp[2][1] - Jp[1][1] * Jp[2][0]);
        }
        *vol = v;
    } else if constexpr (NN == 10) {
        double v = 0.0;
#pragma unroll 1
        for (int gp = 0; gp < 4; ++gp) {
            double sp[3], nv[10], dp[10][3], Jp[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            tet10_point(gp, sp);
            tet10_shape(sp, nv, dp);
            for (int a = 0; a < 10; ++a)
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) Jp[i][j] += x[a][i] * dp[a][j];
            v += (Jp[0][0] * (Jp[1][1] * Jp[2][2] - Jp[1][2] * Jp[2][1]) +
                  Jp[0][1] * (Jp[1][2] * Jp[2][0] - Jp[1][0] * Jp[2][2]) +
                  Jp[0][2] * (Jp[1][0] * Jp[2][1] - Jp[1][1] * Jp[2][0])) / 24.0;
        }
        *vol = v;
    } else {
        *vol = det / 6.0;
    }
}

// Element stiffness C (Voigt, engineering shear): the per-element matrix when
// given, else isotropic from E and nu.
__device__ __forceinline__ void element_cmat(int e, const double* __restrict__ E, const double* __restrict__ nu,
                                             const double* __restrict__ cmat, double (&C)[36]) {
    if (cmat) {
#pragma unroll
        for (int k = 0; k < 36; ++k) C[k] = cmat[(size_t)e * 36 + k];
        return;
    }
    const double ne = nu[e], Ee = E[e];
    const double lam = Ee * ne / ((1.0 + ne) * (1.0 - 2.0 * ne));
    const double mu = Ee / (2.0 * (1.0 + ne));
#pragma unroll
    for (int k = 0; k < 36; ++k) C[k] = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) C[6 * i + j] = lam;
        C[7 * i] += 2.0 * mu;
        C[7 * (i + 3)] = mu;
    }
}

template <int NN>
__device__ __forceinline__ void centroid_strain(const int (&nd)[NN], const double (&g)[NN][3],
                                                const double* __restrict__ u, double (&eps)[6]) {
    double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double u0[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) u0[i] = u[3 * (size_t)nd[0] + i];
#pragma unroll
    for (int a = 1; a < NN; ++a)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double ua = u[3 * (size_t)nd[a] + i] - u0[i];
#pragma unroll
            for (int j = 0; j < 3; ++j) H[i][j] += ua * g[a][j];
        }
    eps[0] = H[0][0];
    eps[1] = H[1][1];
    eps[2] = H[2][2];
    eps[3] = H[0][1] + H[1][0];
    eps[4] = H[0][2] + H[2][0];
    eps[5] = H[1][2] + H[2][1];
}

template <int NN>
__global__ void __launch_bounds__(128)
k_centroid_fields(int n_el, const int32_t* __restrict__ conn, const double* __restrict__ xyz,
                  const double* __restrict__ E, const double* __restrict__ nu, const double* __restrict__ cmat,
                  const double* __restrict__ u, double* __restrict__ eps_out, double* __restrict__ sig_out,
                  double* __restrict__ vol_out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    int nd[NN];
    double g[NN][3], vol = 0.0;
    centroid_gradients<NN>(e, conn, xyz, nd, g, vol_out ? &vol : nullptr);
    if (vol_out) vol_out[e] = vol;
    double eps[6];
    centroid_strain<NN>(nd, g, u, eps);
    if (eps_out)
#pragma unroll
        for (int k = 0; k < 6; ++k) eps_out[(size_t)e * 6 + k] = eps[k];
    if (sig_out) {
        double C[36];
        element_cmat(e, E, nu, cmat, C);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < 6; ++j) s += C[6 * i + j] * eps[j];
            sig_out[(size_t)e * 6 + i] = s;
        }
    }
}

// rhs += sum_e B_c^T (b_e + C_e a_e): the adjoint load of the element term.
template <int NN>
__global__ void __launch_bounds__(128)
k_centroid_rhs(int n_el, const int32_t* __restrict__ conn, const double* __restrict__ xyz,
               const double* __restrict__ E, const double* __restrict__ nu, const double* __restrict__ cmat,
               const double* __restrict__ wa, const double* __restrict__ wb, double* __restrict__ rhs) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    double w[6], a[6];
    bool any = false;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        a[k] = wa[(size_t)e * 6 + k];
        w[k] = wb[(size_t)e * 6 + k];
        any |= (a[k] != 0.0) || (w[k] != 0.0);
    }
    if (!any) return;
    double C[36];
    element_cmat(e, E, nu, cmat, C);
#pragma unroll
    for (int j = 0; j < 6; ++j)
#pragma unroll
        for (int i = 0; i < 6; ++i) w[j] += C[6 * i + j] * a[i];
    int nd[NN];
    double g[NN][3];
    centroid_gradients<NN>(e, conn, xyz, nd, g, nullptr);
#pragma unroll
    for (int n = 0; n < NN; ++n) {
        const double g0 = g[n][0], g1 = g[n][1], g2 = g[n][2];
        atomicAdd(&rhs[3 * (size_t)nd[n] + 0], g0 * w[0] + g1 * w[3] + g2 * w[4]);
        atomicAdd(&rhs[3 * (size_t)nd[n] + 1], g1 * w[1] + g0 * w[3] + g2 * w[5]);
        atomicAdd(&rhs[3 * (size_t)nd[n] + 2], g2 * w[2] + g0 * w[4] + g1 * w[5]);
    }
}

// Explicit terms at fixed u: gE[e] += a_e . sigma_e / E_e (isotropic C = E C1)
// and, when P is given, P_e -= a_e eps_e^T so that -sum (dC/dD) : P_e holds
// both the adjoint and the explicit material derivative.
template <int NN>
__global__ void __launch_bounds__(128)
k_centroid_explicit(int n_el, const int32_t* __restrict__ conn, const double* __restrict__ xyz,
                    const double* __restrict__ E, const double* __restrict__ nu, const double* __restrict__ cmat,
                    const double* __restrict__ wa, const double* __restrict__ u, double* __restrict__ gE,
                    double* __restrict__ P) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    double a[6];
    bool any = false;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        a[k] = wa[(size_t)e * 6 + k];
        any |= a[k] != 0.0;
    }
    if (!any) return;
    int nd[NN];
    double g[NN][3], eps[6];
    centroid_gradients<NN>(e, conn, xyz, nd, g, nullptr);
    centroid_strain<NN>(nd, g, u, eps);
    if (gE) {
        double C[36];
        element_cmat(e, E, nu, cmat, C);
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            double si = 0.0;
#pragma unroll
            for (int j = 0; j < 6; ++j) si += C[6 * i + j] * eps[j];
            s += a[i] * si;
        }
        gE[e] += s / E[e];
    }
    if (P)
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
            for (int j = 0; j < 6; ++j) P[(size_t)e * 36 + 6 * i + j] -= a[i] * eps[j];
}

void check_solid(const Ctx& c) {
    if (c.type != 8 && c.type != 81 && c.type != 4 && c.type != 10)
        throw InputError("element-category objectives are built for hex8, brickIM, tet4 and tet10 meshes");
}

// one launch of a kernel templated on the element's node count
template <typename F>
void by_nodes(const Ctx& c, F&& f) {
    if (c.nn == 8) f(std::integral_constant<int, 8>{});
    else if (c.nn == 10) f(std::integral_constant<int, 10>{});
    else f(std::integral_constant<int, 4>{});
}

const double* cmat_of(const Ctx& c) { return c.ortho.empty() ? nullptr : c.d_cmat.p; }

}  // namespace

void element_fields(Ctx& c, const double* d_u, double* d_eps, double* d_sig, double* d_vol) {
    check_solid(c);
    const int blocks = (c.n_el + 127) / 128;
    by_nodes(c, [&](auto nn) {
        k_centroid_fields<decltype(nn)::value><<<blocks, 128, 0, c.stream>>>(
            c.n_el, c.d_conn.p, c.d_xyz.p, c.d_E.p, c.d_nu.p, cmat_of(c), d_u, d_eps, d_sig, d_vol);
    });
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

void element_objective_rhs(Ctx& c, double* d_rhs) {
    check_solid(c);
    const int blocks = (c.n_el + 127) / 128;
    by_nodes(c, [&](auto nn) {
        k_centroid_rhs<decltype(nn)::value><<<blocks, 128, 0, c.stream>>>(
            c.n_el, c.d_conn.p, c.d_xyz.p, c.d_E.p, c.d_nu.p, cmat_of(c), c.d_obj_wa.p, c.d_obj_wb.p, d_rhs);
    });
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

void element_objective_explicit(Ctx& c, const double* d_u, double* d_gE, double* d_P) {
    check_solid(c);
    const int blocks = (c.n_el + 127) / 128;
    by_nodes(c, [&](auto nn) {
        k_centroid_explicit<decltype(nn)::value><<<blocks, 128, 0, c.stream>>>(
            c.n_el, c.d_conn.p, c.d_xyz.p, c.d_E.p, c.d_nu.p, cmat_of(c), c.d_obj_wa.p, d_u, d_gE, d_P);
    });
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

}  // namespace asend
