// k_beam.cu -- beam2 (type 2) element kernels: stiffness with the two internal
// DOF condensed, consistent section mass, coloured scatter, adjoint contraction.
//
// Reference formulation (solverSrc/asend_run_job/src/):
//   element_meth.rs:371-396        type 2: 2 nodes x 6 DOF, 2 internal DOF (a
//                                  bubble on the section-frame u2 and u3),
//                                  2 Gauss points +-1/sqrt(3), weight 1
//   element_soln_fields.rs:364-379  N1 = (1-s)/2, N2 = (1+s)/2, N3 = 1 - s^2; the
//                                  bubble's derivative -2s belongs to N3 (the
//                                  reference stores it in node 1's slot, which
//                                  leaves the internal block singular)
//   element_soln_fields.rs:415-421  Jacobian: d/dx = (2/L) d/ds, detJ = L/2
//   element_soln_fields.rs:1313-1321 section deformation
//                                  [u1', u2' - th3, u3' + th2, th1', th2', th3']
//   element_properties.rs:878-1017  section stiffness (EA, GA, GA, GJ, E I3, E I4
//                                  and the first-moment / product couplings)
//   element_properties.rs:1410-1500 section mass
//   element_equations.rs:206-418, :19-57, :420-626  K, condensation, M (node DOF)
//   model_analysis.rs:1379-1457     d_relasticd_d: section-strain pairs for material
//                                  DVs (E1 and G1..G3 enter the section stiffness
//                                  separately; nu does not)
// Frame: rows e1 = element axis, e3 = e1 x v / |e1 x v|, e2 = e3 x e1 (the
// section orientation of section_meth.rs:21-50 with the element axis as x).
//
// GB300 mapping: one thread per element of a colour (elements of a colour share
// no node, so the scatter needs no atomics).  The element works in the section
// frame, where the strain-displacement matrix is sparse and fixed, and rotates
// each 3x3 pseudo-node block to global axes on the way out: K_glob = T^T K_loc T
// with T = diag(R, R, R, R).  FP64 throughout; a beam model is small next to
// the solve, so the kernel is built for exactness, not bandwidth.
#include <cmath>
#include <vector>

#include "common.cuh"

namespace asend {
namespace {

constexpr int kBT = 128;
constexpr double kG = 0.57735026918962576451;  // 1/sqrt(3)
// device section table per element: area, I1..I5, J, v (3), then the section
// stiffness and mass given as matrices (6 x 6 each; entry [0] <= 0: computed
// from the area and moments), as the reference's beamProps stiffness / mass
constexpr int kSecC = 10, kSecM = 46, kSecStride = 82;

struct BeamLocal {
    double R[9];        // rows e1 e2 e3
    double a;           // L / 2 = detJ
    double K[12][12];   // condensed stiffness, section-frame DOF 6 k + c
};

// Frame and condensed section-frame stiffness of element e (sec[10] = area,
// I1..I5, J, v); kfull (may be null) receives the uncondensed 14 x 14
// section-frame stiffness.  Returns false on a degenerate frame (rejected on
// the host).
__device__ bool beam_local(BeamLocal& B, const double* x0, const double* x1, double E, double nu, const double* sec,
                           double* kfull = nullptr) {
    double d[3] = {x1[0] - x0[0], x1[1] - x0[1], x1[2] - x0[2]};
    const double L = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (!(L > 0.0)) return false;
    const double e1[3] = {d[0] / L, d[1] / L, d[2] / L};
    const double* v = sec + 7;
    double e3[3] = {e1[1] * v[2] - e1[2] * v[1], e1[2] * v[0] - e1[0] * v[2], e1[0] * v[1] - e1[1] * v[0]};
    const double n3 = sqrt(e3[0] * e3[0] + e3[1] * e3[1] + e3[2] * e3[2]);
    if (!(n3 > 0.0)) return false;
    for (int j = 0; j < 3; ++j) e3[j] /= n3;
    const double e2[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2], e3[0] * e1[1] - e3[1] * e1[0]};
    for (int j = 0; j < 3; ++j) {
        B.R[j] = e1[j];
        B.R[3 + j] = e2[j];
        B.R[6 + j] = e3[j];
    }
    const double a = 0.5 * L;
    B.a = a;
    // section stiffness, symmetric, row-major 6 x 6
    const double G = E / (2.0 * (1.0 + nu));
    double C[36];
    for (int i = 0; i < 36; ++i) C[i] = 0.0;
    C[0] = E * sec[0];
    C[4] = C[24] = E * sec[1];
    C[5] = C[30] = -E * sec[2];
    C[7] = G * sec[0];
    C[9] = C[19] = -G * sec[1];
    C[14] = G * sec[0];
    C[15] = C[20] = G * sec[2];
    C[21] = G * sec[6];
    C[28] = E * sec[3];
    C[29] = C[34] = -E * sec[5];
    C[35] = E * sec[4];
    if (sec[kSecC] > 0.0)  // a given matrix (upper triangle, mirrored)
        for (int i = 0; i < 6; ++i)
            for (int j = i; j < 6; ++j) C[6 * i + j] = C[6 * j + i] = sec[kSecC + 6 * i + j];
    // Section-frame strain rows at a point, as (column, coefficient) lists:
    // node DOF 6k + c (c < 3 translation, c >= 3 rotation), bubbles 12 / 13.
    double K[14][14];
    for (int i = 0; i < 14; ++i)
        for (int j = 0; j < 14; ++j) K[i][j] = 0.0;
#pragma unroll 1
    for (int ip = 0; ip < 2; ++ip) {
        const double s = ip ? kG : -kG;
        const double N[2] = {0.5 * (1.0 - s), 0.5 * (1.0 + s)}, dN[2] = {-0.5 / a, 0.5 / a};
        const double db = -2.0 * s / a;
        double Bm[6][14];
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 14; ++j) Bm[i][j] = 0.0;
        for (int k = 0; k < 2; ++k) {
            Bm[0][6 * k + 0] = dN[k];   // u1'
            Bm[1][6 * k + 1] = dN[k];   // u2'
            Bm[1][6 * k + 5] = -N[k];   // - th3
            Bm[2][6 * k + 2] = dN[k];   // u3'
            Bm[2][6 * k + 4] = N[k];    // + th2
            Bm[3][6 * k + 3] = dN[k];   // th1'
            Bm[4][6 * k + 4] = dN[k];   // th2'
            Bm[5][6 * k + 5] = dN[k];   // th3'
        }
        Bm[1][12] = db;
        Bm[2][13] = db;
        for (int j = 0; j < 14; ++j) {
            double cb[6];
            for (int i = 0; i < 6; ++i) {
                double acc = 0.0;
                for (int q = 0; q < 6; ++q) acc += C[6 * i + q] * Bm[q][j];
                cb[i] = acc * a;
            }
            for (int r = 0; r < 14; ++r) {
                double acc = 0.0;
                for (int i = 0; i < 6; ++i) acc += Bm[i][r] * cb[i];
                K[r][j] += acc;
            }
        }
    }
    if (kfull)
        for (int i = 0; i < 14; ++i)
            for (int j = 0; j < 14; ++j) kfull[14 * i + j] = K[i][j];
    // condense the bubbles: K_nn - K_ni K_ii^-1 K_in (2 x 2 inverse)
    const double det = K[12][12] * K[13][13] - K[12][13] * K[13][12];
    const double i00 = K[13][13] / det, i01 = -K[12][13] / det, i10 = -K[13][12] / det, i11 = K[12][12] / det;
    for (int r = 0; r < 12; ++r) {
        const double x0r = i00 * K[12][r] + i01 * K[13][r];
        const double x1r = i10 * K[12][r] + i11 * K[13][r];
        for (int c2 = 0; c2 < 12; ++c2) B.K[c2][r] = K[c2][r] - (K[c2][12] * x0r + K[c2][13] * x1r);
    }
    return true;
}

// section mass entry (p, q) of the 6 x 6 matrix (symmetric)
__device__ double beam_msec(const double* sec, double rho, int p, int q) {
    if (p > q) {
        const int t = p;
        p = q;
        q = t;
    }
    if (sec[kSecM] > 0.0) return sec[kSecM + 6 * p + q];  // a given matrix (upper triangle)
    switch (6 * p + q) {
        case 0: case 7: case 14: return rho * sec[0];
        case 4: return rho * sec[1];
        case 9: return -rho * sec[1];
        case 5: return -rho * sec[2];
        case 15: return rho * sec[2];
        case 21: return rho * sec[6];
        case 28: return rho * sec[3];
        case 29: return rho * sec[5];
        case 35: return rho * sec[4];
        default: return 0.0;
    }
}

// mass factor sum_ip detJ N_k N_l
__device__ __forceinline__ double beam_mfac(double a, int k, int l) {
    double acc = 0.0;
    for (int ip = 0; ip < 2; ++ip) {
        const double s = ip ? kG : -kG;
        const double N[2] = {0.5 * (1.0 - s), 0.5 * (1.0 + s)};
        acc += a * N[k] * N[l];
    }
    return acc;
}

// global 3x3 block (pa, pb) of pseudo-nodes (2 k + t) of K (and M) from the
// section-frame matrices: R^T X R
__device__ void beam_block(const BeamLocal& B, const double* sec, double rho, int pa, int pb, double* kb,
                           double* mb) {
    double X[3][3];
    for (int p = 0; p < 3; ++p)
        for (int q = 0; q < 3; ++q) X[p][q] = B.K[3 * pa + p][3 * pb + q];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q) acc += B.R[3 * p + i] * X[p][q] * B.R[3 * q + j];
            kb[3 * i + j] = acc;
        }
    if (!mb) return;
    const double f = beam_mfac(B.a, pa >> 1, pb >> 1);
    const int oa = 3 * (pa & 1), ob = 3 * (pb & 1);
    for (int p = 0; p < 3; ++p)
        for (int q = 0; q < 3; ++q) X[p][q] = f * beam_msec(sec, rho, oa + p, ob + q);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q) acc += B.R[3 * p + i] * X[p][q] * B.R[3 * q + j];
            mb[3 * i + j] = acc;
        }
}

__global__ void __launch_bounds__(kBT)
k_beam_assemble(int n, const int32_t* __restrict__ elems, const int32_t* __restrict__ conn2,
                const double* __restrict__ xyz, const double* __restrict__ E, const double* __restrict__ nu,
                const double* __restrict__ rho, const double* __restrict__ sec, const int32_t* __restrict__ slot_map,
                double* __restrict__ vals, double* __restrict__ mvals, double cM) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int e = elems[t];
    BeamLocal B;
    const double* se = sec + kSecStride * (size_t)e;
    if (!beam_local(B, xyz + 3 * (size_t)conn2[2 * (size_t)e], xyz + 3 * (size_t)conn2[2 * (size_t)e + 1], E[e], nu[e],
                    se))
        return;  // frames are validated on the host before assembly
    const double re = mvals ? rho[e] : 0.0;
    for (int pr = 0; pr < 16; ++pr) {
        const int pa = pr >> 2, pb = pr & 3;
        double kb[9], mb[9];
        beam_block(B, se, re, pa, pb, kb, mvals ? mb : nullptr);
        const int32_t slot = slot_map[(size_t)e * 16 + pr];
        const int64_t g = slot >> 5, lane = slot & 31;
        double* vb = vals + (g * 9) * 32 + lane;
        double* mbp = mvals ? mvals + (g * 9) * 32 + lane : nullptr;
        for (int q = 0; q < 9; ++q) {
            double k = kb[q];
            if (mbp) {
                mbp[q * 32] += mb[q];
                k += cM * mb[q];
            }
            vb[q * 32] += k;
        }
    }
}

// g_e = -(lambda_e^T K_e u_e) / E_e (K_e linear in E_e at fixed nu)
__global__ void __launch_bounds__(kBT)
k_beam_adjoint(int n_el, const int32_t* __restrict__ conn2, const double* __restrict__ xyz,
               const double* __restrict__ E, const double* __restrict__ nu, const double* __restrict__ sec,
               const double* __restrict__ u, const double* __restrict__ lam, double* __restrict__ g, int accumulate) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    BeamLocal B;
    const int n0 = conn2[2 * (size_t)e], n1 = conn2[2 * (size_t)e + 1];
    double v = 0.0;
    if (beam_local(B, xyz + 3 * (size_t)n0, xyz + 3 * (size_t)n1, E[e], nu[e], sec + kSecStride * (size_t)e)) {
        double ul[12], ll[12];
        for (int k = 0; k < 2; ++k) {
            const size_t base = 6 * (size_t)(k ? n1 : n0);
            for (int t3 = 0; t3 < 2; ++t3)
                for (int p = 0; p < 3; ++p) {
                    double su = 0.0, sl = 0.0;
                    for (int c = 0; c < 3; ++c) {
                        su += B.R[3 * p + c] * u[base + 3 * t3 + c];
                        sl += B.R[3 * p + c] * lam[base + 3 * t3 + c];
                    }
                    ul[6 * k + 3 * t3 + p] = su;
                    ll[6 * k + 3 * t3 + p] = sl;
                }
        }
        double acc = 0.0;
        for (int r = 0; r < 12; ++r) {
            double kr = 0.0;
            for (int c = 0; c < 12; ++c) kr += B.K[r][c] * ul[c];
            acc += ll[r] * kr;
        }
        v = -acc / E[e];
    }
    g[e] = accumulate ? g[e] + v : v;
}

// node DOF of element e in the section frame: f_loc[6 k + 3 t + p] = R f_glob
__device__ void beam_to_local(const BeamLocal& B, const double* f, int n0, int n1, double* fl) {
    for (int k = 0; k < 2; ++k) {
        const size_t base = 6 * (size_t)(k ? n1 : n0);
        for (int t3 = 0; t3 < 2; ++t3)
            for (int p = 0; p < 3; ++p) {
                double acc = 0.0;
                for (int c = 0; c < 3; ++c) acc += B.R[3 * p + c] * f[base + 3 * t3 + c];
                fl[6 * k + 3 * t3 + p] = acc;
            }
    }
}

// Section-strain pairs P_e[36] = sum_ip detJ eps(a) eps(b)^T with the bubble
// amplitudes recovered (alpha = -K_ii^-1 K_in f, update_internal
// element_equations.rs:147-194), so that a^T (dK_e/dD) b = sum (dC/dD) : P_e
// for any section-stiffness parameter D (d_relasticd_d,
// model_analysis.rs:1379-1457).
__global__ void __launch_bounds__(kBT)
k_beam_pairs(int n_el, const int32_t* __restrict__ conn2, const double* __restrict__ xyz,
             const double* __restrict__ E, const double* __restrict__ nu, const double* __restrict__ sec,
             const double* __restrict__ fa, const double* __restrict__ fb, double* __restrict__ P, int accumulate) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    BeamLocal B;
    double K[196];
    const int n0 = conn2[2 * (size_t)e], n1 = conn2[2 * (size_t)e + 1];
    double acc[36];
    for (int i = 0; i < 36; ++i) acc[i] = 0.0;
    if (beam_local(B, xyz + 3 * (size_t)n0, xyz + 3 * (size_t)n1, E[e], nu[e], sec + kSecStride * (size_t)e, K)) {
        double la[14], lb[14];
        beam_to_local(B, fa, n0, n1, la);
        beam_to_local(B, fb, n0, n1, lb);
        const double det = K[14 * 12 + 12] * K[14 * 13 + 13] - K[14 * 12 + 13] * K[14 * 13 + 12];
        for (double* f : {la, lb}) {
            double r0 = 0.0, r1 = 0.0;
            for (int c = 0; c < 12; ++c) {
                r0 += K[14 * 12 + c] * f[c];
                r1 += K[14 * 13 + c] * f[c];
            }
            f[12] = -(K[14 * 13 + 13] * r0 - K[14 * 12 + 13] * r1) / det;
            f[13] = -(-K[14 * 13 + 12] * r0 + K[14 * 12 + 12] * r1) / det;
        }
        const double a = B.a;
        for (int ip = 0; ip < 2; ++ip) {
            const double s = ip ? kG : -kG;
            const double N0 = 0.5 * (1.0 - s), N1 = 0.5 * (1.0 + s), d0 = -0.5 / a, d1 = 0.5 / a, db = -2.0 * s / a;
            double ea[6], eb[6];
            const double* fs[2] = {la, lb};
            double* es[2] = {ea, eb};
            for (int q = 0; q < 2; ++q) {
                const double* f = fs[q];
                double* ev = es[q];
                ev[0] = d0 * f[0] + d1 * f[6];
                ev[1] = d0 * f[1] + d1 * f[7] - (N0 * f[5] + N1 * f[11]) + db * f[12];
                ev[2] = d0 * f[2] + d1 * f[8] + (N0 * f[4] + N1 * f[10]) + db * f[13];
                ev[3] = d0 * f[3] + d1 * f[9];
                ev[4] = d0 * f[4] + d1 * f[10];
                ev[5] = d0 * f[5] + d1 * f[11];
            }
            for (int i = 0; i < 6; ++i)
                for (int j = 0; j < 6; ++j) acc[6 * i + j] += ea[i] * eb[j] * a;
        }
    }
    double* Pe = P + 36 * (size_t)e;
    for (int i = 0; i < 36; ++i) Pe[i] = accumulate ? Pe[i] + acc[i] : acc[i];
}

// element matrices (checks): ke/me [count][12][12], global DOF 6 a + c
__global__ void __launch_bounds__(kBT)
k_beam_export(int e0, int n, const int32_t* __restrict__ conn2, const double* __restrict__ xyz,
              const double* __restrict__ E, const double* __restrict__ nu, const double* __restrict__ rho,
              const double* __restrict__ sec, double* __restrict__ ke, double* __restrict__ me) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int e = e0 + t;
    BeamLocal B;
    const double* se = sec + kSecStride * (size_t)e;
    double* ko = ke + (size_t)t * 144;
    double* mo = me ? me + (size_t)t * 144 : nullptr;
    if (!beam_local(B, xyz + 3 * (size_t)conn2[2 * (size_t)e], xyz + 3 * (size_t)conn2[2 * (size_t)e + 1], E[e], nu[e],
                    se))
        return;
    for (int pr = 0; pr < 16; ++pr) {
        const int pa = pr >> 2, pb = pr & 3;
        double kb[9], mb[9];
        beam_block(B, se, mo ? rho[e] : 0.0, pa, pb, kb, mo ? mb : nullptr);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                ko[(3 * pa + i) * 12 + 3 * pb + j] = kb[3 * i + j];
                if (mo) mo[(3 * pa + i) * 12 + 3 * pb + j] = mb[3 * i + j];
            }
    }
}

void require_sections(const Ctx& c) {
    if (c.d_beam_sec.n != (size_t)c.n_el * kSecStride)
        throw InputError("beam2 meshes need asend_set_beam_sections before assembly");
}

}  // namespace

void beam_assemble(Ctx& c, double* vals, double* mvals) {
    require_sections(c);
    const int n_col = (int)c.colour_ptr.size() - 1;
    for (int k = 0; k < n_col; ++k) {
        const int n = c.colour_ptr[k + 1] - c.colour_ptr[k];
        if (n == 0) continue;
        k_beam_assemble<<<(n + kBT - 1) / kBT, kBT, 0, c.stream>>>(
            n, c.d_colour_elems.p + c.colour_ptr[k], c.d_shell_conn.p, c.d_shell_xyz.p, c.d_E.p, c.d_nu.p, c.d_rho.p,
            c.d_beam_sec.p, c.d_slot_map.p, vals, mvals, c.cM);
        ASEND_CUDA(cudaGetLastError());
        ++c.launches;
    }
}

void beam_adjoint(Ctx& c, const double* d_u, const double* d_lam, double* d_g, bool accumulate) {
    require_sections(c);
    if (c.beam_given_stiffness())
        throw InputError("given beam section stiffness matrices have no per-element modulus gradient "
                         "(K is not proportional to E)");
    k_beam_adjoint<<<(c.n_el + kBT - 1) / kBT, kBT, 0, c.stream>>>(c.n_el, c.d_shell_conn.p, c.d_shell_xyz.p, c.d_E.p,
                                                                   c.d_nu.p, c.d_beam_sec.p, d_u, d_lam, d_g,
                                                                   accumulate ? 1 : 0);
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

void beam_pairs(Ctx& c, const double* d_a, const double* d_b, double* d_P, bool accumulate) {
    require_sections(c);
    k_beam_pairs<<<(c.n_el + kBT - 1) / kBT, kBT, 0, c.stream>>>(c.n_el, c.d_shell_conn.p, c.d_shell_xyz.p, c.d_E.p,
                                                                 c.d_nu.p, c.d_beam_sec.p, d_a, d_b, d_P,
                                                                 accumulate ? 1 : 0);
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

std::vector<double> beam_device_table(const Ctx& c) {
    std::vector<double> t((size_t)c.n_el * kSecStride, 0.0);
    for (int e = 0; e < c.n_el; ++e) {
        std::copy(c.beam_sec.begin() + (size_t)e * 10, c.beam_sec.begin() + (size_t)e * 10 + 10,
                  t.begin() + (size_t)e * kSecStride);
        if (!c.beam_cm.empty())
            std::copy(c.beam_cm.begin() + (size_t)e * 72, c.beam_cm.begin() + (size_t)e * 72 + 72,
                      t.begin() + (size_t)e * kSecStride + kSecC);
    }
    return t;
}

void beam_section_dC(int category, int component, const double* sec, double E, double nu, double* dC) {
    for (int i = 0; i < 36; ++i) dC[i] = 0.0;
    auto set = [&](int i, int j, double v) { dC[6 * i + j] = dC[6 * j + i] = v; };
    const double G = E / (2.0 * (1.0 + nu));
    if (category == ASEND_DV_AREA) {  // EA, GA, GA
        set(0, 0, E);
        set(1, 1, G);
        set(2, 2, G);
        return;
    }
    if (category == ASEND_DV_AREA_MOMENT) {
        if (component == 1) {  // E I1, -G I1
            set(0, 4, E);
            set(1, 3, -G);
        } else if (component == 2) {  // -E I2, G I2
            set(0, 5, -E);
            set(2, 3, G);
        } else if (component == 3) {
            set(4, 4, E);
        } else if (component == 4) {
            set(5, 5, E);
        } else if (component == 5) {
            set(4, 5, -E);
        }
        return;
    }
    if (category == ASEND_DV_POLAR_MOMENT) {  // GJ
        set(3, 3, G);
        return;
    }
    if (category == ASEND_DV_MODULUS && component == 1) {  // E1: EA, E I1, -E I2, E I3, -E I5, E I4
        set(0, 0, sec[0]);
        set(0, 4, sec[1]);
        set(0, 5, -sec[2]);
        set(4, 4, sec[3]);
        set(4, 5, -sec[5]);
        set(5, 5, sec[4]);
    } else if (category == ASEND_DV_SHEAR_MODULUS && component == 1) {  // G1: GA, -G I1, GJ
        set(1, 1, sec[0]);
        set(1, 3, -sec[1]);
        set(3, 3, sec[6]);
    } else if (category == ASEND_DV_SHEAR_MODULUS && component == 2) {  // G2: GA of the second shear
        set(2, 2, sec[0]);
    } else if (category == ASEND_DV_SHEAR_MODULUS && component == 3) {  // G3: G I2
        set(2, 3, sec[2]);
    }
}

void beam_element_matrices(Ctx& c, int e0, int n, double* ke_host, double* me_host) {
    require_sections(c);
    DArr<double> ke, me;
    ke.alloc((size_t)n * 144);
    if (me_host) me.alloc((size_t)n * 144);
    k_beam_export<<<(n + kBT - 1) / kBT, kBT, 0, c.stream>>>(e0, n, c.d_shell_conn.p, c.d_shell_xyz.p, c.d_E.p,
                                                             c.d_nu.p, c.d_rho.p, c.d_beam_sec.p, ke.p,
                                                             me_host ? me.p : nullptr);
    ++c.launches;
    ASEND_CUDA(cudaGetLastError());
    ASEND_CUDA(cudaMemcpyAsync(ke_host, ke.p, sizeof(double) * n * 144, cudaMemcpyDeviceToHost, c.stream));
    if (me_host)
        ASEND_CUDA(cudaMemcpyAsync(me_host, me.p, sizeof(double) * n * 144, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace asend
