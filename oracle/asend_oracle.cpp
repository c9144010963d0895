// asend_oracle.cpp -- FP64 CPU restatement of the reference's linear-elastic
// solve path.  TEST INFRASTRUCTURE: the checker for the CUDA library, never
// linked into it.  Citations are "file:line" relative to
// solverSrc/asend_run_job/src/ of MSDOToolz/ASenD3D.
//
// Parity status: pinned by the reference's analytic known answers
// (examples/testCases/hexBeam/notes.txt, singleHex) and by central finite
// differences; the reference itself (Rust) cannot be built here.
#include "asend_oracle.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>
#include <vector>

namespace {

constexpr double kTol = 1e-12;                 // constants.rs:13 (TOL)
constexpr double kR1ORt3 = 0.5773502691896257; // constants.rs:3
constexpr double kR1O6 = 0.16666666666666666;  // constants.rs:6
constexpr double kPi = 3.14159265358979323846;
constexpr double kRTet1 = 0.1381966011250071;  // constants.rs:10 (R_TET1)
constexpr double kRTet2 = 0.585410196624929;   // constants.rs:11 (R_TET2)
constexpr double kR1O24 = 0.041666666666666664; // constants.rs:7 (R_1O24)
constexpr double kRPi0180 = 0.017453292519943295;  // constants.rs:9 (R_PI_0180)

// ---------------------------------------------------------------------------
// Element type tables: element_meth.rs:74-448 (initialize_type)
// ---------------------------------------------------------------------------
struct TypeInfo {
    int type = 0, nn = 0, dpn = 3, nip = 0, nfaces = 0;
    double ip[8 * 3] = {};  // at most 8 points (hex8); tet10 uses 4
    double wt[8] = {};
    int faces[6][4] = {};
    int face_nn = 0;
};

TypeInfo type_info(int type) {
    TypeInfo t;
    t.type = type;
    if (type == 8) {
        // hex8: 2x2x2 Gauss points ordered with s0 fastest (element_meth.rs:157-189)
        t.nn = 8; t.dpn = 3; t.nip = 8; t.nfaces = 6; t.face_nn = 4;
        const double sv[2] = {-kR1ORt3, kR1ORt3};
        int k = 0;
        for (int c = 0; c < 2; ++c)
            for (int b = 0; b < 2; ++b)
                for (int a = 0; a < 2; ++a) {
                    t.ip[3 * k + 0] = sv[a];
                    t.ip[3 * k + 1] = sv[b];
                    t.ip[3 * k + 2] = sv[c];
                    t.wt[k] = 1.0;
                    ++k;
                }
        // faces: element_meth.rs:525-591 (initialize_faces, hex branch)
        const int f[6][4] = {{3, 2, 1, 0}, {4, 5, 6, 7}, {0, 1, 5, 4},
                             {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
        std::memcpy(t.faces, f, sizeof(f));
    } else if (type == 81) {
        // brickIM: hex8 points, faces and nodes plus 9 internal DOF
        // (element_meth.rs:157-201)
        t = type_info(8);
        t.type = 81;
    } else if (type == 41) {
        // shell4 as 8 pseudo-nodes of 3 DOF: node a's translations are
        // pseudo-node 2a, its rotations 2a+1, so DOF 6a + c keeps the
        // reference's node-major numbering (element_meth.rs:424-431)
        t.nn = 8; t.dpn = 3; t.nip = 4; t.nfaces = 0; t.face_nn = 0;
    } else if (type == 2) {
        // beam2 as 4 pseudo-nodes of 3 DOF, node a's translations on 2a and
        // rotations on 2a+1, as for shell4; the 2 internal DOF are condensed
        t.nn = 4; t.dpn = 3; t.nip = 2; t.nfaces = 0; t.face_nn = 0;
    } else if (type == 10) {
        // tet10: 4 points (R_TET1 x3 with R_TET2 in turn on each axis after
        // the first), weights 1/24 (element_meth.rs:228-262); face loads are
        // not restated for it
        t.nn = 10; t.dpn = 3; t.nip = 4; t.nfaces = 0; t.face_nn = 0;
        const double pts[4][3] = {{kRTet1, kRTet1, kRTet1}, {kRTet2, kRTet1, kRTet1},
                                  {kRTet1, kRTet2, kRTet1}, {kRTet1, kRTet1, kRTet2}};
        for (int k = 0; k < 4; ++k) {
            for (int j = 0; j < 3; ++j) t.ip[3 * k + j] = pts[k][j];
            t.wt[k] = kR1O24;
        }
    } else if (type == 4) {
        // tet4: one point at (1/4,1/4,1/4), weight 1/6 (element_meth.rs:84-101)
        t.nn = 4; t.dpn = 3; t.nip = 1; t.nfaces = 4; t.face_nn = 3;
        t.ip[0] = t.ip[1] = t.ip[2] = 0.25;
        t.wt[0] = kR1O6;
        const int f[4][4] = {{0, 2, 1, 0}, {0, 1, 3, 0}, {1, 2, 3, 0}, {0, 3, 2, 0}};
        std::memcpy(t.faces, f, sizeof(f));
    }
    return t;
}

// Shape functions and parametric derivatives: element_soln_fields.rs:120-229
// (tet4 :121-140, hex8 :171-211).  dn[3*n + j] = dN_n/ds_j.
void shape(int type, const double* s, double* n, double* dn) {
    if (type == 8) {
        const double sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                 {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
        for (int a = 0; a < 8; ++a) {
            const double f0 = 1.0 + sg[a][0] * s[0];
            const double f1 = 1.0 + sg[a][1] * s[1];
            const double f2 = 1.0 + sg[a][2] * s[2];
            n[a] = 0.125 * f0 * f1 * f2;
            dn[3 * a + 0] = 0.125 * sg[a][0] * f1 * f2;
            dn[3 * a + 1] = 0.125 * sg[a][1] * f0 * f2;
            dn[3 * a + 2] = 0.125 * sg[a][2] * f0 * f1;
        }
    } else if (type == 4) {
        n[0] = 1.0 - s[0] - s[1] - s[2];
        n[1] = s[0]; n[2] = s[1]; n[3] = s[2];
        const double d[12] = {-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1};
        std::memcpy(dn, d, sizeof(d));
    } else if (type == 10) {
        // quadratic tetrahedron (element_soln_fields.rs:229-298): corners
        // 0..3, mid-edge nodes 4 (0-1), 5 (1-2), 6 (0-2), 7 (0-3), 8 (1-3), 9 (2-3)
        const double p1 = 1.0 - s[0] - s[1] - s[2], p2 = p1 - 0.5;
        n[0] = 2.0 * p1 * p2;
        dn[0] = dn[1] = dn[2] = 2.0 * (-p2 - p1);
        for (int k = 0; k < 3; ++k) {
            n[1 + k] = -2.0 * s[k] * (0.5 - s[k]);
            for (int j = 0; j < 3; ++j) dn[3 * (1 + k) + j] = (j == k) ? -2.0 * (0.5 - 2.0 * s[k]) : 0.0;
        }
        // mid-edge node on the edge (0, k): 4 s_k p1
        const int m0[3] = {4, 6, 7};
        for (int k = 0; k < 3; ++k) {
            const int a = m0[k];
            n[a] = 4.0 * s[k] * p1;
            for (int j = 0; j < 3; ++j) dn[3 * a + j] = (j == k) ? 4.0 * (p1 - s[k]) : -4.0 * s[k];
        }
        // mid-edge node on the edge (i, j) of corners 1..3: 4 s_i s_j
        const int mm[3][3] = {{5, 0, 1}, {8, 0, 2}, {9, 1, 2}};
        for (const auto& e : mm) {
            const int a = e[0], i = e[1], j = e[2];
            n[a] = 4.0 * s[i] * s[j];
            for (int q = 0; q < 3; ++q) dn[3 * a + q] = (q == i) ? 4.0 * s[j] : (q == j ? 4.0 * s[i] : 0.0);
        }
    }
}

// ---------------------------------------------------------------------------
// Givens QR with angle storage (matrix_functions.rs:50-105 q_rfactor_ar,
// :107-165 solveq_rx_eqb_ar), full square case (tri_diag = 0), and the
// determinant / inverse built on it (matrix_functions.rs:1707-1729).
// ---------------------------------------------------------------------------
void givens_factor(double* a, int n) {
    for (int c = 0; c < n; ++c) {
        for (int r = c + 1; r < n; ++r) {
            double& piv = a[c * n + c];
            if (std::fabs(piv) < kTol) piv = kTol;
            const double th = std::atan(a[r * n + c] / piv);
            const double sn = std::sin(th), cs = std::cos(th);
            for (int k = c; k < n; ++k) {
                const double top = a[c * n + k], bot = a[r * n + k];
                a[c * n + k] = cs * top + sn * bot;
                a[r * n + k] = -sn * top + cs * bot;
            }
            a[r * n + c] = th;  // the rotation angle replaces the zeroed entry
        }
    }
}

void givens_solve(double* x, const double* a, double* b, int n) {
    for (int c = 0; c < n; ++c) {
        for (int r = c + 1; r < n; ++r) {
            const double th = a[r * n + c];
            const double sn = std::sin(th), cs = std::cos(th);
            const double top = b[c], bot = b[r];
            b[c] = cs * top + sn * bot;
            b[r] = -sn * top + cs * bot;
        }
        x[c] = 0.0;
    }
    for (int c = n - 1; c >= 0; --c) {
        double acc = 0.0;
        for (int k = c + 1; k < n; ++k) acc += a[c * n + k] * x[k];
        x[c] = (b[c] - acc) / a[c * n + c];
    }
}

double det_inv(double* inv, const double* mat_in, int n) {
    double a[36];
    std::memcpy(a, mat_in, sizeof(double) * n * n);
    givens_factor(a, n);
    double det = 1.0, b[6], x[6];
    for (int col = 0; col < n; ++col) {
        for (int k = 0; k < n; ++k) b[k] = (k == col) ? 1.0 : 0.0;
        givens_solve(x, a, b, n);
        for (int k = 0; k < n; ++k) inv[k * n + col] = x[k];
        det *= a[col * n + col];
    }
    return det;
}

// Integration point data: element_soln_fields.rs:383-463 (solid branch).
// xyz[3*nn] node-major.  Returns detJ; dndx[3*a + j] = dN_a/dx_j.
double ip_data(int type, int nn, const double* xyz, const double* s, double* n, double* dndx) {
    double dn[30];
    shape(type, s, n, dn);
    double J[9] = {0};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int a = 0; a < nn; ++a) acc += xyz[3 * a + i] * dn[3 * a + j];
            J[3 * i + j] = acc;
        }
    double Ji[9];
    const double det = det_inv(Ji, J, 3);
    for (int a = 0; a < nn; ++a)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc += dn[3 * a + k] * Ji[3 * k + j];
            dndx[3 * a + j] = acc;
        }
    return det;
}

// Solid 6x6 stiffness from the compliance matrix: element_properties.rs:648-764
// (get_solid_stiff_dfd0, engineering-constant branch).  Voigt order
// 11,22,33,12,13,23.  e/nu/g are (E1,E2,E3), (nu12,nu13,nu23), (G12,G13,G23).
void solid_cmat(const double e[3], const double nu[3], const double g[3], double* C) {
    double S[36] = {0};
    S[0] = 1.0 / e[0];
    S[1] = -nu[0] / e[0];
    S[2] = -nu[1] / e[0];
    S[6] = S[1];
    S[7] = 1.0 / e[1];
    S[8] = -nu[2] / e[1];
    S[12] = S[2];
    S[13] = S[8];
    S[14] = 1.0 / e[2];
    S[21] = 1.0 / g[0];
    S[28] = 1.0 / g[1];
    S[35] = 1.0 / g[2];
    det_inv(C, S, 6);
}

void iso_cmat(double E, double nu, double* C) {
    const double e[3] = {E, E, E};
    const double n3[3] = {nu, nu, nu};
    const double G = E / (2.0 * (1.0 + nu));
    const double g[3] = {G, G, G};
    solid_cmat(e, n3, g, C);
}

// Strain-displacement columns: element_soln_fields.rs:1345-1461
// (get_solid_strain_dfd0, single-DOF derivative branch, identity orientation).
// B[6 * tot + col] layout (row k = strain component).
void solid_bmat(int nn, const double* dndx, double* B) {
    const int tot = 3 * nn;
    std::fill(B, B + 6 * tot, 0.0);
    for (int a = 0; a < nn; ++a) {
        const double* g = dndx + 3 * a;
        for (int d = 0; d < 3; ++d) {
            const int col = 3 * a + d;
            double sm[9] = {0};
            for (int i = 0; i < 3; ++i)
                for (int j = i; j < 3; ++j) {
                    if (i == d) sm[3 * i + j] += g[j];
                    if (j == d) sm[3 * i + j] += g[i];
                }
            B[0 * tot + col] = 0.5 * sm[0];
            B[1 * tot + col] = 0.5 * sm[4];
            B[2 * tot + col] = 0.5 * sm[8];
            B[3 * tot + col] = sm[1];
            B[4 * tot + col] = sm[2];
            B[5 * tot + col] = sm[5];
        }
    }
}

// Element stiffness: element_equations.rs:206-418 (get_ruk_dfd0 with
// get_matrix, linear geometry, dpn == 3): K += B^T (C B) detJ w per point,
// with C*B scaled by detJ*w first (:377-395).
void brickim_ke(const double* xyz, const double* C, double* ke);

void solid_ke(int type, const double* xyz, const double* C, double* ke) {
    if (type == 81) {
        brickim_ke(xyz, C, ke);
        return;
    }
    const TypeInfo t = type_info(type);
    const int nn = t.nn, tot = 3 * nn;
    std::fill(ke, ke + tot * tot, 0.0);
    double n[10], dndx[30], B[6 * 30], CB[6 * 30];
    for (int p = 0; p < t.nip; ++p) {
        const double det = ip_data(type, nn, xyz, t.ip + 3 * p, n, dndx);
        const double djw = det * t.wt[p];
        solid_bmat(nn, dndx, B);
        for (int k = 0; k < 6; ++k)
            for (int c = 0; c < tot; ++c) {
                double acc = 0.0;
                for (int l = 0; l < 6; ++l) acc += C[6 * k + l] * B[l * tot + c];
                CB[k * tot + c] = acc * djw;
            }
        for (int i = 0; i < tot; ++i)
            for (int j = 0; j < tot; ++j) {
                double acc = 0.0;
                for (int k = 0; k < 6; ++k) acc += B[k * tot + i] * CB[k * tot + j];
                ke[i * tot + j] += acc;
            }
    }
}

// brickIM (type 81) stiffness: hex8 plus the bubbles 1-s^2, 1-t^2, 1-u^2 on
// each displacement component (element_soln_fields.rs:212-227, dof_table
// element_meth.rs:192-201), whose derivatives at the point use the centroid
// Jacobian (element_soln_fields.rs:424-461); the 9 internal DOF are condensed
// (element_equations.rs:19-57).
// Inverse Jacobian at the element centroid (the bubbles' derivatives use it).
void brickim_centroid_jinv(const double* xyz, double* Ji0) {
    double n0[8], dn0[24], J0[9] = {0};
    const double s0[3] = {0.0, 0.0, 0.0};
    shape(8, s0, n0, dn0);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int a = 0; a < 8; ++a) J0[3 * i + j] += xyz[3 * a + i] * dn0[3 * a + j];
    det_inv(Ji0, J0, 3);
}

// B (6 x 33: the 24 node DOF, then bubble f = 0..2 x component d) at Gauss
// point p; returns w detJ.
double brickim_bmat(const double* xyz, const double* Ji0, int p, double* B) {
    constexpr int tot = 33, nd = 24;
    const TypeInfo t = type_info(8);
    double n[8], dndx[24], B24[6 * 24];
    const double* sp = t.ip + 3 * p;
    const double det = ip_data(8, 8, xyz, sp, n, dndx);
    solid_bmat(8, dndx, B24);
    std::fill(B, B + 6 * tot, 0.0);
    for (int k = 0; k < 6; ++k)
        for (int c = 0; c < nd; ++c) B[k * tot + c] = B24[k * 24 + c];
    for (int f = 0; f < 3; ++f) {  // bubble f: d/ds_f = -2 s_f
        double g[3];
        for (int j = 0; j < 3; ++j) g[j] = -2.0 * sp[f] * Ji0[3 * f + j];
        for (int d = 0; d < 3; ++d) {
            const int col = nd + 3 * f + d;
            double sm[9] = {0};
            for (int i = 0; i < 3; ++i)
                for (int j = i; j < 3; ++j) {
                    if (i == d) sm[3 * i + j] += g[j];
                    if (j == d) sm[3 * i + j] += g[i];
                }
            B[0 * tot + col] = 0.5 * sm[0];
            B[1 * tot + col] = 0.5 * sm[4];
            B[2 * tot + col] = 0.5 * sm[8];
            B[3 * tot + col] = sm[1];
            B[4 * tot + col] = sm[2];
            B[5 * tot + col] = sm[5];
        }
    }
    return det * t.wt[p];
}

// Full 33 x 33 brickIM stiffness before condensation.
void brickim_kfull(const double* xyz, const double* C, double* K) {
    constexpr int tot = 33;
    const TypeInfo t = type_info(8);
    double Ji0[9];
    brickim_centroid_jinv(xyz, Ji0);
    std::fill(K, K + tot * tot, 0.0);
    std::vector<double> B(6 * tot), CB(6 * tot);
    for (int p = 0; p < t.nip; ++p) {
        const double djw = brickim_bmat(xyz, Ji0, p, B.data());
        for (int k = 0; k < 6; ++k)
            for (int c = 0; c < tot; ++c) {
                double acc = 0.0;
                for (int l = 0; l < 6; ++l) acc += C[6 * k + l] * B[l * tot + c];
                CB[k * tot + c] = acc * djw;
            }
        for (int i = 0; i < tot; ++i)
            for (int j = 0; j < tot; ++j) {
                double acc = 0.0;
                for (int k = 0; k < 6; ++k) acc += B[k * tot + i] * CB[k * tot + j];
                K[i * tot + j] += acc;
            }
    }
}

void brickim_ke(const double* xyz, const double* C, double* ke) {
    constexpr int tot = 33, nd = 24;
    std::vector<double> K(tot * tot);
    brickim_kfull(xyz, C, K.data());
    double Kii[81];
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j) Kii[9 * i + j] = K[(nd + i) * tot + nd + j];
    givens_factor(Kii, 9);
    for (int r = 0; r < nd; ++r) {
        double rhs[9], x[9];
        for (int i = 0; i < 9; ++i) rhs[i] = K[(nd + i) * tot + r];
        givens_solve(x, Kii, rhs, 9);
        for (int c = 0; c < nd; ++c) {
            double acc = 0.0;
            for (int i = 0; i < 9; ++i) acc += K[c * tot + nd + i] * x[i];
            ke[c * nd + r] = K[c * tot + r] - acc;
        }
    }
}

// Consistent mass: element_equations.rs:583-609 (get_rum_dfd0, solid branch)
void solid_me(int type, const double* xyz, double rho, double* me) {
    if (type == 81) type = 8;  // the internal DOF carry no mass (element_equations.rs:420-626)
    const TypeInfo t = type_info(type);
    const int nn = t.nn, tot = 3 * nn;
    std::fill(me, me + tot * tot, 0.0);
    double n[10], dndx[30];
    for (int p = 0; p < t.nip; ++p) {
        const double det = ip_data(type, nn, xyz, t.ip + 3 * p, n, dndx);
        const double djw = det * t.wt[p];
        for (int i = 0; i < tot; ++i)
            for (int j = 0; j < tot; ++j)
                if (i % 3 == j % 3) me[i * tot + j] += n[i / 3] * n[j / 3] * rho * djw;
    }
}

// ---------------------------------------------------------------------------
// shell4 (type 41): 4 nodes x 6 DOF (u v w thx thy thz) + 8 internal DOF,
// 2x2 Gauss points (element_meth.rs:326-370).  Flat elements in a plane
// z = const, where the reference's element frame (correct_orient,
// element_properties.rs:2052-2150) stays the section frame: identity here.
// ---------------------------------------------------------------------------
// Shape functions: element_soln_fields.rs:313-363 (4 bilinear, two in-plane
// incompatible modes 1-s^2, 1-t^2, four edge bubbles for w).
void shell_shape(double s, double t, double* n, double* ds, double* dt) {
    n[0] = 0.25 * (1 - s) * (1 - t); ds[0] = -0.25 * (1 - t); dt[0] = -0.25 * (1 - s);
    n[1] = 0.25 * (1 + s) * (1 - t); ds[1] = 0.25 * (1 - t);  dt[1] = -0.25 * (1 + s);
    n[2] = 0.25 * (1 + s) * (1 + t); ds[2] = 0.25 * (1 + t);  dt[2] = 0.25 * (1 + s);
    n[3] = 0.25 * (1 - s) * (1 + t); ds[3] = -0.25 * (1 + t); dt[3] = 0.25 * (1 - s);
    n[4] = 1 - s * s;             ds[4] = -2 * s;            dt[4] = 0;
    n[5] = 1 - t * t;             ds[5] = 0;                 dt[5] = -2 * t;
    n[6] = (1 - s * s) * (1 - t); ds[6] = -2 * s * (1 - t);  dt[6] = -1 + s * s;
    n[7] = (1 - t * t) * (1 + s); ds[7] = 1 - t * t;         dt[7] = -2 * t * (1 + s);
    n[8] = (1 - s * s) * (1 + t); ds[8] = -2 * s * (1 + t);  dt[8] = 1 - s * s;
    n[9] = (1 - t * t) * (1 - s); ds[9] = -1 + t * t;        dt[9] = -2 * t * (1 - s);
}

// Jacobian with the synthetic third axis (element_soln_fields.rs:404-422):
// J = [x_s x_t 0; y_s y_t 0; z_s z_t +-1], sign of x_s y_t - y_s x_t.
double shell_jac(const double* xyz, const double* ds, const double* dt, double* jinv) {
    double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = 0; a < 4; ++a)
        for (int i = 0; i < 3; ++i) {
            J[3 * i] += xyz[3 * a + i] * ds[a];
            J[3 * i + 1] += xyz[3 * a + i] * dt[a];
        }
    J[8] = (J[0] * J[4] - J[3] * J[1] > 0.0) ? 1.0 : -1.0;
    return det_inv(jinv, J, 3);
}

// Section stiffness ABD (element_properties.rs:766-876, get_abd_dfd0) of one
// isotropic layer of thickness t centred on the reference plane: A = t Q,
// B = 0, D = t^3/12 Q, and the transverse-shear and drilling diagonal entries
// copy A66.  Q = inverse of the plane-stress compliance (get_layer_q_dfd0
// :138-235, inverted by Givens QR).
void shell_abd(double E, double nu, double t, double* C) {
    const double G = E / (2.0 * (1.0 + nu));
    double S[9] = {1.0 / E, -nu / E, 0, -nu / E, 1.0 / E, 0, 0, 0, 1.0 / G}, Q[9];
    det_inv(Q, S, 3);
    for (int i = 0; i < 81; ++i) C[i] = 0.0;
    const double zmin = -0.5 * t, zmax = 0.5 * t;
    const double a = zmax - zmin, d = (zmax * zmax * zmax - zmin * zmin * zmin) / 3.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            C[9 * i + j] = a * Q[3 * i + j];
            C[9 * (i + 3) + j + 3] = d * Q[3 * i + j];
        }
    C[60] = C[70] = C[80] = C[20];
}

// Section deformation columns (element_soln_fields.rs:1160-1343,
// get_section_def_dfd0, single-DOF branches) for the 32 element DOF: node DOF
// 6a + c, then the internal DOF (shape function, component) =
// (4,u) (5,u) (4,v) (5,v) (6,w) (7,w) (8,w) (9,w) (element_meth.rs:357-372).
// Rows: eps_xx, eps_yy, gamma_xy, kappa_xx, kappa_yy, kappa_xy, gamma_xz,
// gamma_yz, drill.
void shell_bmat(const double* n, const double* dndx /* [10][3] */, double* B /* [9][32] */) {
    constexpr int tot = 32;
    for (int i = 0; i < 9 * tot; ++i) B[i] = 0.0;
    auto trans = [&](int col, int f, int c) {
        const double dx = dndx[3 * f], dy = dndx[3 * f + 1];
        if (c == 0) { B[0 * tot + col] = dx; B[2 * tot + col] = dy; B[8 * tot + col] = dy; }
        if (c == 1) { B[1 * tot + col] = dy; B[2 * tot + col] = dx; B[8 * tot + col] = -dx; }
        if (c == 2) { B[6 * tot + col] = dx; B[7 * tot + col] = dy; }
    };
    for (int a = 0; a < 4; ++a) {
        for (int c = 0; c < 3; ++c) trans(6 * a + c, a, c);
        const double dx = dndx[3 * a], dy = dndx[3 * a + 1], N = n[a];
        B[3 * tot + 6 * a + 4] = dx;            // kappa_xx = d thy / dx
        B[5 * tot + 6 * a + 4] = dy;            // kappa_xy = d thy/dy - d thx/dx
        B[6 * tot + 6 * a + 4] = N;             // gamma_xz = dw/dx + thy
        B[4 * tot + 6 * a + 3] = -dy;           // kappa_yy = -d thx / dy
        B[5 * tot + 6 * a + 3] = -dx;
        B[7 * tot + 6 * a + 3] = -N;            // gamma_yz = dw/dy - thx
        B[8 * tot + 6 * a + 5] = 2.0 * N;       // drill = 2 thz - dv/dx + du/dy
    }
    const int fi[8] = {4, 5, 4, 5, 6, 7, 8, 9}, ci[8] = {0, 0, 1, 1, 2, 2, 2, 2};
    for (int k = 0; k < 8; ++k) trans(24 + k, fi[k], ci[k]);
}

// Element stiffness (element_equations.rs:206-418, get_ruk_dfd0 shell branch:
// K += B^T (C B) detJ w) with the internal DOF condensed
// (element_equations.rs:19-57, condense_mat: K_nn - K_ni K_ii^-1 K_in by Givens
// QR), and the consistent mass (get_rum_dfd0 :514-581 with the section mass of
// get_shell_mass_dfd0, element_properties.rs:1354-1408: rho t on the
// translations, rho t^3/12 on the rotations) over the 24 node DOF.
// Layered shell section (get_layer_thk_z_dfd0 element_properties.rs:75-136,
// get_layer_q_dfd0 :138-222, transform_q_dfd0 :581-646, get_abd_dfd0
// :766-876, get_shell_mass_dfd0 :1354-1408).  Layer k: props[7k..7k+6] =
// E1, E2, nu12, G12, density, thickness, angle (degrees).  z_offset = 1 puts
// the reference plane on the upper surface, -1 on the lower one.  Outputs
// the 9x9 ABD (shear and drilling entries = A66) and the 6x6 section mass.
void shell_section(int n_lay, const double* props, double z_offset, double* C, double* msec) {
    for (int i = 0; i < 81; ++i) C[i] = 0.0;
    for (int i = 0; i < 36; ++i) msec[i] = 0.0;
    double tot = 0.0;
    for (int k = 0; k < n_lay; ++k) tot += props[7 * k + 5];
    double zc = -0.5 * tot * (1.0 + z_offset);
    for (int k = 0; k < n_lay; ++k) {
        const double* p = props + 7 * k;
        const double th = p[5], zmid = 0.5 * (zc + zc + th);
        zc += th;
        const double zmin = zmid - 0.5 * th, zmax = zmid + 0.5 * th;
        // layer Q: inverse of the plane-stress compliance
        double S[9] = {1.0 / p[0], -p[2] / p[0], 0.0, -p[2] / p[0], 1.0 / p[1], 0.0, 0.0, 0.0, 1.0 / p[3]}, Q[9];
        det_inv(Q, S, 3);
        // rotation to the section axes: Qbar = Ts Q Te^-1
        const double ang = kRPi0180 * p[6];
        const double c = std::cos(ang), s = std::sin(ang);
        const double a11 = c, a21 = s, a12 = -s, a22 = c;
        const double Ts[9] = {a11 * a11, a12 * a12, 2.0 * a11 * a12, a21 * a21, a22 * a22, 2.0 * a22 * a21,
                              a11 * a21, a12 * a22, a11 * a22 + a12 * a21};
        double Te[9], Tei[9], QT[9], Qb[9];
        std::copy(Ts, Ts + 9, Te);
        Te[2] *= 0.5;
        Te[5] *= 0.5;
        Te[6] *= 2.0;
        Te[7] *= 2.0;
        det_inv(Tei, Te, 3);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double a = 0.0;
                for (int l = 0; l < 3; ++l) a += Q[3 * i + l] * Tei[3 * l + j];
                QT[3 * i + j] = a;
            }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double a = 0.0;
                for (int l = 0; l < 3; ++l) a += Ts[3 * i + l] * QT[3 * l + j];
                Qb[3 * i + j] = a;
            }
        const double fa = zmax - zmin, fb = 0.5 * (zmax * zmax - zmin * zmin),
                     fd = (zmax * zmax * zmax - zmin * zmin * zmin) / 3.0;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                C[9 * i + j] += fa * Qb[3 * i + j];
                C[9 * i + j + 3] += fb * Qb[3 * i + j];
                C[9 * (i + 3) + j + 3] += fd * Qb[3 * i + j];
            }
        const double rho = p[4];
        msec[0] += rho * fa;
        msec[7] += rho * fa;
        msec[14] += rho * fa;
        msec[4] += rho * fb;
        msec[24] += rho * fb;
        msec[9] -= rho * fb;
        msec[19] -= rho * fb;
        msec[21] += rho * fd;
        msec[28] += rho * fd;
        msec[35] += rho * fd;
    }
    // the lower triangle mirrors the upper one; shear and drilling = A66
    for (int i = 1; i < 6; ++i)
        for (int j = 0; j < i; ++j) C[9 * i + j] = C[9 * j + i];
    C[60] = C[70] = C[80] = C[20];
}

void shell_km_sec(const double* xyz, const double* C, const double* msec, double* ke, double* me);

void shell_km(const double* xyz, double E, double nu, double rho, double t, double* ke, double* me) {
    double C[81], msec[36] = {0};
    shell_abd(E, nu, t, C);
    for (int c = 0; c < 3; ++c) {
        msec[7 * c] = rho * t;
        msec[7 * (c + 3)] = rho * t * t * t / 12.0;
    }
    shell_km_sec(xyz, C, msec, ke, me);
}

// Shell element matrices from a section: ABD C[81] and section mass msec[36].
void shell_km_sec(const double* xyz, const double* C, const double* msec, double* ke, double* me) {
    constexpr int tot = 32, nd = 24;
    std::vector<double> K(tot * tot, 0.0), B(9 * tot), CB(9 * tot);
    if (me) for (int i = 0; i < nd * nd; ++i) me[i] = 0.0;
    double n0[10], ds0[10], dt0[10], jinv0[9];
    shell_shape(0.0, 0.0, n0, ds0, dt0);
    shell_jac(xyz, ds0, dt0, jinv0);  // centroid Jacobian for the non-nodal functions
    const double sp[4][2] = {{-kR1ORt3, -kR1ORt3}, {kR1ORt3, -kR1ORt3}, {-kR1ORt3, kR1ORt3}, {kR1ORt3, kR1ORt3}};
    for (int ip = 0; ip < 4; ++ip) {
        double n[10], ds[10], dt[10], jinv[9], dndx[30];
        shell_shape(sp[ip][0], sp[ip][1], n, ds, dt);
        const double detj = shell_jac(xyz, ds, dt, jinv);
        for (int f = 0; f < 10; ++f) {
            const double* ji = (f < 4) ? jinv : jinv0;
            for (int k = 0; k < 3; ++k) dndx[3 * f + k] = ds[f] * ji[k] + dt[f] * ji[3 + k];
        }
        shell_bmat(n, dndx, B.data());
        for (int i = 0; i < 9; ++i)
            for (int c = 0; c < tot; ++c) {
                double acc = 0.0;
                for (int k = 0; k < 9; ++k) acc += C[9 * i + k] * B[k * tot + c];
                CB[i * tot + c] = acc * detj;  // weight 1
            }
        for (int r = 0; r < tot; ++r)
            for (int c = 0; c < tot; ++c) {
                double acc = 0.0;
                for (int k = 0; k < 9; ++k) acc += B[k * tot + r] * CB[k * tot + c];
                K[r * tot + c] += acc;
            }
        if (me)
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b)
                    for (int c = 0; c < 6; ++c)
                        for (int d = 0; d < 6; ++d)
                            me[(6 * a + c) * nd + 6 * b + d] += msec[6 * c + d] * n[a] * n[b] * detj;
    }
    // static condensation of the internal DOF
    double Kii[64];
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j) Kii[8 * i + j] = K[(24 + i) * tot + 24 + j];
    givens_factor(Kii, 8);
    for (int r = 0; r < nd; ++r) {
        double rhs[8], x[8];
        for (int i = 0; i < 8; ++i) rhs[i] = K[(24 + i) * tot + r];
        givens_solve(x, Kii, rhs, 8);
        for (int c = 0; c < nd; ++c) {
            double acc = 0.0;
            for (int i = 0; i < 8; ++i) acc += K[c * tot + 24 + i] * x[i];
            ke[c * nd + r] = K[c * tot + r] - acc;
        }
    }
}

// ---------------------------------------------------------------------------
// beam2 (type 2): 2 nodes x 6 DOF (u1 u2 u3 th1 th2 th3) + 2 internal DOF, a
// transverse bubble 1 - s^2 on the section-frame u2 and u3 (dof_table entries
// (2,1), (2,2)); 2 Gauss points +-1/sqrt(3), weight 1 (element_meth.rs:371-396).
// Shape functions (element_soln_fields.rs:364-379): N1 = (1-s)/2,
// N2 = (1+s)/2, N3 = 1 - s^2.  The reference stores the bubble's derivative
// -2s in node 1's slot (d_nds[0]; node 3's is d_nds[6]), which leaves the
// internal block without stiffness and node 1's axial derivative wrong; here
// the derivative goes to the bubble.  Jacobian (:415-421): [x1_s 0 0; x2_s 1 0;
// x3_s 0 +-1] in the section frame, so d/dx = (2/L) d/ds and detJ = L/2 when
// the frame's first axis is the element axis.  Section deformation
// (:1313-1321): [u1', u2' - th3, u3' + th2, th1', th2', th3'].  Section
// stiffness get_beam_stiff_dfd0 (element_properties.rs:878-1017), section
// mass get_beam_mass_dfd0 (:1410-1500); M uses the node DOF only
// (element_equations.rs:420-626, nd_dof = num_nds * dof_per_nd).
// sec[10] = area, area moments I1..I5 (int z, int y, int z^2, int y^2, int yz
// over the section, y and z along e2 and e3), polar moment J, and v (3), the
// direction fixing the xy plane; frame rows e1 = element axis,
// e3 = e1 x v / |e1 x v|, e2 = e3 x e1 (Section::set_orientation,
// section_meth.rs:21-50, with the element axis as x).
// ---------------------------------------------------------------------------
bool beam_frame(const double* xyz, const double* v, double* R, double* L) {
    double d[3], l2 = 0.0;
    for (int j = 0; j < 3; ++j) {
        d[j] = xyz[3 + j] - xyz[j];
        l2 += d[j] * d[j];
    }
    if (!(l2 > 0.0)) return false;
    *L = std::sqrt(l2);
    double e1[3] = {d[0] / *L, d[1] / *L, d[2] / *L};
    double e3[3] = {e1[1] * v[2] - e1[2] * v[1], e1[2] * v[0] - e1[0] * v[2], e1[0] * v[1] - e1[1] * v[0]};
    const double n3 = std::sqrt(e3[0] * e3[0] + e3[1] * e3[1] + e3[2] * e3[2]);
    const double nv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (!(n3 > 1e-9 * nv)) return false;
    for (int j = 0; j < 3; ++j) e3[j] /= n3;
    const double e2[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2], e3[0] * e1[1] - e3[1] * e1[0]};
    for (int j = 0; j < 3; ++j) {
        R[j] = e1[j];
        R[3 + j] = e2[j];
        R[6 + j] = e3[j];
    }
    return true;
}

// 6x6 section stiffness (element_properties.rs:921-1010, no stiffness-matrix
// override): isotropic E, G = E / (2 (1 + nu)).
void beam_cmat(double E, double nu, const double* sec, double* C) {
    const double G = E / (2.0 * (1.0 + nu));
    for (int i = 0; i < 36; ++i) C[i] = 0.0;
    C[0] = E * sec[0];
    C[4] = E * sec[1];
    C[5] = -E * sec[2];
    C[7] = G * sec[0];
    C[9] = -G * sec[1];
    C[14] = G * sec[0];
    C[15] = G * sec[2];
    C[21] = G * sec[6];
    C[28] = E * sec[3];
    C[29] = -E * sec[5];
    C[35] = E * sec[4];
    for (int i = 1; i < 6; ++i)
        for (int j = 0; j < i; ++j) C[6 * i + j] = C[6 * j + i];
}

// 6x6 section mass (element_properties.rs:1440-1497, no mass-matrix override)
void beam_msec(double rho, const double* sec, double* M) {
    for (int i = 0; i < 36; ++i) M[i] = 0.0;
    M[0] = M[7] = M[14] = rho * sec[0];
    M[4] = rho * sec[1];
    M[9] = -rho * sec[1];
    M[5] = -rho * sec[2];
    M[15] = rho * sec[2];
    M[21] = rho * sec[6];
    M[28] = rho * sec[3];
    M[29] = rho * sec[5];
    M[35] = rho * sec[4];
    for (int i = 1; i < 6; ++i)
        for (int j = 0; j < i; ++j) M[6 * i + j] = M[6 * j + i];
}

// Element stiffness ke[12][12] (internal DOF condensed, condense_mat
// element_equations.rs:19-57) and consistent mass me[12][12] (may be null) in
// global DOF 6 a + c.  The rows of B are built in global components through
// the frame, as get_inst_disp_dfd0 (element_soln_fields.rs:650-690) maps a
// global DOF to section-frame displacements; the internal DOF are section-frame
// amplitudes.  Returns false for a zero-length element or v along the axis.
// Section-strain rows B[6][14] at s: global node DOF 6 k + c, then the two
// section-frame bubble amplitudes.
void beam_bmat(const double* R, double a, double s, double B[6][14]) {
    const double N[2] = {0.5 * (1.0 - s), 0.5 * (1.0 + s)}, dN[2] = {-0.5 / a, 0.5 / a};
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 14; ++j) B[i][j] = 0.0;
    for (int k = 0; k < 2; ++k)
        for (int c = 0; c < 3; ++c) {
            const int ct = 6 * k + c, cr = 6 * k + 3 + c;
            B[0][ct] += dN[k] * R[c];
            B[1][ct] += dN[k] * R[3 + c];
            B[2][ct] += dN[k] * R[6 + c];
            B[1][cr] -= N[k] * R[6 + c];  // - th3
            B[2][cr] += N[k] * R[3 + c];  // + th2
            B[3][cr] += dN[k] * R[c];
            B[4][cr] += dN[k] * R[3 + c];
            B[5][cr] += dN[k] * R[6 + c];
        }
    B[1][12] = -2.0 * s / a;  // bubble on u2
    B[2][13] = -2.0 * s / a;  // bubble on u3
}

// Uncondensed stiffness K[14][14] of a beam2 element with section stiffness C.
void beam_kfull(const double* R, double a, const double* C, double* K) {
    constexpr int tot = 14;
    for (int i = 0; i < tot * tot; ++i) K[i] = 0.0;
    const double sp[2] = {-kR1ORt3, kR1ORt3};
    for (int ip = 0; ip < 2; ++ip) {
        double B[6][tot];
        beam_bmat(R, a, sp[ip], B);
        double CB[6][tot];
        for (int i = 0; i < 6; ++i)
            for (int c = 0; c < tot; ++c) {
                double acc = 0.0;
                for (int k = 0; k < 6; ++k) acc += C[6 * i + k] * B[k][c];
                CB[i][c] = acc * a;  // weight 1
            }
        for (int r = 0; r < tot; ++r)
            for (int c = 0; c < tot; ++c) {
                double acc = 0.0;
                for (int k = 0; k < 6; ++k) acc += B[k][r] * CB[k][c];
                K[r * tot + c] += acc;
            }
    }
}

// Given section matrices ov[72] (stiffness then mass, each used when its [0]
// entry is positive, element_properties.rs:896-920, :1430-1440; symmetric by
// construction, section_meth.rs:61-71) replace the computed ones.
void beam_given(const double* ov, double* C, double* M) {
    if (!ov) return;
    if (C && ov[0] > 0.0) std::copy(ov, ov + 36, C);
    if (M && ov[36] > 0.0) std::copy(ov + 36, ov + 72, M);
}

bool beam_km(const double* xyz, double E, double nu, double rho, const double* sec, double* ke, double* me,
             const double* ov = nullptr) {
    double R[9], L;
    if (!beam_frame(xyz, sec + 7, R, &L)) return false;
    constexpr int tot = 14, nd = 12;
    double C[36], K[tot * tot];
    beam_cmat(E, nu, sec, C);
    beam_given(ov, C, nullptr);
    const double a = 0.5 * L;  // detJ
    beam_kfull(R, a, C, K);
    if (me) {
        for (int i = 0; i < nd * nd; ++i) me[i] = 0.0;
        double Ms[36], RM[36];
        beam_msec(rho, sec, Ms);
        beam_given(ov, nullptr, Ms);
        // Rb^T Ms Rb with Rb = diag(R, R)
        auto rb = [&](int p, int q) { return (p / 3 == q / 3) ? R[3 * (p % 3) + q % 3] : 0.0; };
        for (int c = 0; c < 6; ++c)
            for (int d = 0; d < 6; ++d) {
                double acc = 0.0;
                for (int p = 0; p < 6; ++p)
                    for (int q = 0; q < 6; ++q) acc += rb(p, c) * Ms[6 * p + q] * rb(q, d);
                RM[6 * c + d] = acc;
            }
        const double sp[2] = {-kR1ORt3, kR1ORt3};
        for (int ip = 0; ip < 2; ++ip) {
            const double s = sp[ip];
            const double N[2] = {0.5 * (1.0 - s), 0.5 * (1.0 + s)};
            for (int k = 0; k < 2; ++k)
                for (int l = 0; l < 2; ++l)
                    for (int c = 0; c < 6; ++c)
                        for (int d = 0; d < 6; ++d) me[(6 * k + c) * nd + 6 * l + d] += N[k] * N[l] * a * RM[6 * c + d];
        }
    }
    double Kii[4] = {K[12 * tot + 12], K[12 * tot + 13], K[13 * tot + 12], K[13 * tot + 13]};
    givens_factor(Kii, 2);
    for (int r = 0; r < nd; ++r) {
        double rhs[2] = {K[12 * tot + r], K[13 * tot + r]}, x[2];
        givens_solve(x, Kii, rhs, 2);
        for (int c = 0; c < nd; ++c) ke[c * nd + r] = K[c * tot + r] - (K[c * tot + 12] * x[0] + K[c * tot + 13] * x[1]);
    }
    return true;
}

// Section-strain pairs P[36] = sum_ip detJ eps(lambda) eps(u)^T of one beam2
// element with its bubble amplitudes recovered from the node values
// (alpha = -K_ii^-1 K_in f, update_internal element_equations.rs:147-194), so
// that lambda^T (dK_e/dD) u = sum_ij (dC/dD)_ij P_ij for any section-stiffness
// parameter D (d_relasticd_d, model_analysis.rs:1379-1457).
bool beam_pairs(const double* xyz, double E, double nu, const double* sec, const double* ue, const double* le,
                double* P, const double* ov = nullptr) {
    double R[9], L;
    if (!beam_frame(xyz, sec + 7, R, &L)) return false;
    constexpr int tot = 14;
    double C[36], K[tot * tot];
    beam_cmat(E, nu, sec, C);
    beam_given(ov, C, nullptr);
    const double a = 0.5 * L;
    beam_kfull(R, a, C, K);
    double Kii[4] = {K[12 * tot + 12], K[12 * tot + 13], K[13 * tot + 12], K[13 * tot + 13]};
    givens_factor(Kii, 2);
    double uf[tot], lf[tot];
    for (int c = 0; c < 12; ++c) {
        uf[c] = ue[c];
        lf[c] = le[c];
    }
    for (double* f : {uf, lf}) {
        double rhs[2] = {0.0, 0.0}, x[2];
        for (int i = 0; i < 2; ++i)
            for (int c = 0; c < 12; ++c) rhs[i] += K[(12 + i) * tot + c] * f[c];
        givens_solve(x, Kii, rhs, 2);
        f[12] = -x[0];
        f[13] = -x[1];
    }
    for (int i = 0; i < 36; ++i) P[i] = 0.0;
    const double sp[2] = {-kR1ORt3, kR1ORt3};
    for (int ip = 0; ip < 2; ++ip) {
        double B[6][tot], eu[6] = {0}, el[6] = {0};
        beam_bmat(R, a, sp[ip], B);
        for (int q = 0; q < 6; ++q)
            for (int c = 0; c < tot; ++c) {
                eu[q] += B[q][c] * uf[c];
                el[q] += B[q][c] * lf[c];
            }
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) P[6 * i + j] += el[i] * eu[j] * a;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Sparse matrix with a fixed pattern (sorted columns) and element-order
// accumulation.  The reference keeps row linked lists and add_entry appends or
// accumulates (list_ent_meth.rs:6-18); every (i,j) sum is accumulated in
// element order, which this CSR reproduces.
// ---------------------------------------------------------------------------
struct Csr {
    int n = 0;
    std::vector<int64_t> ptr;
    std::vector<int32_t> col;
    std::vector<double> val;
    int64_t find(int r, int c) const {
        auto b = col.begin() + ptr[r], e = col.begin() + ptr[r + 1];
        auto it = std::lower_bound(b, e, c);
        return (it != e && *it == c) ? (it - col.begin()) : -1;
    }
    void matvec(const double* x, double* y) const {  // y += A x (list_ent_meth.rs:64-79)
        for (int r = 0; r < n; ++r) {
            double acc = y[r];
            for (int64_t k = ptr[r]; k < ptr[r + 1]; ++k) acc += val[k] * x[col[k]];
            y[r] = acc;
        }
    }
    double max_abs() const {  // list_ent_meth.rs:81-94
        double m = 0.0;
        for (double v : val) m = std::max(m, std::fabs(v));
        return m;
    }
};

}  // namespace

struct orc_model {
    TypeInfo ti;
    int n_nodes = 0, n_el = 0, dpn = 3, n_dof = 0;
    std::vector<double> xyz, E, nu, rho, thk;
    std::vector<int32_t> conn;
    // constraint rows (const_meth.rs:30-90 builds C with one row per set member)
    std::vector<int32_t> c_ptr, c_dof;
    std::vector<double> c_coef, c_rhs;
    Csr K, M;           // K holds the full solve matrix (K + c_M M [+ c_D D] when dynamic)
    Csr D;              // damping matrix (Rayleigh c_M M + c_K K + material B^T D B)
    bool dynamic = false;
    double cM = 0.0;    // coefficient of M inside K (Newmark)
    double cD = 0.0;    // coefficient of D inside K (Newmark: dt gamma cM)
    // per-element 6x6 stiffness (engineering constants through the compliance
    // form, element_properties.rs:648-764) replacing the isotropic one
    std::vector<double> cmat;
    // damping (element_equations.rs:628-850): Rayleigh coefficients and the
    // materials' 6x6 damping matrices per element (element_properties.rs:1537-1575)
    double ray_cm = 0.0, ray_ck = 0.0;
    std::vector<double> dmat;
    bool lump = false;  // row-sum lumped mass (element_equations.rs:950-971)
    bool damped() const { return ray_cm != 0.0 || ray_ck != 0.0 || !dmat.empty(); }
    double sf = 0.0;    // penalty scale (model_analysis.rs:255-259)
    bool assembled = false;
    // shell4: physical nodes and connectivity (the assembly view above uses
    // two pseudo-nodes per physical node)
    bool shell = false;
    int n_phys = 0;
    // layered shell sections per element: ABD [n_el][81], section mass [n_el][36]
    std::vector<double> shell_abd81, shell_msec36;
    std::vector<double> phys_xyz;
    std::vector<int32_t> conn4;
    // beam2: the same two-pseudo-node view; 2 physical nodes per element and
    // the section table [n_el][10] (beam_km)
    bool beam = false;
    std::vector<int32_t> conn2;
    std::vector<double> beam_sec;
    std::vector<double> beam_cm;  // given section matrices [n_el][72] (may be empty)
    const double* beam_ov(int e) const { return beam_cm.empty() ? nullptr : &beam_cm[(size_t)e * 72]; }
    bool structural() const { return shell || beam; }
};

namespace {

void elem_xyz(const orc_model* m, int e, double* xyz) {
    const int nn = m->ti.nn;
    for (int a = 0; a < nn; ++a) {
        const int nd = m->conn[(size_t)e * nn + a];
        for (int j = 0; j < 3; ++j) xyz[3 * a + j] = m->xyz[3 * (size_t)nd + j];
    }
}

// Element stiffness (and mass when me != null) in the assembly view's DOF
// order: solids from the isotropic C, shells from the shell4 routine.
void elem_km(const orc_model* m, int e, double* ke, double* me) {
    if (m->beam) {
        double xyz[6];
        for (int a = 0; a < 2; ++a)
            for (int j = 0; j < 3; ++j) xyz[3 * a + j] = m->phys_xyz[3 * (size_t)m->conn2[(size_t)e * 2 + a] + j];
        beam_km(xyz, m->E[e], m->nu[e], m->rho[e], &m->beam_sec[(size_t)e * 10], ke, me, m->beam_ov(e));
        return;
    }
    if (m->shell) {
        double xyz[12];
        for (int a = 0; a < 4; ++a)
            for (int j = 0; j < 3; ++j) xyz[3 * a + j] = m->phys_xyz[3 * (size_t)m->conn4[(size_t)e * 4 + a] + j];
        if (!m->shell_abd81.empty())
            shell_km_sec(xyz, &m->shell_abd81[(size_t)e * 81], &m->shell_msec36[(size_t)e * 36], ke, me);
        else
            shell_km(xyz, m->E[e], m->nu[e], m->rho[e], m->thk[e], ke, me);
        return;
    }
    double xyz[30], C[36];
    elem_xyz(m, e, xyz);
    if (!m->cmat.empty()) std::copy(m->cmat.begin() + (size_t)e * 36, m->cmat.begin() + (size_t)(e + 1) * 36, C);
    else iso_cmat(m->E[e], m->nu[e], C);
    solid_ke(m->ti.type, xyz, C, ke);
    if (me) solid_me(m->ti.type, xyz, m->rho[e], me);
}

// Element damping matrix (get_rud_dfd0, element_equations.rs:628-850, for
// elements without internal DOF): ray_cm M_e + ray_ck K_e + sum_gp B^T D B
// w detJ with the element's material damping matrix D.
void elem_damp(const orc_model* m, int e, const double* ke, const double* me, double* de) {
    const int nn = m->ti.nn, tot = 3 * nn;
    for (int i = 0; i < tot * tot; ++i) de[i] = m->ray_cm * me[i] + m->ray_ck * ke[i];
    if (m->dmat.empty()) return;
    double xyz[30], kd[900];
    elem_xyz(m, e, xyz);
    solid_ke(m->ti.type, xyz, &m->dmat[(size_t)e * 36], kd);
    for (int i = 0; i < tot * tot; ++i) de[i] += kd[i];
}

// Row-sum lumping of an element mass (element_equations.rs:950-971: the
// inertial residual at unit acceleration of every DOF on the diagonal).
void lump_rows(int tot, double* me) {
    for (int i = 0; i < tot; ++i) {
        double s2 = 0.0;
        for (int j = 0; j < tot; ++j) s2 += me[i * tot + j];
        for (int j = 0; j < tot; ++j) me[i * tot + j] = (i == j) ? s2 : 0.0;
    }
}

// Node adjacency from element connectivity, sorted; defines the full 3x3-block
// pattern the reference creates by add_entry on every element DOF pair.
void build_pattern(const orc_model* m, Csr& A) {
    const int nn = m->ti.nn, dpn = m->dpn;
    std::vector<std::vector<int32_t>> adj(m->n_nodes);
    for (int e = 0; e < m->n_el; ++e)
        for (int a = 0; a < nn; ++a)
            for (int b = 0; b < nn; ++b)
                adj[m->conn[(size_t)e * nn + a]].push_back(m->conn[(size_t)e * nn + b]);
    A.n = m->n_dof;
    A.ptr.assign(A.n + 1, 0);
    for (int nd = 0; nd < m->n_nodes; ++nd) {
        auto& v = adj[nd];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        for (int c = 0; c < dpn; ++c) A.ptr[(size_t)nd * dpn + c + 1] = (int64_t)v.size() * dpn;
    }
    for (int r = 0; r < A.n; ++r) A.ptr[r + 1] += A.ptr[r];
    A.col.resize(A.ptr[A.n]);
    for (int nd = 0; nd < m->n_nodes; ++nd)
        for (int c = 0; c < dpn; ++c) {
            int64_t k = A.ptr[(size_t)nd * dpn + c];
            for (int32_t nb : adj[nd])
                for (int cc = 0; cc < dpn; ++cc) A.col[k++] = nb * dpn + cc;
        }
    A.val.assign(A.col.size(), 0.0);
}

// Penalty constraint operator pieces (const_meth.rs:92-119).
// y += sf * C^T (C x)
void constraint_apply(const orc_model* m, const double* x, double* y) {
    const int nr = (int)m->c_rhs.size();
    for (int r = 0; r < nr; ++r) {
        double cx = 0.0;
        for (int k = m->c_ptr[r]; k < m->c_ptr[r + 1]; ++k) cx += m->c_coef[k] * x[m->c_dof[k]];
        cx *= m->sf;
        for (int k = m->c_ptr[r]; k < m->c_ptr[r + 1]; ++k) y[m->c_dof[k]] += m->c_coef[k] * cx;
    }
}
// f += -sf C^T (C u - q)   (const_meth.rs:105-119 get_load)
void constraint_load(const orc_model* m, const double* u, double* f) {
    const int nr = (int)m->c_rhs.size();
    for (int r = 0; r < nr; ++r) {
        double q = -m->c_rhs[r];
        for (int k = m->c_ptr[r]; k < m->c_ptr[r + 1]; ++k) q += m->c_coef[k] * u[m->c_dof[k]];
        q *= -m->sf;
        for (int k = m->c_ptr[r]; k < m->c_ptr[r + 1]; ++k) f[m->c_dof[k]] += m->c_coef[k] * q;
    }
}

void apply_A(const orc_model* m, const double* x, double* y) {
    std::fill(y, y + m->n_dof, 0.0);
    m->K.matvec(x, y);
    constraint_apply(m, x, y);
}

// ---------------------------------------------------------------------------
// Skyline LDL^T restricted to diagonal blocks (lower_tri_mat_meth.rs:15-241).
// Works in the permuted ("reference") DOF numbering given by perm (new->old).
// ---------------------------------------------------------------------------
struct Skyline {
    int dim = 0, max_bw = 0;
    std::vector<int64_t> range;  // start offset per row, size dim+1
    std::vector<int32_t> min_col;
    std::vector<double> mat;
    std::vector<double> z;
};

struct PermOp {
    std::vector<int32_t> new_of_old, old_of_new;  // DOF permutations
};

// allocate_from_sparse_mat :15-90 + populate_from_sparse_mat :96-140
void skyline_build(const orc_model* m, const PermOp& P, int block_dofs, Skyline& S) {
    const int n = m->n_dof;
    S.dim = n;
    std::vector<int64_t> rng(n + 1, 0);
    for (int rn = 0; rn < n; ++rn) rng[rn] = 1;
    // element matrix contributions
    for (int ro = 0; ro < n; ++ro) {
        const int rn = P.new_of_old[ro];
        const int blk_mc = block_dofs * (rn / block_dofs);
        for (int64_t k = m->K.ptr[ro]; k < m->K.ptr[ro + 1]; ++k) {
            const int cn = P.new_of_old[m->K.col[k]];
            if (cn <= rn && cn >= blk_mc) rng[rn] = std::max<int64_t>(rng[rn], rn - cn + 1);
        }
    }
    // constraint couplings (C^T C)
    const int nr = (int)m->c_rhs.size();
    for (int r = 0; r < nr; ++r)
        for (int k = m->c_ptr[r]; k < m->c_ptr[r + 1]; ++k) {
            const int i2 = P.new_of_old[m->c_dof[k]];
            const int blk_mc = block_dofs * (i2 / block_dofs);
            for (int k2 = m->c_ptr[r]; k2 < m->c_ptr[r + 1]; ++k2) {
                const int i3 = P.new_of_old[m->c_dof[k2]];
                if (i3 <= i2 && i3 >= blk_mc) rng[i2] = std::max<int64_t>(rng[i2], i2 - i3 + 1);
            }
        }
    S.min_col.resize(n);
    S.range.assign(n + 1, 0);
    S.max_bw = 0;
    for (int i = 0; i < n; ++i) {
        S.min_col[i] = i - (int)(rng[i] - 1);
        S.max_bw = std::max<int>(S.max_bw, (int)rng[i]);
        S.range[i + 1] = S.range[i] + rng[i];
    }
    S.mat.assign(S.range[n], 0.0);
    S.z.assign(n, 0.0);
    for (int ro = 0; ro < n; ++ro) {
        const int rn = P.new_of_old[ro];
        for (int64_t k = m->K.ptr[ro]; k < m->K.ptr[ro + 1]; ++k) {
            const int cn = P.new_of_old[m->K.col[k]];
            if (cn <= rn && cn >= S.min_col[rn]) S.mat[S.range[rn] + (cn - S.min_col[rn])] += m->K.val[k];
        }
    }
    for (int r = 0; r < nr; ++r)
        for (int k = m->c_ptr[r]; k < m->c_ptr[r + 1]; ++k) {
            const int i2 = P.new_of_old[m->c_dof[k]];
            for (int k2 = m->c_ptr[r]; k2 < m->c_ptr[r + 1]; ++k2) {
                const int i3 = P.new_of_old[m->c_dof[k2]];
                if (i3 <= i2 && i3 >= S.min_col[i2])
                    S.mat[S.range[i2] + (i3 - S.min_col[i2])] += m->sf * m->c_coef[k] * m->c_coef[k2];
            }
        }
}

// ldl_factor :142-192
void skyline_factor(Skyline& S) {
    const int n = S.dim;
    std::vector<double> ld(n, 0.0);
    for (int c = 0; c < n; ++c) {
        int64_t i3 = S.range[c];
        for (int k = S.min_col[c]; k < c; ++k) {
            ld[k] = S.mat[i3] * S.mat[S.range[k + 1] - 1];
            ++i3;
        }
        double sum = 0.0;
        int64_t i2 = S.range[c];
        for (int k = S.min_col[c]; k < c; ++k) sum += ld[k] * S.mat[i2++];
        S.mat[S.range[c + 1] - 1] -= sum;
        const double dcc = S.mat[S.range[c + 1] - 1];
        for (int r = c + 1; r < c + S.max_bw && r < n; ++r) {
            if (S.min_col[r] <= c) {
                const int st = std::max(S.min_col[r], S.min_col[c]);
                int64_t i4 = S.range[r] + (st - S.min_col[r]);
                double s2 = 0.0;
                for (int k = st; k < c; ++k) s2 += ld[k] * S.mat[i4++];
                const int64_t idx = S.range[r] + (c - S.min_col[r]);
                S.mat[idx] = (S.mat[idx] - s2) / dcc;
            }
        }
    }
}

// ldl_solve :194-227
void skyline_solve(Skyline& S, double* x, const double* rhs) {
    const int n = S.dim;
    S.z[0] = rhs[0];
    for (int i = 1; i < n; ++i) {
        int64_t k = S.range[i];
        double sum = 0.0;
        for (int c = S.min_col[i]; c < i; ++c) sum += S.mat[k++] * S.z[c];
        S.z[i] = rhs[i] - sum;
    }
    for (int i = n - 1; i >= 0; --i) {
        double sum = 0.0;
        const int stop = std::min(n, i + S.max_bw + 1);
        for (int r = i + 1; r < stop; ++r)
            if (i >= S.min_col[r]) sum += S.mat[S.range[r] + (i - S.min_col[r])] * x[r];
        x[i] = S.z[i] / S.mat[S.range[i + 1] - 1] - sum;
    }
}

// pos_def :229-241
bool skyline_pos_def(const Skyline& S) {
    for (int i = 0; i < S.dim; ++i)
        if (S.mat[S.range[i + 1] - 1] < 0.0) return false;
    return true;
}

// Node reordering: model_prep.rs:56-303 (reorder_nodes).  Connectivity sets
// keep insertion order (nd_el_set_meth.rs:5-13 add_if_absent); constraint
// couplings per model_prep.rs:20-54 (add_constraint_conn) for rows built from
// one node set with a single term (each constrained node coupled to itself).
std::vector<int32_t> reorder_nodes(const orc_model* m, int block_dim) {
    const int nn = m->ti.nn, N = m->n_nodes;
    std::vector<std::vector<int32_t>> conn(N);
    auto add = [&](int a, int b) {
        auto& v = conn[a];
        if (std::find(v.begin(), v.end(), b) == v.end()) v.push_back(b);
    };
    for (int e = 0; e < m->n_el; ++e)
        for (int i = 0; i < nn; ++i)
            for (int j = i + 1; j < nn; ++j) {
                const int a = m->conn[(size_t)e * nn + i], b = m->conn[(size_t)e * nn + j];
                add(a, b);
                add(b, a);
            }
    const int nr = (int)m->c_rhs.size();
    for (int r = 0; r < nr; ++r)
        for (int k = m->c_ptr[r]; k < m->c_ptr[r + 1]; ++k)
            for (int k2 = m->c_ptr[r]; k2 < m->c_ptr[r + 1]; ++k2) {
                const int a = m->c_dof[k] / m->dpn, b = m->c_dof[k2] / m->dpn;
                add(a, b);
                add(b, a);
            }
    int min_ct = N, min_nd = 0;
    for (int i = 0; i < N; ++i)
        if ((int)conn[i].size() < min_ct) { min_nd = i; min_ct = (int)conn[i].size(); }
    std::vector<int32_t> ordered(N, -1);
    std::vector<char> ins(N, 0);
    ordered[0] = min_nd;
    int on_len = 1, on_i = 0, nd1 = min_nd, since = 0;
    ins[min_nd] = 1;
    while (on_len < N) {
        size_t it = 0;
        bool end = false;
        int nd2 = -1;
        while (!end && since < block_dim) {
            if (it < conn[nd1].size()) nd2 = conn[nd1][it++];
            else end = true;
            // the reference re-tests the last neighbour when the list ends
            if (nd2 >= 0 && !ins[nd2]) {
                ordered[on_len++] = nd2;
                ins[nd2] = 1;
                ++since;
            }
        }
        if (on_len < N) {
            if (since >= block_dim || on_i == on_len - 1) {
                nd1 = ordered[on_len - 1];
                double best = 1e100;
                int best_i = min_nd;
                const double* p1 = &m->xyz[3 * (size_t)nd1];
                for (int i = 0; i < N; ++i)
                    if (!ins[i]) {
                        const double* p2 = &m->xyz[3 * (size_t)i];
                        const double dx = p1[0] - p2[0], dy = p1[1] - p2[1], dz = p1[2] - p2[2];
                        const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
                        if (d < best) { best = d; best_i = i; }
                    }
                min_nd = best_i;
                ordered[on_len++] = min_nd;
                nd1 = min_nd;
                ins[min_nd] = 1;
                ++since;
                on_i = on_len - 1;
                if (since >= block_dim) since = 0;
            } else {
                ++on_i;
                nd1 = ordered[on_i];
            }
        }
    }
    return ordered;
}

// block_dim rule: model_prep.rs:888-902 (smallest multiple of 6 whose square
// reaches the node count); the elastic preconditioner uses 6*block_dim DOFs
// per block (model_prep.rs:610).
int default_block_dim(int n_nodes) {
    int b = 6;
    while (b * b < n_nodes) b += 6;
    return b;
}

struct Precond {
    int kind = ORC_PC_NONE;
    std::vector<double> dinv;
    PermOp P;
    Skyline S;
    std::vector<double> tmp_in, tmp_out;
    void setup(const orc_model* m, int kind_in, int block_dim) {
        kind = kind_in;
        const int n = m->n_dof;
        if (kind == ORC_PC_JACOBI) {
            std::vector<double> d(n, 0.0);
            for (int r = 0; r < n; ++r) {
                const int64_t k = m->K.find(r, r);
                d[r] = (k >= 0) ? m->K.val[k] : 0.0;
            }
            const int nr = (int)m->c_rhs.size();
            for (int r = 0; r < nr; ++r)
                for (int k = m->c_ptr[r]; k < m->c_ptr[r + 1]; ++k)
                    d[m->c_dof[k]] += m->sf * m->c_coef[k] * m->c_coef[k];
            dinv.resize(n);
            for (int r = 0; r < n; ++r) dinv[r] = 1.0 / d[r];
        } else if (kind == ORC_PC_BLOCK_LDL || kind == ORC_PC_DIRECT) {
            int block_dofs;
            std::vector<int32_t> order;
            if (kind == ORC_PC_DIRECT) {
                block_dofs = 2000000000;  // model_prep.rs:885-887
                order = reorder_nodes(m, 2000000000);
            } else {
                const int bd = block_dim > 0 ? block_dim : default_block_dim(m->n_nodes);
                block_dofs = 6 * bd;
                order = reorder_nodes(m, bd);
            }
            P.old_of_new.resize(n);
            P.new_of_old.resize(n);
            for (int i = 0; i < m->n_nodes; ++i)
                for (int c = 0; c < m->dpn; ++c) {
                    const int o = order[i] * m->dpn + c, nw = i * m->dpn + c;
                    P.old_of_new[nw] = o;
                    P.new_of_old[o] = nw;
                }
            skyline_build(m, P, block_dofs, S);
            skyline_factor(S);
            tmp_in.resize(n);
            tmp_out.resize(n);
        }
    }
    void apply(const double* g, double* w) {
        const int n = (int)(kind == ORC_PC_JACOBI ? dinv.size() : tmp_in.size());
        if (kind == ORC_PC_JACOBI) {
            for (int i = 0; i < n; ++i) w[i] = dinv[i] * g[i];
        } else if (kind == ORC_PC_BLOCK_LDL || kind == ORC_PC_DIRECT) {
            for (int i = 0; i < n; ++i) tmp_in[i] = g[P.old_of_new[i]];
            skyline_solve(S, tmp_out.data(), tmp_in.data());
            for (int i = 0; i < n; ++i) w[P.old_of_new[i]] = tmp_out[i];
        }
    }
};


double true_rel_residual(const orc_model* m, const double* f, const double* u) {
    const int n = m->n_dof;
    std::vector<double> y(n);
    apply_A(m, u, y.data());
    double rr = 0.0, ff = 0.0;
    for (int i = 0; i < n; ++i) {
        const double r = f[i] - y[i];
        rr += r * r;
        ff += f[i] * f[i];
    }
    return ff > 0.0 ? std::sqrt(rr / ff) : std::sqrt(rr);
}

// PCG: matrix_functions.rs:285-362 (conj_grad_sparse).  x0 = 0, g = A x - b,
// stop when g^T M^-1 g <= conv_tol (reference rule) or, with the relative
// rule, when ||g||_2 <= tol ||b||_2.
int pcg(orc_model* m, Precond& pc, const double* rhs, double* soln, int stop_rule, double tol,
        int max_it, orc_stats* st) {
    const int n = m->n_dof;
    std::vector<double> h(n), g(n), z(n), w(n);
    double bb = 0.0;
    for (int i = 0; i < n; ++i) {
        soln[i] = 0.0;
        g[i] = -rhs[i];
        bb += rhs[i] * rhs[i];
    }
    const double stop_gg = tol * tol * bb;
    if (pc.kind == ORC_PC_NONE) std::copy(g.begin(), g.end(), w.begin());
    else pc.apply(g.data(), w.data());
    double res = 0.0, gg = 0.0;
    for (int i = 0; i < n; ++i) {
        h[i] = -w[i];
        res += g[i] * w[i];
        gg += g[i] * g[i];
    }
    auto keep_going = [&]() {
        return stop_rule == ORC_STOP_REFERENCE ? (res > tol) : (gg > stop_gg);
    };
    int it = 0, status = 0;
    while (it < max_it && keep_going()) {
        apply_A(m, h.data(), z.data());
        double dp = 0.0;
        for (int i = 0; i < n; ++i) dp += h[i] * z[i];
        const double alpha = res / dp;
        for (int i = 0; i < n; ++i) {
            soln[i] += alpha * h[i];
            g[i] += alpha * z[i];
        }
        if (pc.kind == ORC_PC_NONE) std::copy(g.begin(), g.end(), w.begin());
        else pc.apply(g.data(), w.data());
        double rn = 0.0;
        gg = 0.0;
        for (int i = 0; i < n; ++i) {
            rn += g[i] * w[i];
            gg += g[i] * g[i];
        }
        const double beta = rn / res;
        for (int i = 0; i < n; ++i) h[i] = -w[i] + beta * h[i];
        res = rn;
        ++it;
        if (!std::isfinite(res)) { status = 2; break; }
    }
    if (status == 0 && keep_going()) status = 1;
    if (st) {
        st->iterations += it;
        st->status = status;
        st->final_res = res;
    }
    return status;
}

}  // namespace


// ---------------------------------------------------------------------------
// Modal analysis (frequency job): model_analysis.rs:711-880 and
// matrix_functions.rs:940-1265
// ---------------------------------------------------------------------------
namespace {

// sym_eigen_solve (matrix_functions.rs:940-1097) with tri_diag = 1: pair i
// starts from sin(j (i+1)), is Gram-Schmidt projected off the converged
// vectors and iterated v <- T v / |T v| (T v deflated likewise) until
// |v.Tv| >= (1 - 1e-8) |T v| or 10000 products; eigenvalue = v.Tv; the
// pairs are sorted ascending (bubble sort, stable for ties).  T is row-major
// d x d, read on its tridiagonal band only.
void sym_eigen_tri(const std::vector<double>& T, int d, std::vector<double>& vals, std::vector<double>& vecs) {
    std::vector<double> v1(d), v2(d), tmp((size_t)d * d);
    vals.assign(d, 0.0);
    for (int i = 0; i < d; ++i) {
        for (int j = 0; j < d; ++j) v1[j] = std::sin((double)j * (double)(i + 1));
        for (int k = 0; k < i; ++k) {
            double dp = 0.0;
            for (int j = 0; j < d; ++j) dp += v1[j] * tmp[(size_t)k * d + j];
            for (int j = 0; j < d; ++j) v1[j] -= dp * tmp[(size_t)k * d + j];
        }
        double mag = 0.0;
        for (int j = 0; j < d; ++j) mag += v1[j] * v1[j];
        mag = 1.0 / std::sqrt(mag);
        for (int j = 0; j < d; ++j) v1[j] *= mag;
        double dp = 0.0;
        int loops = 0;
        while (std::fabs(dp) < 0.99999999 * mag && loops < 10000) {
            for (int r = 0; r < d; ++r) {
                const int c0 = r == 0 ? 0 : r - 1, c1 = std::min(r + 2, d);
                double acc = 0.0;
                for (int c = c0; c < c1; ++c) acc += T[(size_t)r * d + c] * v1[c];
                v2[r] = acc;
            }
            for (int k = 0; k < i; ++k) {
                double q = 0.0;
                for (int j = 0; j < d; ++j) q += v2[j] * tmp[(size_t)k * d + j];
                for (int j = 0; j < d; ++j) v2[j] -= q * tmp[(size_t)k * d + j];
            }
            mag = 0.0;
            dp = 0.0;
            for (int j = 0; j < d; ++j) {
                mag += v2[j] * v2[j];
                dp += v1[j] * v2[j];
            }
            mag = std::sqrt(mag);
            for (int j = 0; j < d; ++j) v1[j] = v2[j] / mag;
            ++loops;
        }
        vals[i] = dp;
        std::copy(v1.begin(), v1.end(), tmp.begin() + (size_t)i * d);
    }
    std::vector<int> order(d);
    std::iota(order.begin(), order.end(), 0);
    for (int pass = 0; pass < d; ++pass)
        for (int j = 0; j + 1 < d; ++j)
            if (vals[j + 1] < vals[j]) {
                std::swap(vals[j], vals[j + 1]);
                std::swap(order[j], order[j + 1]);
            }
    vecs.resize((size_t)d * d);
    for (int i = 0; i < d; ++i)
        std::copy(tmp.begin() + (size_t)order[i] * d, tmp.begin() + (size_t)(order[i] + 1) * d,
                  vecs.begin() + (size_t)i * d);
}

// eigen_sparse_direct (matrix_functions.rs:1099-1265): Lanczos on
// D^1/2 A^-1 D^1/2 with h = 5 n_pairs vectors, the first A^-1 s with
// s_i = sin(n + i), each new vector orthogonalised against the previous two
// only; Ritz pairs from the largest Ritz value down (never the smallest),
// eigenvector D^-1/2 Q y scaled to unit 2-norm, a pair skipped when its
// vector has |cos| >= 0.9 with the previously accepted one; eigenvalue
// 1 / Ritz value.
int lanczos_direct(const std::function<void(const double*, double*)>& solve, const std::vector<double>& D,
                   int n_pairs, double* e_vals, double* e_vecs) {
    const int n = (int)D.size();
    const int h = 5 * n_pairs;
    if (h < 2 || h > n) return -2;
    std::vector<double> Q((size_t)h * n), t1(n), t2(n), T((size_t)h * (h - 1), 0.0), sq(n);
    for (int i = 0; i < n; ++i) sq[i] = std::sqrt(D[i]);
    for (int i = 0; i < n; ++i) t2[i] = std::sin((double)(n + i));
    solve(t2.data(), Q.data());
    double mag = 0.0;
    for (int i = 0; i < n; ++i) mag += Q[i] * Q[i];
    mag = 1.0 / std::sqrt(mag);
    for (int i = 0; i < n; ++i) Q[i] *= mag;
    for (int j = 1; j < h; ++j) {
        const double* qp = &Q[(size_t)(j - 1) * n];
        for (int i = 0; i < n; ++i) t1[i] = sq[i] * qp[i];
        solve(t1.data(), t2.data());
        for (int i = 0; i < n; ++i) t1[i] = t2[i] * sq[i];
        for (int k = (j == 1 ? 0 : j - 2); k < j; ++k) {
            const double* qk = &Q[(size_t)k * n];
            double dp = 0.0;
            for (int i = 0; i < n; ++i) dp += t1[i] * qk[i];
            for (int i = 0; i < n; ++i) t1[i] -= dp * qk[i];
            T[(size_t)(h - 1) * k + (j - 1)] = dp;
        }
        mag = 0.0;
        for (int i = 0; i < n; ++i) mag += t1[i] * t1[i];
        mag = std::sqrt(mag);
        T[(size_t)(h - 1) * j + (j - 1)] = mag;
        double* qj = &Q[(size_t)j * n];
        for (int i = 0; i < n; ++i) qj[i] = t1[i] / mag;
    }
    const int d = h - 1;
    std::vector<double> Td(T.begin(), T.begin() + (size_t)d * d), th, S;
    sym_eigen_tri(Td, d, th, S);
    int acc = 0;
    for (int k = d - 1; acc < n_pairs && k > 0; --k) {
        std::fill(t1.begin(), t1.end(), 0.0);
        for (int c = 0; c < d; ++c) {
            const double y = S[(size_t)k * d + c];
            const double* qc = &Q[(size_t)c * n];
            for (int i = 0; i < n; ++i) t1[i] += qc[i] * y;
        }
        mag = 0.0;
        for (int i = 0; i < n; ++i) {
            t2[i] = t1[i] / sq[i];
            mag += t2[i] * t2[i];
        }
        mag = 1.0 / std::sqrt(mag);
        for (int i = 0; i < n; ++i) t2[i] *= mag;
        if (acc > 0) {
            double c = 0.0;
            for (int i = 0; i < n; ++i) c += e_vecs[(size_t)(acc - 1) * n + i] * t2[i];
            if (std::fabs(c) >= 0.9) continue;
        }
        std::copy(t2.begin(), t2.end(), e_vecs + (size_t)acc * n);
        e_vals[acc] = 1.0 / th[k];
        ++acc;
    }
    return acc;
}

}  // namespace

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
extern "C" {

orc_model* orc_create(int32_t elem_type, int32_t n_nodes, const double* coords, int32_t n_elems,
                      const int32_t* conn, const double* E, const double* nu, const double* rho,
                      const double* thickness) {
    if (elem_type != 8 && elem_type != 81 && elem_type != 4 && elem_type != 10 && elem_type != 41 && elem_type != 2)
        return nullptr;
    auto* m = new orc_model();
    m->ti = type_info(elem_type);
    m->n_el = n_elems;
    m->dpn = m->ti.dpn;
    if (elem_type == 41) {
        if (!thickness) { delete m; return nullptr; }
        for (int e = 0; e < n_elems; ++e)  // flat elements in a plane z = const
            for (int a = 1; a < 4; ++a)
                if (coords[3 * (size_t)conn[4 * (size_t)e + a] + 2] != coords[3 * (size_t)conn[4 * (size_t)e] + 2]) {
                    delete m;
                    return nullptr;
                }
        m->shell = true;
        m->n_phys = n_nodes;
        m->phys_xyz.assign(coords, coords + (size_t)3 * n_nodes);
        m->conn4.assign(conn, conn + (size_t)n_elems * 4);
        m->n_nodes = 2 * n_nodes;
        m->xyz.resize((size_t)6 * n_nodes);
        for (int i = 0; i < n_nodes; ++i)
            for (int j = 0; j < 3; ++j) m->xyz[6 * (size_t)i + j] = m->xyz[6 * (size_t)i + 3 + j] = coords[3 * (size_t)i + j];
        m->conn.resize((size_t)n_elems * 8);
        for (size_t k = 0; k < (size_t)n_elems * 4; ++k) {
            m->conn[2 * k] = 2 * conn[k];
            m->conn[2 * k + 1] = 2 * conn[k] + 1;
        }
    } else if (elem_type == 2) {
        m->beam = true;
        m->n_phys = n_nodes;
        m->phys_xyz.assign(coords, coords + (size_t)3 * n_nodes);
        m->conn2.assign(conn, conn + (size_t)n_elems * 2);
        m->n_nodes = 2 * n_nodes;
        m->xyz.resize((size_t)6 * n_nodes);
        for (int i = 0; i < n_nodes; ++i)
            for (int j = 0; j < 3; ++j) m->xyz[6 * (size_t)i + j] = m->xyz[6 * (size_t)i + 3 + j] = coords[3 * (size_t)i + j];
        m->conn.resize((size_t)n_elems * 4);
        for (size_t k = 0; k < (size_t)n_elems * 2; ++k) {
            m->conn[2 * k] = 2 * conn[k];
            m->conn[2 * k + 1] = 2 * conn[k] + 1;
        }
    } else {
        m->n_nodes = n_nodes;
        m->xyz.assign(coords, coords + (size_t)3 * n_nodes);
        m->conn.assign(conn, conn + (size_t)n_elems * m->ti.nn);
    }
    m->n_dof = m->n_nodes * m->dpn;
    m->E.assign(E, E + n_elems);
    m->nu.assign(nu, nu + n_elems);
    if (rho) m->rho.assign(rho, rho + n_elems);
    else m->rho.assign(n_elems, 0.0);
    if (thickness) m->thk.assign(thickness, thickness + n_elems);
    m->c_ptr.assign(1, 0);
    return m;
}

void orc_destroy(orc_model* m) { delete m; }
int32_t orc_dof_per_node(const orc_model* m) { return m->dpn; }
int32_t orc_n_dof(const orc_model* m) { return m->n_dof; }

int orc_set_constraints(orc_model* m, int32_t n_rows, const int32_t* row_ptr, const int32_t* dof,
                        const double* coef, const double* rhs) {
    m->c_ptr.assign(row_ptr, row_ptr + n_rows + 1);
    const int nt = row_ptr[n_rows];
    for (int k = 0; k < nt; ++k)
        if (dof[k] < 0 || dof[k] >= m->n_dof) return -1;
    m->c_dof.assign(dof, dof + nt);
    m->c_coef.assign(coef, coef + nt);
    m->c_rhs.assign(rhs, rhs + n_rows);
    return 0;
}

// Assembly: model_analysis.rs:179-201 (build_elastic_soln_load with the
// matrix) -> element_equations.rs:852-1062 (get_ru_dfd0; Newmark mass term
// c1 = -1/(dt^2 (beta - gamma)) at :977-988) -> add_entry per element DOF pair
// (:1040-1059).  Penalty scale: model_analysis.rs:255-259 over that matrix.
int orc_assemble(orc_model* m, int32_t dynamic, double dt, double beta, double gamma) {
    if (m->beam) {  // beam2 needs its sections, with valid frames
        if (m->beam_sec.size() != (size_t)m->n_el * 10) return -3;
        for (int e = 0; e < m->n_el; ++e) {
            double xyz[6], R[9], L;
            for (int a = 0; a < 2; ++a)
                for (int j = 0; j < 3; ++j) xyz[3 * a + j] = m->phys_xyz[3 * (size_t)m->conn2[(size_t)e * 2 + a] + j];
            if (!beam_frame(xyz, &m->beam_sec[(size_t)e * 10 + 7], R, &L)) return -3;
        }
    }
    build_pattern(m, m->K);
    m->dynamic = dynamic != 0;
    m->cM = 0.0;
    m->cD = 0.0;
    const bool damp = dynamic == 1 && m->damped();
    if ((damp && (m->ray_ck != 0.0 || !m->dmat.empty()) && (m->structural() || m->ti.type == 81)) ||
        (!m->cmat.empty() && m->structural()))
        return -2;  // stiffness / material damping and 6x6 stiffness: elements without internal DOF
    m->D = Csr();
    if (m->dynamic) {
        m->M = m->K;
        // dynamic == 2: modal analysis, K and M kept apart (model_analysis.rs:783-786
        // assembles the static matrix; the mass enters only as the diagonal D)
        if (dynamic != 2) m->cM = -1.0 / (dt * dt * (beta - gamma));
        // damping enters with c2 = dt gamma c1 (element_equations.rs:995-1005)
        if (damp) {
            m->D = m->K;
            m->cD = dt * gamma * m->cM;
        }
    }
    const int nn = m->ti.nn, tot = 3 * nn;
    std::vector<double> ke(tot * tot), me(tot * tot), mc(tot * tot), de(tot * tot);
    std::vector<int32_t> dofs(tot);
    for (int e = 0; e < m->n_el; ++e) {
        elem_km(m, e, ke.data(), m->dynamic ? me.data() : nullptr);
        if (damp) {
            mc = me;  // Rayleigh mass damping uses the consistent mass (get_rud -> get_rum)
            elem_damp(m, e, ke.data(), mc.data(), de.data());
        }
        if (m->dynamic && m->lump) lump_rows(tot, me.data());
        if (m->dynamic)
            for (int i = 0; i < tot * tot; ++i) ke[i] += m->cM * me[i] + (damp ? m->cD * de[i] : 0.0);
        for (int a = 0; a < nn; ++a)
            for (int c = 0; c < 3; ++c) dofs[3 * a + c] = m->conn[(size_t)e * nn + a] * 3 + c;
        for (int i = 0; i < tot; ++i)
            for (int j = 0; j < tot; ++j) {
                const int64_t k = m->K.find(dofs[i], dofs[j]);
                m->K.val[k] += ke[i * tot + j];
                if (m->dynamic) m->M.val[k] += me[i * tot + j];
                if (damp) m->D.val[k] += de[i * tot + j];
            }
    }
    m->sf = 100000.0 * m->K.max_abs();
    m->assembled = true;
    return 0;
}

int64_t orc_nnz(const orc_model* m) { return (int64_t)m->K.col.size(); }
double orc_penalty_scale(const orc_model* m) { return m->sf; }

int orc_set_cmat(orc_model* m, const double* C) {
    if (!C) {
        m->cmat.clear();
        return 0;
    }
    if (m->structural()) return -1;
    m->cmat.assign(C, C + (size_t)m->n_el * 36);
    m->assembled = false;
    return 0;
}

int orc_shell_section(int32_t n_layers, const double* props, double z_offset, double* abd, double* msec) {
    if (n_layers < 1 || !props || !abd || !msec) return -1;
    shell_section(n_layers, props, z_offset, abd, msec);
    return 0;
}

int orc_set_shell_sections(orc_model* m, const double* abd, const double* msec) {
    if (!m->shell) return -1;
    if (!abd) {
        m->shell_abd81.clear();
        m->shell_msec36.clear();
    } else {
        if (!msec) return -1;
        m->shell_abd81.assign(abd, abd + (size_t)m->n_el * 81);
        m->shell_msec36.assign(msec, msec + (size_t)m->n_el * 36);
    }
    m->assembled = false;
    return 0;
}

int orc_set_beam_sections(orc_model* m, const double* sec) {
    if (!m->beam || !sec) return -1;
    m->beam_sec.assign(sec, sec + (size_t)m->n_el * 10);
    m->assembled = false;
    return 0;
}

int orc_beam_element(const double* xyz, double E, double nu, double rho, const double* sec, double* ke,
                     double* me) {
    if (!xyz || !sec || !ke) return -1;
    return beam_km(xyz, E, nu, rho, sec, ke, me) ? 0 : -2;
}

int orc_beam_element_given(const double* xyz, double E, double nu, double rho, const double* sec,
                           const double* given, double* ke, double* me) {
    if (!xyz || !sec || !ke) return -1;
    return beam_km(xyz, E, nu, rho, sec, ke, me, given) ? 0 : -2;
}

int orc_set_beam_section_matrices(orc_model* m, const double* stiffness, const double* mass) {
    if (!m->beam) return -1;
    if (!stiffness && !mass) {
        m->beam_cm.clear();
    } else {
        m->beam_cm.assign((size_t)m->n_el * 72, 0.0);
        for (int e = 0; e < m->n_el; ++e)
            for (int k = 0; k < 36; ++k) {
                if (stiffness) m->beam_cm[(size_t)e * 72 + k] = stiffness[(size_t)e * 36 + k];
                if (mass) m->beam_cm[(size_t)e * 72 + 36 + k] = mass[(size_t)e * 36 + k];
            }
    }
    m->assembled = false;
    return 0;
}

// dC/dD of the beam section stiffness (get_beam_stiff_dfd0,
// element_properties.rs:921-1010) for a unit change of one material DV:
// category 0 modulus (component 1: E1 in EA, E I1, -E I2, E I3, -E I5, E I4;
// components 2, 3 do not enter), 1 shearModulus (component 1: G1 in GA of the
// first shear, -G I1, G J; 2: G2 in GA of the second shear; 3: G3 in G I2),
// 2 poissonRatio (does not enter).
// Categories 3 area (EA, GA, GA), 4 areaMoment component 1-5 (the entries of
// I1..I5), 5 polarMoment (GJ), with the element's E and G = E / (2 (1 + nu)).
int orc_beam_section_dC(int32_t category, int32_t component, double E, double nu, const double* sec, double* dC) {
    if (category < 0 || category > 5 || !sec || !dC) return -1;
    if (category <= 2 && (component < 1 || component > 3)) return -1;
    if (category == 4 && (component < 1 || component > 5)) return -1;
    for (int i = 0; i < 36; ++i) dC[i] = 0.0;
    auto set = [&](int i, int j, double v) { dC[6 * i + j] = dC[6 * j + i] = v; };
    const double G = E / (2.0 * (1.0 + nu));
    if (category == 3) {
        set(0, 0, E);
        set(1, 1, G);
        set(2, 2, G);
        return 0;
    }
    if (category == 4) {
        const int ij[5][2][2] = {{{0, 4}, {1, 3}}, {{0, 5}, {2, 3}}, {{4, 4}, {-1, -1}}, {{5, 5}, {-1, -1}},
                                 {{4, 5}, {-1, -1}}};
        const double v[5][2] = {{E, -G}, {-E, G}, {E, 0.0}, {E, 0.0}, {-E, 0.0}};
        for (int t = 0; t < 2; ++t)
            if (ij[component - 1][t][0] >= 0) set(ij[component - 1][t][0], ij[component - 1][t][1], v[component - 1][t]);
        return 0;
    }
    if (category == 5) {
        set(3, 3, G);
        return 0;
    }
    if (category == 0 && component == 1) {
        set(0, 0, sec[0]);
        set(0, 4, sec[1]);
        set(0, 5, -sec[2]);
        set(4, 4, sec[3]);
        set(4, 5, -sec[5]);
        set(5, 5, sec[4]);
    } else if (category == 1 && component == 1) {
        set(1, 1, sec[0]);
        set(1, 3, -sec[1]);
        set(3, 3, sec[6]);
    } else if (category == 1 && component == 2) {
        set(2, 2, sec[0]);
    } else if (category == 1 && component == 3) {
        set(2, 3, sec[2]);
    }
    return 0;
}

int orc_set_damping(orc_model* m, double ray_cm, double ray_ck, const double* D) {
    m->ray_cm = ray_cm;
    m->ray_ck = ray_ck;
    if (D) m->dmat.assign(D, D + (size_t)m->n_el * 36);
    else m->dmat.clear();
    m->assembled = false;
    return 0;
}

int orc_set_lumped_mass(orc_model* m, int32_t on) {
    m->lump = on != 0;
    m->assembled = false;
    return 0;
}

int orc_orthotropic_cmat(const double* e3, const double* nu3, const double* g3, double* C) {
    solid_cmat(e3, nu3, g3, C);
    return 0;
}

int orc_get_csr(const orc_model* m, int32_t which, int64_t* row_ptr, int32_t* col, double* val) {
    if (!m->assembled) return -1;
    const Csr& A = (which == 1) ? m->M : (which == 3) ? m->D : m->K;
    if (which == 1 && !m->dynamic) return -2;
    if (which == 3 && m->D.val.empty()) return -2;
    if (row_ptr) std::copy(A.ptr.begin(), A.ptr.end(), row_ptr);
    if (col) std::copy(A.col.begin(), A.col.end(), col);
    if (val) {
        std::copy(A.val.begin(), A.val.end(), val);
        if (which == 2) {
            const int nr = (int)m->c_rhs.size();
            for (int r = 0; r < nr; ++r)
                for (int k = m->c_ptr[r]; k < m->c_ptr[r + 1]; ++k)
                    for (int k2 = m->c_ptr[r]; k2 < m->c_ptr[r + 1]; ++k2) {
                        const int64_t idx = A.find(m->c_dof[k], m->c_dof[k2]);
                        if (idx < 0) return -3;
                        val[idx] += m->sf * m->c_coef[k] * m->c_coef[k2];
                    }
        }
    }
    return 0;
}

int orc_element_stiffness(int32_t elem_type, const double* xyz, double E, double nu,
                          double thickness, double* ke) {
    if (elem_type == 41) {
        for (int a = 1; a < 4; ++a)
            if (xyz[3 * a + 2] != xyz[2]) return -2;
        shell_km(xyz, E, nu, 0.0, thickness, ke, nullptr);
        return 0;
    }
    if (elem_type != 8 && elem_type != 81 && elem_type != 4 && elem_type != 10) return -1;
    double C[36];
    iso_cmat(E, nu, C);
    solid_ke(elem_type, xyz, C, ke);
    return 0;
}

int orc_element_mass(int32_t elem_type, const double* xyz, double rho, double thickness,
                     double* me) {
    if (elem_type == 41) {
        for (int a = 1; a < 4; ++a)
            if (xyz[3 * a + 2] != xyz[2]) return -2;
        std::vector<double> ke(24 * 24);
        shell_km(xyz, 1.0, 0.3, rho, thickness, ke.data(), me);
        return 0;
    }
    if (elem_type != 8 && elem_type != 81 && elem_type != 4 && elem_type != 10) return -1;
    solid_me(elem_type, xyz, rho, me);
    return 0;
}

// Surface traction: element_equations.rs:1970-2043 (get_app_load_dfd0,
// surfaceTraction branch).  A face is loaded when it lies on the surface
// (not shared with another element; model_prep.rs:510-554) and its unit
// normal (face_meth.rs:174-221) is within norm_tol degrees of norm_dir.  The
// face load is the unit-density consistent-mass image of the traction applied
// at the face nodes, restricted to the face nodes and scaled so its magnitude
// is area*|t|.  Only the last loaded face of an element survives (the
// reference recomputes the element load per face before accumulating).
int orc_surface_load(const orc_model* m, int32_t n_set, const int32_t* elem_set, const double* norm_dir,
                     double norm_tol_deg, const double* traction_in, double pressure, double* f);

int orc_surface_traction(const orc_model* m, int32_t n_set, const int32_t* elem_set,
                         const double* norm_dir, double norm_tol_deg, const double* traction,
                         double* f) {
    return orc_surface_load(m, n_set, elem_set, norm_dir, norm_tol_deg, traction, 0.0, f);
}

// surfacePressure: the traction -p n of each loaded face (element_equations.rs:1984-1990)
int orc_surface_pressure(const orc_model* m, int32_t n_set, const int32_t* elem_set, const double* norm_dir,
                         double norm_tol_deg, double pressure, double* f) {
    return orc_surface_load(m, n_set, elem_set, norm_dir, norm_tol_deg, nullptr, pressure, f);
}

int orc_surface_load(const orc_model* m, int32_t n_set, const int32_t* elem_set, const double* norm_dir,
                     double norm_tol_deg, const double* traction_in, double pressure, double* f) {
    if (m->shell || m->ti.nfaces == 0) return -1;  // solid element faces only (none restated for tet10)
    const TypeInfo& t = m->ti;
    const int nn = t.nn, tot = 3 * nn;
    // face multiplicity over the whole mesh
    std::vector<std::array<int32_t, 4>> keys;
    keys.reserve((size_t)m->n_el * t.nfaces);
    auto face_key = [&](int e, int fi) {
        std::array<int32_t, 4> k{-1, -1, -1, -1};
        for (int q = 0; q < t.face_nn; ++q) k[q] = m->conn[(size_t)e * nn + t.faces[fi][q]];
        for (int i = 1; i < t.face_nn; ++i)  // insertion sort of the face's node ids
            for (int j = i; j > 0 && k[j - 1] > k[j]; --j) std::swap(k[j - 1], k[j]);
        return k;
    };
    for (int e = 0; e < m->n_el; ++e)
        for (int fi = 0; fi < t.nfaces; ++fi) keys.push_back(face_key(e, fi));
    std::vector<std::array<int32_t, 4>> sorted = keys;
    std::sort(sorted.begin(), sorted.end());
    auto count = [&](const std::array<int32_t, 4>& k) {
        auto r = std::equal_range(sorted.begin(), sorted.end(), k);
        return (int)(r.second - r.first);
    };
    const double cos_tol = std::cos(kPi / 180.0 * norm_tol_deg);
    std::vector<double> me(tot * tot), el_ld(tot);
    double xyz[24];
    for (int s = 0; s < n_set; ++s) {
        const int e = elem_set[s];
        elem_xyz(m, e, xyz);
        bool any = false;
        for (int fi = 0; fi < t.nfaces; ++fi) {
            if (count(keys[(size_t)e * t.nfaces + fi]) != 1) continue;
            const int* ln = t.faces[fi];
            double v1[3], v2[3], nrm[3];
            for (int i = 0; i < 3; ++i) {
                if (t.face_nn == 4) {
                    v1[i] = xyz[3 * ln[2] + i] - xyz[3 * ln[0] + i];
                    v2[i] = xyz[3 * ln[3] + i] - xyz[3 * ln[1] + i];
                } else {
                    v1[i] = xyz[3 * ln[1] + i] - xyz[3 * ln[0] + i];
                    v2[i] = xyz[3 * ln[2] + i] - xyz[3 * ln[0] + i];
                }
            }
            nrm[0] = v1[1] * v2[2] - v1[2] * v2[1];
            nrm[1] = v1[2] * v2[0] - v1[0] * v2[2];
            nrm[2] = v1[0] * v2[1] - v1[1] * v2[0];
            double area = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
            for (double& x : nrm) x /= area;
            area *= 0.5;
            const double dp = norm_dir[0] * nrm[0] + norm_dir[1] * nrm[1] + norm_dir[2] * nrm[2];
            if (!(dp > cos_tol)) continue;
            double traction[3];
            for (int i = 0; i < 3; ++i) traction[i] = traction_in ? traction_in[i] : -pressure * nrm[i];
            // acceleration = traction at face nodes, zero elsewhere
            double acc[24] = {0};
            for (int q = 0; q < t.face_nn; ++q)
                for (int i = 0; i < 3; ++i) acc[3 * ln[q] + i] = traction[i];
            solid_me(t.type, xyz, 1.0, me.data());
            double tot_f[3] = {0, 0, 0};
            for (int i = 0; i < tot; ++i) {
                double a = 0.0;
                for (int j = 0; j < tot; ++j) a += me[i * tot + j] * acc[j];
                bool in_face = false;
                for (int q = 0; q < t.face_nn; ++q) in_face |= (ln[q] == i / 3);
                el_ld[i] = in_face ? a : 0.0;
                tot_f[i % 3] += el_ld[i];
            }
            double vmag = 0.0, imag = 0.0;
            for (int i = 0; i < 3; ++i) {
                vmag += tot_f[i] * tot_f[i];
                imag += traction[i] * traction[i];
            }
            const double scale = area * std::sqrt(imag) / std::sqrt(vmag);
            for (int i = 0; i < tot; ++i) el_ld[i] *= scale;
            any = true;
        }
        if (any)
            for (int i = 0; i < tot; ++i) f[m->conn[(size_t)e * nn + i / 3] * 3 + i % 3] += el_ld[i];
    }
    return 0;
}

// Uniform-acceleration element loads, get_app_load_dfd0
// (element_equations.rs:1875-1968): M_e acc with acc on the translational DOF
// of every node.  kind 0 bodyForce: unit density, then scaled by
// |load| vol / |sum of the element's forces| (:1893-1911); kind 1
// gravitational: the element's density; kind 2 centrifugal: omega^2 times the
// element centroid's offset from the axis (axis normalised on input,
// load_meth.rs:41-51), the element's density.
int orc_body_load(const orc_model* m, int32_t n_set, const int32_t* elem_set, int32_t kind, const double* vec,
                  double omega, const double* center, const double* axis, double* f) {
    if (!m->shell_abd81.empty()) return -2;  // layered sections: not restated
    const int nn = m->ti.nn, tot = 3 * nn;
    std::vector<double> ke(tot * tot), me(tot * tot);
    double ax[3] = {0, 0, 0};
    if (kind == 2) {
        const double l = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
        for (int j = 0; j < 3; ++j) ax[j] = axis[j] / l;
    }
    for (int s = 0; s < n_set; ++s) {
        const int e = elem_set[s];
        double xyz[30];
        elem_xyz(m, e, xyz);
        // element mass at its density, or at unit density for body forces
        if (m->beam) {
            double x2[6];
            for (int a = 0; a < 2; ++a)
                for (int j = 0; j < 3; ++j) x2[3 * a + j] = m->phys_xyz[3 * (size_t)m->conn2[(size_t)e * 2 + a] + j];
            beam_km(x2, m->E[e], m->nu[e], kind == 0 ? 1.0 : m->rho[e], &m->beam_sec[(size_t)e * 10], ke.data(),
                    me.data(), m->beam_ov(e));
        } else if (m->shell) {
            double x4[12];
            for (int a = 0; a < 4; ++a)
                for (int j = 0; j < 3; ++j) x4[3 * a + j] = m->phys_xyz[3 * (size_t)m->conn4[(size_t)e * 4 + a] + j];
            shell_km(x4, m->E[e], m->nu[e], kind == 0 ? 1.0 : m->rho[e], m->thk[e], ke.data(), me.data());
        } else {
            solid_me(m->ti.type, xyz, kind == 0 ? 1.0 : m->rho[e], me.data());
        }
        // physical nodes: shells carry translations on pseudo-node 2a
        const int nphys = m->shell ? 4 : (m->beam ? 2 : nn);
        double acc_e[3];
        if (kind == 2) {
            double cen[3] = {0, 0, 0}, d[3], dp = 0.0;
            for (int a = 0; a < nphys; ++a)
                for (int j = 0; j < 3; ++j) cen[j] += xyz[3 * (m->structural() ? 2 * a : a) + j] / nphys;
            for (int j = 0; j < 3; ++j) {
                d[j] = cen[j] - center[j];
                dp += ax[j] * d[j];
            }
            for (int j = 0; j < 3; ++j) acc_e[j] = omega * omega * (d[j] - ax[j] * dp);
        } else {
            for (int j = 0; j < 3; ++j) acc_e[j] = vec[j];
        }
        std::vector<double> acc(tot, 0.0), ld(tot, 0.0);
        for (int a = 0; a < nphys; ++a)
            for (int j = 0; j < 3; ++j) acc[3 * (m->structural() ? 2 * a : a) + j] = acc_e[j];
        double tot_f[3] = {0, 0, 0};
        for (int i = 0; i < tot; ++i) {
            double v = 0.0;
            for (int j = 0; j < tot; ++j) v += me[i * tot + j] * acc[j];
            ld[i] = v;
            if (!m->structural() || (i / 3) % 2 == 0) tot_f[i % 3] += v;
        }
        if (kind == 0) {
            // element volume: the unit-density mass summed over one direction
            double vol = 0.0;
            for (int i = 0; i < tot; i += 3)
                if (!m->structural() || (i / 3) % 2 == 0)
                    for (int j = 0; j < tot; j += 3) vol += me[i * tot + j];
            double imag = 0.0, vmag = 0.0;
            for (int j = 0; j < 3; ++j) {
                imag += vec[j] * vec[j];
                vmag += tot_f[j] * tot_f[j];
            }
            const double sc = (vmag > 0.0) ? std::sqrt(imag) * vol / std::sqrt(vmag) : 0.0;
            for (double& v : ld) v *= sc;
        }
        for (int i = 0; i < tot; ++i) f[(size_t)m->conn[(size_t)e * nn + i / 3] * 3 + i % 3] += ld[i];
    }
    return 0;
}

int orc_apply_operator(const orc_model* m, const double* x, double* y) {
    if (!m->assembled) return -1;
    apply_A(m, x, y);
    return 0;
}

// Static solve: model_analysis.rs:450-534 (solve_step, elastic linear branch):
// load = f_app - R(u=0) + penalty load (:467-487), solve, u += du (:503-513).
int orc_static_solve(orc_model* m, const double* f, double* u, int32_t precond, int32_t stop_rule,
                     double tol, int32_t max_it, int32_t block_dim, orc_stats* st) {
    if (!m->assembled) return -1;
    const int n = m->n_dof;
    std::vector<double> load(f, f + n), zero(n, 0.0);
    constraint_load(m, zero.data(), load.data());
    if (st) std::memset(st, 0, sizeof(*st));
    auto t0 = std::chrono::steady_clock::now();
    Precond pc;
    pc.setup(m, precond, block_dim);
    int status = 0;
    if (precond == ORC_PC_DIRECT) {
        pc.apply(load.data(), u);
    } else {
        if (precond == ORC_PC_BLOCK_LDL && !skyline_pos_def(pc.S) && st) st->status = 3;
        status = pcg(m, pc, load.data(), u, stop_rule, tol, max_it > 0 ? max_it : n, st);
    }
    auto t1 = std::chrono::steady_clock::now();
    if (st) {
        st->seconds = std::chrono::duration<double>(t1 - t0).count();
        st->rel_residual = true_rel_residual(m, load.data(), u);
    }
    return status;
}

// Several load cases against one preconditioner set-up (one factorization
// for PC_DIRECT): the loop of solve_step over a model's load cases, each as
// orc_static_solve.  st receives the largest iteration count and residual.
int orc_static_solve_multi(orc_model* m, int32_t n_rhs, const double* f, double* u, int32_t precond,
                           int32_t stop_rule, double tol, int32_t max_it, int32_t block_dim, orc_stats* st) {
    if (!m->assembled) return -1;
    const int n = m->n_dof;
    if (st) std::memset(st, 0, sizeof(*st));
    auto t0 = std::chrono::steady_clock::now();
    Precond pc;
    pc.setup(m, precond, block_dim);
    int status = 0;
    double relmax = 0.0;
    for (int r = 0; r < n_rhs; ++r) {
        std::vector<double> load(f + (size_t)r * n, f + (size_t)(r + 1) * n), zero(n, 0.0);
        constraint_load(m, zero.data(), load.data());
        double* ur = u + (size_t)r * n;
        orc_stats sr;
        std::memset(&sr, 0, sizeof(sr));
        if (precond == ORC_PC_DIRECT) {
            pc.apply(load.data(), ur);
        } else {
            std::fill(ur, ur + n, 0.0);
            status = std::max(status, pcg(m, pc, load.data(), ur, stop_rule, tol, max_it > 0 ? max_it : n, &sr));
        }
        relmax = std::max(relmax, true_rel_residual(m, load.data(), ur));
        if (st) st->iterations = std::max(st->iterations, sr.iterations);
    }
    auto t1 = std::chrono::steady_clock::now();
    if (st) {
        st->seconds = std::chrono::duration<double>(t1 - t0).count();
        st->rel_residual = relmax;
        st->status = status;
    }
    return status;
}

// Static adjoint: model_analysis.rs:1065-1126 (solve_for_adjoint: same
// operator and solver for lambda = A^-1 dL/du) and :1632-1704 with
// d_relasticd_d :1379-1457; for a modulus DV on element e the only nonzero
// dR/dD is the element's internal force, so dL/dE_e = -lambda_e^T dK_e/dE_e u_e
// (isotropic at fixed nu: dK_e/dE_e = K_e / E_e).
int orc_adjoint_modulus_gradient(orc_model* m, const double* u, const double* dLdu,
                                 const double* lambda_in, double* lambda_out, double* gE,
                                 int32_t precond, int32_t stop_rule, double tol, int32_t max_it,
                                 orc_stats* st) {
    if (!m->assembled) return -1;
    if (!m->shell_abd81.empty()) return -2;  // layered sections are not proportional to E
    for (size_t e = 0; e < m->beam_cm.size() / 72; ++e)
        if (m->beam_cm[e * 72] > 0.0) return -2;  // nor are given beam section stiffnesses
    const int n = m->n_dof;
    std::vector<double> lam(n, 0.0);
    int status = 0;
    if (st) std::memset(st, 0, sizeof(*st));
    if (dLdu) {
        Precond pc;
        pc.setup(m, precond, 0);
        if (precond == ORC_PC_DIRECT) pc.apply(dLdu, lam.data());
        else status = pcg(m, pc, dLdu, lam.data(), stop_rule, tol, max_it > 0 ? max_it : n, st);
        if (st) st->rel_residual = true_rel_residual(m, dLdu, lam.data());
    } else if (lambda_in) {
        std::copy(lambda_in, lambda_in + n, lam.begin());
    } else {
        return -2;
    }
    if (lambda_out) std::copy(lam.begin(), lam.end(), lambda_out);
    const int nn = m->ti.nn, tot = 3 * nn;
    std::vector<double> ke(tot * tot);
    for (int e = 0; e < m->n_el; ++e) {
        elem_km(m, e, ke.data(), nullptr);
        double acc = 0.0;
        for (int i = 0; i < tot; ++i) {
            const int gi = m->conn[(size_t)e * nn + i / 3] * 3 + i % 3;
            double ki = 0.0;
            for (int j = 0; j < tot; ++j) ki += ke[i * tot + j] * u[m->conn[(size_t)e * nn + j / 3] * 3 + j % 3];
            acc += lam[gi] * ki;
        }
        gE[e] = -acc / m->E[e];
    }
    return status;
}

// Orthotropic "modulus" DV component k (element_properties.rs:700-711 adds the
// DV to E_k; dC/dE_k = -C (dS/dE_k) C by differentiating the compliance
// inverse of :724-760).
int orc_adjoint_modulus_component_gradient(orc_model* m, const double* u, const double* lambda,
                                           int32_t component, double* gD) {
    if (component < 1 || component > 3 || m->structural() || m->ti.type == 81) return -1;
    const int k = component - 1;
    const TypeInfo& t = m->ti;
    const int nn = t.nn, tot = 3 * nn;
    double xyz[30], C[36], dS[36], tmp[36], dC[36], n[10], dndx[30], B[6 * 30];
    for (int e = 0; e < m->n_el; ++e) {
        elem_xyz(m, e, xyz);
        const double E = m->E[e], nu = m->nu[e];
        iso_cmat(E, nu, C);
        std::fill(dS, dS + 36, 0.0);
        // compliance entries depending on E_k: S[k][k] = 1/E_k; S[k][j] = -nu/E_k
        dS[7 * k] = -1.0 / (E * E);
        const int pair[3][2] = {{1, 2}, {0, 2}, {0, 1}};
        (void)pair;
        if (k == 0) { dS[1] = dS[6] = nu / (E * E); dS[2] = dS[12] = nu / (E * E); }
        if (k == 1) { dS[8] = dS[13] = nu / (E * E); }
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                double a = 0.0;
                for (int l = 0; l < 6; ++l) a += dS[6 * i + l] * C[6 * l + j];
                tmp[6 * i + j] = a;
            }
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                double a = 0.0;
                for (int l = 0; l < 6; ++l) a += C[6 * i + l] * tmp[6 * l + j];
                dC[6 * i + j] = -a;
            }
        double acc = 0.0;
        for (int p = 0; p < t.nip; ++p) {
            const double det = ip_data(t.type, nn, xyz, t.ip + 3 * p, n, dndx);
            solid_bmat(nn, dndx, B);
            double eu[6] = {0}, el[6] = {0};
            for (int q = 0; q < 6; ++q)
                for (int c = 0; c < tot; ++c) {
                    const int gdof = m->conn[(size_t)e * nn + c / 3] * 3 + c % 3;
                    eu[q] += B[q * tot + c] * u[gdof];
                    el[q] += B[q * tot + c] * lambda[gdof];
                }
            for (int i = 0; i < 6; ++i)
                for (int j = 0; j < 6; ++j) acc += el[i] * dC[6 * i + j] * eu[j] * det * t.wt[p];
        }
        gD[e] = -acc;
    }
    return 0;
}

// Newmark transient: model_analysis.rs:591-624 (solve, dynamic loop) with
// solve_step :450-534 and node_meth.rs:127-138 (update_vel_acc),
// :158-165 (advance_disp).  a = c1 (u_prev - u + dt v_prev + c2 a_prev),
// c1 = 1/(dt^2 (beta - gamma)), c2 = dt^2 (0.5 + beta - gamma);
// v = v_prev + dt ((1 - gamma) a_prev + gamma a).
int orc_newmark_run(orc_model* m, int32_t n_steps, double dt, double beta, double gamma,
                    const double* f_shape, const double* amp, int32_t probe_dof,
                    double* probe_hist, int32_t precond, int32_t stop_rule, double tol,
                    int32_t max_it, double* u_final, int32_t* total_iters) {
    if (!m->assembled || !m->dynamic || m->cM == 0.0) return -1;
    const int n = m->n_dof;
    std::vector<double> u(n, 0.0), v(n, 0.0), a(n, 0.0), up(n, 0.0), vp(n, 0.0), ap(n, 0.0);
    std::vector<double> load(n), du(n), tmp(n), ku(n);
    const double c1 = 1.0 / (dt * dt * (beta - gamma));
    const double c2 = dt * dt * (0.5 + beta - gamma);
    auto update_vel_acc = [&]() {
        for (int i = 0; i < n; ++i) {
            a[i] = c1 * (up[i] - u[i] + dt * vp[i] + c2 * ap[i]);
            v[i] = vp[i] + dt * ((1.0 - gamma) * ap[i] + gamma * a[i]);
        }
    };
    update_vel_acc();  // prep_matrix_factorizations, model_prep.rs:584-590
    Precond pc;
    pc.setup(m, precond, 0);
    orc_stats st{};
    int status = 0;
    const bool damp = !m->D.val.empty() && m->cD != 0.0;
    for (int s = 0; s < n_steps; ++s) {
        // residual R = K u + M a + D v (K here is K + cM M + cD D, so
        // subtract cM M u and cD D u)
        std::fill(ku.begin(), ku.end(), 0.0);
        m->K.matvec(u.data(), ku.data());
        for (int i = 0; i < n; ++i) tmp[i] = a[i] - m->cM * u[i];
        m->M.matvec(tmp.data(), ku.data());
        if (damp) {
            for (int i = 0; i < n; ++i) tmp[i] = v[i] - m->cD * u[i];
            m->D.matvec(tmp.data(), ku.data());
        }
        for (int i = 0; i < n; ++i) load[i] = amp[s] * f_shape[i] - ku[i];
        constraint_load(m, u.data(), load.data());
        if (precond == ORC_PC_DIRECT) {
            pc.apply(load.data(), du.data());
        } else {
            const int rc = pcg(m, pc, load.data(), du.data(), stop_rule, tol, max_it > 0 ? max_it : n, &st);
            if (rc == 2) { status = 2; break; }
            if (rc == 1) status = 1;
        }
        for (int i = 0; i < n; ++i) u[i] += du[i];
        update_vel_acc();
        if (probe_hist) probe_hist[s] = u[probe_dof];
        up = u; vp = v; ap = a;
        update_vel_acc();
    }
    if (u_final) std::copy(u.begin(), u.end(), u_final);
    if (total_iters) *total_iters = st.iterations;
    return status;
}

int orc_reorder_nodes(const orc_model* m, int32_t block_dim, int32_t* order_out) {
    const auto o = reorder_nodes(m, block_dim > 0 ? block_dim : default_block_dim(m->n_nodes));
    std::copy(o.begin(), o.end(), order_out);
    return 0;
}


// Frequency job (model_analysis.rs:711-880, eigen_solve):
//   D = row sums of the consistent mass (get_rum with unit acceleration,
//   :748-766), entries below 1e-6 mean|D| raised to it (:768-779);
//   A = K - shift D with the penalty terms (:783-789), factored directly
//   (:790-795); eigen_sparse_direct; eigenvalue += shift (:803-805);
//   frequency sqrt(lambda) / (2 pi), -1 for a negative eigenvalue (:874-879).
// Needs orc_assemble(m, 2, ...).  Returns the number of pairs found, or < 0.
int orc_eigen_solve(orc_model* m, int32_t n_modes, double shift, double* eig, double* freq, double* modes,
                    double* diag_mass) {
    if (!m->assembled || !m->dynamic || m->cM != 0.0) return -1;
    const int n = m->n_dof;
    std::vector<double> D(n, 0.0), ones(n, 1.0);
    m->M.matvec(ones.data(), D.data());
    double avg = 0.0;
    for (int i = 0; i < n; ++i) avg += std::fabs(D[i]);
    avg /= (double)n;
    const double dmin = 1e-6 * avg;
    for (int i = 0; i < n; ++i)
        if (D[i] < dmin) D[i] = dmin;
    if (diag_mass) std::copy(D.begin(), D.end(), diag_mass);
    std::vector<double> dsave(n);
    for (int i = 0; i < n; ++i) {
        const int64_t k = m->K.find(i, i);
        dsave[i] = m->K.val[k];
        m->K.val[k] += -shift * D[i];
    }
    Precond pc;
    pc.setup(m, ORC_PC_DIRECT, 0);
    for (int i = 0; i < n; ++i) m->K.val[m->K.find(i, i)] = dsave[i];
    std::vector<double> vecs((size_t)n_modes * n, 0.0);
    auto solve = [&](const double* b, double* x) { pc.apply(b, x); };
    const int found = lanczos_direct(solve, D, n_modes, eig, vecs.data());
    if (found < 0) return found;
    for (int k = 0; k < found; ++k) {
        eig[k] += shift;
        if (freq) freq[k] = eig[k] >= 0.0 ? 0.159154943091895335 * std::sqrt(eig[k]) : -1.0;
    }
    if (modes) std::copy(vecs.begin(), vecs.begin() + (size_t)found * n, modes);
    return found;
}


// Transient adjoint, elastic Newmark (model_analysis.rs:1544-1631 dynamic
// branch; augmentd_ld_u :936-1063; solve_for_adjoint :1065-1126) for
//   L = sum_{n=1..N} sum_k w_k u_n[dof_k]
// (a displacement powerNorm of exponent 1 evaluated at every saved step) and
// per-element isotropic modulus DVs.  The forward run is orc_newmark_run's
// with a direct solve and every step's (u, v, a) kept, as the solnTStep
// history; the sweep runs n = N..1:
//   step n < N adds the coupling to step n+1's adjoints (augmentd_ld_u):
//     dL/du -= (d_ad_up M) u_adj, dL/dv -= (d_ad_vp M) u_adj,
//     dL/da -= (d_ad_ap M) u_adj (no damping on this path), then
//     dL/du += c1 a_adj, dL/da += c2 a_adj + c3 v_adj, dL/dv += c4 a_adj + v_adj
//     with d_ad_up = c1 = 1/(dt^2 (beta - gamma)), d_ad_vp = dt d_ad_up,
//     d_ad_ap = c2 = dt^2 (0.5 + beta - gamma) d_ad_up, c3 = dt (1 - gamma),
//     c4 = 1/(dt (beta - gamma));
//   dL/du += w (the step's objective term); v_adj = dL/dv;
//   a_adj = dL/da + dt gamma v_adj; dL/du -= a_adj / (dt^2 (beta - gamma));
//   A u_adj = dL/du with the step operator A = K + c_M M + penalty;
//   dL/dE_e -= u_adj_e^T (K_e / E_e) u_n,e (only K depends on E).
// The reference holds `time` at the end time through the sweep (:1563-1566);
// with the objective and loads active at all times that changes nothing here.
// Needs orc_assemble(m, 1, dt, beta, gamma).  gE[n_el], *L_out.
int orc_newmark_adjoint(orc_model* m, int32_t n_steps, double dt, double beta, double gamma,
                        const double* f_shape, const double* amp, int32_t n_obj, const int32_t* obj_dof,
                        const double* obj_w, double* L_out, double* gE) {
    if (!m->assembled || !m->dynamic || m->cM == 0.0 || n_steps < 1) return -1;
    if (m->cD != 0.0 || m->lump || !m->cmat.empty()) return -2;  // undamped consistent-mass isotropic models
    if (!m->shell_abd81.empty()) return -2;                        // K proportional to E only
    for (size_t e = 0; e < m->beam_cm.size() / 72; ++e)
        if (m->beam_cm[e * 72] > 0.0) return -2;
    const int n = m->n_dof;
    std::vector<double> u(n, 0.0), v(n, 0.0), a(n, 0.0), up(n, 0.0), vp(n, 0.0), ap(n, 0.0);
    std::vector<double> load(n), du(n), tmp(n), ku(n);
    const double c1n = 1.0 / (dt * dt * (beta - gamma));
    const double c2n = dt * dt * (0.5 + beta - gamma);
    auto update_vel_acc = [&]() {
        for (int i = 0; i < n; ++i) {
            a[i] = c1n * (up[i] - u[i] + dt * vp[i] + c2n * ap[i]);
            v[i] = vp[i] + dt * ((1.0 - gamma) * ap[i] + gamma * a[i]);
        }
    };
    update_vel_acc();
    Precond pc;
    pc.setup(m, ORC_PC_DIRECT, 0);
    std::vector<std::vector<double>> hist_u(n_steps + 1, std::vector<double>(n, 0.0));
    for (int s = 0; s < n_steps; ++s) {
        std::fill(ku.begin(), ku.end(), 0.0);
        m->K.matvec(u.data(), ku.data());
        for (int i = 0; i < n; ++i) tmp[i] = a[i] - m->cM * u[i];
        m->M.matvec(tmp.data(), ku.data());
        for (int i = 0; i < n; ++i) load[i] = amp[s] * f_shape[i] - ku[i];
        constraint_load(m, u.data(), load.data());
        pc.apply(load.data(), du.data());
        for (int i = 0; i < n; ++i) u[i] += du[i];
        update_vel_acc();
        hist_u[s + 1] = u;
        up = u; vp = v; ap = a;
        update_vel_acc();
    }
    double L = 0.0;
    for (int s = 1; s <= n_steps; ++s)
        for (int k = 0; k < n_obj; ++k) L += obj_w[k] * hist_u[s][obj_dof[k]];
    if (L_out) *L_out = L;
    // backward sweep
    const double d_ad_up = 1.0 / (dt * dt * (beta - gamma));
    const double d_ad_vp = d_ad_up * dt;
    const double d_ad_ap = d_ad_up * dt * dt * (0.5 + beta - gamma);
    const double c1 = d_ad_up, c2 = d_ad_ap, c3 = dt * (1.0 - gamma), c4 = 1.0 / (dt * (beta - gamma));
    std::vector<double> u_adj(n, 0.0), v_adj(n, 0.0), a_adj(n, 0.0), dldu(n), dldv(n), dlda(n), mu(n);
    std::fill(gE, gE + m->n_el, 0.0);
    const int nn = m->ti.nn, tot = 3 * nn;
    std::vector<double> ke(tot * tot);
    for (int s = n_steps; s >= 1; --s) {
        std::fill(dldu.begin(), dldu.end(), 0.0);
        std::fill(dldv.begin(), dldv.end(), 0.0);
        std::fill(dlda.begin(), dlda.end(), 0.0);
        if (s < n_steps) {
            std::fill(mu.begin(), mu.end(), 0.0);
            m->M.matvec(u_adj.data(), mu.data());
            for (int i = 0; i < n; ++i) {
                dldu[i] -= d_ad_up * mu[i];
                dlda[i] -= d_ad_ap * mu[i];
                dldv[i] -= d_ad_vp * mu[i];
                dldu[i] += c1 * a_adj[i];
                dlda[i] += c2 * a_adj[i] + c3 * v_adj[i];
                dldv[i] += c4 * a_adj[i] + v_adj[i];
            }
        }
        for (int k = 0; k < n_obj; ++k) dldu[obj_dof[k]] += obj_w[k];
        for (int i = 0; i < n; ++i) {
            v_adj[i] = dldv[i];
            a_adj[i] = dlda[i] + dt * gamma * v_adj[i];
            dldu[i] -= d_ad_up * a_adj[i];
        }
        pc.apply(dldu.data(), u_adj.data());
        const std::vector<double>& us = hist_u[s];
        for (int e = 0; e < m->n_el; ++e) {
            elem_km(m, e, ke.data(), nullptr);
            double acc = 0.0;
            for (int i = 0; i < tot; ++i) {
                const int gi = m->conn[(size_t)e * nn + i / 3] * 3 + i % 3;
                double ki = 0.0;
                for (int j = 0; j < tot; ++j) ki += ke[i * tot + j] * us[m->conn[(size_t)e * nn + j / 3] * 3 + j % 3];
                acc += u_adj[gi] * ki;
            }
            gE[e] -= acc / m->E[e];
        }
    }
    return 0;
}


// Strain-pair tensors of an adjoint pair (u, lambda): per element
// P_e = sum_gp w detJ eps(lambda_e) eps(u_e)^T (Voigt 11,22,33,12,13,23,
// engineering shear), so that lambda_e^T dR_e/dD = sum_ij (dC/dD)_ij P_e[i][j]
// for any material derivative of a solid element (d_relasticd_d,
// model_analysis.rs:1379-1457, with C constant over the element).  brickIM:
// the strains include the condensed modes, recovered as
// x_i = -K_ii^-1 K_ie x_e for both fields (update_internal,
// element_equations.rs:147-194), since d(K_ee - K_ei K_ii^-1 K_ie)/dD
// contracted with (lambda_e, u_e) equals the full dK/dD contracted with the
// recovered (lambda, u).  Solid types (8, 81, 4, 10); P[n_el][36].
int orc_adjoint_strain_pairs(const orc_model* m, const double* u, const double* lam, double* P) {
    if (!m->assembled || m->shell) return -1;
    if (m->beam) {  // section strains of beam2 (beam_pairs)
        for (int e = 0; e < m->n_el; ++e) {
            double xyz[6], ue[12], le[12];
            for (int a = 0; a < 2; ++a) {
                const int nd = m->conn2[(size_t)e * 2 + a];
                for (int j = 0; j < 3; ++j) xyz[3 * a + j] = m->phys_xyz[3 * (size_t)nd + j];
                for (int c = 0; c < 6; ++c) {
                    ue[6 * a + c] = u[6 * (size_t)nd + c];
                    le[6 * a + c] = lam[6 * (size_t)nd + c];
                }
            }
            beam_pairs(xyz, m->E[e], m->nu[e], &m->beam_sec[(size_t)e * 10], ue, le, P + (size_t)e * 36,
                       m->beam_ov(e));
        }
        return 0;
    }
    const TypeInfo& t = m->ti;
    const int nn = t.nn;
    for (int e = 0; e < m->n_el; ++e) {
        double xyz[30];
        elem_xyz(m, e, xyz);
        double acc[36] = {0};
        if (t.type == 81) {
            constexpr int tot = 33, nd = 24;
            double C[36];
            iso_cmat(m->E[e], m->nu[e], C);
            std::vector<double> K(tot * tot), B(6 * tot);
            brickim_kfull(xyz, C, K.data());
            double Kii[81];
            for (int i = 0; i < 9; ++i)
                for (int j = 0; j < 9; ++j) Kii[9 * i + j] = K[(nd + i) * tot + nd + j];
            givens_factor(Kii, 9);
            double uf[tot], lf[tot];
            for (int c = 0; c < nd; ++c) {
                const int g = m->conn[(size_t)e * nn + c / 3] * 3 + c % 3;
                uf[c] = u[g];
                lf[c] = lam[g];
            }
            for (double* f : {uf, lf}) {
                double rhs[9], x[9];
                for (int i = 0; i < 9; ++i) {
                    double a = 0.0;
                    for (int c = 0; c < nd; ++c) a += K[(nd + i) * tot + c] * f[c];
                    rhs[i] = a;
                }
                givens_solve(x, Kii, rhs, 9);
                for (int i = 0; i < 9; ++i) f[nd + i] = -x[i];
            }
            double Ji0[9];
            brickim_centroid_jinv(xyz, Ji0);
            for (int p = 0; p < t.nip; ++p) {
                const double djw = brickim_bmat(xyz, Ji0, p, B.data());
                double eu[6] = {0}, el[6] = {0};
                for (int q = 0; q < 6; ++q)
                    for (int c = 0; c < tot; ++c) {
                        eu[q] += B[q * tot + c] * uf[c];
                        el[q] += B[q * tot + c] * lf[c];
                    }
                for (int i = 0; i < 6; ++i)
                    for (int j = 0; j < 6; ++j) acc[6 * i + j] += el[i] * eu[j] * djw;
            }
        } else {
            const int tot = 3 * nn;
            double n[10], dndx[30], B[6 * 30];
            for (int p = 0; p < t.nip; ++p) {
                const double djw = ip_data(t.type, nn, xyz, t.ip + 3 * p, n, dndx) * t.wt[p];
                solid_bmat(nn, dndx, B);
                double eu[6] = {0}, el[6] = {0};
                for (int q = 0; q < 6; ++q)
                    for (int c = 0; c < tot; ++c) {
                        const int g = m->conn[(size_t)e * nn + c / 3] * 3 + c % 3;
                        eu[q] += B[q * tot + c] * u[g];
                        el[q] += B[q * tot + c] * lam[g];
                    }
                for (int i = 0; i < 6; ++i)
                    for (int j = 0; j < 6; ++j) acc[6 * i + j] += el[i] * eu[j] * djw;
            }
        }
        std::copy(acc, acc + 36, P + (size_t)e * 36);
    }
    return 0;
}

// Element-category objective terms (categories stress / strain /
// strainEnergy) evaluated at the element centroid s_cent, with the operators
// powerNorm, ks, volumeIntegral and volumeAverage:
//   values      ObjectiveTerm::get_obj_val, objective_meth.rs:665-720, with
//               get_stress_strain_dfd0 element_soln_fields.rs:1463-1576 and
//               get_volume_dfd0 :1118-1155 (sum_ip w detJ);
//   operators   get_power_norm :329-337, get_ks :390-398,
//               get_vol_integral :442-449, get_vol_average :504-516;
//   dL/du       getd_ld_u :1051-1160 (dq/du = b^T B + a^T C B with
//               a = dq/dsigma, b = dq/deps at the centroid);
//   dL/dD       getd_ld_d :1372-1500: dq/dD = a^T (dC/dD) eps at fixed u.
// Targets: one value for all elements, one per element, or none (0; 1 for
// ks), get_tgt_vec :94-215.  The incompatible modes of brickIM have zero
// derivatives at the centroid (element_soln_fields.rs:212-227), so its
// centroid strain is the hex8 one.  Outputs: L; dLdu[n_dof] (may be null);
// Q[n_el][36] with dL/dD|explicit = sum_e sum_ij (dC/dD)_ij Q_e[i][j] (may be
// null); dLdE[n_el], the explicit isotropic-modulus term (C = E C1) (may be
// null).  Elements outside the set get zeros.
int orc_element_objective(const orc_model* m, const double* u, int32_t n_set, const int32_t* elem_set,
                          int32_t category, int32_t component, int32_t optr, double coef, double expnt,
                          int32_t n_tgt, const double* tgt, double* L_out, double* dLdu, double* Q,
                          double* dLdE) {
    if (!m->assembled || m->structural() || n_set <= 0) return -1;
    if (category < 0 || category > 2 || optr < 0 || optr > 3) return -1;
    if (category != 2 && (component < 1 || component > 6)) return -1;
    if (n_tgt != 0 && n_tgt != 1 && n_tgt != n_set) return -1;
    const TypeInfo& t = m->ti;
    const int nn = t.nn, tot = 3 * nn;
    const int stype = (t.type == 81) ? 8 : t.type;
    const TypeInfo ts = type_info(stype);
    // s_cent: 0 for hex8 / brickIM / tet4 (element_meth.rs:81-83), 1/4 for tet10 (:257-259)
    const double sc = (t.type == 10) ? 0.25 : 0.0;
    const double s_cent[3] = {sc, sc, sc};
    std::vector<double> q(n_set), vol(n_set), tg(n_set), eps(6 * (size_t)n_set), sig(6 * (size_t)n_set);
    std::vector<double> Bc((size_t)n_set * 6 * tot), Cs((size_t)n_set * 36);
    for (int k = 0; k < n_set; ++k) {
        const int e = elem_set[k];
        if (e < 0 || e >= m->n_el) return -1;
        double xyz[30], nv[10], dndx[30], C[36];
        elem_xyz(m, e, xyz);
        ip_data(stype, nn, xyz, s_cent, nv, dndx);
        double* B = &Bc[(size_t)k * 6 * tot];
        solid_bmat(nn, dndx, B);
        if (!m->cmat.empty()) std::copy(m->cmat.begin() + (size_t)e * 36, m->cmat.begin() + (size_t)(e + 1) * 36, C);
        else iso_cmat(m->E[e], m->nu[e], C);
        std::copy(C, C + 36, &Cs[(size_t)k * 36]);
        double* ep = &eps[6 * (size_t)k];
        double* sp = &sig[6 * (size_t)k];
        for (int i = 0; i < 6; ++i) {
            double a = 0.0;
            for (int c = 0; c < tot; ++c) a += B[i * tot + c] * u[m->conn[(size_t)e * nn + c / 3] * 3 + c % 3];
            ep[i] = a;
        }
        for (int i = 0; i < 6; ++i) {
            double a = 0.0;
            for (int j = 0; j < 6; ++j) a += C[6 * i + j] * ep[j];
            sp[i] = a;
        }
        if (category == 0) q[k] = sp[component - 1];
        else if (category == 1) q[k] = ep[component - 1];
        else {
            double se = 0.0;
            for (int i = 0; i < 6; ++i) se += sp[i] * ep[i];
            q[k] = 0.5 * se;
        }
        double v = 0.0;
        for (int p = 0; p < ts.nip; ++p) v += ip_data(stype, nn, xyz, ts.ip + 3 * p, nv, dndx) * ts.wt[p];
        vol[k] = v;
        tg[k] = (n_tgt == 0) ? (optr == 1 ? 1.0 : 0.0) : (n_tgt == 1 ? tgt[0] : tgt[k]);
    }
    // operator value and the per-element weights g_k = dL/dq_k
    std::vector<double> g(n_set);
    double L = 0.0;
    if (optr == 0) {
        double ps = 0.0;
        for (int k = 0; k < n_set; ++k) ps += std::pow(q[k] - tg[k], expnt);
        L = coef * std::pow(ps, 1.0 / expnt);
        const double f = coef * std::pow(ps, 1.0 / expnt - 1.0);
        for (int k = 0; k < n_set; ++k) g[k] = f * std::pow(q[k] - tg[k], expnt - 1.0);
    } else if (optr == 1) {
        double ps = 0.0;
        for (int k = 0; k < n_set; ++k) ps += std::exp(expnt * q[k] / tg[k]);
        L = (coef / expnt) * std::log(ps);
        for (int k = 0; k < n_set; ++k) g[k] = coef * std::exp(expnt * q[k] / tg[k]) / ps / tg[k];
    } else {
        double vi = 0.0, tv = 0.0;
        for (int k = 0; k < n_set; ++k) {
            vi += q[k] * vol[k];
            tv += vol[k];
        }
        const double base = (optr == 2) ? vi - tg[0] : vi / tv - tg[0];
        L = coef * std::pow(base, expnt);
        const double f = coef * expnt * std::pow(base, expnt - 1.0) / (optr == 2 ? 1.0 : tv);
        for (int k = 0; k < n_set; ++k) g[k] = f * vol[k];
    }
    if (L_out) *L_out = L;
    if (dLdu) std::fill(dLdu, dLdu + m->n_dof, 0.0);
    if (Q) std::fill(Q, Q + (size_t)m->n_el * 36, 0.0);
    if (dLdE) std::fill(dLdE, dLdE + m->n_el, 0.0);
    for (int k = 0; k < n_set; ++k) {
        const int e = elem_set[k];
        const double* ep = &eps[6 * (size_t)k];
        const double* sp = &sig[6 * (size_t)k];
        double a[6] = {0}, b[6] = {0};
        if (category == 0) a[component - 1] = 1.0;
        else if (category == 1) b[component - 1] = 1.0;
        else
            for (int i = 0; i < 6; ++i) {
                a[i] = 0.5 * ep[i];
                b[i] = 0.5 * sp[i];
            }
        if (dLdu) {
            // w = b + C^T a (strain-space weight), dL/du_e += g B^T w
            const double* C = &Cs[(size_t)k * 36];
            const double* B = &Bc[(size_t)k * 6 * tot];
            double w[6];
            for (int j = 0; j < 6; ++j) {
                double s = b[j];
                for (int i = 0; i < 6; ++i) s += C[6 * i + j] * a[i];
                w[j] = g[k] * s;
            }
            for (int c = 0; c < tot; ++c) {
                double s = 0.0;
                for (int i = 0; i < 6; ++i) s += B[i * tot + c] * w[i];
                dLdu[m->conn[(size_t)e * nn + c / 3] * 3 + c % 3] += s;
            }
        }
        if (Q)
            for (int i = 0; i < 6; ++i)
                for (int j = 0; j < 6; ++j) Q[(size_t)e * 36 + 6 * i + j] += g[k] * a[i] * ep[j];
        if (dLdE) {
            double s = 0.0;
            for (int i = 0; i < 6; ++i) s += a[i] * sp[i];
            dLdE[e] += g[k] * s / m->E[e];
        }
    }
    return 0;
}

}  // extern "C"
