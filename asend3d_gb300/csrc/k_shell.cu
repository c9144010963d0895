// k_shell.cu -- shell4 (type 41) element kernels: stiffness with condensed
// internal DOF, consistent section mass, coloured scatter, adjoint contraction;
// isotropic E, nu, t sections or per-element layered ABD and section mass.
//
// Reference formulation (solverSrc/asend_run_job/src/):
//   element_meth.rs:326-370      type 41: 4 nodes x 6 DOF, 8 internal DOF, 2x2 points
//   element_soln_fields.rs:313-363  shape functions (bilinear, in-plane
//                                incompatible modes 1-s^2 / 1-t^2, four w bubbles)
//   element_soln_fields.rs:383-463  Jacobian with a synthetic third axis; the
//                                non-nodal functions' derivatives at the point
//                                use the centroid Jacobian
//   element_soln_fields.rs:1160-1343 section deformation (membrane strains,
//                                curvatures, transverse shears, drilling)
//   element_properties.rs:766-876  ABD (A = tQ, B = 0, D = t^3/12 Q, shear and
//                                drill entries = A66), :1354-1408 section mass
//   element_equations.rs:206-418   K = sum B^T C B detJ w;  :19-57 condensation
//   element_equations.rs:514-581   M = sum Bm^T Msec Bm detJ w (node DOF only)
// Flat elements in a plane z = const (the element frame is the section frame).
//
// GB300 mapping: one 64-thread CTA per element, all element matrices in
// shared memory, FP64 (the operator is assembled once per transient run);
// each shell node is two 3-DOF pseudo-nodes, so the 24x24 element matrix is
// an 8x8 grid of 3x3 blocks scattered with the hex8 slot map and colouring.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace asend {
namespace {

constexpr int kST = 64;  // threads per element CTA
constexpr double kG = 0.57735026918962576451;  // 1/sqrt(3)

struct ShellSmem {
    double xyz[4][3];
    double C[81];
    double n[4][10];
    double ds[4][10], dt[4][10];  // parametric derivatives per point
    double ji[5][4];              // inverse 2D Jacobian per point (4 = centroid)
    double dx[4][10], dy[4][10];  // dN/dx, dN/dy per point
    double det[4];
    double B[9][32];
    double CB[9][32];
    double K[32][32];
    double Kii[8][8];
    double X[8][24];              // K_ii^-1 K_in
    double K24[24][24];
    double msec[36];              // section mass 6 x 6 (u v w thx thy thz)
};

// Layered sections (per-element ABD [81] and section mass [36]); null
// pointers: the isotropic E, nu, t section.
struct ShellSec {
    const double* abd;
    const double* msec;
};

__device__ void shape(double s, double t, double* n, double* ds, double* dt) {
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

// Builds the condensed 24x24 stiffness (and the section mass terms) of element
// e in shared memory.  All threads of the CTA must call it.
__device__ void shell_element(ShellSmem& S, int e, const int32_t* __restrict__ conn4, const double* __restrict__ xyz,
                              const double* __restrict__ Ev, const double* __restrict__ nuv,
                              const double* __restrict__ rhov, const double* __restrict__ thkv, ShellSec sec) {
    const int t = threadIdx.x;
    if (t < 12) S.xyz[t / 3][t % 3] = xyz[3 * (size_t)conn4[4 * (size_t)e + t / 3] + t % 3];
    if (sec.abd) {
        for (int q = t; q < 81; q += kST) S.C[q] = sec.abd[(size_t)e * 81 + q];
        for (int q = t; q < 36; q += kST) S.msec[q] = rhov ? sec.msec[(size_t)e * 36 + q] : 0.0;
    } else if (t == 12) {
        const double E = Ev[e], nu = nuv[e], h = thkv[e];
        const double G = E / (2.0 * (1.0 + nu)), q = E / (1.0 - nu * nu);
        const double Q[9] = {q, nu * q, 0, nu * q, q, 0, 0, 0, G};
        for (int i = 0; i < 81; ++i) S.C[i] = 0.0;
        const double d = h * h * h / 12.0;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                S.C[9 * i + j] = h * Q[3 * i + j];
                S.C[9 * (i + 3) + j + 3] = d * Q[3 * i + j];
            }
        S.C[60] = S.C[70] = S.C[80] = S.C[20];
        const double r = rhov ? rhov[e] : 0.0;
        for (int i = 0; i < 36; ++i) S.msec[i] = 0.0;
        S.msec[0] = S.msec[7] = S.msec[14] = r * h;
        S.msec[21] = S.msec[28] = S.msec[35] = r * d;
    }
    __syncthreads();
    if (t < 5) {  // points 0..3 and the centroid
        const double sp = (t == 4) ? 0.0 : ((t & 1) ? kG : -kG);
        const double tp = (t == 4) ? 0.0 : ((t & 2) ? kG : -kG);
        double n[10], ds[10], dt[10];
        shape(sp, tp, n, ds, dt);
        double xs = 0, xt = 0, ys = 0, yt = 0;
        for (int a = 0; a < 4; ++a) {
            xs += S.xyz[a][0] * ds[a];
            xt += S.xyz[a][0] * dt[a];
            ys += S.xyz[a][1] * ds[a];
            yt += S.xyz[a][1] * dt[a];
        }
        const double d2 = xs * yt - ys * xt;
        // inverse of [xs xt 0; ys yt 0; 0 0 +-1]: the x/y block
        S.ji[t][0] = yt / d2;
        S.ji[t][1] = -xt / d2;
        S.ji[t][2] = -ys / d2;
        S.ji[t][3] = xs / d2;
        if (t < 4) {
            S.det[t] = fabs(d2);
            for (int f = 0; f < 10; ++f) {
                S.n[t][f] = n[f];
                S.ds[t][f] = ds[f];
                S.dt[t][f] = dt[f];
            }
        }
    }
    for (int q = t; q < 32 * 32; q += kST) S.K[q / 32][q % 32] = 0.0;
    __syncthreads();
    // x/y derivatives at each point: the nodal functions with that point's
    // Jacobian, the non-nodal ones (their derivatives at the point) with the
    // centroid Jacobian (element_soln_fields.rs:424-461)
    if (t < 40) {
        const int ip = t / 10, f = t % 10;
        const double* J = S.ji[f < 4 ? ip : 4];
        S.dx[ip][f] = S.ds[ip][f] * J[0] + S.dt[ip][f] * J[2];
        S.dy[ip][f] = S.ds[ip][f] * J[1] + S.dt[ip][f] * J[3];
    }
    __syncthreads();
    for (int ip = 0; ip < 4; ++ip) {
        // B columns (thread = column)
        if (t < 32) {
            double col[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            int f, c;
            bool rot = false;
            if (t < 24) {
                f = t / 6;
                c = t % 6;
                rot = c >= 3;
            } else {
                const int k = t - 24;
                const int fi[8] = {4, 5, 4, 5, 6, 7, 8, 9}, ci[8] = {0, 0, 1, 1, 2, 2, 2, 2};
                f = fi[k];
                c = ci[k];
            }
            const double dx = S.dx[ip][f], dy = S.dy[ip][f];
            if (!rot) {
                if (c == 0) { col[0] = dx; col[2] = dy; col[8] = dy; }
                if (c == 1) { col[1] = dy; col[2] = dx; col[8] = -dx; }
                if (c == 2) { col[6] = dx; col[7] = dy; }
            } else {
                const double N = S.n[ip][f];
                if (c == 3) { col[4] = -dy; col[5] = -dx; col[7] = -N; }
                if (c == 4) { col[3] = dx; col[5] = dy; col[6] = N; }
                if (c == 5) { col[8] = 2.0 * N; }
            }
            for (int k = 0; k < 9; ++k) S.B[k][t] = col[k];
        }
        __syncthreads();
        for (int q = t; q < 9 * 32; q += kST) {
            const int i = q / 32, c = q % 32;
            double acc = 0.0;
            for (int k = 0; k < 9; ++k) acc += S.C[9 * i + k] * S.B[k][c];
            S.CB[i][c] = acc * S.det[ip];
        }
        __syncthreads();
        for (int q = t; q < 32 * 32; q += kST) {
            const int r = q / 32, c = q % 32;
            double acc = 0.0;
            for (int k = 0; k < 9; ++k) acc += S.B[k][r] * S.CB[k][c];
            S.K[r][c] += acc;
        }
        __syncthreads();
    }
    // condensation: K24 = K_nn - K_ni K_ii^-1 K_in
    if (t < 64) S.Kii[t / 8][t % 8] = S.K[24 + t / 8][24 + t % 8];
    __syncthreads();
    if (t == 0) {  // in-place Gauss-Jordan inverse of the SPD 8x8 block
        for (int p = 0; p < 8; ++p) {
            const double piv = 1.0 / S.Kii[p][p];
            S.Kii[p][p] = 1.0;
            for (int j = 0; j < 8; ++j) S.Kii[p][j] *= piv;
            for (int i = 0; i < 8; ++i) {
                if (i == p) continue;
                const double f = S.Kii[i][p];
                S.Kii[i][p] = 0.0;
                for (int j = 0; j < 8; ++j) S.Kii[i][j] -= f * S.Kii[p][j];
            }
        }
    }
    __syncthreads();
    for (int q = t; q < 8 * 24; q += kST) {
        const int i = q / 24, c = q % 24;
        double acc = 0.0;
        for (int k = 0; k < 8; ++k) acc += S.Kii[i][k] * S.K[24 + k][c];
        S.X[i][c] = acc;
    }
    __syncthreads();
    for (int q = t; q < 24 * 24; q += kST) {
        const int r = q / 24, c = q % 24;
        double acc = 0.0;
        for (int k = 0; k < 8; ++k) acc += S.K[r][24 + k] * S.X[k][c];
        S.K24[r][c] = S.K[r][c] - acc;
    }
    __syncthreads();
}

// mass entry between node DOF (a, ca) and (b, cb): the section mass couples
// the components, the shape functions the nodes
__device__ __forceinline__ double mass_entry(const ShellSmem& S, int a, int ca, int b, int cb) {
    const double m = S.msec[6 * ca + cb];
    if (m == 0.0) return 0.0;
    double acc = 0.0;
    for (int ip = 0; ip < 4; ++ip) acc += S.n[ip][a] * S.n[ip][b] * S.det[ip];
    return m * acc;
}

__global__ void __launch_bounds__(kST)
k_shell_assemble(const int32_t* __restrict__ elems, const int32_t* __restrict__ conn4, const double* __restrict__ xyz,
                 const double* __restrict__ E, const double* __restrict__ nu, const double* __restrict__ rho,
                 const double* __restrict__ thk, const int32_t* __restrict__ slot_map, double* __restrict__ vals,
                 double* __restrict__ mvals, double cM, ShellSec sec) {
    __shared__ ShellSmem S;
    const int e = elems[blockIdx.x];
    shell_element(S, e, conn4, xyz, E, nu, mvals ? rho : nullptr, thk, sec);
    const int pr = threadIdx.x;  // pseudo-node pair (pa, pb)
    const int pa = pr >> 3, pb = pr & 7;
    const int32_t slot = slot_map[(size_t)e * 64 + pr];
    const int64_t g = slot >> 5, lane = slot & 31;
    double* vb = vals + (g * 9) * 32 + lane;
    double* mb = mvals ? mvals + (g * 9) * 32 + lane : nullptr;
    const int a = pa >> 1, b = pb >> 1, oa = 3 * (pa & 1), ob = 3 * (pb & 1);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double k = S.K24[3 * pa + i][3 * pb + j];
            if (mb) {
                const double m = mass_entry(S, a, oa + i, b, ob + j);
                mb[(i * 3 + j) * 32] += m;
                k += cM * m;
            }
            vb[(i * 3 + j) * 32] += k;
        }
}

// g_e = -(lambda_e^T K_e u_e) / E_e (K_e linear in E_e at fixed nu)
__global__ void __launch_bounds__(kST)
k_shell_adjoint(const int32_t* __restrict__ conn4, const double* __restrict__ xyz, const double* __restrict__ E,
                const double* __restrict__ nu, const double* __restrict__ thk, const double* __restrict__ u,
                const double* __restrict__ lam, double* __restrict__ g, int accumulate) {
    __shared__ ShellSmem S;
    __shared__ double red[kST];
    const int e = blockIdx.x;
    shell_element(S, e, conn4, xyz, E, nu, nullptr, thk, ShellSec{nullptr, nullptr});
    double acc = 0.0;
    for (int q = threadIdx.x; q < 24 * 24; q += kST) {
        const int r = q / 24, c = q % 24;
        const size_t dr = 6 * (size_t)conn4[4 * (size_t)e + r / 6] + r % 6;
        const size_t dc = 6 * (size_t)conn4[4 * (size_t)e + c / 6] + c % 6;
        acc += lam[dr] * S.K24[r][c] * u[dc];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kST / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double v = -red[0] / E[e];
        g[e] = accumulate ? g[e] + v : v;
    }
}

// element matrices (checks): ke/me [count][24][24]
__global__ void __launch_bounds__(kST)
k_shell_export(int e0, const int32_t* __restrict__ conn4, const double* __restrict__ xyz, const double* __restrict__ E,
               const double* __restrict__ nu, const double* __restrict__ rho, const double* __restrict__ thk,
               double* __restrict__ ke, double* __restrict__ me, ShellSec sec) {
    __shared__ ShellSmem S;
    const int e = e0 + blockIdx.x;
    shell_element(S, e, conn4, xyz, E, nu, rho, thk, sec);
    for (int q = threadIdx.x; q < 576; q += kST) {
        const int r = q / 24, c = q % 24;
        ke[(size_t)blockIdx.x * 576 + q] = S.K24[r][c];
        if (me) me[(size_t)blockIdx.x * 576 + q] = mass_entry(S, r / 6, r % 6, c / 6, c % 6);
    }
}

ShellSec sections_of(const Ctx& c) {
    return c.shell_layered ? ShellSec{c.d_shell_abd.p, c.d_shell_msec.p} : ShellSec{nullptr, nullptr};
}

}  // namespace

void shell_assemble(Ctx& c, double* vals, double* mvals) {
    const int n_col = (int)c.colour_ptr.size() - 1;
    for (int k = 0; k < n_col; ++k) {
        const int n = c.colour_ptr[k + 1] - c.colour_ptr[k];
        if (n == 0) continue;
        k_shell_assemble<<<n, kST, 0, c.stream>>>(c.d_colour_elems.p + c.colour_ptr[k], c.d_shell_conn.p,
                                                 c.d_shell_xyz.p, c.d_E.p, c.d_nu.p, c.d_rho.p, c.d_thk.p,
                                                 c.d_slot_map.p, vals, mvals, c.cM, sections_of(c));
        ASEND_CUDA(cudaGetLastError());
        ++c.launches;
    }
}

void shell_adjoint(Ctx& c, const double* d_u, const double* d_lam, double* d_g, bool accumulate) {
    if (c.shell_layered)
        throw InputError("layered shell sections have no per-element modulus gradient (K is not proportional to E)");
    k_shell_adjoint<<<c.n_el, kST, 0, c.stream>>>(c.d_shell_conn.p, c.d_shell_xyz.p, c.d_E.p, c.d_nu.p, c.d_thk.p,
                                                 d_u, d_lam, d_g, accumulate ? 1 : 0);
    ASEND_CUDA(cudaGetLastError());
    ++c.launches;
}

void shell_element_matrices(Ctx& c, int e0, int n, double* ke_host, double* me_host) {
    DArr<double> ke, me;
    ke.alloc((size_t)n * 576);
    if (me_host) me.alloc((size_t)n * 576);
    k_shell_export<<<n, kST, 0, c.stream>>>(e0, c.d_shell_conn.p, c.d_shell_xyz.p, c.d_E.p, c.d_nu.p, c.d_rho.p,
                                            c.d_thk.p, ke.p, me_host ? me.p : nullptr, sections_of(c));
    ++c.launches;
    ASEND_CUDA(cudaGetLastError());
    ASEND_CUDA(cudaMemcpyAsync(ke_host, ke.p, sizeof(double) * n * 576, cudaMemcpyDeviceToHost, c.stream));
    if (me_host)
        ASEND_CUDA(cudaMemcpyAsync(me_host, me.p, sizeof(double) * n * 576, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace asend
