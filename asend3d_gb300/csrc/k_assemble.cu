// k_assemble.cu -- K1 element integration fused with K2 coloured scatter.
//
// Reference path (solverSrc/asend_run_job/src/):
//   per-element K_e: element_equations.rs:206-418 (get_ruk_dfd0, Gauss loop
//   K += B^T C B detJ w), shape functions element_soln_fields.rs:120-229,
//   Jacobian / dN/dx element_soln_fields.rs:383-463, solid C
//   element_properties.rs:648-764, consistent mass element_equations.rs:583-609,
//   Newmark mass term element_equations.rs:977-988, scatter to the global
//   matrix element_equations.rs:1040-1059 (SparseMat::add_entry,
//   list_ent_meth.rs:6-18), penalty scale model_analysis.rs:255-259 and the
//   penalty operator const_meth.rs:92-103.
//
// GB300 design: a CTA integrates EB elements; each thread owns one node pair
// (a <= b) of one element and forms the 3x3 block
//     K_ab = lambda S + mu S^T + mu tr(S) I,   S = sum_gp w detJ g_a g_b^T
// (the isotropic B^T C B product in closed form), then scatters K_ab and its
// transpose into the sliced block-ELL values through a precomputed slot map.
// Elements of one colour share no node, so the scatter needs no atomics and
// the summation order is fixed (deterministic).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "pcg_common.cuh"

namespace asend {
namespace {

// Reference-element tables (filled once from the host).
__constant__ double c_hex_dn[8][8][3];  // [gp][node][ds_j]
__constant__ double c_hex_n[8][8];      // [gp][node]
__constant__ int c_hex_pair[36][2];
__constant__ int c_tet_pair[10][2];
__constant__ double c_t10_dn[4][10][3];  // tet10 at its 4 points
__constant__ double c_t10_n[4][10];
__constant__ int c_t10_pair[55][2];
bool g_tables_ready = false;


void init_tables() {
    if (g_tables_ready) return;
    const double g = 0.5773502691896257;
    const double sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                             {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    double dn[8][8][3], nv[8][8];
    int k = 0;
    for (int zc = 0; zc < 2; ++zc)
        for (int yc = 0; yc < 2; ++yc)
            for (int xc = 0; xc < 2; ++xc) {
                const double s[3] = {xc ? g : -g, yc ? g : -g, zc ? g : -g};
                for (int a = 0; a < 8; ++a) {
                    const double f0 = 1 + sg[a][0] * s[0], f1 = 1 + sg[a][1] * s[1], f2 = 1 + sg[a][2] * s[2];
                    nv[k][a] = 0.125 * f0 * f1 * f2;
                    dn[k][a][0] = 0.125 * sg[a][0] * f1 * f2;
                    dn[k][a][1] = 0.125 * sg[a][1] * f0 * f2;
                    dn[k][a][2] = 0.125 * sg[a][2] * f0 * f1;
                }
                ++k;
            }
    int hp[36][2], tp[10][2];
    k = 0;
    for (int a = 0; a < 8; ++a)
        for (int b = a; b < 8; ++b) { hp[k][0] = a; hp[k][1] = b; ++k; }
    k = 0;
    for (int a = 0; a < 4; ++a)
        for (int b = a; b < 4; ++b) { tp[k][0] = a; tp[k][1] = b; ++k; }
    ASEND_CUDA(cudaMemcpyToSymbol(c_hex_dn, dn, sizeof(dn)));
    ASEND_CUDA(cudaMemcpyToSymbol(c_hex_n, nv, sizeof(nv)));
    ASEND_CUDA(cudaMemcpyToSymbol(c_hex_pair, hp, sizeof(hp)));
    ASEND_CUDA(cudaMemcpyToSymbol(c_tet_pair, tp, sizeof(tp)));
    double t10dn[4][10][3], t10n[4][10];
    for (int gp = 0; gp < 4; ++gp) {
        double sp[3];
        tet10_point(gp, sp);
        tet10_shape(sp, t10n[gp], t10dn[gp]);
    }
    int t10p[55][2];
    k = 0;
    for (int a = 0; a < 10; ++a)
        for (int b = a; b < 10; ++b) { t10p[k][0] = a; t10p[k][1] = b; ++k; }
    ASEND_CUDA(cudaMemcpyToSymbol(c_t10_dn, t10dn, sizeof(t10dn)));
    ASEND_CUDA(cudaMemcpyToSymbol(c_t10_n, t10n, sizeof(t10n)));
    ASEND_CUDA(cudaMemcpyToSymbol(c_t10_pair, t10p, sizeof(t10p)));
    g_tables_ready = true;
}

// Optional element data of the colour assembly: per-element 6x6 stiffness
// (replacing the isotropic E, nu), material damping matrices, Rayleigh
// coefficients, the damping coefficient of the Newmark operator and the
// damping values (nullptr: no damping).
struct ElemExtra {
    const double* cmat;
    const double* dmat;
    double rcm, rck, cD;
    double* dvals;
};

__constant__ int c_voigt[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};

template <int NN>
struct ElemTraits;
template <>
struct ElemTraits<8> {
    static constexpr int NIP = 8, NP = 36, EB = 8;
};
template <>
struct ElemTraits<4> {
    static constexpr int NIP = 1, NP = 10, EB = 32;
};
template <>
struct ElemTraits<10> {
    static constexpr int NIP = 4, NP = 55, EB = 8;
};

template <int NN>
__device__ __forceinline__ void pair_of(int p, int& a, int& b) {
    if constexpr (NN == 8) {
        a = c_hex_pair[p][0];
        b = c_hex_pair[p][1];
    } else if constexpr (NN == 10) {
        a = c_t10_pair[p][0];
        b = c_t10_pair[p][1];
    } else {
        a = c_tet_pair[p][0];
        b = c_tet_pair[p][1];
    }
}

template <int NN, typename T>
__device__ __forceinline__ void shape_ref(int gp, int a, T& n, T (&dn)[3]) {
    if constexpr (NN == 8) {
        n = (T)c_hex_n[gp][a];
        dn[0] = (T)c_hex_dn[gp][a][0];
        dn[1] = (T)c_hex_dn[gp][a][1];
        dn[2] = (T)c_hex_dn[gp][a][2];
    } else if constexpr (NN == 10) {
        n = (T)c_t10_n[gp][a];
        dn[0] = (T)c_t10_dn[gp][a][0];
        dn[1] = (T)c_t10_dn[gp][a][1];
        dn[2] = (T)c_t10_dn[gp][a][2];
    } else {
        n = (T)0.25;
        dn[0] = (a == 1) ? (T)1 : (a == 0 ? (T)-1 : (T)0);
        dn[1] = (a == 2) ? (T)1 : (a == 0 ? (T)-1 : (T)0);
        dn[2] = (a == 3) ? (T)1 : (a == 0 ? (T)-1 : (T)0);
    }
}

// One CTA = EB elements of one colour; thread = (element, node pair).
template <int NN, typename T>
__global__ void __launch_bounds__(ElemTraits<NN>::EB * ElemTraits<NN>::NP)
assemble_colour_kernel(int n_el, const int32_t* __restrict__ el_list, const int32_t* __restrict__ conn,
                       const double* __restrict__ xyz, const double* __restrict__ E,
                       const double* __restrict__ nu, const double* __restrict__ rho,
                       const int32_t* __restrict__ slot_map, T* __restrict__ vals,
                       double* __restrict__ mvals, double cM, ElemExtra X) {
    constexpr int NIP = ElemTraits<NN>::NIP, NP = ElemTraits<NN>::NP, EB = ElemTraits<NN>::EB;
    __shared__ T s_x[EB][NN][3];
    __shared__ T s_g[EB][NIP][NN][3];
    __shared__ T s_w[EB][NIP];
    __shared__ int s_el[EB];
    const int tid = threadIdx.x;
    const int base = blockIdx.x * EB;
    if (tid < EB) s_el[tid] = (base + tid < n_el) ? el_list[base + tid] : -1;
    __syncthreads();
    // coordinates relative to the element's first node (translation invariant)
    for (int t = tid; t < EB * NN * 3; t += blockDim.x) {
        const int el = t / (NN * 3), a = (t / 3) % NN, j = t % 3;
        const int e = s_el[el];
        T v = 0;
        if (e >= 0) {
            const int n0 = conn[(size_t)e * NN], na = conn[(size_t)e * NN + a];
            v = (T)(xyz[3 * (size_t)na + j] - xyz[3 * (size_t)n0 + j]);
        }
        s_x[el][a][j] = v;
    }
    __syncthreads();
    // Gauss-point data: J = sum_a x_a dN_a^T, dN/dx = dN/ds J^-1
    if (tid < EB * NIP) {
        const int el = tid / NIP, gp = tid % NIP;
        T J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int a = 0; a < NN; ++a) {
            T n, dn[3];
            shape_ref<NN, T>(gp, a, n, dn);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) J[i][j] += s_x[el][a][i] * dn[j];
        }
        const T c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const T c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const T c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const T det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        const T id = (T)1 / det;
        T Ji[3][3];
        Ji[0][0] = c00 * id;
        Ji[1][0] = c01 * id;
        Ji[2][0] = c02 * id;
        Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
        Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
        Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
        Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
        for (int a = 0; a < NN; ++a) {
            T n, dn[3];
            shape_ref<NN, T>(gp, a, n, dn);
#pragma unroll
            for (int j = 0; j < 3; ++j) s_g[el][gp][a][j] = dn[0] * Ji[0][j] + dn[1] * Ji[1][j] + dn[2] * Ji[2][j];
        }
        s_w[el][gp] = det * ((NN == 8) ? (T)1 : (NN == 10 ? (T)(1.0 / 24.0) : (T)(1.0 / 6.0)));
    }
    __syncthreads();
    if (tid >= EB * NP) return;
    const int el = tid / NP, p = tid % NP;
    const int e = s_el[el];
    if (e < 0) return;
    int a, b;
    pair_of<NN>(p, a, b);
    T S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    T m = 0;
#pragma unroll
    for (int gp = 0; gp < NIP; ++gp) {
        const T w = s_w[el][gp];
        const T ga0 = s_g[el][gp][a][0] * w, ga1 = s_g[el][gp][a][1] * w, ga2 = s_g[el][gp][a][2] * w;
        const T gb0 = s_g[el][gp][b][0], gb1 = s_g[el][gp][b][1], gb2 = s_g[el][gp][b][2];
        S[0][0] += ga0 * gb0; S[0][1] += ga0 * gb1; S[0][2] += ga0 * gb2;
        S[1][0] += ga1 * gb0; S[1][1] += ga1 * gb1; S[1][2] += ga1 * gb2;
        S[2][0] += ga2 * gb0; S[2][1] += ga2 * gb1; S[2][2] += ga2 * gb2;
        if (mvals) {
            T na, nb, dn[3];
            shape_ref<NN, T>(gp, a, na, dn);
            shape_ref<NN, T>(gp, b, nb, dn);
            m += na * nb * w;
        }
    }
    const T mass = mvals ? m * (T)rho[e] : (T)0;
    // K_ab: isotropic closed form, or a general 6x6 C contracted with S,
    // K_ab[i][j] = sum_kl C[v(i,k)][v(j,l)] S[k][l] (v: the Voigt index of a
    // symmetric index pair), which is B_a^T C B_b integrated
    T Kab[3][3], Dab[3][3];
    if (X.cmat) {
        const double* Ce = X.cmat + (size_t)e * 36;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                T acc = 0;
#pragma unroll
                for (int k = 0; k < 3; ++k)
#pragma unroll
                    for (int l = 0; l < 3; ++l) acc += (T)Ce[6 * c_voigt[i][k] + c_voigt[j][l]] * S[k][l];
                Kab[i][j] = acc;
            }
    } else {
        const double Ee = E[e], ne = nu[e];
        const T lam = (T)(Ee * ne / ((1.0 + ne) * (1.0 - 2.0 * ne)));
        const T mu = (T)(Ee / (2.0 * (1.0 + ne)));
        const T tr = mu * (S[0][0] + S[1][1] + S[2][2]);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Kab[i][j] = lam * S[i][j] + mu * S[j][i] + ((i == j) ? tr : (T)0);
    }
    // damping block (Rayleigh mass / stiffness terms + material B^T D B)
    if (X.dvals) {
        const double* De = X.dmat ? X.dmat + (size_t)e * 36 : nullptr;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                T acc = (T)X.rck * Kab[i][j] + ((i == j) ? (T)X.rcm * mass : (T)0);
                if (De) {
#pragma unroll
                    for (int k = 0; k < 3; ++k)
#pragma unroll
                        for (int l = 0; l < 3; ++l) acc += (T)De[6 * c_voigt[i][k] + c_voigt[j][l]] * S[k][l];
                }
                Dab[i][j] = acc;
            }
    }
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1 && a == b) break;
        // pass 0: block (a, b); pass 1: its transpose at (b, a)
        const int32_t slot = pass ? slot_map[((size_t)e * NN + b) * NN + a] : slot_map[((size_t)e * NN + a) * NN + b];
        const int64_t g = slot >> 5, lane = slot & 31;
        T* vb = vals + (g * 9) * 32 + lane;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                T kij = Kab[i][j];
                if (i == j) kij += (T)cM * mass;
                if (X.dvals) kij += (T)X.cD * Dab[i][j];
                vb[(pass ? (j * 3 + i) : (i * 3 + j)) * 32] += kij;
            }
        if (mvals) {
            double* mb = mvals + (g * 9) * 32 + lane;
#pragma unroll
            for (int i = 0; i < 3; ++i) mb[(i * 3 + i) * 32] += (double)mass;
        }
        if (X.dvals) {
            double* db = X.dvals + (g * 9) * 32 + lane;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) db[(pass ? (j * 3 + i) : (i * 3 + j)) * 32] += (double)Dab[i][j];
        }
    }
}

__global__ void max_abs_kernel(size_t n, const double* __restrict__ v, unsigned long long* out) {
    double m = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(v[i]));
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

__global__ void penalty_kernel(int n, const int64_t* __restrict__ idx, const double* __restrict__ coef,
                               double sf, double* vals) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) atomicAdd(&vals[idx[k]], sf * coef[k]);
}

__global__ void unit_kernel(int n, const int64_t* __restrict__ idx, double* vals) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) vals[idx[k]] = 1.0;
}

// per-instance max |value| over contiguous value ranges (blockIdx.y = instance)
__global__ void max_abs_seg_kernel(const int64_t* __restrict__ seg, const double* __restrict__ v,
                                   unsigned long long* out) {
    const int inst = blockIdx.y;
    const int64_t b = seg[inst], e = seg[inst + 1];
    double m = 0.0;
    for (int64_t i = b + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < e; i += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(v[i]));
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) atomicMax(&out[inst], (unsigned long long)__double_as_longlong(m));
}

__global__ void penalty_val_kernel(int n, const int64_t* __restrict__ idx, const double* __restrict__ val,
                                   double* vals) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) atomicAdd(&vals[idx[k]], val[k]);
}

// FP32 copy (high parts) and the low parts of the FP64 values
__global__ void round_kernel(size_t n, const double* __restrict__ src, float* __restrict__ dst,
                             float* __restrict__ lo) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = src[i];
        const float hi = (float)v;
        dst[i] = hi;
        lo[i] = (float)(v - (double)hi);
    }
}
__global__ void widen_kernel(size_t n, const float* __restrict__ src, double* __restrict__ dst) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}

// ---- geometry classes and the gather assembly --------------------------------
// Unit-modulus (E = 1) stiffness and unit-density mass of hex8 elements
// reps[r] (one per geometry class): the closed-form isotropic blocks of
// assemble_colour_kernel at E = 1.  One CTA (64 threads = node pairs) per
// element.
__global__ void __launch_bounds__(64) k_hex8_unit(const int32_t* __restrict__ reps, const int32_t* __restrict__ conn,
                                                  const double* __restrict__ xyz, const double* __restrict__ nu,
                                                  double* __restrict__ ke, double* __restrict__ me) {
    __shared__ double s_x[8][3];
    __shared__ double s_g[8][8][3];
    __shared__ double s_w[8];
    const int r = blockIdx.x, t = threadIdx.x;
    const int e = reps[r];
    if (t < 24) {
        const int a = t / 3, j = t % 3;
        const int n0 = conn[(size_t)e * 8], na = conn[(size_t)e * 8 + a];
        s_x[a][j] = xyz[3 * (size_t)na + j] - xyz[3 * (size_t)n0 + j];
    }
    __syncthreads();
    if (t < 8) {
        const int gp = t;
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int a = 0; a < 8; ++a)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) J[i][j] += s_x[a][i] * c_hex_dn[gp][a][j];
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
        for (int a = 0; a < 8; ++a)
            for (int j = 0; j < 3; ++j)
                s_g[gp][a][j] = c_hex_dn[gp][a][0] * Ji[0][j] + c_hex_dn[gp][a][1] * Ji[1][j] + c_hex_dn[gp][a][2] * Ji[2][j];
        s_w[gp] = det;
    }
    __syncthreads();
    const int a = t >> 3, b = t & 7;
    double S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double m = 0.0;
    for (int gp = 0; gp < 8; ++gp) {
        const double w = s_w[gp];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) S[i][j] += s_g[gp][a][i] * w * s_g[gp][b][j];
        m += c_hex_n[gp][a] * c_hex_n[gp][b] * w;
    }
    const double ne = nu[e];
    const double lam = ne / ((1.0 + ne) * (1.0 - 2.0 * ne));
    const double mu = 1.0 / (2.0 * (1.0 + ne));
    const double tr = mu * (S[0][0] + S[1][1] + S[2][2]);
    double* K = ke + (size_t)r * 576;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            K[(3 * a + i) * 24 + 3 * b + j] = lam * S[i][j] + mu * S[j][i] + ((i == j) ? tr : 0.0);
    me[(size_t)r * 64 + t] = m;
}

// Gather assembly: one CTA per slice of 32 node rows; thread (lane, jj)
// forms the slots j = jj, jj + 8, ... of row slice*32 + lane.  Each value is
// summed once from its contributing (element, a, b) entries,
//   K_slot = sum E_e Khat_class(e)[a, b] (+ c_M rho_e Mhat_class(e)[a, b] I),
// and written once in FP64 and as FP32 hi / lo parts (no colouring, no
// read-modify-write, no zeroing pass); the largest |value| of the slice's
// instance is reduced on the way (the penalty scale).  A slot's entries are
// fetched up to 8 at a time (independent loads in flight).
__global__ void __launch_bounds__(256)
k_gather_assemble(const int64_t* __restrict__ slice_off, const int32_t* __restrict__ gat_ptr,
                  const int32_t* __restrict__ gat, const int32_t* __restrict__ cls_of,
                  const double* __restrict__ cls_ke, const double* __restrict__ cls_me, const double* __restrict__ E,
                  const double* __restrict__ rho, double cM, double* __restrict__ v64, float* __restrict__ v32,
                  float* __restrict__ v32lo, double* __restrict__ m64, const int32_t* __restrict__ slice_inst,
                  unsigned long long* __restrict__ max_out) {
    __shared__ double s_max[8];
    const int sl = blockIdx.x, lane = threadIdx.x & 31, jj = threadIdx.x >> 5;
    const int64_t g0 = slice_off[sl];
    const int W = (int)(slice_off[sl + 1] - g0);
    double mx = 0.0;
    for (int j = jj; j < W; j += 8) {
        const int64_t g = g0 + j;
        const int64_t slot = g * 32 + lane;
        double k[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) k[q] = 0.0;
        double m = 0.0;
        const int q0 = gat_ptr[slot], q1 = gat_ptr[slot + 1];
        for (int base = q0; base < q1; base += 8) {
            int ent[8], cl[8];
            double Ee[8], re[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) ent[u] = (base + u < q1) ? gat[base + u] : -1;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                cl[u] = 0;
                Ee[u] = 0.0;
                re[u] = 0.0;
                if (ent[u] >= 0) {
                    const int e = ent[u] >> 6;
                    cl[u] = cls_of[e];
                    Ee[u] = E[e];
                    if (m64) re[u] = rho[e];
                }
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (ent[u] < 0) continue;
                const int a = (ent[u] >> 3) & 7, b = ent[u] & 7;
                const double* K = cls_ke + (size_t)cl[u] * 576 + (3 * a) * 24 + 3 * b;
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int c2 = 0; c2 < 3; ++c2) k[i * 3 + c2] = fma(Ee[u], K[i * 24 + c2], k[i * 3 + c2]);
                if (m64) m = fma(re[u], cls_me[(size_t)cl[u] * 64 + a * 8 + b], m);
            }
        }
        if (m64) {
            k[0] += cM * m;
            k[4] += cM * m;
            k[8] += cM * m;
        }
        double* vb = v64 + (g * 9) * 32 + lane;
        float* wb = v32 + (g * 9) * 32 + lane;
        float* lb = v32lo + (g * 9) * 32 + lane;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const float hi = (float)k[q];
            vb[q * 32] = k[q];
            wb[q * 32] = hi;
            lb[q * 32] = (float)(k[q] - (double)hi);
            mx = fmax(mx, fabs(k[q]));
        }
        if (m64) {
            double* mb = m64 + (g * 9) * 32 + lane;
#pragma unroll
            for (int q = 0; q < 9; ++q) mb[q * 32] = (q == 0 || q == 4 || q == 8) ? m : 0.0;
        }
    }
    mx = warp_max(mx);
    if (lane == 0) s_max[jj] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t = fmax(t, s_max[w]);
        atomicMax(&max_out[slice_inst ? slice_inst[sl] : 0], (unsigned long long)__double_as_longlong(t));
    }
}

// ---------------------------------------------------------------------------
// Split-only gather assembly (precision 48, statics): the same sums
// K_slot = sum E_e Khat_class(e)[a, b] as k_gather_assemble, in FP32 pairs
// (E_e and Khat as pairs, FMA-exact products, TwoSum accumulation) on the
// FP32 pipes, written as the hi / lo values only.  On this GPU the FP64 gather
// was bound by its FP64 sums and conversions, not by its writes.  The largest
// |value| per instance (the penalty scale) is compared exactly on the pairs
// and converted to FP64 once per thread.
// ---------------------------------------------------------------------------
__global__ void k_pairs_of(size_t n, const double* __restrict__ v, float2* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const pcg::F2 a = pcg::f2_of(v[i]);
        out[i] = make_float2(a.h, a.l);
    }
}

__device__ __forceinline__ bool pair_abs_greater(pcg::F2 a, pcg::F2 b) {  // |a| > |b| for normalised pairs
    const float ah = fabsf(a.h), bh = fabsf(b.h);
    if (ah != bh) return ah > bh;
    return copysignf(1.f, a.h) * a.l > copysignf(1.f, b.h) * b.l;
}

__global__ void __launch_bounds__(256)
k_gather_assemble_pair(const int64_t* __restrict__ slice_off, const int32_t* __restrict__ gat_ptr,
                       const int32_t* __restrict__ gat, const int32_t* __restrict__ cls_of,
                       const float2* __restrict__ cls_ke2, const float2* __restrict__ E2, float* __restrict__ v32,
                       float* __restrict__ v32lo, const int32_t* __restrict__ slice_inst,
                       unsigned long long* __restrict__ max_out) {
    __shared__ double s_max[8];
    const int sl = blockIdx.x, lane = threadIdx.x & 31, jj = threadIdx.x >> 5;
    const int64_t g0 = slice_off[sl];
    const int W = (int)(slice_off[sl + 1] - g0);
    pcg::F2 mx{0.f, 0.f};
    for (int j = jj; j < W; j += 8) {
        const int64_t g = g0 + j;
        const int64_t slot = g * 32 + lane;
        pcg::F2 k[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) k[q] = {0.f, 0.f};
        const int q0 = gat_ptr[slot], q1 = gat_ptr[slot + 1];
        for (int base = q0; base < q1; base += 8) {
            int ent[8], cl[8];
            float2 Ee[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) ent[u] = (base + u < q1) ? gat[base + u] : -1;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                cl[u] = 0;
                Ee[u] = make_float2(0.f, 0.f);
                if (ent[u] >= 0) {
                    const int e = ent[u] >> 6;
                    cl[u] = cls_of[e];
                    Ee[u] = E2[e];
                }
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (ent[u] < 0) continue;
                const int a = (ent[u] >> 3) & 7, b = ent[u] & 7;
                const float2* K = cls_ke2 + (size_t)cl[u] * 576 + (3 * a) * 24 + 3 * b;
                const pcg::F2 E{Ee[u].x, Ee[u].y};
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int c2 = 0; c2 < 3; ++c2) {
                        const float2 kv = K[i * 24 + c2];
                        k[i * 3 + c2] = pcg::f2_add(k[i * 3 + c2], pcg::f2_mul(E, pcg::F2{kv.x, kv.y}));
                    }
            }
        }
        float* wb = v32 + (g * 9) * 32 + lane;
        float* lb = v32lo + (g * 9) * 32 + lane;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            wb[q * 32] = k[q].h;
            lb[q * 32] = k[q].l;
            if (pair_abs_greater(k[q], mx)) mx = k[q];
        }
    }
    double m = fabs(pcg::f2_dbl(mx));
    m = warp_max(m);
    if (lane == 0) s_max[jj] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t = fmax(t, s_max[w]);
        atomicMax(&max_out[slice_inst ? slice_inst[sl] : 0], (unsigned long long)__double_as_longlong(t));
    }
}

// FP64 values at the listed slots from their pairs (the penalty and unit
// slots, before the FP64 penalty update of a split-only assembly)
__global__ void k_slots_to64(int n, const int64_t* __restrict__ idx, const float* __restrict__ v32,
                             const float* __restrict__ v32lo, double* __restrict__ v64) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) v64[idx[k]] = (double)v32[idx[k]] + (double)v32lo[idx[k]];
}

// every FP64 value from its pair
__global__ void k_pairs_to64(size_t n, const float* __restrict__ v32, const float* __restrict__ v32lo,
                             double* __restrict__ v64) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        v64[i] = (double)v32[i] + (double)v32lo[i];
}

// Row-sum lumping of the assembled mass (the reference lumps each element's
// mass by its rows, element_equations.rs:950-971; summed over the elements
// that is the row sum of the global mass): m := diag(row sums), and the
// operator's diagonal gains cM times it.
__global__ void k_lump_mass(int n_rows, const int64_t* __restrict__ slice_off, const uint8_t* __restrict__ row_len,
                            const uint8_t* __restrict__ diag, double* __restrict__ m64, double* __restrict__ v64,
                            double cM) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    const int lane = row & 31;
    const int64_t g0 = slice_off[row >> 5];
    const int len = row_len[row];
    double s3[3] = {0, 0, 0};
    for (int j = 0; j < len; ++j)
        for (int q = 0; q < 9; ++q) {
            double* mq = m64 + ((g0 + j) * 9 + q) * 32 + lane;
            s3[q / 3] += *mq;
            *mq = 0.0;
        }
    const int64_t gd = g0 + diag[row];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        m64[(gd * 9 + 4 * a) * 32 + lane] = s3[a];
        v64[(gd * 9 + 4 * a) * 32 + lane] += cM * s3[a];
    }
}

// d := cm * m (Rayleigh mass-proportional damping of elements whose kernels
// form no damping block), operator += cD d
__global__ void k_mass_damping(size_t n, const double* __restrict__ m64, double cm, double cD, double* __restrict__ d64,
                               double* __restrict__ v64) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double d = cm * m64[i];
        d64[i] = d;
        v64[i] += cD * d;
    }
}

// FP32 hi / lo copies of the entries the penalty or the unit diagonal changed
__global__ void k_refresh32(int n, const int64_t* __restrict__ idx, const double* __restrict__ v64,
                            float* __restrict__ v32, float* __restrict__ v32lo) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double v = v64[idx[k]];
    const float hi = (float)v;
    v32[idx[k]] = hi;
    v32lo[idx[k]] = (float)(v - (double)hi);
}

int stream_grid(size_t n) {
    size_t b = (n + 255) / 256;
    return (int)std::min<size_t>(b, 152 * 16);
}

template <int NN, typename T>
void launch_colours(Ctx& c, T* vals, double* mvals, double cM, const ElemExtra& X) {
    constexpr int EB = ElemTraits<NN>::EB, NP = ElemTraits<NN>::NP;
    const int n_col = (int)c.colour_ptr.size() - 1;
    for (int k = 0; k < n_col; ++k) {
        const int n = c.colour_ptr[k + 1] - c.colour_ptr[k];
        if (n == 0) continue;
        const int blocks = (n + EB - 1) / EB;
        assemble_colour_kernel<NN, T><<<blocks, EB * NP, 0, c.stream>>>(
            n, c.d_colour_elems.p + c.colour_ptr[k], c.d_conn.p, c.d_xyz.p, c.d_E.p, c.d_nu.p, c.d_rho.p,
            c.d_slot_map.p, vals, mvals, cM, X);
        ASEND_CUDA(cudaGetLastError());
        ++c.launches;
    }
}

}  // namespace

// Geometry classes of a hex8 / brickIM mesh and the per-slot gather lists.
// Two elements share a class when their corner offsets from corner 0 agree
// to 1e-12 of the element size and their Poisson ratios are equal; their
// matrices at unit modulus and density then agree to that relative level, so
// K_e = E_e Khat_class and M_e = rho_e Mhat_class.  A structured block has
// one class (a batch of blocks one per instance); an unstructured mesh has up
// to one per element.  Without classes (other element types, or more class
// matrices than fit the memory cap) the colour scatter assembles instead.
void build_classes(Ctx& c, const std::vector<int32_t>& slot_map) {
    c.cls_ready = false;
    c.n_cls = 0;
    c.cls_ke.release();
    c.cls_me.release();
    c.cls_ke32.release();
    c.cls_ke2.release();
    c.d_cls_of.release();
    c.d_gat_ptr.release();
    c.d_gat.release();
    c.h_cls_of.clear();
    if ((c.type != 8 && c.type != 81) || c.n_el >= (1 << 25)) return;
    init_tables();
    const int nn = 8, ne = c.n_el;
    std::vector<double> rel((size_t)ne * 24), scale(ne);
    double hmax = 0.0;
    for (int e = 0; e < ne; ++e) {
        const int n0 = c.conn[(size_t)e * nn];
        double s2 = 0.0;
        for (int a = 0; a < nn; ++a) {
            const int na = c.conn[(size_t)e * nn + a];
            for (int j = 0; j < 3; ++j) {
                const double d = c.xyz[3 * (size_t)na + j] - c.xyz[3 * (size_t)n0 + j];
                rel[(size_t)e * 24 + 3 * a + j] = d;
                s2 = std::max(s2, std::fabs(d));
            }
        }
        scale[e] = s2;
        hmax = std::max(hmax, s2);
    }
    if (!(hmax > 0.0)) return;
    const double grid = 1e-9 * hmax;
    std::unordered_map<uint64_t, std::vector<int32_t>> buckets;
    std::vector<int32_t> reps;
    c.h_cls_of.assign(ne, 0);
    const size_t cap_bytes = (size_t)1 << 30;
    for (int e = 0; e < ne; ++e) {
        const double* r = &rel[(size_t)e * 24];
        uint64_t h = 1469598103934665603ull;
        auto mix = [&](uint64_t v) {
            h ^= v;
            h *= 1099511628211ull;
        };
        for (int i = 0; i < 24; ++i) mix((uint64_t)std::llround(r[i] / grid));
        uint64_t nub;
        std::memcpy(&nub, &c.nu[e], sizeof(nub));
        mix(nub);
        auto& cand = buckets[h];
        int found = -1;
        for (int cl : cand) {
            const int rp = reps[cl];
            if (c.nu[rp] != c.nu[e]) continue;
            const double* q = &rel[(size_t)rp * 24];
            double d = 0.0;
            for (int i = 0; i < 24; ++i) d = std::max(d, std::fabs(r[i] - q[i]));
            if (d <= 1e-12 * scale[e]) {
                found = cl;
                break;
            }
        }
        if (found < 0) {
            found = (int)reps.size();
            reps.push_back(e);
            cand.push_back(found);
            if (reps.size() * 576 * sizeof(double) > cap_bytes || (c.type == 81 && reps.size() > 4096)) {
                c.h_cls_of.clear();
                return;
            }
        }
        c.h_cls_of[e] = found;
    }
    const int ncl = (int)reps.size();
    c.cls_ke.alloc((size_t)ncl * 576);
    c.cls_me.alloc((size_t)ncl * 64);
    if (c.type == 8) {
        DArr<int32_t> d_reps;
        d_reps.upload(reps, c.stream);
        k_hex8_unit<<<ncl, 64, 0, c.stream>>>(d_reps.p, c.d_conn.p, c.d_xyz.p, c.d_nu.p, c.cls_ke.p, c.cls_me.p);
        ++c.launches;
        ASEND_CUDA(cudaGetLastError());
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
    } else {
        // brickIM: the condensed matrices of each class's element, scaled to
        // unit modulus and density (the condensation is linear in E)
        std::vector<double> ke((size_t)ncl * 576), me((size_t)ncl * 64, 0.0), kt(576), mt(576);
        const bool mass = !c.rho.empty();
        for (int cl = 0; cl < ncl; ++cl) {
            const int e = reps[cl];
            brickim_element_matrices(c, e, 1, kt.data(), mass ? mt.data() : nullptr);
            for (int q = 0; q < 576; ++q) ke[(size_t)cl * 576 + q] = kt[q] / c.E[e];
            if (mass && c.rho[e] != 0.0)
                for (int a = 0; a < 8; ++a)
                    for (int b = 0; b < 8; ++b) me[(size_t)cl * 64 + a * 8 + b] = mt[(3 * a) * 24 + 3 * b] / c.rho[e];
        }
        ASEND_CUDA(cudaMemcpyAsync(c.cls_ke.p, ke.data(), sizeof(double) * ke.size(), cudaMemcpyHostToDevice, c.stream));
        ASEND_CUDA(cudaMemcpyAsync(c.cls_me.p, me.data(), sizeof(double) * me.size(), cudaMemcpyHostToDevice, c.stream));
    }
    {
        std::vector<double> k64((size_t)ncl * 576);
        ASEND_CUDA(cudaMemcpyAsync(k64.data(), c.cls_ke.p, sizeof(double) * k64.size(), cudaMemcpyDeviceToHost,
                                   c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        std::vector<float> k32(k64.begin(), k64.end());
        c.cls_ke32.upload(k32, c.stream);
    }
    // per-slot lists of contributing (element, a, b), in element order
    const Sbell& A = c.A;
    const size_t n_slots = (size_t)A.n_groups * kSlice;
    std::vector<int32_t> ptr(n_slots + 1, 0);
    for (size_t q = 0; q < slot_map.size(); ++q) ptr[(size_t)slot_map[q] + 1]++;
    for (size_t q = 0; q < n_slots; ++q) ptr[q + 1] += ptr[q];
    std::vector<int32_t> gat(slot_map.size()), fill(ptr.begin(), ptr.end() - 1);
    for (int e = 0; e < ne; ++e)
        for (int ab = 0; ab < 64; ++ab) gat[fill[slot_map[(size_t)e * 64 + ab]]++] = e * 64 + ab;
    c.d_gat_ptr.upload(ptr, c.stream);
    c.d_gat.upload(gat, c.stream);
    c.d_cls_of.upload(c.h_cls_of, c.stream);
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    c.n_cls = ncl;
    c.cls_type = c.type;
    c.cls_ready = true;
}

void assemble_operator(Ctx& c, int precision) {
    init_tables();
    Sbell& A = c.A;
    const size_t nval = (size_t)A.n_groups * 9 * kSlice;
    A.v64.alloc(nval);
    A.v32.alloc(nval);
    A.v32lo.alloc(nval);
    // damping (Newmark only): a damping value array and its operator term
    const bool damp = c.dynamic && !c.modal && (c.ray_cm != 0.0 || c.ray_ck != 0.0 || !c.dmat.empty());
    const bool lump = c.dynamic && !c.modal && c.lump;
    c.cD = damp ? c.dt * c.gamma * c.cM : 0.0;
    // gather path: FP64 hex8 / brickIM with geometry classes and isotropic
    // material, no damping or lumping (every value written once, the penalty
    // scale reduced on the way)
    const bool gather_ok = c.cls_ready && c.cls_type == c.type && c.ortho.empty() && !damp && !lump;
    // split-only (precision 48): statics on the class gather; anything else
    // takes the FP64 assembly
    const bool split_only = precision == 48 && gather_ok && !c.dynamic;
    if (precision == 48 && !split_only) precision = 64;
    const bool gather = precision == 64 && gather_ok;
    double* mvals = nullptr;
    if (c.dynamic) {
        A.m64.alloc(nval);
        if (!gather) A.m64.zero(c.stream);
        mvals = A.m64.p;
    } else {
        A.m64.release();
    }
    if (damp) {
        A.d64.alloc(nval);
        A.d64.zero(c.stream);
    } else {
        A.d64.release();
    }
    // lumped mass: elements assemble K (and M apart), the lumped mass enters after
    const double cM_el = lump ? 0.0 : c.cM;
    ElemExtra X{};
    X.cmat = c.ortho.empty() ? nullptr : c.d_cmat.p;
    if (damp && (c.ray_ck != 0.0 || !c.dmat.empty())) {  // damping blocks formed by the element kernel
        X.dmat = c.dmat.empty() ? nullptr : c.d_dmat.p;
        X.rcm = c.ray_cm;
        X.rck = c.ray_ck;
        X.cD = c.cD;
        X.dvals = A.d64.p;
    }
    if (!gather && !split_only) {  // the scatter paths accumulate into zeroed values
        A.v64.zero(c.stream);
        A.v32.zero(c.stream);
    }
    const int ni = c.n_inst > 1 ? c.n_inst : 1;
    ASEND_CUDA(cudaEventRecord(c.ev0, c.stream));
    c.d_max_partial.alloc(ni);
    c.d_max_partial.zero(c.stream);
    unsigned long long* dmax = reinterpret_cast<unsigned long long*>(c.d_max_partial.p);
    if (split_only) {
        const int32_t* slice_inst = nullptr;
        DArr<int32_t> d_si;
        if (ni > 1) {
            std::vector<int32_t> si(A.n_slices);
            for (int s2 = 0; s2 < A.n_slices; ++s2) si[s2] = instance_of_node(c, s2 * kSlice);
            d_si.upload(si, c.stream);
            slice_inst = d_si.p;
        }
        const size_t n_cls_vals = (size_t)c.n_cls * 576;
        if (c.cls_ke2.n != n_cls_vals) {
            c.cls_ke2.alloc(n_cls_vals);
            k_pairs_of<<<stream_grid(n_cls_vals), 256, 0, c.stream>>>(n_cls_vals, c.cls_ke.p, c.cls_ke2.p);
            ++c.launches;
        }
        c.d_E2.alloc(c.n_el);
        k_pairs_of<<<stream_grid(c.n_el), 256, 0, c.stream>>>((size_t)c.n_el, c.d_E.p, c.d_E2.p);
        k_gather_assemble_pair<<<A.n_slices, 256, 0, c.stream>>>(A.slice_off.p, c.d_gat_ptr.p, c.d_gat.p,
                                                                 c.d_cls_of.p, c.cls_ke2.p, c.d_E2.p, A.v32.p,
                                                                 A.v32lo.p, slice_inst, dmax);
        c.launches += 2;
        ASEND_CUDA(cudaGetLastError());
        ASEND_CUDA(cudaStreamSynchronize(c.stream));  // d_si
        // the FP64 penalty / unit updates below work on FP64 values at their slots
        const int np0 = (int)c.d_pen_idx.n, nu0 = (int)c.d_unit_idx.n;
        if (np0 > 0)
            k_slots_to64<<<(np0 + 255) / 256, 256, 0, c.stream>>>(np0, c.d_pen_idx.p, A.v32.p, A.v32lo.p, A.v64.p);
        if (nu0 > 0)
            k_slots_to64<<<(nu0 + 255) / 256, 256, 0, c.stream>>>(nu0, c.d_unit_idx.p, A.v32.p, A.v32lo.p, A.v64.p);
        c.launches += (np0 > 0) + (nu0 > 0);
    } else if (gather) {
        const int32_t* slice_inst = nullptr;
        DArr<int32_t> d_si;
        if (ni > 1) {
            std::vector<int32_t> si(A.n_slices);
            for (int s2 = 0; s2 < A.n_slices; ++s2) si[s2] = instance_of_node(c, s2 * kSlice);
            d_si.upload(si, c.stream);
            slice_inst = d_si.p;
        }
        k_gather_assemble<<<A.n_slices, 256, 0, c.stream>>>(A.slice_off.p, c.d_gat_ptr.p, c.d_gat.p, c.d_cls_of.p,
                                                            c.cls_ke.p, c.cls_me.p, c.d_E.p, c.d_rho.p, c.cM,
                                                            A.v64.p, A.v32.p, A.v32lo.p, mvals, slice_inst, dmax);
        ++c.launches;
        ASEND_CUDA(cudaGetLastError());
        ASEND_CUDA(cudaStreamSynchronize(c.stream));  // d_si
    } else {
        const double cM_save = c.cM;
        c.cM = cM_el;  // the shell / brickIM kernels read the context's coefficient
        if (c.type == 41) {
            shell_assemble(c, A.v64.p, mvals);  // FP64 element matrices at either precision
        } else if (c.type == 2) {
            beam_assemble(c, A.v64.p, mvals);  // FP64 element matrices at either precision
        } else if (c.type == 81) {
            brickim_assemble(c, A.v64.p, mvals);  // FP64 condensed element matrices at either precision
        } else if (precision == 64) {
            if (c.nn == 8) launch_colours<8, double>(c, A.v64.p, mvals, cM_el, X);
            else if (c.nn == 10) launch_colours<10, double>(c, A.v64.p, mvals, cM_el, X);
            else launch_colours<4, double>(c, A.v64.p, mvals, cM_el, X);
        } else {
            if (c.nn == 8) launch_colours<8, float>(c, A.v32.p, mvals, cM_el, X);
            else if (c.nn == 10) launch_colours<10, float>(c, A.v32.p, mvals, cM_el, X);
            else launch_colours<4, float>(c, A.v32.p, mvals, cM_el, X);
            widen_kernel<<<stream_grid(nval), 256, 0, c.stream>>>(nval, A.v32.p, A.v64.p);
            ++c.launches;
        }
        c.cM = cM_save;
        if (damp && !X.dvals) {  // mass-proportional damping only
            k_mass_damping<<<stream_grid(nval), 256, 0, c.stream>>>(nval, A.m64.p, c.ray_cm, c.cD, A.d64.p, A.v64.p);
            ++c.launches;
        }
        if (lump) {
            k_lump_mass<<<(A.n_rows + 127) / 128, 128, 0, c.stream>>>(A.n_rows, A.slice_off.p, A.row_len.p, A.diag.p,
                                                                      A.m64.p, A.v64.p, c.cM);
            ++c.launches;
        }
        // penalty scale over the element matrix (K [+ cM M]): one per
        // instance of a batched stack (each instance is its own model)
        if (ni > 1) {
            std::vector<int64_t> seg(ni + 1);
            for (int i = 0; i <= ni; ++i) {
                const int node = c.inst_node_ptr[i];
                const int s2 = std::min((node + kSlice - 1) / kSlice, A.n_slices);
                seg[i] = A.h_slice_off[s2] * 9 * kSlice;
            }
            DArr<int64_t> d_seg;
            d_seg.upload(seg, c.stream);
            max_abs_seg_kernel<<<dim3(64, ni), 256, 0, c.stream>>>(d_seg.p, A.v64.p, dmax);
            ASEND_CUDA(cudaStreamSynchronize(c.stream));  // d_seg
        } else {
            max_abs_kernel<<<stream_grid(nval), 256, 0, c.stream>>>(nval, A.v64.p, dmax);
        }
        ++c.launches;
    }
    std::vector<double> mx(ni);
    ASEND_CUDA(cudaMemcpyAsync(mx.data(), c.d_max_partial.p, sizeof(double) * ni, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    const int npen = (int)c.d_pen_idx.n;
    if (ni > 1) {
        c.sf_inst.resize(ni);
        c.sf = 0.0;
        for (int i = 0; i < ni; ++i) {
            c.sf_inst[i] = 100000.0 * mx[i];
            c.sf = std::max(c.sf, c.sf_inst[i]);
        }
        if (npen > 0) {
            std::vector<double> val(npen);
            for (int k = 0; k < npen; ++k)
                val[k] = c.sf_inst[instance_of_node(c, c.pen_dof[k] / c.dpn)] * c.pen_coef_host[k];
            c.d_pen_val.upload(val, c.stream);
            penalty_val_kernel<<<(npen + 255) / 256, 256, 0, c.stream>>>(npen, c.d_pen_idx.p, c.d_pen_val.p, A.v64.p);
            ++c.launches;
        }
    } else {
        c.sf_inst.clear();
        c.sf = 100000.0 * mx[0];
        if (npen > 0) {
            penalty_kernel<<<(npen + 255) / 256, 256, 0, c.stream>>>(npen, c.d_pen_idx.p, c.d_pen_coef.p, c.sf,
                                                                     A.v64.p);
            ++c.launches;
        }
    }
    const int nunit = (int)c.d_unit_idx.n;
    if (nunit > 0) {
        unit_kernel<<<(nunit + 255) / 256, 256, 0, c.stream>>>(nunit, c.d_unit_idx.p, A.v64.p);
        ++c.launches;
    }
    if (gather || split_only) {  // FP32 copies of the entries changed after the gather
        if (npen > 0)
            k_refresh32<<<(npen + 255) / 256, 256, 0, c.stream>>>(npen, c.d_pen_idx.p, A.v64.p, A.v32.p, A.v32lo.p);
        if (nunit > 0)
            k_refresh32<<<(nunit + 255) / 256, 256, 0, c.stream>>>(nunit, c.d_unit_idx.p, A.v64.p, A.v32.p,
                                                                   A.v32lo.p);
        c.launches += (npen > 0) + (nunit > 0);
    } else {
        round_kernel<<<stream_grid(nval), 256, 0, c.stream>>>(nval, A.v64.p, A.v32.p, A.v32lo.p);
        ++c.launches;
    }
    ASEND_CUDA(cudaGetLastError());
    ASEND_CUDA(cudaEventRecord(c.ev1, c.stream));
    ASEND_CUDA(cudaEventSynchronize(c.ev1));
    float ms = 0.f;
    ASEND_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.assembled_precision = precision;
    c.v64_valid = !split_only;
    ++c.assembly_epoch;
    c.last_assemble_ms = ms;
}

cudaError_t ensure_v64_rc(Ctx& c) {
    if (c.v64_valid) return cudaSuccess;
    const size_t nval = (size_t)c.A.n_groups * 9 * kSlice;
    k_pairs_to64<<<stream_grid(nval), 256, 0, c.stream>>>(nval, c.A.v32.p, c.A.v32lo.p, c.A.v64.p);
    ++c.launches;
    const cudaError_t rc = cudaGetLastError();
    if (rc == cudaSuccess) c.v64_valid = true;
    return rc;
}

void ensure_v64(Ctx& c) { ASEND_CUDA(ensure_v64_rc(c)); }

}  // namespace asend
