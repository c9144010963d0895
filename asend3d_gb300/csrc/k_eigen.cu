// k_eigen.cu -- modal analysis (frequency job): the lowest eigenpairs of
// (K + sf C^T C) x = lambda D x with D the row-sum diagonal mass.
//
// Reference (solverSrc/asend_run_job/src/):
//   Model::eigen_solve model_analysis.rs:711-880 (frequency branch):
//     D = row sums of the consistent mass (get_rum with unit acceleration,
//     :748-766), entries below 1e-6 mean|D| raised to it (:768-779);
//     A = K - tgt_eval D with the penalty terms (:783-789), factored by a
//     direct LDL^T (:790-795), then eigen_sparse_direct
//     (matrix_functions.rs:1099-1265): Lanczos on D^1/2 A^-1 D^1/2 with
//     5 n_modes vectors and local orthogonalisation; eigenvalue = 1/theta
//     + tgt_eval (:803-805); frequency sqrt(lambda) / (2 pi) (:874-879);
//     mode shapes D^-1/2 Q y at unit 2-norm.
//
// GB300 design: the same operator and shift-invert, with the inner solves
// done by this library's PCG or multigrid-preconditioned CG on the assembled
// SBELL operator instead of a direct factor, block Lanczos (block size
// 1..4 right-hand sides per solve; a block captures repeated eigenvalues,
// e.g. the two bending families of a symmetric section) with full
// reorthogonalisation (two classical Gram-Schmidt passes against the whole
// basis, so no spurious copies), and a stopping test on the Ritz residuals
// instead of a fixed basis size.  The basis lives in HBM as FP64 columns
// [m][n]; the Gram-Schmidt dots are column-parallel CTA reductions with a
// fixed-order second pass (bit-reproducible); the projected matrix is solved
// on the host.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"

namespace asend {
namespace {

constexpr int kEt = 256;

__global__ void __launch_bounds__(128)
k_mass_rowsum(int n_rows, const int64_t* __restrict__ slice_off, const uint8_t* __restrict__ row_len,
              const double* __restrict__ m64, double* __restrict__ D) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    const int lane = row & 31;
    const int64_t g0 = slice_off[row >> 5];
    const int len = row_len[row];
    double s[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < len; ++j) {
        const double* v = m64 + ((g0 + j) * 9) * 32 + lane;
#pragma unroll
        for (int r = 0; r < 3; ++r) s[r] += v[(3 * r) * 32] + v[(3 * r + 1) * 32] + v[(3 * r + 2) * 32];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) D[3 * (size_t)row + r] = s[r];
}

// Diagonal entries of the node-diagonal blocks: save (mode 0), add s (mode 1)
// or restore from the saved copy (mode 2); the FP32 copy follows the FP64 one.
__global__ void k_diag_entries(int n_rows, const int64_t* __restrict__ slice_off, const uint8_t* __restrict__ diag,
                               double* __restrict__ v64, float* __restrict__ v32, float* __restrict__ v32lo,
                               const double* __restrict__ s, double* __restrict__ saved, int mode) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    const int lane = row & 31;
    const int64_t g = slice_off[row >> 5] + diag[row];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const size_t idx = (size_t)(g * 9 + 4 * r) * 32 + lane;
        const size_t i = 3 * (size_t)row + r;
        if (mode == 0) {
            saved[i] = v64[idx];
        } else {
            const double v = (mode == 1) ? v64[idx] + s[i] : saved[i];
            v64[idx] = v;
            v32[idx] = (float)v;
            v32lo[idx] = (float)(v - (double)(float)v);
        }
    }
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    v = 0.0;
    if (w == 0) {
        v = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;
}

// part[j][bx] = sum over CTA bx's rows of Q_j . w  (grid: x row chunks, y columns)
__global__ void __launch_bounds__(kEt) k_basis_dots(int n, const double* __restrict__ Q, size_t ldq,
                                                    const double* __restrict__ w, double* __restrict__ part) {
    __shared__ double sh[kEt / 32];
    const int j = blockIdx.y;
    const double* q = Q + (size_t)j * ldq;
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * kEt + threadIdx.x; i < (size_t)n; i += (size_t)gridDim.x * kEt)
        acc += q[i] * w[i];
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) part[(size_t)j * gridDim.x + blockIdx.x] = acc;
}

// h[j] = sum_b part[j][b] in a fixed order (one CTA per column)
__global__ void __launch_bounds__(kEt) k_reduce_parts(int nb, const double* __restrict__ part,
                                                      double* __restrict__ h) {
    __shared__ double sh[kEt / 32];
    const int j = blockIdx.x;
    double acc = 0.0;
    for (int b = threadIdx.x; b < nb; b += kEt) acc += part[(size_t)j * nb + b];
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) h[j] = acc;
}

// w -= sum_j h[j] Q_j
__global__ void k_basis_axpy(int n, int m, const double* __restrict__ Q, size_t ldq, const double* __restrict__ h,
                             double* __restrict__ w) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n) return;
    double acc = w[i];
    for (int j = 0; j < m; ++j) acc -= h[j] * Q[(size_t)j * ldq + i];
    w[i] = acc;
}

// r = A x - lambda D x (in place in ax)
__global__ void k_eig_residual(int n, const double* __restrict__ D, const double* __restrict__ x, double lam,
                               double* __restrict__ ax) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n) return;
    ax[i] -= lam * D[i] * x[i];
}

// out = a * x (elementwise a[i] when a_vec, else the scalar s)
__global__ void k_scale(int n, const double* __restrict__ a_vec, double s, const double* x, double* out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n) return;
    out[i] = (a_vec ? a_vec[i] : s) * x[i];
}

// Seeded start / restart vector in [-1, 1): an integer hash of (i, seed).
__global__ void k_fill_hash(int n, uint32_t seed, double* __restrict__ x) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n) return;
    uint32_t h = (uint32_t)i * 0x9E3779B1u + seed * 0x85EBCA77u + 0x165667B1u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    x[i] = (double)h * (2.0 / 4294967296.0) - 1.0;
}

// X_k = sum_j S[j][k] Q_j for k < nk (S column-major per Ritz vector: S[k*m + j])
__global__ void k_basis_combine(int n, int m, int nk, const double* __restrict__ Q, size_t ldq,
                                const double* __restrict__ S, double* __restrict__ X) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n) return;
    for (int k = 0; k < nk; ++k) {
        double acc = 0.0;
        for (int j = 0; j < m; ++j) acc += S[(size_t)k * m + j] * Q[(size_t)j * ldq + i];
        X[(size_t)k * n + i] = acc;
    }
}

inline int egrid(size_t n) { return (int)((n + kEt - 1) / kEt); }

// Dense basis algebra on the stream, with the host copy of the coefficients.
struct Basis {
    Ctx& c;
    int n;
    size_t ldq;
    DArr<double> Q, part, h;
    int nb;  // CTAs per column in k_basis_dots
    Basis(Ctx& cc, int n_in, int cols) : c(cc), n(n_in), ldq((size_t)n_in) {
        Q.alloc((size_t)cols * ldq);
        nb = std::max(1, std::min(4 * 152, (n + kEt * 8 - 1) / (kEt * 8)));
        part.alloc((size_t)cols * nb);
        h.alloc(cols);
    }
    double* col(int j) { return Q.p + (size_t)j * ldq; }
    // h = Q[0..m)^T w on the device (and *host if given)
    void dots(const double* Qb, int m, const double* w, double* host) {
        k_basis_dots<<<dim3(nb, m), kEt, 0, c.stream>>>(n, Qb, ldq, w, part.p);
        k_reduce_parts<<<m, kEt, 0, c.stream>>>(nb, part.p, h.p);
        c.launches += 2;
        if (host) {
            ASEND_CUDA(cudaMemcpyAsync(host, h.p, sizeof(double) * m, cudaMemcpyDeviceToHost, c.stream));
            ASEND_CUDA(cudaStreamSynchronize(c.stream));
        }
    }
    double norm(const double* w) {
        double v = 0.0;
        dots(w, 1, w, &v);
        return std::sqrt(v);
    }
    // two classical Gram-Schmidt passes of w against columns [0, m); the
    // coefficients are added into coef[0..m)
    void orthogonalise(int m, double* w, double* coef) {
        if (m == 0) return;
        std::vector<double> hh(m);
        for (int pass = 0; pass < 2; ++pass) {
            dots(Q.p, m, w, hh.data());
            k_basis_axpy<<<egrid(n), kEt, 0, c.stream>>>(n, m, Q.p, ldq, h.p, w);
            ++c.launches;
            if (coef)
                for (int j = 0; j < m; ++j) coef[j] += hh[j];
        }
    }
    void scale(double s, const double* x, double* out) {
        k_scale<<<egrid(n), kEt, 0, c.stream>>>(n, nullptr, s, x, out);
        ++c.launches;
    }
};

}  // namespace

// Dense symmetric eigenproblem (row-major a, m x m): Householder reduction to
// tridiagonal form and implicit symmetric QR steps with Wilkinson shifts
// (Golub & Van Loan, Matrix Computations, Algorithms 8.3.1 and 8.3.3).
// Eigenvalues ascending in vals[m]; vecs[k*m + i] = component i of vector k.
// Returns 0, or -1 if the QR iteration did not converge.
int sym_eigen_dense(int m, const double* a_in, double* vals, double* vecs) {
    if (m <= 0) return 0;
    std::vector<double> a(a_in, a_in + (size_t)m * m), Z((size_t)m * m, 0.0), v(m), p(m), q(m);
    for (int i = 0; i < m; ++i) Z[(size_t)i * m + i] = 1.0;
    for (int k = 0; k + 2 < m; ++k) {
        double xn = 0.0;
        for (int i = k + 1; i < m; ++i) xn += a[(size_t)i * m + k] * a[(size_t)i * m + k];
        xn = std::sqrt(xn);
        if (xn == 0.0) continue;
        const double alpha = a[(size_t)(k + 1) * m + k] > 0.0 ? -xn : xn;
        double vn = 0.0;
        for (int i = k + 1; i < m; ++i) {
            v[i] = a[(size_t)i * m + k] - (i == k + 1 ? alpha : 0.0);
            vn += v[i] * v[i];
        }
        vn = std::sqrt(vn);
        if (vn == 0.0) continue;
        for (int i = k + 1; i < m; ++i) v[i] /= vn;
        double kk = 0.0;
        for (int i = k + 1; i < m; ++i) {
            double s = 0.0;
            for (int j = k + 1; j < m; ++j) s += a[(size_t)i * m + j] * v[j];
            p[i] = 2.0 * s;
            kk += v[i] * p[i];
        }
        for (int i = k + 1; i < m; ++i) q[i] = p[i] - kk * v[i];
        for (int i = k + 1; i < m; ++i)
            for (int j = k + 1; j < m; ++j) a[(size_t)i * m + j] -= v[i] * q[j] + q[i] * v[j];
        a[(size_t)(k + 1) * m + k] = a[(size_t)k * m + k + 1] = alpha;
        for (int i = k + 2; i < m; ++i) a[(size_t)i * m + k] = a[(size_t)k * m + i] = 0.0;
        for (int r = 0; r < m; ++r) {
            double s = 0.0;
            for (int j = k + 1; j < m; ++j) s += Z[(size_t)r * m + j] * v[j];
            s *= 2.0;
            for (int j = k + 1; j < m; ++j) Z[(size_t)r * m + j] -= s * v[j];
        }
    }
    std::vector<double> d(m), e(std::max(1, m - 1), 0.0);
    for (int i = 0; i < m; ++i) d[i] = a[(size_t)i * m + i];
    for (int i = 0; i + 1 < m; ++i) e[i] = a[(size_t)(i + 1) * m + i];
    const double eps = 2.220446049250313e-16;
    int hi = m - 1, steps = 0;
    const int max_steps = 60 * m + 60;
    while (hi > 0) {
        for (int i = 0; i < hi; ++i)
            if (std::fabs(e[i]) <= eps * (std::fabs(d[i]) + std::fabs(d[i + 1]))) e[i] = 0.0;
        if (e[hi - 1] == 0.0) {
            --hi;
            continue;
        }
        if (++steps > max_steps) return -1;
        int lo = hi - 1;
        while (lo > 0 && e[lo - 1] != 0.0) --lo;
        const double dd = 0.5 * (d[hi - 1] - d[hi]), b2 = e[hi - 1] * e[hi - 1];
        const double den = dd + std::copysign(std::sqrt(dd * dd + b2), dd);
        const double mu = den != 0.0 ? d[hi] - b2 / den : d[hi];
        double x = d[lo] - mu, z = e[lo];
        for (int k = lo; k < hi; ++k) {
            const double r = std::hypot(x, z);
            const double c = r != 0.0 ? x / r : 1.0, s = r != 0.0 ? z / r : 0.0;
            if (k > lo) e[k - 1] = r;
            const double ak = d[k], bk = e[k], ck = d[k + 1];
            d[k] = c * c * ak + 2.0 * c * s * bk + s * s * ck;
            d[k + 1] = s * s * ak - 2.0 * c * s * bk + c * c * ck;
            e[k] = c * s * (ck - ak) + (c * c - s * s) * bk;
            if (k + 1 < hi) {
                z = s * e[k + 1];
                e[k + 1] *= c;
            }
            x = e[k];
            for (int r2 = 0; r2 < m; ++r2) {
                const double zk = Z[(size_t)r2 * m + k], zk1 = Z[(size_t)r2 * m + k + 1];
                Z[(size_t)r2 * m + k] = c * zk + s * zk1;
                Z[(size_t)r2 * m + k + 1] = -s * zk + c * zk1;
            }
        }
    }
    std::vector<int> order(m);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int i, int j) { return d[i] < d[j]; });
    for (int k = 0; k < m; ++k) {
        vals[k] = d[order[k]];
        if (vecs)
            for (int i = 0; i < m; ++i) vecs[(size_t)k * m + i] = Z[(size_t)i * m + order[k]];
    }
    return 0;
}

int eigen_solve(Ctx& c, const asend_eigen_opts& eo, double* eig_out, double* freq_out, double* modes_out,
                double* diag_mass_out, asend_eigen_stats* st) {
    ensure_v64(c);
    const int n = c.n_dof, rows = c.A.n_rows;
    const int nm = eo.n_modes;
    const int b = eo.block_size > 0 ? eo.block_size : 2;
    if (nm < 1) throw InputError("n_modes must be positive");
    if (b > 4) throw InputError("block_size must be 1..4");
    // default cap: the reference's 5 n_modes vectors (at least n_modes + 20),
    // scaled with the block size so that larger blocks keep the Krylov degree
    int m_max = eo.max_subspace > 0 ? eo.max_subspace : std::max(5 * nm, nm + 20) * std::max(2, b) / 2;
    m_max = ((m_max + b - 1) / b) * b;
    if (m_max + b > n) m_max = ((n - b) / b) * b;
    if (m_max < nm) throw InputError("the model has too few DOF for that many modes");
    const double tol = eo.tol > 0.0 ? eo.tol : 1e-8;
    const double shift = eo.shift;
    if (!std::isfinite(shift)) throw InputError("shift must be finite");
    cudaEvent_t e0, e1;
    ASEND_CUDA(cudaEventCreate(&e0));
    ASEND_CUDA(cudaEventCreate(&e1));
    ASEND_CUDA(cudaEventRecord(e0, c.stream));
    // diagonal mass (row sums of M) with the reference's floor
    DArr<double> D, dh, dhinv;
    D.alloc(n);
    k_mass_rowsum<<<(rows + 127) / 128, 128, 0, c.stream>>>(rows, c.A.slice_off.p, c.A.row_len.p, c.A.m64.p, D.p);
    ++c.launches;
    std::vector<double> hD(n), hs(n), hsi(n);
    ASEND_CUDA(cudaMemcpyAsync(hD.data(), D.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    double avg = 0.0;
    for (int i = 0; i < n; ++i) avg += std::fabs(hD[i]);
    avg /= (double)n;
    const double dmin = 1e-6 * avg;
    for (int i = 0; i < n; ++i) {
        if (hD[i] < dmin) hD[i] = dmin;
        hs[i] = std::sqrt(hD[i]);
        hsi[i] = 1.0 / hs[i];
    }
    if (diag_mass_out) std::copy(hD.begin(), hD.end(), diag_mass_out);
    D.upload(hD, c.stream);
    dh.upload(hs, c.stream);
    dhinv.upload(hsi, c.stream);
    // A - shift D on the diagonal for the shift-invert solves
    DArr<double> saved, sD;
    if (shift != 0.0) {
        std::vector<double> s(n);
        for (int i = 0; i < n; ++i) s[i] = -shift * hD[i];
        sD.upload(s, c.stream);
        saved.alloc(n);
        k_diag_entries<<<(rows + 127) / 128, 128, 0, c.stream>>>(rows, c.A.slice_off.p, c.A.diag.p, c.A.v64.p,
                                                                c.A.v32.p, c.A.v32lo.p, nullptr, saved.p, 0);
        k_diag_entries<<<(rows + 127) / 128, 128, 0, c.stream>>>(rows, c.A.slice_off.p, c.A.diag.p, c.A.v64.p,
                                                                c.A.v32.p, c.A.v32lo.p, sD.p, saved.p, 1);
        c.launches += 2;
        ++c.assembly_epoch;  // preconditioners and multigrid levels follow the shifted values
    }
    struct Restore {  // puts the unshifted diagonal back, also on an exception
        Ctx& c;
        DArr<double>& saved;
        bool on;
        void run() {
            if (!on) return;
            on = false;
            const int rows = c.A.n_rows;
            k_diag_entries<<<(rows + 127) / 128, 128, 0, c.stream>>>(rows, c.A.slice_off.p, c.A.diag.p, c.A.v64.p,
                                                                    c.A.v32.p, c.A.v32lo.p, nullptr, saved.p, 2);
            ++c.launches;
            ++c.assembly_epoch;
        }
        ~Restore() { run(); }
    } restore{c, saved, shift != 0.0};

    const int cols = m_max + b;
    Basis B(c, n, cols);
    DArr<double> rhs, y;
    rhs.alloc((size_t)b * n);
    y.alloc((size_t)b * n);
    std::vector<double> H((size_t)cols * m_max, 0.0);  // H[i * m_max + j]: coefficient of q_i in Op q_j
    auto Hc = [&](int i, int j) -> double& { return H[(size_t)i * m_max + j]; };
    uint32_t seed = 1;
    // new basis vector from a seeded random direction, orthonormal to [0, q)
    auto random_column = [&](int q) {
        for (int attempt = 0; attempt < 4; ++attempt) {
            k_fill_hash<<<egrid(n), kEt, 0, c.stream>>>(n, seed++, B.col(q));
            ++c.launches;
            const double n0 = B.norm(B.col(q));
            B.orthogonalise(q, B.col(q), nullptr);
            const double n1 = B.norm(B.col(q));
            if (n1 > 1e-8 * n0) {
                B.scale(1.0 / n1, B.col(q), B.col(q));
                return;
            }
        }
        throw InputError("could not extend the Lanczos basis");
    };
    for (int k = 0; k < b; ++k) random_column(k);
    int q = b, m = 0, solves = 0, inner_capped = 0;
    long long inner_its = 0;
    std::vector<double> T, th, S, coef;
    std::vector<int> top;  // indices (into th) of the wanted Ritz values, best first
    std::vector<double> ritz_res;  // their relative Ritz residuals
    int n_conv = 0;
    while (m < m_max) {
        // W = D^1/2 A^-1 D^1/2 Q[m .. m+b)
        for (int k = 0; k < b; ++k) {
            k_scale<<<egrid(n), kEt, 0, c.stream>>>(n, dh.p, 0.0, B.col(m + k), rhs.p + (size_t)k * n);
            ++c.launches;
        }
        asend_solve_opts io = eo.inner;
        io.warm_start = 0;
        asend_solve_stats ps{};
        const int rc = pcg_solve(c, io, &ps, false, rhs.p, y.p, b);
        solves += b;
        inner_its += ps.iterations;
        if (rc == ASEND_NONFINITE) throw InputError("shift-invert solve turned non-finite (is A - shift D positive definite?)");
        if (rc == ASEND_MAX_ITER) ++inner_capped;  // recorded; the Ritz residuals decide
        for (int k = 0; k < b; ++k) {
            k_scale<<<egrid(n), kEt, 0, c.stream>>>(n, dh.p, 0.0, y.p + (size_t)k * n, y.p + (size_t)k * n);
            ++c.launches;
        }
        for (int k = 0; k < b; ++k) {
            const int j = m + k;
            double* w = y.p + (size_t)k * n;
            coef.assign(q, 0.0);
            const double n0 = B.norm(w);
            B.orthogonalise(q, w, coef.data());
            for (int i = 0; i < q; ++i) Hc(i, j) = coef[i];
            const double n1 = B.norm(w);
            if (q < cols) {
                if (n1 > 1e-10 * n0 && n1 > 0.0) {
                    B.scale(1.0 / n1, w, B.col(q));
                    Hc(q, j) = n1;
                } else {
                    random_column(q);  // invariant subspace or dependent block member
                }
                ++q;
            }
        }
        m += b;
        if (m < nm) continue;
        // Rayleigh-Ritz on the symmetric part of H[0..m, 0..m)
        T.assign((size_t)m * m, 0.0);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j) T[(size_t)i * m + j] = 0.5 * (Hc(i, j) + Hc(j, i));
        th.assign(m, 0.0);
        S.assign((size_t)m * m, 0.0);
        if (sym_eigen_dense(m, T.data(), th.data(), S.data()) != 0)
            throw InputError("projected eigenproblem did not converge");
        top.clear();
        ritz_res.clear();
        n_conv = 0;
        bool all = true;
        for (int k = m - 1; k >= 0 && (int)top.size() < nm; --k) {
            top.push_back(k);
            double r2 = 0.0;  // || H[m..q, 0..m) s_k ||
            for (int i = m; i < q; ++i) {
                double s = 0.0;
                for (int j = 0; j < m; ++j) s += Hc(i, j) * S[(size_t)k * m + j];
                r2 += s * s;
            }
            ritz_res.push_back(std::sqrt(r2) / std::fabs(th[k]));
            const bool conv = ritz_res.back() <= tol;
            n_conv += conv;
            all &= conv;
        }
        if (all) break;
    }
    // Ritz vectors x_k = D^-1/2 Q s_k at unit 2-norm; eigenvalues 1/theta + shift
    const int nk = (int)top.size();
    std::vector<double> Ssel((size_t)nk * m);
    for (int k = 0; k < nk; ++k)
        std::copy(S.begin() + (size_t)top[k] * m, S.begin() + (size_t)(top[k] + 1) * m, Ssel.begin() + (size_t)k * m);
    DArr<double> dS, X, AX;
    dS.upload(Ssel, c.stream);
    X.alloc((size_t)nk * n);
    k_basis_combine<<<egrid(n), kEt, 0, c.stream>>>(n, m, nk, B.Q.p, B.ldq, dS.p, X.p);
    ++c.launches;
    restore.run();
    AX.alloc(n);
    double max_res = 0.0;
    std::vector<double> lam(nk);
    for (int k = 0; k < nk; ++k) {
        double* x = X.p + (size_t)k * n;
        k_scale<<<egrid(n), kEt, 0, c.stream>>>(n, dhinv.p, 0.0, x, x);
        ++c.launches;
        const double nx = B.norm(x);
        B.scale(1.0 / nx, x, x);
        lam[k] = 1.0 / th[top[k]] + shift;
        // true residual ||A x - lambda D x|| / ||A x|| with the unshifted operator
        apply_operator_device(c, 64, x, AX.p);
        const double nax = B.norm(AX.p);
        k_eig_residual<<<egrid(n), kEt, 0, c.stream>>>(n, D.p, x, lam[k], AX.p);
        ++c.launches;
        const double nr = B.norm(AX.p);
        max_res = std::max(max_res, nax > 0.0 ? nr / nax : nr);
    }
    if (modes_out) {
        ASEND_CUDA(cudaMemcpyAsync(modes_out, X.p, sizeof(double) * (size_t)nk * n, cudaMemcpyDeviceToHost,
                                   c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        // sign: the largest-magnitude component of each mode is positive
        for (int k = 0; k < nk; ++k) {
            double* x = modes_out + (size_t)k * n;
            int im = 0;
            for (int i = 1; i < n; ++i)
                if (std::fabs(x[i]) > std::fabs(x[im])) im = i;
            if (x[im] < 0.0)
                for (int i = 0; i < n; ++i) x[i] = -x[i];
        }
    }
    for (int k = 0; k < nk; ++k) {
        if (eig_out) eig_out[k] = lam[k];
        if (freq_out) freq_out[k] = lam[k] >= 0.0 ? std::sqrt(lam[k]) / (2.0 * 3.14159265358979323846) : -1.0;
    }
    ASEND_CUDA(cudaEventRecord(e1, c.stream));
    ASEND_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    ASEND_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const int status = n_conv < nm ? ASEND_MAX_ITER : ASEND_OK;
    if (st) {
        st->n_found = nk;
        st->n_converged = n_conv;
        st->subspace = m;
        st->n_solves = solves;
        st->inner_iterations = inner_its;
        st->max_rel_residual = ritz_res.empty() ? 0.0 : *std::max_element(ritz_res.begin(), ritz_res.end());
        st->max_pencil_residual = max_res;
        st->ms = ms;
        st->status = status;
        st->inner_capped = inner_capped;
    }
    return status;
}

}  // namespace asend
