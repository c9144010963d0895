// k_learned.cu -- K6: learned nodal preconditioner blocks (BF16 MLP).
//
// No counterpart in the reference (its CG is preconditioned by block LDL^T
// factors, lower_tri_mat_meth.rs:15-241).  A 3-layer MLP (16 -> 64 -> 64 -> 8,
// ReLU, BF16 weights and activations, FP32 accumulation) maps per-node
// features -- the node's 3x3 diagonal stiffness block normalised by its trace,
// the log trace relative to the mesh mean, and the log-modulus statistics of
// the adjacent elements -- to a lower-triangular correction U of the
// block-Jacobi inverse:
//     M_n = C_n U_n U_n^T C_n^T,   C_n C_n^T = D_n^-1 (Cholesky),
//     U_n = [[e^t0, 0, 0], [t3, e^t1, 0], [t4, t5, e^t2]].
// M_n is SPD for any output and equals the block-Jacobi inverse at zero
// output, so the network only learns a correction and the plain method
// remains the fallback.
//
// Training (on the GPU, by these kernels) minimises, over residual samples r
// that the plain Jacobi PCG produces on fresh fields,
//     loss = sum_s || r_s - A M r_s ||^2 / || r_s ||^2,
// whose gradient with respect to block M_n is G_n = -2 sym((A e_s)_n r_{s,n}^T)
// / ||r_s||^2 with e_s = r_s - A M r_s (A symmetric).  Inference runs the
// forward pass on BF16 tensor cores (mma.sync m16n8k16, FP32 accumulate);
// the backward pass stages each 128-node tile in shared memory and forms the
// weight gradients as small FP32-accumulated products (SIMT); Adam updates
// FP32 master weights and refreshes the BF16 copies.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "common.cuh"

namespace asend {

constexpr int kF = 16, kH = 64, kO = 8;  // features (12 used), hidden, outputs (6 used)
constexpr int kNW1 = kH * kF, kNW2 = kH * kH, kNW3 = kO * kH;
constexpr int kNParam = kNW1 + kH + kNW2 + kH + kNW3 + kO;  // W1 b1 W2 b2 W3 b3

struct LearnedState {
    DArr<float> master, m1, m2, grad;  // FP32 parameters, Adam moments, gradient
    DArr<__nv_bfloat16> wbf;           // BF16 copy of the weights (W1, W2, W3, W2^T, W3^T)
    DArr<__nv_bfloat16> feat;          // [N][16]
    DArr<float> y, dy;                 // [N][8] outputs / output gradients
    DArr<float> cfac, gblk;            // [N][6] Cholesky of D^-1, [N][6] block gradient
    DArr<float> samples;               // [S][n_dof] residual samples (unit norm)
    DArr<float> z4, e4;                // work vectors (M r, r - A M r)
    DArr<int32_t> nel_ptr, nel;        // node -> adjacent elements
    DArr<float> gpart, binv;           // per-CTA gradient partials, training blocks
    DArr<double> part;
    int n_samples = 0, step = 0;
    int objective = ASEND_LEARN_BLOCK;  // loss the training minimises
    bool have_weights = false;
    int64_t feat_epoch = -1;
};

namespace {

constexpr int kLT = 128;
inline int lgrid(int n) { return (n + kLT - 1) / kLT; }

// parameter offsets
constexpr int oW1 = 0, ob1 = oW1 + kNW1, oW2 = ob1 + kH, ob2 = oW2 + kNW2, oW3 = ob2 + kH, ob3 = oW3 + kNW3;
// BF16 weight buffer offsets: W1 [64][16], W2 [64][64], W3 [8][64] (row-major [out][in])
constexpr int bW1 = 0, bW2 = bW1 + kNW1, bW3 = bW2 + kNW2, bEnd = bW3 + kNW3;

// ---------------------------------------------------------------------------
// features
// ---------------------------------------------------------------------------
__device__ __forceinline__ void diag_block(const int64_t* slice_off, const uint8_t* diag, const double* v64, int row,
                                           double (&m)[9]) {
    const int64_t g = slice_off[row >> 5] + diag[row];
    const int lane = row & 31;
#pragma unroll
    for (int q = 0; q < 9; ++q) m[q] = v64[(g * 9 + q) * 32 + lane];
}

__global__ void k_logtrace_sum(int n, const int64_t* slice_off, const uint8_t* diag, const double* v64,
                               double* part) {
    __shared__ double sm[32];
    double v[1] = {0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        double m[9];
        diag_block(slice_off, diag, v64, row, m);
        v[0] += log((m[0] + m[4] + m[8]) / 3.0);
    }
    block_sum<1>(v, sm);
    if (threadIdx.x == 0) atomicAdd(part, v[0]);
}

// features [N][16] (BF16) and the Cholesky factor of the inverse diagonal block
__global__ void k_features(int n, const int64_t* slice_off, const uint8_t* diag, const double* v64,
                           const int32_t* nel_ptr, const int32_t* nel, const double* E, double mean_logtr,
                           double mean_logE, __nv_bfloat16* feat, float* cfac) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    double m[9];
    diag_block(slice_off, diag, v64, row, m);
    const double tr = (m[0] + m[4] + m[8]) / 3.0;
    float f[kF];
    f[0] = (float)(m[0] / tr);
    f[1] = (float)(m[4] / tr);
    f[2] = (float)(m[8] / tr);
    f[3] = (float)(m[1] / tr);
    f[4] = (float)(m[2] / tr);
    f[5] = (float)(m[5] / tr);
    f[6] = (float)(0.1 * (log(tr) - mean_logtr));
    double s = 0.0, s2 = 0.0, lo = 1e300, hi = -1e300;
    const int b = nel_ptr[row], e = nel_ptr[row + 1];
    for (int k = b; k < e; ++k) {
        const double le = log(E[nel[k]]) - mean_logE;
        s += le;
        s2 += le * le;
        lo = fmin(lo, le);
        hi = fmax(hi, le);
    }
    const int cnt = e - b;
    const double mean = cnt ? s / cnt : 0.0;
    f[7] = (float)mean;
    f[8] = (float)(cnt ? sqrt(fmax(s2 / cnt - mean * mean, 0.0)) : 0.0);
    f[9] = (float)(cnt ? hi - lo : 0.0);
    f[10] = (float)cnt / 8.f;
    // penalty-dominated node (a constrained DOF makes the diagonal very large)
    const double mx = fmax(m[0], fmax(m[4], m[8])), mn = fmin(m[0], fmin(m[4], m[8]));
    f[11] = (mx > 1e3 * mn) ? 1.f : 0.f;
    for (int q = 12; q < kF; ++q) f[q] = 0.f;
#pragma unroll
    for (int q = 0; q < kF; ++q) feat[(size_t)row * kF + q] = __float2bfloat16(f[q]);
    // D^-1 (cofactors) and its Cholesky factor C (lower): stored c00 c10 c11 c20 c21 c22
    const double c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8], c02 = m[3] * m[7] - m[4] * m[6];
    const double id = 1.0 / (m[0] * c00 + m[1] * c01 + m[2] * c02);
    const double i00 = c00 * id, i01 = (m[2] * m[7] - m[1] * m[8]) * id, i02 = (m[1] * m[5] - m[2] * m[4]) * id;
    const double i11 = (m[0] * m[8] - m[2] * m[6]) * id, i12 = (m[2] * m[3] - m[0] * m[5]) * id;
    const double i22 = (m[0] * m[4] - m[1] * m[3]) * id;
    const double l00 = sqrt(i00);
    const double l10 = i01 / l00, l20 = i02 / l00;
    const double l11 = sqrt(fmax(i11 - l10 * l10, 1e-300));
    const double l21 = (i12 - l20 * l10) / l11;
    const double l22 = sqrt(fmax(i22 - l20 * l20 - l21 * l21, 1e-300));
    float* C = cfac + 6 * (size_t)row;
    C[0] = (float)l00;
    C[1] = (float)l10;
    C[2] = (float)l11;
    C[3] = (float)l20;
    C[4] = (float)l21;
    C[5] = (float)l22;
}

// ---------------------------------------------------------------------------
// MLP forward on tensor cores: one warp = 16 nodes; mma.sync m16n8k16 BF16,
// FP32 accumulate.  C-fragments of one layer become the next layer's
// A-fragments in registers (the m16n8 C layout matches the m16k16 A layout
// pairwise), so activations never leave the SM.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
// B fragment (k16 x n8, "col"): element (k, n) = W[n0 + n][k0 + k] of a row-major
// [out][in] weight matrix with leading dimension ld.
__device__ __forceinline__ void load_b(const __nv_bfloat16* W, int ld, int n0, int k0, int lane, uint32_t& b0,
                                       uint32_t& b1) {
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* row = W + (size_t)(n0 + g) * ld + k0 + 2 * t;
    b0 = *reinterpret_cast<const uint32_t*>(row);
    b1 = *reinterpret_cast<const uint32_t*>(row + 8);
}

__global__ void __launch_bounds__(128) k_mlp_forward(int n, const __nv_bfloat16* __restrict__ feat,
                                                     const __nv_bfloat16* __restrict__ wbf,
                                                     const float* __restrict__ params, float* __restrict__ y) {
    __shared__ __align__(16) __nv_bfloat16 sw[bEnd];  // W1, W2, W3
    __shared__ float sb[kH + kH + kO];
    for (int q = threadIdx.x; q < bEnd; q += blockDim.x) sw[q] = wbf[q];
    for (int q = threadIdx.x; q < kH; q += blockDim.x) {
        sb[q] = params[ob1 + q];
        sb[kH + q] = params[ob2 + q];
    }
    if (threadIdx.x < kO) sb[2 * kH + threadIdx.x] = params[ob3 + threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int tiles = (n + 15) / 16;
    for (int tile = blockIdx.x * 4 + warp; tile < tiles; tile += gridDim.x * 4) {
        const int r0 = tile * 16 + g, r1 = r0 + 8;
        // A fragment of X (16 x 16)
        uint32_t a[4];
        auto ld2 = [&](int r, int c) -> uint32_t {
            if (r >= n) return 0u;
            return *reinterpret_cast<const uint32_t*>(feat + (size_t)r * kF + c);
        };
        a[0] = ld2(r0, 2 * t);
        a[1] = ld2(r1, 2 * t);
        a[2] = ld2(r0, 2 * t + 8);
        a[3] = ld2(r1, 2 * t + 8);
        // layer 1: 8 n-tiles of 8 hidden units
        float h[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float bj0 = sb[8 * j + 2 * t], bj1 = sb[8 * j + 2 * t + 1];
            h[j][0] = bj0; h[j][1] = bj1; h[j][2] = bj0; h[j][3] = bj1;
            uint32_t b0, b1;
            load_b(sw + bW1, kF, 8 * j, 0, lane, b0, b1);
            mma_bf16(h[j], a, b0, b1);
        }
        // layer 2
        uint32_t ah[4][4];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            ah[kk][0] = pack_bf16(fmaxf(h[2 * kk][0], 0.f), fmaxf(h[2 * kk][1], 0.f));
            ah[kk][1] = pack_bf16(fmaxf(h[2 * kk][2], 0.f), fmaxf(h[2 * kk][3], 0.f));
            ah[kk][2] = pack_bf16(fmaxf(h[2 * kk + 1][0], 0.f), fmaxf(h[2 * kk + 1][1], 0.f));
            ah[kk][3] = pack_bf16(fmaxf(h[2 * kk + 1][2], 0.f), fmaxf(h[2 * kk + 1][3], 0.f));
        }
        float h2[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float bj0 = sb[kH + 8 * j + 2 * t], bj1 = sb[kH + 8 * j + 2 * t + 1];
            h2[j][0] = bj0; h2[j][1] = bj1; h2[j][2] = bj0; h2[j][3] = bj1;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                uint32_t b0, b1;
                load_b(sw + bW2, kH, 8 * j, 16 * kk, lane, b0, b1);
                mma_bf16(h2[j], ah[kk], b0, b1);
            }
        }
        // layer 3 (8 outputs)
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            ah[kk][0] = pack_bf16(fmaxf(h2[2 * kk][0], 0.f), fmaxf(h2[2 * kk][1], 0.f));
            ah[kk][1] = pack_bf16(fmaxf(h2[2 * kk][2], 0.f), fmaxf(h2[2 * kk][3], 0.f));
            ah[kk][2] = pack_bf16(fmaxf(h2[2 * kk + 1][0], 0.f), fmaxf(h2[2 * kk + 1][1], 0.f));
            ah[kk][3] = pack_bf16(fmaxf(h2[2 * kk + 1][2], 0.f), fmaxf(h2[2 * kk + 1][3], 0.f));
        }
        float o[4] = {sb[2 * kH + 2 * t], sb[2 * kH + 2 * t + 1], sb[2 * kH + 2 * t], sb[2 * kH + 2 * t + 1]};
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            uint32_t b0, b1;
            load_b(sw + bW3, kH, 0, 16 * kk, lane, b0, b1);
            mma_bf16(o, ah[kk], b0, b1);
        }
        if (r0 < n) {
            y[(size_t)r0 * kO + 2 * t] = o[0];
            y[(size_t)r0 * kO + 2 * t + 1] = o[1];
        }
        if (r1 < n) {
            y[(size_t)r1 * kO + 2 * t] = o[2];
            y[(size_t)r1 * kO + 2 * t + 1] = o[3];
        }
    }
}

// ---------------------------------------------------------------------------
// blocks M = C U U^T C^T from the outputs, and their backward
// ---------------------------------------------------------------------------
__device__ __forceinline__ void make_u(const float* yo, float (&U)[3][3]) {
    U[0][0] = __expf(yo[0]); U[0][1] = 0.f; U[0][2] = 0.f;
    U[1][0] = yo[3]; U[1][1] = __expf(yo[1]); U[1][2] = 0.f;
    U[2][0] = yo[4]; U[2][1] = yo[5]; U[2][2] = __expf(yo[2]);
}
__device__ __forceinline__ void make_c(const float* C6, float (&C)[3][3]) {
    C[0][0] = C6[0]; C[0][1] = 0.f; C[0][2] = 0.f;
    C[1][0] = C6[1]; C[1][1] = C6[2]; C[1][2] = 0.f;
    C[2][0] = C6[3]; C[2][1] = C6[4]; C[2][2] = C6[5];
}

__global__ void k_make_blocks(int n, const float* __restrict__ y, const float* __restrict__ cfac, float* __restrict__ binv,
                              int use_net) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    float U[3][3], C[3][3], L[3][3];
    const float zero[kO] = {0, 0, 0, 0, 0, 0, 0, 0};
    make_u(use_net ? y + (size_t)row * kO : zero, U);
    make_c(cfac + 6 * (size_t)row, C);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            float s = 0.f;
            for (int k = 0; k < 3; ++k) s += C[i][k] * U[k][j];
            L[i][j] = s;
        }
    float* B = binv + 9 * (size_t)row;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            float s = 0.f;
            for (int k = 0; k < 3; ++k) s += L[i][k] * L[j][k];
            B[3 * i + j] = s;
        }
}

// dL/dy from the block gradient G (symmetric, stored g00 g11 g22 g01 g02 g12),
// times scale: dL/dU = 2 C^T G C U; dy_diag = (dL/dU)_ii e^{t_i}; dy_off = (dL/dU)_ij.
__global__ void k_block_backward(int n, const float* __restrict__ y, const float* __restrict__ cfac,
                                 const float* __restrict__ gblk, float scale, float* __restrict__ dy) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    float U[3][3], C[3][3], G[3][3];
    make_u(y + (size_t)row * kO, U);
    make_c(cfac + 6 * (size_t)row, C);
    const float* g6 = gblk + 6 * (size_t)row;
    G[0][0] = g6[0]; G[1][1] = g6[1]; G[2][2] = g6[2];
    G[0][1] = G[1][0] = g6[3];
    G[0][2] = G[2][0] = g6[4];
    G[1][2] = G[2][1] = g6[5];
    float T1[3][3], T2[3][3], D[3][3];
    for (int i = 0; i < 3; ++i)  // T1 = G C
        for (int j = 0; j < 3; ++j) {
            float s = 0.f;
            for (int k = 0; k < 3; ++k) s += G[i][k] * C[k][j];
            T1[i][j] = s;
        }
    for (int i = 0; i < 3; ++i)  // T2 = C^T T1
        for (int j = 0; j < 3; ++j) {
            float s = 0.f;
            for (int k = 0; k < 3; ++k) s += C[k][i] * T1[k][j];
            T2[i][j] = s;
        }
    for (int i = 0; i < 3; ++i)  // D = 2 T2 U
        for (int j = 0; j < 3; ++j) {
            float s = 0.f;
            for (int k = 0; k < 3; ++k) s += T2[i][k] * U[k][j];
            D[i][j] = 2.f * scale * s;
        }
    float* d = dy + (size_t)row * kO;
    d[0] = D[0][0] * U[0][0];
    d[1] = D[1][1] * U[1][1];
    d[2] = D[2][2] * U[2][2];
    d[3] = D[1][0];
    d[4] = D[2][0];
    d[5] = D[2][1];
    d[6] = 0.f;
    d[7] = 0.f;
}

// ---------------------------------------------------------------------------
// loss and block gradient over residual samples (FP32 SBELL products)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sb_row_f(const int64_t* slice_off, const uint8_t* row_len, const int32_t* col,
                                         const float* v, int row, const float* __restrict__ x, float (&y)[3]) {
    y[0] = y[1] = y[2] = 0.f;
    const int lane = row & 31;
    const int64_t g0 = slice_off[row >> 5];
    const int len = row_len[row];
    for (int j = 0; j < len; ++j) {
        const int64_t g = g0 + j;
        const int c = col[g * 32 + lane];
        const float* vv = v + (g * 9) * 32 + lane;
        const float x0 = x[3 * (size_t)c], x1 = x[3 * (size_t)c + 1], x2 = x[3 * (size_t)c + 2];
#pragma unroll
        for (int a = 0; a < 3; ++a) y[a] = fmaf(vv[(a * 3) * 32], x0, fmaf(vv[(a * 3 + 1) * 32], x1, fmaf(vv[(a * 3 + 2) * 32], x2, y[a])));
    }
}

__global__ void k_apply_blocks(int n, const float* __restrict__ binv, const float* __restrict__ r, float* __restrict__ z) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    const float* B = binv + 9 * (size_t)row;
    const float r0 = r[3 * row], r1 = r[3 * row + 1], r2 = r[3 * row + 2];
    z[3 * row] = B[0] * r0 + B[1] * r1 + B[2] * r2;
    z[3 * row + 1] = B[3] * r0 + B[4] * r1 + B[5] * r2;
    z[3 * row + 2] = B[6] * r0 + B[7] * r1 + B[8] * r2;
}

// e = r - A z, accumulates sum e.e into *loss
__global__ void __launch_bounds__(kLT) k_residual_e(int n, const int64_t* slice_off, const uint8_t* row_len,
                                                    const int32_t* col, const float* v, const float* __restrict__ r,
                                                    const float* __restrict__ z, float* __restrict__ e, double* loss) {
    __shared__ double sm[32];
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[1] = {0.0};
    if (row < n) {
        float y[3];
        sb_row_f(slice_off, row_len, col, v, row, z, y);
        for (int a = 0; a < 3; ++a) {
            const float ev = r[3 * row + a] - y[a];
            e[3 * row + a] = ev;
            acc[0] += (double)ev * ev;
        }
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) atomicAdd(loss, acc[0]);
}

// q = A e; G_n += -2 sym(q_n r_n^T)
__global__ void __launch_bounds__(kLT) k_block_grad(int n, const int64_t* slice_off, const uint8_t* row_len,
                                                    const int32_t* col, const float* v, const float* __restrict__ e,
                                                    const float* __restrict__ r, float* __restrict__ gblk) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    float q[3];
    sb_row_f(slice_off, row_len, col, v, row, e, q);
    const float r0 = r[3 * row], r1 = r[3 * row + 1], r2 = r[3 * row + 2];
    float* G = gblk + 6 * (size_t)row;
    G[0] += -2.f * q[0] * r0;
    G[1] += -2.f * q[1] * r1;
    G[2] += -2.f * q[2] * r2;
    G[3] += -(q[0] * r1 + q[1] * r0);
    G[4] += -(q[0] * r2 + q[2] * r0);
    G[5] += -(q[1] * r2 + q[2] * r1);
}

// ---------------------------------------------------------------------------
// MLP backward (SIMT).  Each CTA walks 128-node tiles; per tile the node
// activations are recomputed in FP32 from the BF16 weights (one thread per
// node), kept in padded shared rows, and the weight gradients are summed over
// the tile's nodes into per-thread register partials (thread t owns
// parameters t, t+128, ...).  Partials go to part[cta][param]; k_grad_reduce
// adds them in CTA order, so the gradient is deterministic.
// ---------------------------------------------------------------------------
constexpr int kBT = 128;                       // nodes per tile = threads per CTA
constexpr int kPad = kH + 1;                   // padded row (floats)
constexpr size_t kBwdSmem =
    sizeof(float) * ((size_t)kBT * (17 + 4 * kPad + 9) + (kNW1 + kNW2 + kNW3) + 2 * kH + kO + kNParam);
static_assert(kBwdSmem <= 227 * 1024, "backward tile exceeds the shared-memory limit");

__global__ void __launch_bounds__(kBT) k_mlp_backward(int n, const __nv_bfloat16* __restrict__ feat,
                                                      const __nv_bfloat16* __restrict__ wbf,
                                                      const float* __restrict__ params, const float* __restrict__ dy,
                                                      float* __restrict__ part) {
    extern __shared__ float smem[];
    float* sx = smem;                    // [kBT][17]
    float* sa1 = sx + kBT * 17;          // [kBT][kPad]  bf16-rounded relu(h1)
    float* sa2 = sa1 + kBT * kPad;       // [kBT][kPad]  bf16-rounded relu(h2)
    float* sd2 = sa2 + kBT * kPad;       // [kBT][kPad]  dL/dh2
    float* sd1 = sd2 + kBT * kPad;       // [kBT][kPad]  dL/dh1
    float* sdy = sd1 + kBT * kPad;       // [kBT][9]
    float* sw = sdy + kBT * 9;           // W1 W2 W3 (float copies of the BF16 weights)
    float* sb = sw + kNW1 + kNW2 + kNW3; // b1 b2 b3
    float* sacc = sb + 2 * kH + kO;      // [kNParam] this CTA's gradient sums; entry q belongs to thread q % kBT
    const int t = threadIdx.x;
    for (int q = t; q < kNW1 + kNW2 + kNW3; q += kBT) sw[q] = __bfloat162float(wbf[q]);
    for (int q = t; q < kH; q += kBT) {
        sb[q] = params[ob1 + q];
        sb[kH + q] = params[ob2 + q];
    }
    if (t < kO) sb[2 * kH + t] = params[ob3 + t];
    const float* W1 = sw;
    const float* W2 = sw + kNW1;
    const float* W3 = sw + kNW1 + kNW2;
    for (int q = t; q < kNParam; q += kBT) sacc[q] = 0.f;
    const int tiles = (n + kBT - 1) / kBT;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        __syncthreads();  // previous tile's gradient sums are done with the rows
        const int node = tile * kBT + t;
        const bool valid = node < n;
        float x[kF];
#pragma unroll
        for (int k = 0; k < kF; ++k) x[k] = valid ? __bfloat162float(feat[(size_t)node * kF + k]) : 0.f;
#pragma unroll
        for (int k = 0; k < kF; ++k) sx[t * 17 + k] = x[k];
        float g[kO];
#pragma unroll
        for (int o = 0; o < kO; ++o) {
            g[o] = valid ? dy[(size_t)node * kO + o] : 0.f;
            sdy[t * 9 + o] = g[o];
        }
        float* a1 = sa1 + t * kPad;
        float* a2 = sa2 + t * kPad;
        float* d2 = sd2 + t * kPad;
        float* d1 = sd1 + t * kPad;
        for (int j = 0; j < kH; ++j) {
            float s = sb[j];
#pragma unroll
            for (int k = 0; k < kF; ++k) s = fmaf(W1[j * kF + k], x[k], s);
            a1[j] = __bfloat162float(__float2bfloat16(fmaxf(s, 0.f)));
        }
        for (int j = 0; j < kH; ++j) {
            float s = sb[kH + j];
            for (int k = 0; k < kH; ++k) s = fmaf(W2[j * kH + k], a1[k], s);
            a2[j] = __bfloat162float(__float2bfloat16(fmaxf(s, 0.f)));
        }
        for (int j = 0; j < kH; ++j) {
            float s = 0.f;
#pragma unroll
            for (int o = 0; o < kO; ++o) s = fmaf(W3[o * kH + j], g[o], s);
            d2[j] = a2[j] > 0.f ? s : 0.f;
        }
        for (int j = 0; j < kH; ++j) {
            float s = 0.f;
            for (int k = 0; k < kH; ++k) s = fmaf(W2[k * kH + j], d2[k], s);
            d1[j] = a1[j] > 0.f ? s : 0.f;
        }
        __syncthreads();
        // Kept rolled: fully unrolled over the 46 parameters a thread owns, the 128-row sums
        // below made the compiler's optimiser run for minutes.
#pragma unroll 1
        for (int q = t; q < kNParam; q += kBT) {
            const float* lhs;  // per-node factor (stride ls), rhs per-node factor (stride rs)
            const float* rhs = nullptr;
            int ls, rs = 0;
            if (q < ob1) {
                lhs = sd1 + q / kF; ls = kPad; rhs = sx + q % kF; rs = 17;
            } else if (q < oW2) {
                lhs = sd1 + (q - ob1); ls = kPad;
            } else if (q < ob2) {
                const int w = q - oW2;
                lhs = sd2 + w / kH; ls = kPad; rhs = sa1 + w % kH; rs = kPad;
            } else if (q < oW3) {
                lhs = sd2 + (q - ob2); ls = kPad;
            } else if (q < ob3) {
                const int w = q - oW3;
                lhs = sdy + w / kH; ls = 9; rhs = sa2 + w % kH; rs = kPad;
            } else {
                lhs = sdy + (q - ob3); ls = 9;
            }
            float s = 0.f;
            if (rhs) {
                for (int r = 0; r < kBT; ++r) s = fmaf(lhs[r * ls], rhs[r * rs], s);
            } else {
                for (int r = 0; r < kBT; ++r) s += lhs[r * ls];
            }
            sacc[q] += s;
        }
    }
    for (int q = t; q < kNParam; q += kBT) part[(size_t)blockIdx.x * kNParam + q] = sacc[q];
}

__global__ void k_grad_reduce(int n_part, const float* __restrict__ part, float* __restrict__ grad) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= kNParam) return;
    float s = 0.f;
    for (int b = 0; b < n_part; ++b) s += part[(size_t)b * kNParam + q];
    grad[q] = s;
}

// Adam on FP32 master weights; refresh the BF16 copies (W1, W2, W3, W2^T, W3^T)
__global__ void k_adam(int np, float* __restrict__ w, float* __restrict__ m1, float* __restrict__ m2,
                       const float* __restrict__ g, float lr, float b1, float b2, float eps, float c1, float c2,
                       float gscale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float gi = g[i] * gscale;
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    w[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}
__global__ void k_refresh_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ wbf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kNW1) wbf[bW1 + i] = __float2bfloat16(w[oW1 + i]);
    if (i < kNW2) wbf[bW2 + i] = __float2bfloat16(w[oW2 + i]);
    if (i < kNW3) wbf[bW3 + i] = __float2bfloat16(w[oW3 + i]);
}

LearnedState& state(Ctx& c) {
    if (!c.learned) c.learned = std::make_shared<LearnedState>();
    return *c.learned;
}

void ensure_buffers(Ctx& c) {
    LearnedState& L = state(c);
    const int n = c.n_nodes;
    if (L.feat.n != (size_t)n * kF) {
        L.feat.alloc((size_t)n * kF);
        L.y.alloc((size_t)n * kO);
        L.dy.alloc((size_t)n * kO);
        L.cfac.alloc((size_t)n * 6);
        L.gblk.alloc((size_t)n * 6);
        L.z4.alloc(c.n_dof);
        L.e4.alloc(c.n_dof);
        L.feat_epoch = -1;
        // node -> adjacent elements
        std::vector<int32_t> ptr(n + 1, 0), el;
        for (size_t k = 0; k < c.conn.size(); ++k) ptr[c.conn[k] + 1]++;
        for (int i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
        el.resize(ptr[n]);
        std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
        for (int e = 0; e < c.n_el; ++e)
            for (int a = 0; a < c.nn; ++a) el[fill[c.conn[(size_t)e * c.nn + a]]++] = e;
        L.nel_ptr.upload(ptr, c.stream);
        L.nel.upload(el, c.stream);
    }
    if (!L.master.n) {
        L.master.alloc(kNParam);
        L.m1.alloc(kNParam);
        L.m2.alloc(kNParam);
        L.grad.alloc(kNParam);
        L.wbf.alloc(bEnd);
        L.part.alloc(1);
    }
}

void require_weights(const LearnedState& L) {
    if (!L.have_weights) throw InputError("no learned weights (init, train or set them first)");
}

void launch_forward(Ctx& c, int n, const __nv_bfloat16* feat, float* y) {
    LearnedState& L = state(c);
    const int warps = (n + 15) / 16;
    k_mlp_forward<<<std::max(1, std::min((warps + 3) / 4, 152 * 8)), 128, 0, c.stream>>>(n, feat, L.wbf.p, L.master.p, y);
    ++c.launches;
}

// parameter gradient (sum over nodes) of dy into L.grad
void launch_backward(Ctx& c, int n, const __nv_bfloat16* feat, const float* dy) {
    LearnedState& L = state(c);
    static bool attr_set = false;
    if (!attr_set) {
        ASEND_CUDA(cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem));
        attr_set = true;
    }
    const int tiles = (n + kBT - 1) / kBT;
    const int ctas = std::max(1, std::min(tiles, 152 * 2));
    if (L.gpart.n < (size_t)ctas * kNParam) L.gpart.alloc((size_t)ctas * kNParam);
    k_mlp_backward<<<ctas, kBT, kBwdSmem, c.stream>>>(n, feat, L.wbf.p, L.master.p, dy, L.gpart.p);
    k_grad_reduce<<<(kNParam + 255) / 256, 256, 0, c.stream>>>(ctas, L.gpart.p, L.grad.p);
    c.launches += 2;
}

void refresh(Ctx& c) {
    LearnedState& L = state(c);
    k_refresh_bf16<<<(kNW2 + 255) / 256, 256, 0, c.stream>>>(L.master.p, L.wbf.p);
    ++c.launches;
}

}  // namespace

bool learned_ready(const Ctx& c) { return c.learned && c.learned->have_weights; }

// a new mesh keeps the weights and drops the per-mesh buffers and samples
void learned_mesh_changed(Ctx& c) {
    if (!c.learned) return;
    LearnedState& L = *c.learned;
    L.feat.release();
    L.samples.release();
    L.n_samples = 0;
    L.feat_epoch = -1;
}

void learned_init(Ctx& c, uint64_t seed) {
    ensure_buffers(c);
    LearnedState& L = state(c);
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::vector<float> w(kNParam, 0.f);
    for (int i = 0; i < kNW1; ++i) w[oW1 + i] = nd(rng) * std::sqrt(2.f / 12.f);
    for (int i = 0; i < kNW2; ++i) w[oW2 + i] = nd(rng) * std::sqrt(2.f / kH);
    for (int i = 0; i < kNW3; ++i) w[oW3 + i] = nd(rng) * 1e-3f;  // start at block Jacobi
    L.master.upload(w, c.stream);
    L.m1.zero(c.stream);
    L.m2.zero(c.stream);
    refresh(c);
    L.step = 0;
    L.have_weights = true;
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
}

void learned_set_params(Ctx& c, const float* params) {
    ensure_buffers(c);
    LearnedState& L = state(c);
    L.master.upload(params, kNParam, c.stream);
    L.m1.zero(c.stream);
    L.m2.zero(c.stream);
    L.step = 0;
    refresh(c);
    L.have_weights = true;
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
}

void learned_get_params(Ctx& c, float* params) {
    LearnedState& L = state(c);
    require_weights(L);
    ASEND_CUDA(cudaMemcpyAsync(params, L.master.p, sizeof(float) * kNParam, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
}

int learned_n_params() { return kNParam; }

void learned_set_objective(Ctx& c, int kind) {
    if (kind != ASEND_LEARN_BLOCK && kind != ASEND_LEARN_MG) throw InputError("unknown learning objective");
    if (kind == ASEND_LEARN_MG && ((c.type != 8 && c.type != 81) || c.bx <= 0))
        throw InputError("the multigrid objective needs a structured hex8 block");
    state(c).objective = kind;
}
int learned_n_features() { return kF; }
int learned_n_outputs() { return kO; }

// features for the current assembly
void learned_features(Ctx& c) {
    ensure_v64(c);
    ensure_buffers(c);
    LearnedState& L = state(c);
    if (L.feat_epoch == c.assembly_epoch) return;
    const int n = c.n_nodes;
    double mean_logE = 0.0;
    for (double e : c.E) mean_logE += std::log(e);
    mean_logE /= std::max<size_t>(1, c.E.size());
    L.part.zero(c.stream);
    k_logtrace_sum<<<256, 256, 0, c.stream>>>(n, c.A.slice_off.p, c.A.diag.p, c.A.v64.p, L.part.p);
    double s = 0.0;
    ASEND_CUDA(cudaMemcpyAsync(&s, L.part.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    k_features<<<lgrid(n), kLT, 0, c.stream>>>(n, c.A.slice_off.p, c.A.diag.p, c.A.v64.p, L.nel_ptr.p, L.nel.p,
                                               c.d_E.p, s / n, mean_logE, L.feat.p, L.cfac.p);
    c.launches += 2;
    L.feat_epoch = c.assembly_epoch;
}

// nodal blocks M_n (FP32, row-major 3x3) from the network, or the plain
// block-Jacobi inverse when use_net is false
void learned_blocks(Ctx& c, float* d_binv, bool use_net) {
    learned_features(c);
    LearnedState& L = state(c);
    const int n = c.n_nodes;
    if (use_net) {
        require_weights(L);
        launch_forward(c, n, L.feat.p, L.y.p);
    }
    k_make_blocks<<<lgrid(n), kLT, 0, c.stream>>>(n, L.y.p, L.cfac.p, d_binv, use_net ? 1 : 0);
    ++c.launches;
    ASEND_CUDA(cudaGetLastError());
}

// Residual samples: sample s is the FP64 residual of the plain method
// (Jacobi PCG on load case 0) after iters[s] > 0 iterations; for iters[s] == 0
// a seeded standard normal vector; for iters[s] < 0 the residual after
// -iters[s] stationary V-cycle iterations from a seeded normal vector (with
// the learned finest-level smoother when the multigrid objective is selected
// and weights exist).  Each is scaled to unit norm.
void learned_add_samples(Ctx& c, int n_samples, const int32_t* iters, bool append, uint64_t seed) {
    if (n_samples <= 0) throw InputError("n_samples must be positive");
    if (!c.assembled) throw InputError("assemble first");
    ensure_buffers(c);
    LearnedState& L = state(c);
    const int nd = c.n_dof;
    const int first = append ? L.n_samples : 0;
    const int total = first + n_samples;
    if (L.samples.n < (size_t)total * nd) {
        DArr<float> bigger;
        bigger.alloc((size_t)total * nd);
        if (first)
            ASEND_CUDA(cudaMemcpyAsync(bigger.p, L.samples.p, sizeof(float) * (size_t)first * nd,
                                       cudaMemcpyDeviceToDevice, c.stream));
        std::swap(bigger.p, L.samples.p);
        std::swap(bigger.n, L.samples.n);
    }
    upload_rhs(c);
    DArr<double> x;
    x.alloc(nd);
    std::vector<double> hr(nd);
    std::vector<float> hf(nd);
    std::mt19937_64 rng(seed);
    std::normal_distribution<double> gauss(0.0, 1.0);
    for (int s = 0; s < n_samples; ++s) {
        if (iters[s] < 0) {
            std::vector<float> rf(nd);
            for (float& v : rf) v = (float)gauss(rng);
            mg_stationary_residual(c, rf.data(), -iters[s], L.objective == ASEND_LEARN_MG && L.have_weights);
            for (int i = 0; i < nd; ++i) hr[i] = rf[i];
        } else if (iters[s] > 0) {
            asend_solve_opts o{ASEND_METHOD_FP64, ASEND_PC_JACOBI, 1e-14, (int)iters[s], std::min(8, (int)iters[s]), 0, 0};
            asend_solve_stats st{};
            pcg_solve(c, o, &st, false, c.d_f.p, x.p, 1);
            ASEND_CUDA(cudaMemcpyAsync(hr.data(), c.d_r.p, sizeof(double) * nd, cudaMemcpyDeviceToHost, c.stream));
            ASEND_CUDA(cudaStreamSynchronize(c.stream));
        } else {
            for (double& v : hr) v = gauss(rng);
        }
        double nrm = 0.0;
        for (double v : hr) nrm += v * v;
        nrm = std::sqrt(std::max(nrm, 1e-300));
        for (int i = 0; i < nd; ++i) hf[i] = (float)(hr[i] / nrm);
        ASEND_CUDA(cudaMemcpyAsync(L.samples.p + (size_t)(first + s) * nd, hf.data(), sizeof(float) * nd,
                                   cudaMemcpyHostToDevice, c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
    }
    L.n_samples = total;
}

// caller-supplied samples [n_samples][n_dof], each scaled to unit norm (FP64 norm)
void learned_set_samples(Ctx& c, int n_samples, const float* samples) {
    if (n_samples <= 0) throw InputError("n_samples must be positive");
    ensure_buffers(c);
    LearnedState& L = state(c);
    const int nd = c.n_dof;
    std::vector<float> hf((size_t)n_samples * nd);
    for (int s = 0; s < n_samples; ++s) {
        const float* r = samples + (size_t)s * nd;
        double nrm = 0.0;
        for (int i = 0; i < nd; ++i) {
            if (!std::isfinite(r[i])) throw InputError("non-finite sample value");
            nrm += (double)r[i] * r[i];
        }
        if (!(nrm > 0.0)) throw InputError("zero sample");
        nrm = std::sqrt(nrm);
        for (int i = 0; i < nd; ++i) hf[(size_t)s * nd + i] = (float)(r[i] / nrm);
    }
    L.samples.upload(hf, c.stream);
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    L.n_samples = n_samples;
}

// mean loss over the samples; with grad, the mean parameter gradient in L.grad
double learned_loss_grad(Ctx& c, bool grad) {
    LearnedState& L = state(c);
    require_weights(L);
    if (L.n_samples <= 0) throw InputError("no residual samples");
    const int n = c.n_nodes, nd = c.n_dof, S = L.n_samples;
    if (L.objective == ASEND_LEARN_MG) {
        // residual after one V-cycle with the learned finest-level smoother
        mg_prepare(c);
        mg_select_smoother(c, true);
        L.gblk.zero(c.stream);
        L.part.zero(c.stream);
        mg_learned_loss_grad(c, L.samples.p, S, L.gblk.p, L.part.p);
        double loss = 0.0;
        ASEND_CUDA(cudaMemcpyAsync(&loss, L.part.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if (grad) {
            k_block_backward<<<lgrid(n), kLT, 0, c.stream>>>(n, L.y.p, L.cfac.p, L.gblk.p, 1.f / (float)S, L.dy.p);
            ++c.launches;
            launch_backward(c, n, L.feat.p, L.dy.p);
        }
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        ASEND_CUDA(cudaGetLastError());
        return loss / S;
    }
    L.binv.alloc((size_t)9 * n);
    learned_blocks(c, L.binv.p, true);
    if (grad) L.gblk.zero(c.stream);
    L.part.zero(c.stream);
    for (int s = 0; s < S; ++s) {
        const float* r = L.samples.p + (size_t)s * nd;
        k_apply_blocks<<<lgrid(n), kLT, 0, c.stream>>>(n, L.binv.p, r, L.z4.p);
        k_residual_e<<<lgrid(n), kLT, 0, c.stream>>>(n, c.A.slice_off.p, c.A.row_len.p, c.A.col.p, c.A.v32.p, r,
                                                     L.z4.p, L.e4.p, L.part.p);
        if (grad)
            k_block_grad<<<lgrid(n), kLT, 0, c.stream>>>(n, c.A.slice_off.p, c.A.row_len.p, c.A.col.p, c.A.v32.p,
                                                         L.e4.p, r, L.gblk.p);
        c.launches += grad ? 3 : 2;
    }
    double loss = 0.0;
    ASEND_CUDA(cudaMemcpyAsync(&loss, L.part.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    if (grad) {
        k_block_backward<<<lgrid(n), kLT, 0, c.stream>>>(n, L.y.p, L.cfac.p, L.gblk.p, 1.f / (float)S, L.dy.p);
        ++c.launches;
        launch_backward(c, n, L.feat.p, L.dy.p);
    }
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    ASEND_CUDA(cudaGetLastError());
    return loss / S;
}

// n_steps Adam steps on the current samples; returns the loss before the last step
double learned_train(Ctx& c, int n_steps, float lr) {
    LearnedState& L = state(c);
    require_weights(L);
    if (n_steps <= 0) return learned_loss_grad(c, false);
    double loss = 0.0;
    for (int it = 0; it < n_steps; ++it) {
        loss = learned_loss_grad(c, true);
        ++L.step;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)L.step), c2 = 1.f - std::pow(b2, (float)L.step);
        k_adam<<<(kNParam + 255) / 256, 256, 0, c.stream>>>(kNParam, L.master.p, L.m1.p, L.m2.p, L.grad.p, lr, b1, b2,
                                                            1e-8f, c1, c2, 1.f);
        ++c.launches;
        refresh(c);
    }
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    ASEND_CUDA(cudaGetLastError());
    return loss;
}

void learned_get_grad(Ctx& c, float* out) {
    LearnedState& L = state(c);
    require_weights(L);
    ASEND_CUDA(cudaMemcpyAsync(out, L.grad.p, sizeof(float) * kNParam, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
}

// features [n][16] (BF16 values as float), Cholesky factors [n][6], outputs [n][8]
void learned_get_features(Ctx& c, float* feat, float* cfac, float* y) {
    learned_features(c);
    LearnedState& L = state(c);
    const int n = c.n_nodes;
    if (y) {
        require_weights(L);
        launch_forward(c, n, L.feat.p, L.y.p);
    }
    std::vector<__nv_bfloat16> fb;
    if (feat) fb.resize((size_t)n * kF);
    if (feat)
        ASEND_CUDA(cudaMemcpyAsync(fb.data(), L.feat.p, sizeof(__nv_bfloat16) * fb.size(), cudaMemcpyDeviceToHost, c.stream));
    if (cfac) ASEND_CUDA(cudaMemcpyAsync(cfac, L.cfac.p, sizeof(float) * 6 * n, cudaMemcpyDeviceToHost, c.stream));
    if (y) ASEND_CUDA(cudaMemcpyAsync(y, L.y.p, sizeof(float) * kO * n, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    for (size_t i = 0; i < fb.size(); ++i) feat[i] = __bfloat162float(fb[i]);
}

// kernel checks: forward on given features; parameter gradient for given
// output gradients (sum over the n nodes)
void learned_forward_host(Ctx& c, int n, const float* feat, float* y_out) {
    LearnedState& L = state(c);
    require_weights(L);
    if (n <= 0) throw InputError("n must be positive");
    std::vector<__nv_bfloat16> fb((size_t)n * kF);
    for (size_t i = 0; i < fb.size(); ++i) fb[i] = __float2bfloat16(feat[i]);
    DArr<__nv_bfloat16> df;
    DArr<float> dyo;
    df.upload(fb, c.stream);
    dyo.alloc((size_t)n * kO);
    launch_forward(c, n, df.p, dyo.p);
    ASEND_CUDA(cudaMemcpyAsync(y_out, dyo.p, sizeof(float) * n * kO, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    ASEND_CUDA(cudaGetLastError());
}

void learned_backward_host(Ctx& c, int n, const float* feat, const float* dy, float* grad_out) {
    LearnedState& L = state(c);
    require_weights(L);
    if (n <= 0) throw InputError("n must be positive");
    std::vector<__nv_bfloat16> fb((size_t)n * kF);
    for (size_t i = 0; i < fb.size(); ++i) fb[i] = __float2bfloat16(feat[i]);
    DArr<__nv_bfloat16> df;
    DArr<float> ddy;
    df.upload(fb, c.stream);
    ddy.upload(dy, (size_t)n * kO, c.stream);
    launch_backward(c, n, df.p, ddy.p);
    ASEND_CUDA(cudaMemcpyAsync(grad_out, L.grad.p, sizeof(float) * kNParam, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    ASEND_CUDA(cudaGetLastError());
}

}  // namespace asend
