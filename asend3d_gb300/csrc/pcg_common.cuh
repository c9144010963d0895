// pcg_common.cuh -- data structures and device helpers shared by the PCG
// drivers (k_pcg.cu: Jacobi / block-Jacobi; k_mg.cu: multigrid-preconditioned).
#pragma once
#include <type_traits>

#include "common.cuh"

namespace asend {
namespace pcg {

constexpr int kThreads = 128;
constexpr int kMaxRhs = 4;

struct RhsScalars {
    double rz, rz_new, pAp, rr, bb, alpha, beta, target, rr_last_true;
    int32_t iter, done, finished, replace, nonfinite;
    int32_t restart;  // done by convergence: that iteration's p update was skipped
    int32_t refresh;  // multigrid CG: rz (and p when restarting) to be re-formed after a V-cycle
    int32_t n_repl;   // true-residual replacements made on the device (Jacobi / block PCG)
    float alpha2[2], beta2[2];  // alpha and beta as FP32 pairs (the split method's vector updates)
};
struct Control {
    int32_t all_done;
    uint32_t ticket[4];
    int32_t pad[3];  // pad[0]: instances still iterating (multigrid CG)
};

struct PcgArgs {
    int n_rows, nrhs, n_dof;
    const int64_t* slice_off;
    const uint8_t* row_len;
    const int32_t* col;
    const float* v32;    // FP32 values (the high part of each FP64 value)
    const float* v32lo;  // low parts: v64 = v32 + v32lo to 2^-48 relative (split method)
    const double* v64;
    const double* f;
    double* x;
    double* r;
    void* p;      // node-padded direction (float4 or 2 x double2 per node)
    void* ap;     // natural layout A p (float or double)
    const double* dinv;
    const float* binv;
    double* partials;  // [gridDim.x][kMaxRhs][3]
    RhsScalars* sc;    // [n_inst][kMaxRhs]
    Control* ctl;
    // Independent instances (disconnected sub-systems stacked in one
    // operator, each starting on a CTA boundary): CTA -> instance map, first
    // CTA and CTA count per instance, 4 reduction tickets per instance.
    // nullptr = a single instance spanning the whole grid.
    const int32_t* cta_inst;
    const int32_t* inst_cta0;
    const int32_t* inst_ncta;
    uint32_t* tickets;
};

__device__ __forceinline__ int cta_instance(const PcgArgs& A) { return A.cta_inst ? A.cta_inst[blockIdx.x] : 0; }

// True when this CTA has nothing left to do: everything converged (single
// instance) or every right-hand side of the CTA's instance is done.
template <int NR>
__device__ __forceinline__ bool cta_done(const PcgArgs& A, const RhsScalars* S) {
    if (A.ctl->all_done) return true;
    if (!A.cta_inst) return false;
#pragma unroll
    for (int k = 0; k < NR; ++k)
        if (!S[k].done) return false;
    return true;
}

// Split precision (ASEND_METHOD_SPLIT): the search direction is stored as
// FP32 hi + lo pairs (a node: hi float4 then lo float4, 32 bytes like the
// padded FP64 direction) and products with the hi + lo operator values run
// in compensated FP32 arithmetic, FP64-accurate on the FP32 pipes.
struct SplitP {};

// Type in which a direction element is loaded and A p is stored.
template <typename TP>
struct ApOf {
    using T = TP;
};
template <>
struct ApOf<SplitP> {
    using T = double;
};

template <typename TP>
struct PadVec;
template <>
struct PadVec<SplitP> {
    __device__ static void load(const void* p, size_t node, double (&v)[3]) {
        const float4 h = reinterpret_cast<const float4*>(p)[2 * node];
        const float4 l = reinterpret_cast<const float4*>(p)[2 * node + 1];
        v[0] = (double)h.x + (double)l.x;
        v[1] = (double)h.y + (double)l.y;
        v[2] = (double)h.z + (double)l.z;
    }
    __device__ static void store(void* p, size_t node, const double (&v)[3]) {
        const float h0 = (float)v[0], h1 = (float)v[1], h2 = (float)v[2];
        reinterpret_cast<float4*>(p)[2 * node] = make_float4(h0, h1, h2, 0.f);
        reinterpret_cast<float4*>(p)[2 * node + 1] =
            make_float4((float)(v[0] - (double)h0), (float)(v[1] - (double)h1), (float)(v[2] - (double)h2), 0.f);
    }
};
template <>
struct PadVec<float> {
    __device__ static void load(const void* p, size_t node, float (&v)[3]) {
        const float4 q = reinterpret_cast<const float4*>(p)[node];
        v[0] = q.x; v[1] = q.y; v[2] = q.z;
    }
    __device__ static void store(void* p, size_t node, const double (&v)[3]) {
        reinterpret_cast<float4*>(p)[node] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.f);
    }
};
template <>
struct PadVec<double> {
    __device__ static void load(const void* p, size_t node, double (&v)[3]) {
        const double2* q = reinterpret_cast<const double2*>(p) + 2 * node;
        const double2 a = q[0], b = q[1];
        v[0] = a.x; v[1] = a.y; v[2] = b.x;
    }
    __device__ static void store(void* p, size_t node, const double (&v)[3]) {
        double2* q = reinterpret_cast<double2*>(p) + 2 * node;
        q[0] = make_double2(v[0], v[1]);
        q[1] = make_double2(v[2], 0.0);
    }
};

// One compensated product term: (h + l)(xh + xl) added to the running sum
// (S, C).  p = h xh exactly equals pr + e (e from an FMA); pr enters S by
// TwoSum (its rounding error goes to C); e, h xl and l xh go to C.  The
// intrinsics keep the compiler from contracting the error-free steps.
__device__ __forceinline__ void split_term(float h, float l, float xh, float xl, float& S, float& C) {
    const float pr = __fmul_rn(h, xh);
    const float e = __fmaf_rn(h, xh, -pr);
    const float s = __fadd_rn(S, pr);
    const float bp = __fsub_rn(s, S);
    const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(s, bp)), __fsub_rn(pr, bp));
    S = s;
    C = __fadd_rn(C, __fadd_rn(err, e));
    C = __fmaf_rn(h, xl, C);
    C = __fmaf_rn(l, xh, C);
}

// ---------------------------------------------------------------------------
// FP32 pairs (double-float): a value v = h + l with |l| <= ulp(h) / 2, a
// 48-bit significand carried by two FP32 numbers.  The arithmetic below is
// built from error-free transformations -- Knuth's TwoSum, Dekker's
// Fast2Sum and the FMA-exact product -- so it runs on the FP32 pipes, which
// on this GPU issue many times faster than its FP64 pipe.  The intrinsics
// keep the compiler from contracting or reassociating the steps.
// ---------------------------------------------------------------------------
struct F2 {
    float h, l;
};
__device__ __forceinline__ F2 fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ F2 two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp))};
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    const F2 s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ F2 f2_neg(F2 a) { return {-a.h, -a.l}; }
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
    const float p = __fmul_rn(a.h, b.h);
    const float e = __fmaf_rn(a.h, b.h, -p);
    return fast_two_sum(p, __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e)));
}
__device__ __forceinline__ F2 f2_mul_f(F2 a, float b) {  // pair times an FP32 number
    const float p = __fmul_rn(a.h, b);
    const float e = __fmaf_rn(a.h, b, -p);
    return fast_two_sum(p, __fmaf_rn(a.l, b, e));
}
__device__ __forceinline__ F2 f2_of(double v) {  // FP64 -> pair (FP64 pipe: conversions)
    const float h = (float)v;
    return {h, (float)(v - (double)h)};
}
__device__ __forceinline__ double f2_dbl(F2 a) { return (double)a.h + (double)a.l; }

// FP64-accurate row product from FP32 hi / lo values and a split direction:
// the running sums S and their compensations Cc (y = S + Cc).
template <int NR>
__device__ __forceinline__ void spmv_row_split_sc(int row, const PcgArgs& A, const void* __restrict__ p,
                                                  float (&S)[NR][3], float (&Cc)[NR][3]) {
#pragma unroll
    for (int k = 0; k < NR; ++k)
#pragma unroll
        for (int a = 0; a < 3; ++a) S[k][a] = Cc[k][a] = 0.f;
    const float4* P = reinterpret_cast<const float4*>(p);
    const int lane = row & 31;
    const int64_t g0 = A.slice_off[row >> 5];
    const int len = A.row_len[row];
    int j = 0;
    if constexpr (NR == 1) {
        // two block columns in flight per step (independent loads overlap)
        for (; j + 2 <= len; j += 2) {
            const int64_t g = g0 + j;
            int c[2];
            float h[2][9], l[2][9];
#pragma unroll
            for (int u = 0; u < 2; ++u) c[u] = A.col[(g + u) * 32 + lane];
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    h[u][q] = A.v32[((g + u) * 9 + q) * 32 + lane];
                    l[u][q] = A.v32lo[((g + u) * 9 + q) * 32 + lane];
                }
            float4 xh[2], xl[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                xh[u] = P[2 * (size_t)c[u]];
                xl[u] = P[2 * (size_t)c[u] + 1];
            }
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    split_term(h[u][3 * a], l[u][3 * a], xh[u].x, xl[u].x, S[0][a], Cc[0][a]);
                    split_term(h[u][3 * a + 1], l[u][3 * a + 1], xh[u].y, xl[u].y, S[0][a], Cc[0][a]);
                    split_term(h[u][3 * a + 2], l[u][3 * a + 2], xh[u].z, xl[u].z, S[0][a], Cc[0][a]);
                }
        }
    }
    for (; j < len; ++j) {
        const int64_t g = g0 + j;
        const int c = A.col[g * 32 + lane];
        float h[9], l[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            h[q] = A.v32[(g * 9 + q) * 32 + lane];
            l[q] = A.v32lo[(g * 9 + q) * 32 + lane];
        }
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            const size_t nd = (size_t)k * A.n_rows + c;
            const float4 xh = P[2 * nd], xl = P[2 * nd + 1];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                split_term(h[3 * a], l[3 * a], xh.x, xl.x, S[k][a], Cc[k][a]);
                split_term(h[3 * a + 1], l[3 * a + 1], xh.y, xl.y, S[k][a], Cc[k][a]);
                split_term(h[3 * a + 2], l[3 * a + 2], xh.z, xl.z, S[k][a], Cc[k][a]);
            }
        }
    }
}

template <int NR>
__device__ __forceinline__ void spmv_row_split(int row, const PcgArgs& A, const void* __restrict__ p,
                                               double (&y)[NR][3]) {
    float S[NR][3], Cc[NR][3];
    spmv_row_split_sc<NR>(row, A, p, S, Cc);
#pragma unroll
    for (int k = 0; k < NR; ++k)
#pragma unroll
        for (int a = 0; a < 3; ++a) y[k][a] = (double)S[k][a] + (double)Cc[k][a];
}

// y[k][a] = sum_j sum_c A[r][j](a,c) * p_k[col_j](c) for NR right-hand sides.
template <typename TV, typename TP, int NR>
__device__ __forceinline__ void spmv_row(int row, const PcgArgs& A, const TV* __restrict__ vals,
                                         const void* __restrict__ p, typename ApOf<TP>::T (&y)[NR][3]) {
    if constexpr (std::is_same<TP, SplitP>::value) {
        spmv_row_split<NR>(row, A, p, y);
        return;
    } else {
#pragma unroll
    for (int k = 0; k < NR; ++k) y[k][0] = y[k][1] = y[k][2] = (TP)0;
    const int lane = row & 31;
    const int64_t g0 = A.slice_off[row >> 5];
    const int len = A.row_len[row];
    int j = 0;
    if constexpr (NR == 1) {
        // three block columns in flight per step (independent loads overlap)
        for (; j + 3 <= len; j += 3) {
            const int64_t g = g0 + j;
            int c[3];
            TV m[3][9];
#pragma unroll
            for (int u = 0; u < 3; ++u) c[u] = A.col[(g + u) * 32 + lane];
#pragma unroll
            for (int u = 0; u < 3; ++u)
#pragma unroll
                for (int q = 0; q < 9; ++q) m[u][q] = vals[((g + u) * 9 + q) * 32 + lane];
            TP pv[3][3];
#pragma unroll
            for (int u = 0; u < 3; ++u) PadVec<TP>::load(p, (size_t)c[u], pv[u]);
#pragma unroll
            for (int u = 0; u < 3; ++u)
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    y[0][a] = fma((TP)m[u][a * 3 + 0], pv[u][0],
                                  fma((TP)m[u][a * 3 + 1], pv[u][1], fma((TP)m[u][a * 3 + 2], pv[u][2], y[0][a])));
        }
    }
    for (; j < len; ++j) {
        const int64_t g = g0 + j;
        const int c = A.col[g * 32 + lane];
        const TV* v = vals + (g * 9) * 32 + lane;
        TV m[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) m[q] = v[q * 32];
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            TP pv[3];
            PadVec<TP>::load(p, (size_t)k * A.n_rows + c, pv);
#pragma unroll
            for (int a = 0; a < 3; ++a)
                y[k][a] = fma((TP)m[a * 3 + 0], pv[0], fma((TP)m[a * 3 + 1], pv[1], fma((TP)m[a * 3 + 2], pv[2], y[k][a])));
        }
    }
    }
}

// ---------------------------------------------------------------------------
// Staged split product.  A warp owns one slice (32 rows); the slice's block
// column groups -- 288 FP32 hi values, 288 lo values and 32 column indices
// each, contiguous in HBM group after group -- stream through a ring of
// shared-memory stages that cp.async.bulk copies fill and that complete on
// one mbarrier per stage.  The bytes in flight per SM are then set by the
// ring depth (warps x stages x stage bytes) instead of by how many loads the
// resident warps' registers can hold, which left the register-fed product
// latency-bound near half of the HBM bandwidth.  The arithmetic and its
// order per row are those of spmv_row_split (bit-identical results).
// ---------------------------------------------------------------------------
template <int G, int S>
struct SplitStage {
    static constexpr int kVal = 9 * 32;                            // floats per group and value part
    static constexpr int kStage = G * (2 * kVal * 4 + 32 * 4);     // bytes per stage
    static constexpr int kWarp = S * kStage;                       // ring bytes per warp
    static constexpr int kBar = 128;                               // mbarrier area (16 x 8 B max)
    static constexpr int smem(int threads) { return kBar + (threads / 32) * kWarp; }
    static_assert((kThreads / 32) * S <= kBar / 8, "one mbarrier per warp and stage must fit the barrier area");
    static_assert(kStage % 16 == 0 && (G * kVal * 4) % 16 == 0, "bulk copies need 16-byte aligned stages");
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false after kSpinLimit polls (each poll may suspend the
// thread for a hardware-chosen interval), so a copy that never lands ends
// the kernel with an error instead of a hang.
constexpr int kSpinLimit = 1 << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (int i = 0; i < kSpinLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// global -> shared bulk copy (16-byte aligned addresses, size a multiple of
// 16) completing on bar; the executing CTA's shared::cta address is a valid
// shared::cluster address
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Persistent staged split product.  Warp w of CTA b owns the slices
// b * W + w + j * (gridDim.x * W), j = 0, 1, ... (W warps per CTA), so thread
// t of CTA b meets the rows b * blockDim.x + t + j * gridDim.x * blockDim.x,
// as a grid-stride loop over rows does.  The warp's groups, slice after
// slice, form one stream of stages: lane 0 keeps S stages in flight across
// slice boundaries, every lane consumes them in order.  After each slice
// the lane's row (if any) is handed to epi(row, y) with y = A p as FP32
// pairs.  Returns false in every lane of a warp whose copies did not land
// within the wait limit (the remaining slices are then skipped).
// smem: SplitStage<G, S>::smem(blockDim.x) bytes, 16-aligned.
template <int G, int S, typename Epi>
__device__ __forceinline__ bool split_staged_slices(const PcgArgs& A, const void* __restrict__ p, unsigned char* smem,
                                                    Epi&& epi) {
    using St = SplitStage<G, S>;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpc = blockDim.x >> 5;
    const int n_sl = (A.n_rows + 31) >> 5;
    const int sl0 = blockIdx.x * wpc + warp, sl_step = gridDim.x * wpc;
    if (sl0 >= n_sl) return true;  // warp-uniform: no slice for this warp
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem) + warp * S;
    unsigned char* ring = smem + St::kBar + warp * St::kWarp;
    const float4* P = reinterpret_cast<const float4*>(p);
    // producer cursor (lane 0): slice pj, its first group pg0 and group count
    // png, next stage pk within it; issued = stages issued so far
    int psl = sl0, pk = 0, issued = 0;
    int64_t pg0 = 0;
    int png = 0;
    auto load_slice = [&](int sl) {
        pg0 = A.slice_off[sl];
        png = (int)(A.slice_off[sl + 1] - pg0);
    };
    auto issue_next = [&]() {  // lane 0: the next stage of the stream, if any
        if (psl >= n_sl) return;
        const int s = issued % S;
        const int cnt = min(G, png - pk * G);
        const int64_t gk = pg0 + (int64_t)pk * G;
        unsigned char* st = ring + s * St::kStage;
        mbar_expect_tx(bars + s, (uint32_t)cnt * (2 * St::kVal * 4 + 32 * 4));
        bulk_g2s(st, A.v32 + gk * St::kVal, cnt * St::kVal * 4, bars + s);
        bulk_g2s(st + G * St::kVal * 4, A.v32lo + gk * St::kVal, cnt * St::kVal * 4, bars + s);
        bulk_g2s(st + 2 * G * St::kVal * 4, A.col + gk * 32, cnt * 32 * 4, bars + s);
        ++issued;
        if (++pk * G >= png) {  // next slice of this warp
            pk = 0;
            psl += sl_step;
            if (psl < n_sl) load_slice(psl);
        }
    };
    if (lane == 0) {
#pragma unroll
        for (int s = 0; s < S; ++s) mbar_init(bars + s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_async_shared();
        load_slice(psl);
        for (int s = 0; s < S; ++s) issue_next();
    }
    __syncwarp();
    int used = 0;  // stages consumed
    bool ok = true;
    for (int sl = sl0; sl < n_sl && ok; sl += sl_step) {
        const int row = sl * 32 + lane;
        const int64_t g0 = A.slice_off[sl];
        const int ng = (int)(A.slice_off[sl + 1] - g0);
        const int len = row < A.n_rows ? A.row_len[row] : 0;
        const int nst = (ng + G - 1) / G;
        float Sm[3] = {0.f, 0.f, 0.f}, Cc[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < nst; ++k) {
            const int s = used % S;
            if (!__all_sync(0xffffffffu, mbar_wait(bars + s, (uint32_t)((used / S) & 1)))) {
                ok = false;
                break;
            }
            const float* hv = reinterpret_cast<const float*>(ring + s * St::kStage);
            const float* lv = hv + G * St::kVal;
            const int* cv = reinterpret_cast<const int*>(lv + G * St::kVal);
            const int cnt = min(G, ng - k * G);
            float4 xh[G], xl[G];
#pragma unroll
            for (int u = 0; u < G; ++u) {
                if (u < cnt && k * G + u < len) {
                    const int c = cv[u * 32 + lane];
                    xh[u] = P[2 * (size_t)c];
                    xl[u] = P[2 * (size_t)c + 1];
                }
            }
#pragma unroll
            for (int u = 0; u < G; ++u) {
                if (u < cnt && k * G + u < len) {
                    const float* h = hv + u * St::kVal + lane;
                    const float* l = lv + u * St::kVal + lane;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        split_term(h[(3 * a) * 32], l[(3 * a) * 32], xh[u].x, xl[u].x, Sm[a], Cc[a]);
                        split_term(h[(3 * a + 1) * 32], l[(3 * a + 1) * 32], xh[u].y, xl[u].y, Sm[a], Cc[a]);
                        split_term(h[(3 * a + 2) * 32], l[(3 * a + 2) * 32], xh[u].z, xl[u].z, Sm[a], Cc[a]);
                    }
                }
            }
            ++used;
            __syncwarp();  // every lane is done reading stage s before it is refilled
            if (lane == 0) {
                fence_async_shared();
                issue_next();
            }
        }
        if (!ok) break;
        if (row < A.n_rows) {
            const F2 y[3] = {two_sum(Sm[0], Cc[0]), two_sum(Sm[1], Cc[1]), two_sum(Sm[2], Cc[2])};
            epi(row, y);
        }
    }
    if (!ok) {
        // stages used .. issued - 1 may still be in flight: wait for them
        // (bounded) before the CTA can leave and its shared memory be reused
        const int upto = __shfl_sync(0xffffffffu, issued, 0);
        if (lane == 0)
            for (int q = used; q < upto; ++q) mbar_wait(bars + q % S, (uint32_t)((q / S) & 1));
        __syncwarp();
    }
    return ok;
}

// Programmatic dependent launch: a kernel launched with the programmatic
// stream-serialization attribute may start while its predecessor in the
// stream drains.  It first waits for the predecessor's completion and memory
// (griddepcontrol.wait; a no-op without the attribute), then lets its own
// successor launch early (griddepcontrol.launch_dependents), so only the
// launch and CTA set-up overlap; every read and write comes after the wait.
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Preconditioner application z = M^-1 r for one node.
template <int PC>
__device__ __forceinline__ void precond(const PcgArgs& A, int row, const double (&r)[3], double (&z)[3]) {
    if constexpr (PC == ASEND_PC_JACOBI) {
#pragma unroll
        for (int a = 0; a < 3; ++a) z[a] = A.dinv[3 * (size_t)row + a] * r[a];
    } else {
        const float* B = A.binv + 9 * (size_t)row;
        const float r0 = (float)r[0], r1 = (float)r[1], r2 = (float)r[2];
#pragma unroll
        for (int a = 0; a < 3; ++a) z[a] = (double)fmaf(B[3 * a], r0, fmaf(B[3 * a + 1], r1, B[3 * a + 2] * r2));
    }
}

// Last-CTA reduction of NV values per RHS; returns true in the last CTA
// (all its threads) with tot[k][v] valid in every thread.
template <int NR, int NV>
__device__ __forceinline__ bool last_block_reduce(const PcgArgs& A, double (&val)[NR][NV], int ticket_id,
                                  double (&tot)[NR][NV]) {
    __shared__ double sm[32 * NR * NV];
    __shared__ bool is_last;
    double flat[NR * NV];
#pragma unroll
    for (int k = 0; k < NR; ++k)
#pragma unroll
        for (int v = 0; v < NV; ++v) flat[k * NV + v] = val[k][v];
    block_sum<NR * NV>(flat, sm);
    // the CTAs of this CTA's instance reduce together (whole grid if single)
    const int inst = cta_instance(A);
    const int b0 = A.cta_inst ? A.inst_cta0[inst] : 0;
    const int nb = A.cta_inst ? A.inst_ncta[inst] : (int)gridDim.x;
    uint32_t* ticket = A.tickets ? &A.tickets[inst * 4 + ticket_id] : &A.ctl->ticket[ticket_id];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NR * NV; ++q) A.partials[(size_t)blockIdx.x * (kMaxRhs * 3) + q] = flat[q];
        __threadfence();
        const uint32_t t = atomicAdd(ticket, 1u);
        is_last = (t == (uint32_t)nb - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    double acc[NR * NV];
#pragma unroll
    for (int q = 0; q < NR * NV; ++q) acc[q] = 0.0;
    // L2 reads (ld.global.cg: no stale L1 line after the fence) that may all
    // be in flight together, unlike volatile loads, which issue one by one
#pragma unroll 4
    for (int b = b0 + threadIdx.x; b < b0 + nb; b += blockDim.x) {
        const double* pp = A.partials + (size_t)b * (kMaxRhs * 3);
#pragma unroll
        for (int q = 0; q < NR * NV; ++q) acc[q] += __ldcg(pp + q);
    }
    __syncthreads();
    block_sum<NR * NV>(acc, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NR * NV; ++q) sm[q] = acc[q];
        *ticket = 0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NR; ++k)
#pragma unroll
        for (int v = 0; v < NV; ++v) tot[k][v] = sm[k * NV + v];
    return true;
}


}  // namespace pcg
}  // namespace asend
