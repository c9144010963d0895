// k_noalloc.cu -- operator application with the strain energy x^T A x, for
// callers that cannot allocate device memory.
//
// Who needs it: host applications that hand all device memory to their own
// pool allocator (or run several solvers under a fixed HBM budget) and forbid
// libraries from calling cudaMalloc, and optimisation / line-search loops that
// evaluate y = A x and x^T A x many thousands of times, where an allocation
// inside the loop could fail or stall.  The regular entry point
// asend_apply_operator copies host buffers through temporary device arrays;
// this one works on caller-provided device buffers and keeps its only scratch
// (the per-CTA partial sums and the arrival counter of the deterministic
// last-CTA reduction) in a fixed array compiled into the library.
#include <mutex>

#include "common.cuh"

namespace asend {
namespace {

constexpr int kNaThreads = 128;
// Limit: 4,194,304 node rows (12,582,912 DOF) -> 32,768 CTAs of 128 rows.
constexpr int kNaMaxRows = 1 << 22;
constexpr int kNaMaxBlocks = kNaMaxRows / kNaThreads;
// [0, kNaMaxBlocks): per-CTA partial energies; [kNaMaxBlocks]: arrival
// counter (as unsigned int).  256 KiB + 256 B, held by every GPU that loads
// the library until the process exits.  Shared by all calls: calls that
// overlap on the GPU (different streams, or contexts on one device) race on it.
static __device__ __align__(256) double g_noalloc_scratch[kNaMaxBlocks + 32];

std::mutex g_na_mutex;
void* g_na_ptr[64] = {nullptr};  // device address of the scratch, per device

__global__ void __launch_bounds__(kNaThreads)
k_energy_noalloc(int n_rows, const int64_t* __restrict__ slice_off, const uint8_t* __restrict__ row_len,
                 const int32_t* __restrict__ col, const double* __restrict__ v64, const double* __restrict__ x,
                 double* __restrict__ y, double* __restrict__ energy, double* __restrict__ scratch) {
    __shared__ double sm[32];
    __shared__ bool is_last;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    double e[1] = {0.0};
    if (row < n_rows) {
        const int lane = row & 31;
        const int64_t g0 = slice_off[row >> 5];
        const int len = row_len[row];
        double acc[3] = {0.0, 0.0, 0.0};
        for (int j = 0; j < len; ++j) {
            const int64_t g = g0 + j;
            const int c = col[g * 32 + lane];
            const double* v = v64 + (g * 9) * 32 + lane;
            const double x0 = x[3 * (size_t)c], x1 = x[3 * (size_t)c + 1], x2 = x[3 * (size_t)c + 2];
#pragma unroll
            for (int a = 0; a < 3; ++a)
                acc[a] = fma(v[(a * 3) * 32], x0, fma(v[(a * 3 + 1) * 32], x1, fma(v[(a * 3 + 2) * 32], x2, acc[a])));
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            y[3 * (size_t)row + a] = acc[a];
            e[0] += x[3 * (size_t)row + a] * acc[a];
        }
    }
    block_sum<1>(e, sm);
    unsigned int* ticket = reinterpret_cast<unsigned int*>(scratch + kNaMaxBlocks);
    if (threadIdx.x == 0) {
        scratch[blockIdx.x] = e[0];
        __threadfence();
        is_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double s[1] = {0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s[0] += ((volatile double*)scratch)[b];
    __syncthreads();
    block_sum<1>(s, sm);
    if (threadIdx.x == 0) {
        *energy = s[0];
        *ticket = 0u;
    }
}

}  // namespace
}  // namespace asend

using namespace asend;

extern "C" int asend_operator_energy_noalloc(asend_ctx* ctx, const double* d_x, double* d_y, double* d_energy) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c) return ASEND_EINVAL;
    c->err.clear();
    if (!c->assembled) {
        c->err = "assemble first";
        return ASEND_ESTATE;
    }
    if (!d_x || !d_y || !d_energy) {
        c->err = "null device buffer";
        return ASEND_EINVAL;
    }
    {  // the rows read other rows' x after those rows wrote y: no overlap allowed
        const uintptr_t x0 = reinterpret_cast<uintptr_t>(d_x), y0 = reinterpret_cast<uintptr_t>(d_y);
        const uintptr_t e0 = reinterpret_cast<uintptr_t>(d_energy), nb = sizeof(double) * (uintptr_t)c->n_dof;
        const bool xy = x0 < y0 + nb && y0 < x0 + nb;
        const bool ex = e0 + sizeof(double) > x0 && e0 < x0 + nb;
        const bool ey = e0 + sizeof(double) > y0 && e0 < y0 + nb;
        if (xy || ex || ey) {
            c->err = "asend_operator_energy_noalloc: x, y and energy must not overlap";
            return ASEND_EINVAL;
        }
    }
    if (c->A.n_rows > kNaMaxRows || c->A.b != 3) {
        c->err = "operator too large for asend_operator_energy_noalloc: at most 4194304 node rows "
                 "(12582912 DOF) with 3 DOF per node; use asend_apply_operator";
        return ASEND_EINVAL;
    }
    if (c->device < 0 || c->device >= 64) {
        c->err = "device index out of range";
        return ASEND_EINVAL;
    }
    cudaError_t rc = cudaSetDevice(c->device);
    if (rc != cudaSuccess) {
        c->err = cudaGetErrorString(rc);
        return ASEND_ECUDA;
    }
    // One-time set-up per device (made on the first call, with the device
    // current): the device address of the scratch array.
    void* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_ptr[c->device]) {
            rc = cudaGetSymbolAddress(&g_na_ptr[c->device], g_noalloc_scratch);
            if (rc != cudaSuccess) {
                g_na_ptr[c->device] = nullptr;
                c->err = std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(rc);
                return ASEND_ECUDA;
            }
        }
        scratch = g_na_ptr[c->device];
    }
    double* sc = static_cast<double*>(scratch);
    // the arrival counter must start at zero
    rc = cudaMemsetAsync(sc + kNaMaxBlocks, 0, sizeof(unsigned int), c->stream);
    if (rc != cudaSuccess) {
        c->err = cudaGetErrorString(rc);
        return ASEND_ECUDA;
    }
    const int blocks = (c->A.n_rows + kNaThreads - 1) / kNaThreads;
    rc = ensure_v64_rc(*c);  // after a split-only assembly: the FP64 values from the pairs (no allocation)
    if (rc != cudaSuccess) {
        c->err = cudaGetErrorString(rc);
        return ASEND_ECUDA;
    }
    k_energy_noalloc<<<blocks, kNaThreads, 0, c->stream>>>(c->A.n_rows, c->A.slice_off.p, c->A.row_len.p,
                                                            c->A.col.p, c->A.v64.p, d_x, d_y, d_energy, sc);
    rc = cudaGetLastError();
    if (rc != cudaSuccess) {
        c->err = cudaGetErrorString(rc);
        return ASEND_ECUDA;
    }
    ++c->launches;
    return ASEND_OK;
}
