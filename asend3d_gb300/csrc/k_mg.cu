// k_mg.cu -- geometric multigrid preconditioner for structured hex8 blocks and
// the multigrid-preconditioned (flexible) CG driver.
//
// The reference preconditions its CG with LDL^T factors of diagonal blocks of
// the stiffness matrix (lower_tri_mat_meth.rs:15-241, block size from
// model_prep.rs:888-902) and otherwise follows conj_grad_sparse
// (matrix_functions.rs:285-362).  A block factorization has no efficient GPU
// form; this module replaces it by a V-cycle whose cost per application is a
// few SpMVs and whose iteration count is nearly independent of the mesh size.
//
// Hierarchy (structured block nx x ny x nz, node (i,j,k) = (i*(ny+1)+j)*(nz+1)+k):
//  * each level halves the element count per axis (an odd count leaves one
//    coarse element spanning a single fine element), down to <= 256 DOFs;
//  * prolongation is trilinear interpolation in index space, per component;
//  * coarse operators are Galerkin, formed element by element:
//        K_C = sum_{e child of C} Q_e^T K_e Q_e,
//    Q_e the 24x24 trilinear map from C's corners to e's corners.  For nested
//    grids this equals P^T A P exactly (without the penalty rows), and unlike
//    rediscretised coarse hex8 grids it does not lock in bending;
//  * penalty constraints enter coarse levels lumped: pen_c = P^T pen_f row sums;
//  * smoothing: one pre- and one post-sweep of damped nodal block Jacobi;
//  * coarsest level: explicit inverse (Gauss-Jordan, one CTA);
//  * all level arithmetic in FP32; the outer CG keeps the FP64 operator,
//    FP64 vectors and dots, and uses the Polak-Ribiere (flexible) beta
//    beta = -alpha (z . Ap) / (r_old . z_old), which tolerates the FP32
//    preconditioner's rounding asymmetry.
#include <algorithm>
#include <array>
#include <cstring>
#include <cmath>
#include <memory>
#include <utility>

#include "pcg_common.cuh"

namespace asend {

struct MgAxis {
    int n_f = 0, n_c = 0;         // fine / coarse element counts
    std::vector<int32_t> xs;      // coarse node -> fine node index (n_c + 1)
    std::vector<int32_t> lo;      // fine node -> lower coarse node (n_f + 1)
    std::vector<float> w;         // fine node -> weight of lo + 1
};

// One structured block of a level: a single model's grid, or one instance of
// a batched stack.  Block b of every level belongs to instance b; blocks are
// coarsened independently, and a block that needs no further coarsening is
// carried down unchanged (identity maps) until every block is coarse enough.
struct MgBlk {
    int nx = 0, ny = 0, nz = 0;   // cells
    int node0 = 0, el0 = 0;       // first node / element in the level numbering
    MgAxis ax[3];                 // maps from the finer level's block (levels >= 1)
    int ox[3] = {0, 0, 0}, ol[3] = {0, 0, 0};  // offsets into the level's packed xs / lo, w
    double h[3] = {0, 0, 0};      // cell spacing per axis
    bool done = false;            // coarse enough: identity maps below this level
    int n_nodes() const { return (nx + 1) * (ny + 1) * (nz + 1); }
    int n_el() const { return nx * ny * nz; }
};

// Device descriptor of block b of a level; levels >= 1 also describe the
// finer level's block b (f*) and the block's axis maps.
struct BlkDev {
    int nx, ny, nz, node0, el0;
    int fnx, fny, fnz, fnode0, fel0;
    int ox0, ox1, ox2, ol0, ol1, ol2;
    int dense0, pad;
};

struct MgLevel {
    int n_nodes = 0, n_el = 0, n_dof = 0;  // totals (level 0 of a batch includes padding nodes)
    std::vector<MgBlk> blk;
    DArr<BlkDev> d_blk;
    DArr<int32_t> pre_node, pre_el;  // per-block starts (+ total)
    DArr<int32_t> d_xs, d_lo;     // packed per block and axis
    DArr<float> d_w;
    Sbell own;                    // pattern + FP32 values (levels >= 1)
    Sbell* A = nullptr;
    std::vector<int32_t> colour_ptr;
    DArr<int32_t> colour_elems, slot_map, conn;
    DArr<float> Ke;               // Galerkin element matrices [n_el][24][24]
    std::vector<float> h_pen;     // lumped penalty per DOF (in units of sf)
    DArr<float> pen;
    DArr<float> binv, b, r, x4, y4;
    DArr<float> pow_vec;          // last power-iteration vector (warm start)
    bool pow_warm = false;
    int pow_steps = 0;            // steps of the last estimate
};

struct MgHierarchy {
    std::vector<std::unique_ptr<MgLevel>> L;
    DArr<float> dense, ainv;      // coarsest operators, one dense block per instance, inverted in place
    int n_coarse = 0;             // largest coarsest block (DOF)
    int n_blk = 1;
    std::vector<int32_t> h_dense0;  // offset of each block's dense matrix (floats)
    DArr<double> blk_sf;          // penalty scale per block (instance)
    DArr<float> child;            // projected class matrices of the first coarsening [n_cls][27][576]
    bool child_ready = false;
    // captured outer iterations, reused while the launch arguments match
    std::vector<std::pair<std::vector<uint8_t>, cudaGraphExec_t>> graphs;
    ~MgHierarchy() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    }
    int64_t epoch = -1;
    float omega = 0.6f;           // damping used when the eigenvalue estimate fails
    bool l0_learned = false;      // finest-level smoother blocks come from the learned model
    bool l0_damped = false;       // finest-level eigenvalue-damped blocks are current
    DArr<float> pow_nrm;          // power-iteration norms per level [levels][kPowSteps + 1]
    DArr<uint32_t> pow_ticket;    // last-CTA tickets per level and step
    DArr<double> pow_part;        // per-CTA partial sums
    DArr<unsigned int> pow_bound; // ||D^-1 A||_inf per level (float bits)
    DArr<float> pow_omega;        // damping in use per level
    bool safe_damping = false;    // omega from the guaranteed bound (after a failed solve)
    int tail = 0;                 // first level of the fused coarse tail (0: none)
    DArr<float> vl_q, vl_mw, vl_t4, vl_r2, vl_w;  // learned-smoother training vectors
};

constexpr int kPowSteps = 10;      // from a hashed start vector
constexpr int kPowWarmSteps = 4;   // from the previous assembly's vector

namespace {
using namespace pcg;

constexpr int kT = 128;
inline int grid_of(int n) { return (n + kT - 1) / kT; }
// Grid of the split method's CG kernels on a single instance: grid-stride
// loops over 4 CTAs per SM (152 SMs) instead of one CTA per 128 rows, so the
// last-CTA reductions sum 608 partials, not thousands.
constexpr int kPersistCtas = 152 * 4;

// Launch on the context's stream, with programmatic dependent launch when the
// context allows it (the kernel then starts while its predecessor drains and
// waits for it in pdl_begin(); every kernel launched here calls it first).
template <typename... KArgs, typename... Args>
void launch_k(const Ctx& c, void (*k)(KArgs...), int grid, int block, size_t smem, Args&&... args) {
    if (!c.pdl) {
        k<<<grid, block, smem, c.stream>>>(std::forward<Args>(args)...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = c.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    ASEND_CUDA(cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...));
}
// classes up to which the first coarsening uses projected class matrices
// (27 x 576 floats each, 62 KB)
constexpr int kMaxChildClasses = 512;
// dynamic shared memory of the blocked coarsest inverse (227 KB per CTA less
// the 4 KB panel inverse and static data)
constexpr size_t kGjSmem = 220 * 1024;

__device__ __forceinline__ int nid(int i, int j, int k, int ny, int nz) { return (i * (ny + 1) + j) * (nz + 1) + k; }

// hex8 corner offsets in the reference's corner order
__constant__ int c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                   {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

struct LevelView {  // kernel-side view of a coarse level's blocks and maps from the finer level
    int n_blk;
    const BlkDev* blk;
    const int32_t* xs;
    const int32_t* lo;
    const float* w;
};

// Block of index idx: the largest b with pre[b] <= idx (pre ascending).
__device__ __forceinline__ int find_blk(const int32_t* __restrict__ pre, int n_blk, int idx) {
    int lo = 0, hi = n_blk - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= idx) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// Galerkin coarsening by elements
// ---------------------------------------------------------------------------
// One CTA (512 threads) per coarse element C of level l.  Its <= 8 children
// (elements of level l-1) are processed together: each child's FP32 stiffness
// comes from the stored Galerkin matrices of level l-1, or for l = 1 is
// integrated here from the fine geometry (2x2x2 Gauss points, closed-form
// isotropic blocks as in the assembly kernel); then T_e = K_e (Q_e x I3) and
// K_C = sum_e (Q_e x I3)^T T_e.
__global__ void __launch_bounds__(512)
k_coarsen(LevelView cv, const int32_t* __restrict__ pre_el, const float* __restrict__ fine_ke,
          const float* __restrict__ cls_ke, const int32_t* __restrict__ cls_of, const double* __restrict__ xyz,
          const int32_t* __restrict__ conn0, const double* __restrict__ E, const double* __restrict__ nu,
          float* __restrict__ coarse_ke) {
    __shared__ float Ke[8][576];
    __shared__ float T[8][576];
    __shared__ float Q[8][8][8];
    __shared__ float g[8][8][8][3];
    __shared__ float wdet[8][8];
    __shared__ float xl[8][8][3];
    __shared__ int fe[8];
    const int t = threadIdx.x;
    const int C = blockIdx.x;
    const BlkDev& d = cv.blk[find_blk(pre_el, cv.n_blk, C)];
    const int Cl = C - d.el0;
    const int ci = Cl / (d.ny * d.nz), cj = (Cl / d.nz) % d.ny, ck = Cl % d.nz;
    const int s0 = cv.xs[d.ox0 + ci], w0 = cv.xs[d.ox0 + ci + 1] - s0;
    const int s1 = cv.xs[d.ox1 + cj], w1 = cv.xs[d.ox1 + cj + 1] - s1;
    const int s2 = cv.xs[d.ox2 + ck], w2 = cv.xs[d.ox2 + ck + 1] - s2;
    const int nch = w0 * w1 * w2;
    if (t < nch * 64) {  // interpolation weights of child ch: fine corner a <- coarse corner b
        const int ch = t >> 6, a = (t >> 3) & 7, b = t & 7;
        const int o0 = ch / (w1 * w2), o1 = (ch / w2) % w1, o2 = ch % w2;
        const float xi0 = (float)(o0 + c_corner[a][0]) / w0;
        const float xi1 = (float)(o1 + c_corner[a][1]) / w1;
        const float xi2 = (float)(o2 + c_corner[a][2]) / w2;
        Q[ch][a][b] = (c_corner[b][0] ? xi0 : 1.f - xi0) * (c_corner[b][1] ? xi1 : 1.f - xi1) *
                      (c_corner[b][2] ? xi2 : 1.f - xi2);
        if (a == 0 && b == 0) fe[ch] = d.fel0 + ((s0 + o0) * d.fny + (s1 + o1)) * d.fnz + (s2 + o2);
    }
    __syncthreads();
    if (cls_ke) {  // K_e = E_e * (unit-modulus matrix of the element's geometry class)
        for (int q = t; q < nch * 576; q += blockDim.x) {
            const int e = fe[q / 576];
            Ke[q / 576][q % 576] = (float)E[e] * cls_ke[(size_t)cls_of[e] * 576 + q % 576];
        }
    } else if (fine_ke) {
        for (int q = t; q < nch * 576; q += blockDim.x) Ke[q / 576][q % 576] = fine_ke[(size_t)fe[q / 576] * 576 + q % 576];
    } else {
        if (t < nch * 24) {
            const int ch = t / 24, a = (t / 3) % 8, j = t % 3;
            const int e = fe[ch];
            const int n0 = conn0[(size_t)e * 8], na = conn0[(size_t)e * 8 + a];
            xl[ch][a][j] = (float)(xyz[3 * (size_t)na + j] - xyz[3 * (size_t)n0 + j]);
        }
        __syncthreads();
        if (t < nch * 8) {  // Gauss-point data of child ch, point gp
            const int ch = t >> 3, gp = t & 7;
            const float gq = 0.5773502691896257f;
            const float s[3] = {(gp & 1) ? gq : -gq, (gp & 2) ? gq : -gq, (gp & 4) ? gq : -gq};
            float dn[8][3];
            float J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int a = 0; a < 8; ++a) {
                const float sg0 = c_corner[a][0] ? 1.f : -1.f, sg1 = c_corner[a][1] ? 1.f : -1.f,
                            sg2 = c_corner[a][2] ? 1.f : -1.f;
                const float f0 = 1 + sg0 * s[0], f1 = 1 + sg1 * s[1], f2 = 1 + sg2 * s[2];
                dn[a][0] = 0.125f * sg0 * f1 * f2;
                dn[a][1] = 0.125f * sg1 * f0 * f2;
                dn[a][2] = 0.125f * sg2 * f0 * f1;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) J[i][j] += xl[ch][a][i] * dn[a][j];
            }
            const float c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
            const float c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
            const float c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
            const float det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
            const float id = 1.f / det;
            float Ji[3][3];
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
                    g[ch][gp][a][j] = dn[a][0] * Ji[0][j] + dn[a][1] * Ji[1][j] + dn[a][2] * Ji[2][j];
            wdet[ch][gp] = det;
        }
        __syncthreads();
        if (t < nch * 64) {  // node-pair block (a, b) of child ch
            const int ch = t >> 6, a = (t >> 3) & 7, b = t & 7;
            const double Ee = E[fe[ch]], ne = nu[fe[ch]];
            const float lam = (float)(Ee * ne / ((1.0 + ne) * (1.0 - 2.0 * ne)));
            const float mu = (float)(Ee / (2.0 * (1.0 + ne)));
            float S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int gp = 0; gp < 8; ++gp)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) S[i][j] += wdet[ch][gp] * g[ch][gp][a][i] * g[ch][gp][b][j];
            const float tr = mu * (S[0][0] + S[1][1] + S[2][2]);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    Ke[ch][(3 * a + i) * 24 + 3 * b + j] = lam * S[i][j] + mu * S[j][i] + ((i == j) ? tr : 0.f);
        }
    }
    __syncthreads();
    // T_ch = K_ch (Q_ch x I3)
    for (int q = t; q < nch * 576; q += blockDim.x) {
        const int ch = q / 576, r = q % 576, row = r / 24, col = r % 24, b = col / 3, c2 = col % 3;
        float acc = 0.f;
#pragma unroll
        for (int a2 = 0; a2 < 8; ++a2) acc = fmaf(Ke[ch][row * 24 + 3 * a2 + c2], Q[ch][a2][b], acc);
        T[ch][r] = acc;
    }
    __syncthreads();
    // K_C = sum_ch (Q_ch x I3)^T T_ch
    for (int q = t; q < 576; q += blockDim.x) {
        const int row = q / 24, col = q % 24, b = row / 3, c1 = row % 3;
        float acc = 0.f;
        for (int ch = 0; ch < nch; ++ch)
#pragma unroll
            for (int a = 0; a < 8; ++a) acc = fmaf(Q[ch][a][b], T[ch][(3 * a + c1) * 24 + col], acc);
        coarse_ke[(size_t)C * 576 + q] = acc;
    }
}

// First coarsening of a level-0 block made of geometry classes: with
// K_e = E_e K^_cls, the coarse matrix K_C = sum_ch E_ch (Q_ch x I3)^T K^ (Q_ch x I3)
// is linear in the children's moduli, and the projected class matrix depends
// only on the child's place in its coarse element.  Per axis a child is one
// of three cases (coarse cell of width 1; width 2, first or second half), so
// 27 projected matrices per class, built once per hierarchy in FP64 from the
// FP64 class matrices (CTA = (case, class)).
__global__ void __launch_bounds__(256) k_child_mats(const double* __restrict__ cls_ke, float* __restrict__ out) {
    __shared__ double K[576];
    __shared__ double T[576];
    __shared__ double Q[8][8];
    const int tc = blockIdx.x, cls = blockIdx.y, t = threadIdx.x;
    int w[3], o[3];
    for (int ax = 0, v = tc; ax < 3; ++ax, v /= 3) {
        const int s = v % 3;
        w[ax] = s == 0 ? 1 : 2;
        o[ax] = s == 2 ? 1 : 0;
    }
    for (int q = t; q < 576; q += blockDim.x) K[q] = cls_ke[(size_t)cls * 576 + q];
    if (t < 64) {
        const int a = t >> 3, b = t & 7;
        double q = 1.0;
        for (int ax = 0; ax < 3; ++ax) {
            const double xi = (double)(o[ax] + c_corner[a][ax]) / w[ax];
            q *= c_corner[b][ax] ? xi : 1.0 - xi;
        }
        Q[a][b] = q;
    }
    __syncthreads();
    for (int q = t; q < 576; q += blockDim.x) {  // T = K (Q x I3)
        const int row = q / 24, col = q % 24, b = col / 3, c2 = col % 3;
        double acc = 0.0;
        for (int a = 0; a < 8; ++a) acc += K[row * 24 + 3 * a + c2] * Q[a][b];
        T[q] = acc;
    }
    __syncthreads();
    for (int q = t; q < 576; q += blockDim.x) {  // (Q x I3)^T T
        const int row = q / 24, col = q % 24, b = row / 3, c1 = row % 3;
        double acc = 0.0;
        for (int a = 0; a < 8; ++a) acc += Q[a][b] * T[(3 * a + c1) * 24 + col];
        out[((size_t)cls * 27 + tc) * 576 + q] = (float)acc;
    }
}

// K_C = sum_ch E_ch B[cls_ch][case_ch]: one CTA of 144 threads per coarse
// element, four consecutive entries per thread.
__global__ void __launch_bounds__(144) k_coarsen_lin(LevelView cv, const int32_t* __restrict__ pre_el,
                                                     const double* __restrict__ E, const int32_t* __restrict__ cls_of,
                                                     const float* __restrict__ child, float* __restrict__ coarse_ke) {
    __shared__ float ew[8];
    __shared__ int bi[8];
    __shared__ int nch_s;
    const int t = threadIdx.x, C = blockIdx.x;
    if (t < 8) {
        const BlkDev& d = cv.blk[find_blk(pre_el, cv.n_blk, C)];
        const int Cl = C - d.el0;
        const int ci = Cl / (d.ny * d.nz), cj = (Cl / d.nz) % d.ny, ck = Cl % d.nz;
        const int s0 = cv.xs[d.ox0 + ci], w0 = cv.xs[d.ox0 + ci + 1] - s0;
        const int s1 = cv.xs[d.ox1 + cj], w1 = cv.xs[d.ox1 + cj + 1] - s1;
        const int s2 = cv.xs[d.ox2 + ck], w2 = cv.xs[d.ox2 + ck + 1] - s2;
        const int nch = w0 * w1 * w2;
        if (t == 0) nch_s = nch;
        if (t < nch) {
            const int o0 = t / (w1 * w2), o1 = (t / w2) % w1, o2 = t % w2;
            const int e = d.fel0 + ((s0 + o0) * d.fny + (s1 + o1)) * d.fnz + (s2 + o2);
            const int tc = (w0 == 1 ? 0 : 1 + o0) + 3 * (w1 == 1 ? 0 : 1 + o1) + 9 * (w2 == 1 ? 0 : 1 + o2);
            ew[t] = (float)E[e];
            bi[t] = cls_of[e] * 27 + tc;
        }
    }
    __syncthreads();
    const int nch = nch_s;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int ch = 0; ch < nch; ++ch) {
        const float4 b = reinterpret_cast<const float4*>(child + (size_t)bi[ch] * 576)[t];
        const float e = ew[ch];
        acc.x = fmaf(e, b.x, acc.x);
        acc.y = fmaf(e, b.y, acc.y);
        acc.z = fmaf(e, b.z, acc.z);
        acc.w = fmaf(e, b.w, acc.w);
    }
    reinterpret_cast<float4*>(coarse_ke + (size_t)C * 576)[t] = acc;
}

// Coloured scatter of stored element matrices into a level's FP32 values.
__global__ void k_scatter_ke(int n, const int32_t* __restrict__ elems, const int32_t* __restrict__ slot_map,
                             const float* __restrict__ ke, float* __restrict__ vals) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * 64) return;
    const int e = elems[t >> 6], pr = t & 63, a = pr >> 3, b = pr & 7;
    const int32_t slot = slot_map[(size_t)e * 64 + pr];
    const int64_t g = slot >> 5, lane = slot & 31;
    float* vb = vals + (g * 9) * 32 + lane;
    const float* K = ke + (size_t)e * 576;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) vb[(i * 3 + j) * 32] += K[(3 * a + i) * 24 + 3 * b + j];
}

// Lumped penalty of a coarse level, scaled by the penalty scale of the
// node's block (instance).
__global__ void k_add_pen(int n_rows, const int64_t* __restrict__ slice_off, const uint8_t* __restrict__ diag,
                          const float* __restrict__ pen, const int32_t* __restrict__ pre_node, int n_blk,
                          const double* __restrict__ blk_sf, float* __restrict__ vals) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    const float sf = (float)blk_sf[find_blk(pre_node, n_blk, row)];
    const int64_t g = slice_off[row >> 5] + diag[row];
    const int lane = row & 31;
#pragma unroll
    for (int a = 0; a < 3; ++a) vals[(g * 9 + a * 4) * 32 + lane] += sf * pen[3 * row + a];
}

template <typename TV>
__global__ void k_smoother_blocks(int n_rows, const int64_t* __restrict__ slice_off, const uint8_t* __restrict__ diag,
                                  const TV* __restrict__ vals, float omega, float* __restrict__ binv) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    const int64_t g = slice_off[row >> 5] + diag[row];
    const int lane = row & 31;
    double m[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) m[q] = (double)vals[(g * 9 + q) * 32 + lane];
    const double c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8], c02 = m[3] * m[7] - m[4] * m[6];
    const double id = omega / (m[0] * c00 + m[1] * c01 + m[2] * c02);
    float* B = binv + 9 * (size_t)row;
    B[0] = (float)(c00 * id);
    B[1] = (float)((m[2] * m[7] - m[1] * m[8]) * id);
    B[2] = (float)((m[1] * m[5] - m[2] * m[4]) * id);
    B[3] = (float)(c01 * id);
    B[4] = (float)((m[0] * m[8] - m[2] * m[6]) * id);
    B[5] = (float)((m[2] * m[3] - m[0] * m[5]) * id);
    B[6] = (float)(c02 * id);
    B[7] = (float)((m[1] * m[6] - m[0] * m[7]) * id);
    B[8] = (float)((m[0] * m[4] - m[1] * m[3]) * id);
}

// Coarsest level: one dense matrix per block (n_b = 3 x the block's nodes,
// at offset dense0), filled row by row (one CTA per node row), then inverted
// in place by Gauss-Jordan (SPD, no pivoting), one CTA per block.
__global__ void k_dense_build(int n_rows, const int64_t* __restrict__ slice_off, const uint8_t* __restrict__ row_len,
                              const int32_t* __restrict__ col, const float* __restrict__ vals, LevelView cv,
                              const int32_t* __restrict__ pre_node, float* __restrict__ D) {
    const int row = blockIdx.x;
    const BlkDev& d = cv.blk[find_blk(pre_node, cv.n_blk, row)];
    const int n = 3 * (d.nx + 1) * (d.ny + 1) * (d.nz + 1);
    const int lr = row - d.node0;
    if (lr >= n / 3) return;  // padding node between instances
    float* Db = D + d.dense0;
    for (int q = threadIdx.x; q < 3 * n; q += blockDim.x) Db[(size_t)(3 * lr) * n + q] = 0.f;
    __syncthreads();
    const int lane = row & 31, len = row_len[row];
    const int64_t g0 = slice_off[row >> 5];
    for (int q = threadIdx.x; q < len * 9; q += blockDim.x) {
        const int j = q / 9, v = q % 9, a = v / 3, c = v % 3;
        const int64_t g = g0 + j;
        const int cn = col[g * 32 + lane] - d.node0;
        Db[(size_t)(3 * lr + a) * n + 3 * cn + c] = vals[(g * 9 + v) * 32 + lane];
    }
}

// In-place Gauss-Jordan inverse of block blockIdx.x's matrix.  The 1024
// threads form a 32 x 32 grid; thread (ty, tx) updates the entries (ty + 32i,
// tx + 32j), so consecutive threads touch consecutive addresses and no index
// is divided.  With in_smem the matrix lives in dynamic shared memory for
// the n steps (n <= 234); otherwise it is updated in global memory.
__global__ void __launch_bounds__(1024) k_gauss_jordan(LevelView cv, float* __restrict__ Dall, int in_smem) {
    extern __shared__ float dyn[];
    __shared__ float colk[1024];
    __shared__ float rowk[1024];
    const BlkDev& d = cv.blk[blockIdx.x];
    const int n = 3 * (d.nx + 1) * (d.ny + 1) * (d.nz + 1);
    float* Ag = Dall + d.dense0;
    float* A = in_smem ? dyn : Ag;
    if (in_smem) {
        for (int q = threadIdx.x; q < n * n; q += blockDim.x) dyn[q] = Ag[q];
        __syncthreads();
    }
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int k = 0; k < n; ++k) {
        const float inv = 1.f / A[(size_t)k * n + k];
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            colk[i] = A[(size_t)i * n + k];
            rowk[i] = A[(size_t)k * n + i] * inv;
        }
        __syncthreads();
        for (int i = ty; i < n; i += 32) {
            const float ci = colk[i];
            float* Ar = A + (size_t)i * n;
            if (i == k) {
                for (int j = tx; j < n; j += 32) Ar[j] = (j == k) ? inv : rowk[j];
            } else {
                for (int j = tx; j < n; j += 32) Ar[j] = (j == k) ? -ci * inv : fmaf(-ci, rowk[j], Ar[j]);
            }
        }
        __syncthreads();
    }
    // the exact inverse is symmetric: average the FP32 rounding asymmetry out,
    // so the coarse solve (and with it the V-cycle) is a symmetric operator
    for (int q = threadIdx.x; q < n * n; q += blockDim.x) {
        const int i = q / n, j = q % n;
        if (j <= i) continue;
        const float v = 0.5f * (A[(size_t)i * n + j] + A[(size_t)j * n + i]);
        A[(size_t)i * n + j] = v;
        A[(size_t)j * n + i] = v;
    }
    __syncthreads();
    if (in_smem)
        for (int q = threadIdx.x; q < n * n; q += blockDim.x) Ag[q] = dyn[q];
}

// Blocked Gauss-Jordan inverse in shared memory (row stride ld, a multiple
// of 4), 32-column panels: for panel P (rows / columns k0..k0+kb)
//   D = A_PP^-1 (warp 0, in registers, lane = row), R = D A_P,rest (row
//   panel), A_rest,rest -= A_rest,P R, A_rest,P = -A_rest,P D, A_PP = D,
// which is the unblocked in-place elimination regrouped, so a panel costs
// four CTA barriers instead of 2 kb, and the trailing update runs as 2 x 4
// register tiles.  No pivoting: the coarse operators are SPD.
__device__ __forceinline__ void gj_panel_inverse(float* __restrict__ A, int ld, int k0, int kb, float* __restrict__ D) {
    const int lane = threadIdx.x & 31;
    float d[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) d[j] = (lane < kb && j < kb) ? A[(size_t)(k0 + lane) * ld + k0 + j] : (lane == j ? 1.f : 0.f);
#pragma unroll
    for (int p = 0; p < 32; ++p) {
        const float piv = __shfl_sync(0xffffffffu, d[p], p);
        const float inv = 1.f / piv;
        const float cp = d[p];  // this row's entry in column p
        if (lane == p) {
#pragma unroll
            for (int j = 0; j < 32; ++j) d[j] = (j == p) ? inv : d[j] * inv;
        }
        // row p (already scaled) from lane p, entry by entry; lane p keeps its row
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const float rpj = __shfl_sync(0xffffffffu, d[j], p);
            if (lane != p) d[j] = (j == p) ? -cp * inv : fmaf(-cp, rpj, d[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < 32; ++j) D[lane * 32 + j] = d[j];
}

__global__ void __launch_bounds__(1024) k_gauss_jordan_blk(LevelView cv, float* __restrict__ Dall, int ld) {
    extern __shared__ float dyn[];
    __shared__ float D[32 * 32];
    const BlkDev& dv = cv.blk[blockIdx.x];
    const int n = 3 * (dv.nx + 1) * (dv.ny + 1) * (dv.nz + 1);
    float* Ag = Dall + dv.dense0;
    float* A = dyn;
    const int t = threadIdx.x, nt = blockDim.x;
    for (int q = t; q < n * ld; q += nt) {
        const int i = q / ld, j = q % ld;
        A[q] = (j < n) ? Ag[(size_t)i * n + j] : 0.f;
    }
    __syncthreads();
    for (int k0 = 0; k0 < n; k0 += 32) {
        const int kb = min(32, n - k0);
        if (t < 32) gj_panel_inverse(A, ld, k0, kb, D);
        __syncthreads();
        // row panel: A_P,j = D A_P,j for the columns j outside the panel
        for (int j = t; j < n; j += nt) {
            if (j >= k0 && j < k0 + kb) continue;
            float a[32];
#pragma unroll
            for (int q = 0; q < 32; ++q) a[q] = (q < kb) ? A[(size_t)(k0 + q) * ld + j] : 0.f;
#pragma unroll 4
            for (int p = 0; p < kb; ++p) {
                float s = 0.f;
#pragma unroll
                for (int q = 0; q < 32; ++q) s = fmaf(D[p * 32 + q], a[q], s);
                A[(size_t)(k0 + p) * ld + j] = s;
            }
        }
        __syncthreads();
        // trailing block: A_ij -= sum_q A_iq R_qj, rows and columns outside
        // the panel, 2 x 4 tiles (columns in float4 groups; ld % 4 == 0)
        const int ncg = ld / 4, nrg = (n + 1) / 2;
        for (int tile = t; tile < nrg * ncg; tile += nt) {
            const int i0 = 2 * (tile / ncg), j0 = 4 * (tile % ncg);
            if (j0 >= n) continue;
            const bool r0 = (i0 < k0 || i0 >= k0 + kb), r1 = (i0 + 1 < n) && (i0 + 1 < k0 || i0 + 1 >= k0 + kb);
            if (!r0 && !r1) continue;
            float4 acc0 = *reinterpret_cast<const float4*>(A + (size_t)i0 * ld + j0);
            float4 acc1 = (i0 + 1 < n) ? *reinterpret_cast<const float4*>(A + (size_t)(i0 + 1) * ld + j0)
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
            for (int q = 0; q < kb; ++q) {
                const float4 rq = *reinterpret_cast<const float4*>(A + (size_t)(k0 + q) * ld + j0);
                const float a0 = A[(size_t)i0 * ld + k0 + q];
                const float a1 = (i0 + 1 < n) ? A[(size_t)(i0 + 1) * ld + k0 + q] : 0.f;
                acc0.x = fmaf(-a0, rq.x, acc0.x); acc0.y = fmaf(-a0, rq.y, acc0.y);
                acc0.z = fmaf(-a0, rq.z, acc0.z); acc0.w = fmaf(-a0, rq.w, acc0.w);
                acc1.x = fmaf(-a1, rq.x, acc1.x); acc1.y = fmaf(-a1, rq.y, acc1.y);
                acc1.z = fmaf(-a1, rq.z, acc1.z); acc1.w = fmaf(-a1, rq.w, acc1.w);
            }
            // columns of the panel keep their old values here (they are
            // rewritten below); columns beyond n stay zero
            float* o0 = A + (size_t)i0 * ld + j0;
            float* o1 = A + (size_t)(i0 + 1) * ld + j0;
            const float v0[4] = {acc0.x, acc0.y, acc0.z, acc0.w}, v1[4] = {acc1.x, acc1.y, acc1.z, acc1.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int j = j0 + c;
                if (j >= n || (j >= k0 && j < k0 + kb)) continue;
                if (r0) o0[c] = v0[c];
                if (r1) o1[c] = v1[c];
            }
        }
        __syncthreads();
        // column panel A_i,P = -A_i,P D for the rows outside the panel; the
        // diagonal block becomes D
        for (int i = t; i < n; i += nt) {
            float* Ar = A + (size_t)i * ld + k0;
            if (i >= k0 && i < k0 + kb) {
                const int p = i - k0;
                for (int q = 0; q < kb; ++q) Ar[q] = D[p * 32 + q];
                continue;
            }
            float a[32];
#pragma unroll
            for (int q = 0; q < 32; ++q) a[q] = (q < kb) ? Ar[q] : 0.f;
#pragma unroll 4
            for (int p = 0; p < kb; ++p) {
                float s = 0.f;
#pragma unroll
                for (int q = 0; q < 32; ++q) s = fmaf(a[q], D[q * 32 + p], s);
                Ar[p] = -s;
            }
        }
        __syncthreads();
    }
    // symmetrise (the exact inverse is symmetric) and store
    for (int q = t; q < n * n; q += nt) {
        const int i = q / n, j = q % n;
        Ag[q] = 0.5f * (A[(size_t)i * ld + j] + A[(size_t)j * ld + i]);
    }
}

// ---------------------------------------------------------------------------
// V-cycle kernels (all FP32; x4/y4 node-padded float4)
// ---------------------------------------------------------------------------
struct SbView {
    int n_rows;
    const int64_t* slice_off;
    const uint8_t* row_len;
    const int32_t* col;
    const float* v;
};

// Row product with three block columns in flight per step: the column
// indices, 27 values and three gathers of a step are independent loads, so
// their latencies overlap instead of forming one 27-long dependent chain.
__device__ __forceinline__ void sb_row(const SbView& A, int row, const float4* __restrict__ x, float (&y)[3]) {
    y[0] = y[1] = y[2] = 0.f;
    const int lane = row & 31;
    const int64_t g0 = A.slice_off[row >> 5];
    const int len = A.row_len[row];
    int j = 0;
    for (; j + 3 <= len; j += 3) {
        const int64_t g = g0 + j;
        int c[3];
        float m[3][9];
#pragma unroll
        for (int u = 0; u < 3; ++u) c[u] = A.col[(g + u) * 32 + lane];
#pragma unroll
        for (int u = 0; u < 3; ++u)
#pragma unroll
            for (int q = 0; q < 9; ++q) m[u][q] = A.v[((g + u) * 9 + q) * 32 + lane];
        float4 p[3];
#pragma unroll
        for (int u = 0; u < 3; ++u) p[u] = x[c[u]];
#pragma unroll
        for (int u = 0; u < 3; ++u)
#pragma unroll
            for (int a = 0; a < 3; ++a)
                y[a] = fmaf(m[u][a * 3], p[u].x, fmaf(m[u][a * 3 + 1], p[u].y, fmaf(m[u][a * 3 + 2], p[u].z, y[a])));
    }
    for (; j < len; ++j) {
        const int64_t g = g0 + j;
        const int c = A.col[g * 32 + lane];
        const float* v = A.v + (g * 9) * 32 + lane;
        const float4 p = x[c];
#pragma unroll
        for (int a = 0; a < 3; ++a)
            y[a] = fmaf(v[(a * 3) * 32], p.x, fmaf(v[(a * 3 + 1) * 32], p.y, fmaf(v[(a * 3 + 2) * 32], p.z, y[a])));
    }
}

// The share of row `row`'s product held by lane t of its T lanes (block
// columns t, t + T, ...); the T lanes of a row are consecutive threads of one
// warp and are summed by xor shuffles, which every lane of the warp executes.
template <int T>
__device__ __forceinline__ void sb_row_part(const SbView& A, int row, int t, const float4* __restrict__ x,
                                            float (&y)[3]) {
    y[0] = y[1] = y[2] = 0.f;
    const int lane = row & 31;
    const int64_t g0 = A.slice_off[row >> 5];
    const int len = A.row_len[row];
    for (int j = t; j < len; j += T) {
        const int64_t g = g0 + j;
        const int c = A.col[g * 32 + lane];
        const float* v = A.v + (g * 9) * 32 + lane;
        float m[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) m[q] = v[q * 32];
        const float4 p = x[c];
#pragma unroll
        for (int a = 0; a < 3; ++a) y[a] = fmaf(m[a * 3], p.x, fmaf(m[a * 3 + 1], p.y, fmaf(m[a * 3 + 2], p.z, y[a])));
    }
}

template <int T>
__device__ __forceinline__ void sum_lanes(float (&y)[3]) {
#pragma unroll
    for (int o = T / 2; o >= 1; o >>= 1)
#pragma unroll
        for (int a = 0; a < 3; ++a) y[a] += __shfl_xor_sync(0xffffffffu, y[a], o);
}

__global__ void k_vc_smooth0(int n, const float* __restrict__ binv, const float* __restrict__ b, float4* __restrict__ x,
                             const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    const float* B = binv + 9 * (size_t)row;
    const float b0 = b[3 * row], b1 = b[3 * row + 1], b2 = b[3 * row + 2];
    x[row] = make_float4(B[0] * b0 + B[1] * b1 + B[2] * b2, B[3] * b0 + B[4] * b1 + B[5] * b2,
                         B[6] * b0 + B[7] * b1 + B[8] * b2, 0.f);
}

__global__ void __launch_bounds__(kT) k_vc_resid(SbView A, const float* __restrict__ b, const float4* __restrict__ x,
                                                 float* __restrict__ r, const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= A.n_rows) return;
    float y[3];
    sb_row(A, row, x, y);
#pragma unroll
    for (int a = 0; a < 3; ++a) r[3 * row + a] = b[3 * row + a] - y[a];
}

// ---------------------------------------------------------------------------
// Staged FP32 level products (the finest level's residual and post-smoothing
// sweep).  As the split outer product: warp w of CTA b owns the slices
// b * W + w + j * gridDim.x * W, and the slices' FP32 values and column
// indices stream through a per-warp ring of shared-memory stages filled by
// cp.async.bulk and completed on mbarriers; the gathered x stays a plain
// load.  Per row the products are summed in the order of sb_row.
// ---------------------------------------------------------------------------
template <int G, int S>
struct F32Stage {
    static constexpr int kVal = 9 * 32;                      // floats per group
    static constexpr int kStage = G * (kVal * 4 + 32 * 4);   // bytes per stage
    static constexpr int kWarp = S * kStage;
    static constexpr int kBar = 128;
    static constexpr int smem(int threads) { return kBar + (threads / 32) * kWarp; }
    static_assert((kT / 32) * S <= kBar / 8, "one mbarrier per warp and stage must fit the barrier area");
    static_assert(kStage % 16 == 0 && (G * kVal * 4) % 16 == 0, "bulk copies need 16-byte aligned stages");
};
constexpr int kVcG = 4, kVcS = 2;  // stage shape of the finest level's products

template <int G, int S, typename Epi>
__device__ __forceinline__ bool f32_staged_slices(const SbView& A, const float4* __restrict__ x, unsigned char* smem,
                                                  Epi&& epi) {
    using St = F32Stage<G, S>;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpc = blockDim.x >> 5;
    const int n_sl = (A.n_rows + 31) >> 5;
    const int sl0 = blockIdx.x * wpc + warp, sl_step = gridDim.x * wpc;
    if (sl0 >= n_sl) return true;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem) + warp * S;
    unsigned char* ring = smem + St::kBar + warp * St::kWarp;
    int psl = sl0, pk = 0, issued = 0;
    int64_t pg0 = 0;
    int png = 0;
    auto load_slice = [&](int sl) {
        pg0 = A.slice_off[sl];
        png = (int)(A.slice_off[sl + 1] - pg0);
    };
    auto issue_next = [&]() {  // lane 0
        if (psl >= n_sl) return;
        const int s = issued % S;
        const int cnt = min(G, png - pk * G);
        const int64_t gk = pg0 + (int64_t)pk * G;
        unsigned char* st = ring + s * St::kStage;
        mbar_expect_tx(bars + s, (uint32_t)cnt * (St::kVal * 4 + 32 * 4));
        bulk_g2s(st, A.v + gk * St::kVal, cnt * St::kVal * 4, bars + s);
        bulk_g2s(st + G * St::kVal * 4, A.col + gk * 32, cnt * 32 * 4, bars + s);
        ++issued;
        if (++pk * G >= png) {
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
    int used = 0;
    bool ok = true;
    for (int sl = sl0; sl < n_sl && ok; sl += sl_step) {
        const int row = sl * 32 + lane;
        const int64_t g0 = A.slice_off[sl];
        const int ng = (int)(A.slice_off[sl + 1] - g0);
        const int len = row < A.n_rows ? A.row_len[row] : 0;
        const int nst = (ng + G - 1) / G;
        float y[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < nst; ++k) {
            const int s = used % S;
            if (!__all_sync(0xffffffffu, mbar_wait(bars + s, (uint32_t)((used / S) & 1)))) {
                ok = false;
                break;
            }
            const float* hv = reinterpret_cast<const float*>(ring + s * St::kStage);
            const int* cv = reinterpret_cast<const int*>(hv + G * St::kVal);
            const int cnt = min(G, ng - k * G);
            float4 p[G];
#pragma unroll
            for (int u = 0; u < G; ++u)
                if (u < cnt && k * G + u < len) p[u] = x[cv[u * 32 + lane]];
#pragma unroll
            for (int u = 0; u < G; ++u) {
                if (u < cnt && k * G + u < len) {
                    const float* m = hv + u * St::kVal + lane;
#pragma unroll
                    for (int a = 0; a < 3; ++a)
                        y[a] = fmaf(m[(a * 3) * 32], p[u].x,
                                    fmaf(m[(a * 3 + 1) * 32], p[u].y, fmaf(m[(a * 3 + 2) * 32], p[u].z, y[a])));
                }
            }
            ++used;
            __syncwarp();
            if (lane == 0) {
                fence_async_shared();
                issue_next();
            }
        }
        if (!ok) break;
        if (row < A.n_rows) epi(row, y);
    }
    if (!ok) {
        const int upto = __shfl_sync(0xffffffffu, issued, 0);
        if (lane == 0)
            for (int q = used; q < upto; ++q) mbar_wait(bars + q % S, (uint32_t)((q / S) & 1));
        __syncwarp();
        // poison this warp's first row: the V-cycle output turns non-finite
        // and the solve reports it
        const int row = sl0 * 32 + lane;
        if (row < A.n_rows) epi(row, {__int_as_float(0x7fc00000), 0.f, 0.f});
    }
    return ok;
}

// r = b - A x over the level's rows (staged)
__global__ void __launch_bounds__(kT) k_vc_resid_staged(SbView A, const float* __restrict__ b,
                                                        const float4* __restrict__ x, float* __restrict__ r,
                                                        const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    extern __shared__ __align__(128) unsigned char vc_smem[];
    f32_staged_slices<kVcG, kVcS>(A, x, vc_smem, [&](int row, const float (&y)[3]) {
#pragma unroll
        for (int a = 0; a < 3; ++a) r[3 * row + a] = b[3 * row + a] - y[a];
    });
}

// y4 = x + B^-1 (b - A x) over the level's rows (staged)
__global__ void __launch_bounds__(kT) k_vc_post_staged(SbView A, const float* __restrict__ binv,
                                                       const float* __restrict__ b, const float4* __restrict__ x,
                                                       float4* __restrict__ y4, const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    extern __shared__ __align__(128) unsigned char vc_smem[];
    f32_staged_slices<kVcG, kVcS>(A, x, vc_smem, [&](int row, const float (&y)[3]) {
        const float d0 = b[3 * row] - y[0], d1 = b[3 * row + 1] - y[1], d2 = b[3 * row + 2] - y[2];
        const float* B = binv + 9 * (size_t)row;
        const float4 xv = x[row];
        y4[row] = make_float4(xv.x + B[0] * d0 + B[1] * d1 + B[2] * d2, xv.y + B[3] * d0 + B[4] * d1 + B[5] * d2,
                              xv.z + B[6] * d0 + B[7] * d1 + B[8] * d2, 0.f);
    });
}

// Coarse-level variants with T lanes per row: a coarse level has too few
// rows to fill the GPU with one thread each, and a row's 27 block columns
// then form a long chain of dependent loads; T lanes split the chain.
template <int T>
__global__ void __launch_bounds__(kT) k_vc_resid_t(SbView A, const float* __restrict__ b, const float4* __restrict__ x,
                                                   float* __restrict__ r, const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = gt / T, t = gt % T;
    const bool ok = row < A.n_rows;
    float y[3] = {0.f, 0.f, 0.f};
    if (ok) sb_row_part<T>(A, row, t, x, y);
    sum_lanes<T>(y);
    if (!ok || t != 0) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) r[3 * row + a] = b[3 * row + a] - y[a];
}

template <int T>
__global__ void __launch_bounds__(kT) k_vc_post_t(SbView A, const float* __restrict__ binv, const float* __restrict__ b,
                                                  const float4* __restrict__ x, float4* __restrict__ y4,
                                                  const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = gt / T, t = gt % T;
    const bool ok = row < A.n_rows;
    float y[3] = {0.f, 0.f, 0.f};
    if (ok) sb_row_part<T>(A, row, t, x, y);
    sum_lanes<T>(y);
    if (!ok || t != 0) return;
    const float d0 = b[3 * row] - y[0], d1 = b[3 * row + 1] - y[1], d2 = b[3 * row + 2] - y[2];
    const float* B = binv + 9 * (size_t)row;
    const float4 xv = x[row];
    y4[row] = make_float4(xv.x + B[0] * d0 + B[1] * d1 + B[2] * d2, xv.y + B[3] * d0 + B[4] * d1 + B[5] * d2,
                          xv.z + B[6] * d0 + B[7] * d1 + B[8] * d2, 0.f);
}

__global__ void __launch_bounds__(kT) k_vc_post(SbView A, const float* __restrict__ binv, const float* __restrict__ b,
                                                const float4* __restrict__ x, float4* __restrict__ y4,
                                                const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= A.n_rows) return;
    float y[3];
    sb_row(A, row, x, y);
    const float d0 = b[3 * row] - y[0], d1 = b[3 * row + 1] - y[1], d2 = b[3 * row + 2] - y[2];
    const float* B = binv + 9 * (size_t)row;
    const float4 xv = x[row];
    y4[row] = make_float4(xv.x + B[0] * d0 + B[1] * d1 + B[2] * d2, xv.y + B[3] * d0 + B[4] * d1 + B[5] * d2,
                          xv.z + B[6] * d0 + B[7] * d1 + B[8] * d2, 0.f);
}

// ---------------------------------------------------------------------------
// Gradient of the V-cycle residual loss with respect to the finest-level
// smoother blocks M (learned smoother training).  With z = V(b), x2 the
// level-0 iterate before post-smoothing, q = b - A z, r2 = b - A x2,
// w = A q, t = w - A M w and v = t - A P C R t (C: coarse V-cycle,
// R = P^T), the loss ||q||^2 has dL/dM_n = -2 (v_n b_n^T + w_n r2_n^T).
// ---------------------------------------------------------------------------
// q = b - A z, r2 = b - A x2; loss += ||q||^2
__global__ void __launch_bounds__(kT) k_vl_resid(SbView A, const float* __restrict__ b, const float4* __restrict__ z,
                                                 const float4* __restrict__ x2, float4* __restrict__ q,
                                                 float* __restrict__ r2, double* __restrict__ loss) {
    __shared__ double sm[32];
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[1] = {0.0};
    if (row < A.n_rows) {
        float y[3], u[3];
        sb_row(A, row, z, y);
        sb_row(A, row, x2, u);
        const float q0 = b[3 * row] - y[0], q1 = b[3 * row + 1] - y[1], q2 = b[3 * row + 2] - y[2];
        q[row] = make_float4(q0, q1, q2, 0.f);
#pragma unroll
        for (int a = 0; a < 3; ++a) r2[3 * row + a] = b[3 * row + a] - u[a];
        acc[0] = (double)q0 * q0 + (double)q1 * q1 + (double)q2 * q2;
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0 && acc[0] != 0.0) atomicAdd(loss, acc[0]);
}

// w = A q (stored as float[3n]); mw = M w (float4)
__global__ void __launch_bounds__(kT) k_vl_w(SbView A, const float* __restrict__ M, const float4* __restrict__ q,
                                             float* __restrict__ w, float4* __restrict__ mw) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= A.n_rows) return;
    float y[3];
    sb_row(A, row, q, y);
#pragma unroll
    for (int a = 0; a < 3; ++a) w[3 * row + a] = y[a];
    const float* B = M + 9 * (size_t)row;
    mw[row] = make_float4(B[0] * y[0] + B[1] * y[1] + B[2] * y[2], B[3] * y[0] + B[4] * y[1] + B[5] * y[2],
                          B[6] * y[0] + B[7] * y[1] + B[8] * y[2], 0.f);
}

// t = w - A mw (float[3n] and float4 copies)
__global__ void __launch_bounds__(kT) k_vl_t(SbView A, const float* __restrict__ w, const float4* __restrict__ mw,
                                             float* __restrict__ t, float4* __restrict__ t4) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= A.n_rows) return;
    float y[3];
    sb_row(A, row, mw, y);
    const float t0 = w[3 * row] - y[0], t1 = w[3 * row + 1] - y[1], t2 = w[3 * row + 2] - y[2];
    t[3 * row] = t0;
    t[3 * row + 1] = t1;
    t[3 * row + 2] = t2;
    t4[row] = make_float4(t0, t1, t2, 0.f);
}

// r := r - A z (stationary multigrid iteration on residuals)
__global__ void __launch_bounds__(kT) k_vl_rstep(SbView A, const float4* __restrict__ z, float* __restrict__ r) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= A.n_rows) return;
    float y[3];
    sb_row(A, row, z, y);
#pragma unroll
    for (int a = 0; a < 3; ++a) r[3 * row + a] -= y[a];
}

// v = t - A cc (cc = P C R t); G_n += -sym(2 (v b^T + w r2^T)), G stored g00 g11 g22 g01 g02 g12
__global__ void __launch_bounds__(kT) k_vl_grad(SbView A, const float4* __restrict__ t4, const float4* __restrict__ cc,
                                                const float* __restrict__ b, const float* __restrict__ w,
                                                const float* __restrict__ r2, float* __restrict__ G) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= A.n_rows) return;
    float y[3];
    sb_row(A, row, cc, y);
    const float4 tv = t4[row];
    const float v[3] = {tv.x - y[0], tv.y - y[1], tv.z - y[2]};
    const float bb[3] = {b[3 * row], b[3 * row + 1], b[3 * row + 2]};
    const float ww[3] = {w[3 * row], w[3 * row + 1], w[3 * row + 2]};
    const float rr[3] = {r2[3 * row], r2[3 * row + 1], r2[3 * row + 2]};
    auto gij = [&](int i, int j) { return -(v[i] * bb[j] + v[j] * bb[i] + ww[i] * rr[j] + ww[j] * rr[i]); };
    float* g = G + 6 * (size_t)row;
    g[0] += gij(0, 0);
    g[1] += gij(1, 1);
    g[2] += gij(2, 2);
    g[3] += gij(0, 1);
    g[4] += gij(0, 2);
    g[5] += gij(1, 2);
}

// ---------------------------------------------------------------------------
// Smoother damping: omega = 4 / (3 lambda), lambda an estimate of the largest
// eigenvalue of D^-1 A by power iteration (D = nodal diagonal blocks), so the
// damped block-Jacobi sweep stays a contraction on elongated or strongly
// heterogeneous elements.  All on the device: step k computes
// y = D^-1 A (x / nrm[k]) and nrm[k+1] = ||y||; the last CTA of a step sums
// the per-CTA partials in CTA order (deterministic).
// ---------------------------------------------------------------------------
__global__ void k_pow_init(int n, float4* __restrict__ x, float* __restrict__ nrm, int fill) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row == 0) nrm[0] = 1.f;
    if (row >= n || !fill) return;
    auto h = [](uint32_t v) {  // integer hash -> [-1, 1)
        v ^= v >> 16; v *= 0x7feb352du; v ^= v >> 15; v *= 0x846ca68bu; v ^= v >> 16;
        return (float)(v >> 8) * (2.f / 16777216.f) - 1.f;
    };
    x[row] = make_float4(h(3u * row + 1u), h(3u * row + 2u), h(3u * row + 3u), 0.f);
}

__global__ void __launch_bounds__(kT) k_pow_step(SbView A, const float* __restrict__ dinv, const float4* __restrict__ x,
                                                 float4* __restrict__ y4, float* __restrict__ nrm, int k,
                                                 double* __restrict__ part, uint32_t* __restrict__ ticket) {
    __shared__ double sm[32];
    __shared__ bool last;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    const float inv = 1.f / nrm[k];
    double acc[1] = {0.0};
    if (row < A.n_rows) {
        float y[3];
        sb_row(A, row, x, y);
        const float* B = dinv + 9 * (size_t)row;
        const float z0 = inv * (B[0] * y[0] + B[1] * y[1] + B[2] * y[2]);
        const float z1 = inv * (B[3] * y[0] + B[4] * y[1] + B[5] * y[2]);
        const float z2 = inv * (B[6] * y[0] + B[7] * y[1] + B[8] * y[2]);
        y4[row] = make_float4(z0, z1, z2, 0.f);
        acc[0] = (double)z0 * z0 + (double)z1 * z1 + (double)z2 * z2;
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = acc[0];
        __threadfence();
        last = atomicAdd(ticket + k, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s[1] = {0.0};
#pragma unroll 4
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s[0] += __ldcg(part + b);
    block_sum<1>(s, sm);
    if (threadIdx.x == 0) nrm[k + 1] = (float)sqrt(s[0]);
}

// Guaranteed bound ||D^-1 A||_inf >= lambda_max(D^-1 A): the largest absolute
// row sum of D_n^-1 A_nm over the row's blocks (binv holds D^-1), as the
// float bits of a non-negative value under atomicMax.
__global__ void __launch_bounds__(kT) k_inf_bound(SbView A, const float* __restrict__ dinv,
                                                  unsigned int* __restrict__ bound_bits) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    float best = 0.f;
    if (row < A.n_rows) {
        const float* B = dinv + 9 * (size_t)row;
        const int lane = row & 31;
        const int64_t g0 = A.slice_off[row >> 5];
        const int len = A.row_len[row];
        float sum[3] = {0.f, 0.f, 0.f};
        for (int j = 0; j < len; ++j) {
            const float* v = A.v + ((g0 + j) * 9) * 32 + lane;
            float m[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) m[q] = v[q * 32];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b)
                    sum[a] += fabsf(B[3 * a] * m[b] + B[3 * a + 1] * m[3 + b] + B[3 * a + 2] * m[6 + b]);
        }
        best = fmaxf(sum[0], fmaxf(sum[1], sum[2]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0 && best > 0.f) atomicMax(bound_bits, __float_as_uint(best));
}

// binv := omega * binv (binv held D^-1) with omega = scale / lambda, lambda =
// the power estimate nrm[k], or the guaranteed bound when safe is set
__global__ void k_scale_blocks(int n, float* __restrict__ binv, const float* __restrict__ nrm, int k,
                               const unsigned int* __restrict__ bound_bits, int safe, float scale,
                               float* __restrict__ omega_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * n) return;
    const float est = nrm[k], bound = __uint_as_float(*bound_bits);
    float lam = safe ? bound : est;
    if (!(lam > 0.f) || !isfinite(lam)) lam = bound;
    const float omega = (lam > 0.f && isfinite(lam)) ? scale / lam : 0.5f;
    binv[i] *= omega;
    if (i == 0) *omega_out = omega;
}

// x_f[i] += sum_I w_iI y_c[I] over the fine level's nodes (a fine node outside
// every block -- padding between instances -- is left alone); cv describes
// the coarse level, pre_fnode the fine blocks' first nodes.
__device__ __forceinline__ void prolong_row(const LevelView& cv, const BlkDev& d, int f, const float4* __restrict__ yc,
                                            float4* __restrict__ xf) {
    const int fl = f - d.fnode0;
    if (fl >= (d.fnx + 1) * (d.fny + 1) * (d.fnz + 1)) return;
    const int i = fl / ((d.fny + 1) * (d.fnz + 1)), j = (fl / (d.fnz + 1)) % (d.fny + 1), k = fl % (d.fnz + 1);
    const int li = cv.lo[d.ol0 + i], lj = cv.lo[d.ol1 + j], lk = cv.lo[d.ol2 + k];
    const float wi = cv.w[d.ol0 + i], wj = cv.w[d.ol1 + j], wk = cv.w[d.ol2 + k];
    float4 acc = xf[f];
#pragma unroll
    for (int di = 0; di < 2; ++di) {
        const float a = di ? wi : 1.f - wi;
        if (a == 0.f) continue;
#pragma unroll
        for (int dj = 0; dj < 2; ++dj) {
            const float b = dj ? wj : 1.f - wj;
            if (b == 0.f) continue;
#pragma unroll
            for (int dk = 0; dk < 2; ++dk) {
                const float c = dk ? wk : 1.f - wk;
                if (c == 0.f) continue;
                const float4 y = yc[d.node0 + nid(li + di, lj + dj, lk + dk, d.ny, d.nz)];
                const float ww = a * b * c;
                acc.x += ww * y.x;
                acc.y += ww * y.y;
                acc.z += ww * y.z;
            }
        }
    }
    xf[f] = acc;
}

__global__ void k_vc_prolong(LevelView cv, const int32_t* __restrict__ pre_fnode, int n_fine,
                             const float4* __restrict__ yc, float4* __restrict__ xf, const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_fine) return;
    prolong_row(cv, cv.blk[find_blk(pre_fnode, cv.n_blk, f)], f, yc, xf);
}

// Coarsest solve y = A_b^-1 b per block (CTA = block): one warp per row,
// lanes stride the row (coalesced), shuffle reduction.  y is node-padded.
// sb: shared staging of the block's b (at least n floats); the CTA's threads
// all call this (it synchronises them).
__device__ __forceinline__ void dense_block(const BlkDev& d, const float* __restrict__ ainv, const float* __restrict__ b,
                                            float* __restrict__ y4, float* sb) {
    const int n = 3 * (d.nx + 1) * (d.ny + 1) * (d.nz + 1);
    const float* bb = b + 3 * (size_t)d.node0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) sb[i] = bb[i];
    __syncthreads();
    const float* Ab = ainv + d.dense0;
    float* yb = y4 + 4 * (size_t)d.node0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    // eight loads per lane issued together (a 256-wide row in one pass): the
    // row's loads overlap instead of waiting on each other
    for (int row = warp; row < n; row += nw) {
        const float* ar = Ab + (size_t)row * n;
        float acc = 0.f;
        for (int j0 = 0; j0 < n; j0 += 256) {
            float a[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int j = j0 + lane + 32 * t;
                a[t] = j < n ? ar[j] : 0.f;
            }
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int j = j0 + lane + 32 * t;
                if (j < n) acc = fmaf(a[t], sb[j], acc);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) yb[4 * (row / 3) + row % 3] = acc;
    }
}

__global__ void __launch_bounds__(1024) k_vc_dense(LevelView cv, const float* __restrict__ ainv,
                                                   const float* __restrict__ b, float* __restrict__ y4,
                                                   const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    __shared__ float sb[1024];
    dense_block(cv.blk[blockIdx.x], ainv, b, y4, sb);
}

// Trilinear restriction R = P^T over every block at once, one coarse node per
// thread: b_c[m] = sum over the fine nodes f of w_x w_y w_z r_f, where along
// each axis the fine nodes between xs[m-1] and xs[m+1] contribute with the
// prolongation weight of m (1 - w on the node's lower coarse neighbour, w on
// the upper one).  The coarse level's first smoothing sweep x4 = B^-1 b is
// fused in (binv non-null).
// The taps of coarse node m on one axis: fine nodes xs[m] - 1, xs[m] and
// xs[m] + 1, each present when it lies strictly between xs[m - 1] and
// xs[m + 1] (coarse spacing is one or two fine cells, so no other fine node
// has a non-zero weight); weights w[xs[m] - 1], 1 and 1 - w[xs[m] + 1], the
// prolongation weights of m.  Fixed slots keep the taps in registers and let
// the 27 loads of a coarse node issue together.
struct Taps {
    int f[3];
    float w[3];
    bool on[3];
};
__device__ __forceinline__ Taps axis_taps(const int32_t* __restrict__ xs, const float* __restrict__ w, int m,
                                          int n_c) {
    Taps t;
    const int x = xs[m];
    t.on[0] = m > 0 && x - 1 > xs[m - 1];
    t.on[1] = true;
    t.on[2] = m < n_c && x + 1 < xs[m + 1];
    t.f[0] = t.on[0] ? x - 1 : x;  // an absent tap points at x: every address formed stays in range
    t.f[1] = x;
    t.f[2] = t.on[2] ? x + 1 : x;
    t.w[0] = t.on[0] ? w[x - 1] : 0.f;
    t.w[1] = 1.f;
    t.w[2] = t.on[2] ? 1.f - w[x + 1] : 0.f;
    return t;
}

__device__ __forceinline__ void restrict_row(const LevelView& cv, const BlkDev& d, int o, const float* __restrict__ in,
                                             float* __restrict__ out, const float* __restrict__ binv,
                                             float4* __restrict__ x4) {
    const int ol = o - d.node0;
    const int i0 = ol / ((d.ny + 1) * (d.nz + 1)), i1 = (ol / (d.nz + 1)) % (d.ny + 1), i2 = ol % (d.nz + 1);
    const Taps tx = axis_taps(cv.xs + d.ox0, cv.w + d.ol0, i0, d.nx);
    const Taps ty = axis_taps(cv.xs + d.ox1, cv.w + d.ol1, i1, d.ny);
    const Taps tz = axis_taps(cv.xs + d.ox2, cv.w + d.ol2, i2, d.nz);
    float v[3][3][3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const bool on = tx.on[a] && ty.on[b] && tz.on[c];
                const size_t src = 3 * (size_t)(d.fnode0 + (tx.f[a] * (d.fny + 1) + ty.f[b]) * (d.fnz + 1) + tz.f[c]);
#pragma unroll
                for (int q = 0; q < 3; ++q) v[a][b][c][q] = on ? in[src + q] : 0.f;
            }
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const float wab = tx.w[a] * ty.w[b];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (!(tx.on[a] && ty.on[b] && tz.on[c])) continue;
                const float ww = wab * tz.w[c];
                s0 = fmaf(ww, v[a][b][c][0], s0);
                s1 = fmaf(ww, v[a][b][c][1], s1);
                s2 = fmaf(ww, v[a][b][c][2], s2);
            }
        }
    out[3 * (size_t)o] = s0;
    out[3 * (size_t)o + 1] = s1;
    out[3 * (size_t)o + 2] = s2;
    if (binv) {
        const float* B = binv + 9 * (size_t)o;
        x4[o] = make_float4(B[0] * s0 + B[1] * s1 + B[2] * s2, B[3] * s0 + B[4] * s1 + B[5] * s2,
                            B[6] * s0 + B[7] * s1 + B[8] * s2, 0.f);
    }
}

__global__ void __launch_bounds__(kT) k_vc_restrict(LevelView cv, const int32_t* __restrict__ pre_node, int n_out,
                                                    const float* __restrict__ in, float* __restrict__ out,
                                                    const float* __restrict__ binv, float4* __restrict__ x4,
                                                    const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n_out) return;
    restrict_row(cv, cv.blk[find_blk(pre_node, cv.n_blk, o)], o, in, out, binv, x4);
}

// ---------------------------------------------------------------------------
// Fused coarse tail of the V-cycle.  Below a size threshold every level of an
// instance fits one CTA, and an instance's rows couple only to its own rows
// on every level (the stacked operator is block diagonal), so one CTA per
// block runs the tail's residuals, restrictions, the coarsest dense solve,
// prolongations and post-smoothing in sequence with CTA barriers between the
// steps, in place of a dozen small grid-wide launches whose latency, not
// their few hundred kilobytes, set their time.  Per row the arithmetic and
// its order are those of the separate kernels (same lanes per row).
// ---------------------------------------------------------------------------
constexpr int kMaxTail = 8;       // levels a fused tail may hold
constexpr int kTailNodes = 512;   // largest block (nodes) of a level in the tail
constexpr int kTailThreads = 1024;
constexpr int kTailMinBlocks = 16;  // instances a stack needs before its tail is fused

struct TailLevel {
    SbView A;
    LevelView V;   // blocks of this level (with their finer blocks' maps)
    const float* binv;
    float* b;
    float* r;
    float4* x4;
    float4* y4;
    int lanes;     // lanes per row of this level's products (as the separate kernels)
};
struct TailArgs {
    int n_lev;     // levels lt .. nl - 1; the last one is solved by its dense inverse
    TailLevel L[kMaxTail];
    const float* ainv;
};

// r = b - A x (post == false) or y = x + B^-1 (b - A x) (post == true) over
// the rows [row0, row0 + nn) of one block, T lanes per row.
template <int T>
__device__ __forceinline__ void tail_rows(const TailLevel& L, int row0, int nn, bool post) {
    const int tot = nn * T;
    const float4* x = L.x4;
    for (int base = 0; base < tot; base += blockDim.x) {  // same trip count in every thread
        const int gt = base + threadIdx.x;
        const int row = row0 + gt / T, t = gt % T;
        const bool ok = gt < tot;
        float y[3] = {0.f, 0.f, 0.f};
        if (ok) sb_row_part<T>(L.A, row, t, x, y);
        sum_lanes<T>(y);
        if (!ok || t != 0) continue;
        if (!post) {
#pragma unroll
            for (int a = 0; a < 3; ++a) L.r[3 * row + a] = L.b[3 * row + a] - y[a];
        } else {
            const float d0 = L.b[3 * row] - y[0], d1 = L.b[3 * row + 1] - y[1], d2 = L.b[3 * row + 2] - y[2];
            const float* B = L.binv + 9 * (size_t)row;
            const float4 xv = x[row];
            L.y4[row] = make_float4(xv.x + B[0] * d0 + B[1] * d1 + B[2] * d2, xv.y + B[3] * d0 + B[4] * d1 + B[5] * d2,
                                    xv.z + B[6] * d0 + B[7] * d1 + B[8] * d2, 0.f);
        }
    }
}
__device__ __forceinline__ void tail_level_rows(const TailLevel& L, int row0, int nn, bool post) {
    switch (L.lanes) {
        case 1: tail_rows<1>(L, row0, nn, post); break;
        case 2: tail_rows<2>(L, row0, nn, post); break;
        case 4: tail_rows<4>(L, row0, nn, post); break;
        case 8: tail_rows<8>(L, row0, nn, post); break;
        default: tail_rows<16>(L, row0, nn, post); break;
    }
}

__global__ void __launch_bounds__(kTailThreads) k_vc_tail(TailArgs ta, const Control* ctl) {
    pdl_begin();
    if (ctl && ctl->all_done) return;
    __shared__ float sb[1024];
    const int b = blockIdx.x;
    const int nl = ta.n_lev;
    auto nodes = [](const BlkDev& d) { return (d.nx + 1) * (d.ny + 1) * (d.nz + 1); };
    for (int l = 0; l + 1 < nl; ++l) {
        const BlkDev& d = ta.L[l].V.blk[b];
        tail_level_rows(ta.L[l], d.node0, nodes(d), false);
        __syncthreads();
        const TailLevel& C = ta.L[l + 1];
        const BlkDev& dc = C.V.blk[b];
        const bool last = (l + 2 == nl);  // the coarsest level takes no smoothing sweep
        for (int q = threadIdx.x; q < nodes(dc); q += blockDim.x)
            restrict_row(C.V, dc, dc.node0 + q, ta.L[l].r, C.b, last ? nullptr : C.binv, C.x4);
        __syncthreads();
    }
    dense_block(ta.L[nl - 1].V.blk[b], ta.ainv, ta.L[nl - 1].b, reinterpret_cast<float*>(ta.L[nl - 1].y4), sb);
    __syncthreads();
    for (int l = nl - 2; l >= 0; --l) {
        const TailLevel& C = ta.L[l + 1];
        const BlkDev& dc = C.V.blk[b];
        const int nf = (dc.fnx + 1) * (dc.fny + 1) * (dc.fnz + 1);
        for (int q = threadIdx.x; q < nf; q += blockDim.x) prolong_row(C.V, dc, dc.fnode0 + q, C.y4, ta.L[l].x4);
        __syncthreads();
        const BlkDev& d = ta.L[l].V.blk[b];
        tail_level_rows(ta.L[l], d.node0, nodes(d), true);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// multigrid-preconditioned flexible CG kernels (one right-hand side; every
// instance of a batched stack at once, with its own scalars and tickets)
// ---------------------------------------------------------------------------
struct MgPcg {
    PcgArgs a;            // outer operator, x, r, p, ap, partials, sc, ctl (nrhs = 1)
    float4* xp;           // split method: the correction e of x since its last true residual,
                          // node-padded FP32 pairs (hi float4, lo float4)
    float4* xt;           // split method on a split-only operator: x as three node-padded FP32
                          // parts (hi, lo, remainder) for the true residual (else nullptr)
    float* b0;            // V-cycle input (level-0 rhs, FP32 r)
    const float4* z;      // V-cycle output (level-0 y4)
    const float* binv0;   // level-0 smoother blocks: the first sweep
    float4* x40;          // x4 = B^-1 r is fused into the kernels writing b0
    int n_inst;           // instances (1: a single model)
};

// Instances still iterating are counted in ctl->pad[0]; the one whose
// recurrence converges last sets all_done, which ends every kernel of the
// remaining captured iterations at once.
__device__ __forceinline__ void retire_instance(const PcgArgs& A) {
    if (atomicSub(&A.ctl->pad[0], 1) == 1) A.ctl->all_done = 1;
}

// First kernel of a captured chunk of iterations: count the instances not
// done (all_done when none is left).
__global__ void k_mg_count_active(MgPcg M) {
    pdl_begin();
    const PcgArgs& A = M.a;
    int n = 0;
    for (int i = threadIdx.x; i < M.n_inst; i += blockDim.x) n += A.sc[(size_t)i * kMaxRhs].done ? 0 : 1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    if (threadIdx.x == 0) {
        A.ctl->pad[0] = n;
        A.ctl->all_done = (n == 0) ? 1 : 0;
    }
}

__device__ __forceinline__ void fused_smooth0(const MgPcg& M, int row, const double (&r)[3]) {
    const float* B = M.binv0 + 9 * (size_t)row;
    const float r0 = (float)r[0], r1 = (float)r[1], r2 = (float)r[2];
    M.x40[row] = make_float4(B[0] * r0 + B[1] * r1 + B[2] * r2, B[3] * r0 + B[4] * r1 + B[5] * r2,
                             B[6] * r0 + B[7] * r1 + B[8] * r2, 0.f);
}

template <typename TV, typename TP>
__global__ void __launch_bounds__(kThreads) k_mg_spmv_dot(MgPcg M) {
    using PV = typename ApOf<TP>::T;
    const PcgArgs& A = M.a;
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (cta_done<1>(A, S)) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    double d[1][1] = {{0.0}};
    if (row < A.n_rows) {
        PV y[1][3];
        const TV* vals;
        if constexpr (sizeof(TV) == 4) vals = A.v32; else vals = A.v64;
        spmv_row<TV, TP, 1>(row, A, vals, A.p, y);
        PV pv[3];
        PadVec<TP>::load(A.p, row, pv);
        PV* ap = reinterpret_cast<PV*>(A.ap) + 3 * (size_t)row;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            ap[q] = y[0][q];
            d[0][0] += (double)pv[q] * (double)y[0][q];
        }
    }
    double tot[1][1];
    if (last_block_reduce<1, 1>(A, d, 0, tot) && threadIdx.x == 0) {
        RhsScalars& s = S[0];
        s.pAp = tot[0][0];
        s.alpha = s.rz / s.pAp;
    }
}

// ---------------------------------------------------------------------------
// Split method, vector side: the correction e of x (node-padded), r and A p
// (natural layout) are FP32 pairs and every per-row update and dot product is
// pair arithmetic on the FP32 pipes; FP64 is left to the per-CTA reductions
// (one value per thread), the scalars, and the true residuals (x64 += e, then
// r = f - A64 x64), formed two or three times per solve.
// ---------------------------------------------------------------------------
__device__ __forceinline__ F2 ld_pair(const float2* v, size_t i) {
    const float2 q = v[i];
    return {q.x, q.y};
}
__device__ __forceinline__ void st_pair(float2* v, size_t i, F2 a) { v[i] = make_float2(a.h, a.l); }
__device__ __forceinline__ void ld_pad_pair(const void* p, size_t node, F2 (&v)[3]) {
    const float4 h = reinterpret_cast<const float4*>(p)[2 * node];
    const float4 l = reinterpret_cast<const float4*>(p)[2 * node + 1];
    v[0] = {h.x, l.x};
    v[1] = {h.y, l.y};
    v[2] = {h.z, l.z};
}
__device__ __forceinline__ void st_pad_pair(void* p, size_t node, const F2 (&v)[3]) {
    reinterpret_cast<float4*>(p)[2 * node] = make_float4(v[0].h, v[1].h, v[2].h, 0.f);
    reinterpret_cast<float4*>(p)[2 * node + 1] = make_float4(v[0].l, v[1].l, v[2].l, 0.f);
}

// Store A p of this row (pairs) and return p . A p over the row's 3 DOF (a
// pair: a thread sums its rows in pairs and converts to FP64 once).
__device__ __forceinline__ F2 pair_ap_dot(const PcgArgs& A, int row, const F2 (&y)[3]) {
    F2 pv[3];
    ld_pad_pair(A.p, row, pv);
    float2* ap = reinterpret_cast<float2*>(A.ap);
    F2 acc{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        st_pair(ap, 3 * (size_t)row + q, y[q]);
        acc = f2_add(acc, f2_mul(pv[q], y[q]));
    }
    return acc;
}

__device__ __forceinline__ void set_alpha(RhsScalars& s, double pAp) {
    s.pAp = pAp;
    s.alpha = s.rz / s.pAp;
    const F2 a = f2_of(s.alpha);
    s.alpha2[0] = a.h;
    s.alpha2[1] = a.l;
}

// The register-fed split product with the pair epilogue.
__global__ void __launch_bounds__(kThreads) k_mg_spmv_dot_pair(MgPcg M) {
    pdl_begin();
    const PcgArgs& A = M.a;
    RhsScalars* Sc = A.sc + cta_instance(A) * kMaxRhs;
    if (cta_done<1>(A, Sc)) return;
    F2 acc{0.f, 0.f};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n_rows; row += gridDim.x * blockDim.x) {
        float Sm[1][3], Cc[1][3];
        spmv_row_split_sc<1>(row, A, A.p, Sm, Cc);
        const F2 y[3] = {two_sum(Sm[0][0], Cc[0][0]), two_sum(Sm[0][1], Cc[0][1]), two_sum(Sm[0][2], Cc[0][2])};
        acc = f2_add(acc, pair_ap_dot(A, row, y));
    }
    double d[1][1] = {{f2_dbl(acc)}};
    double tot[1][1];
    if (last_block_reduce<1, 1>(A, d, 0, tot) && threadIdx.x == 0) set_alpha(Sc[0], tot[0][0]);
}

// The split method iterates on x = x64 + e: x64 (FP64) changes only when a
// true residual is formed, and the correction e gathered since then is an
// FP32 pair.  Folding e into x64 there (and at the end) keeps the stored
// solution in FP64, so the pairs' 48-bit rounding of e stays far below the
// solve's tolerance (x itself as a pair left a noise floor near 1e-9).
__global__ void k_zero_pairs(int n, float4* __restrict__ e) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 2 * n) e[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// x64 += e, e = 0 for the instances whose true residual is formed next (all
// rows when all is set)
__global__ void __launch_bounds__(kThreads) k_fold_pairs(MgPcg M, int all) {
    pdl_begin();
    const PcgArgs& A = M.a;
    const RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (!all && !S[0].replace) return;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n_rows; row += gridDim.x * blockDim.x) {
        F2 e[3];
        ld_pad_pair(M.xp, row, e);
        float t[3][3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double xv = A.x[3 * (size_t)row + q] + f2_dbl(e[q]);
            A.x[3 * (size_t)row + q] = xv;
            if (M.xt) {  // x = hi + lo + remainder, each FP32
                const float h = (float)xv;
                const double r1 = xv - (double)h;
                const float l = (float)r1;
                t[0][q] = h;
                t[1][q] = l;
                t[2][q] = (float)(r1 - (double)l);
            }
        }
        const F2 z[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
        st_pad_pair(M.xp, row, z);
        if (M.xt)
#pragma unroll
            for (int k = 0; k < 3; ++k) M.xt[3 * (size_t)row + k] = make_float4(t[k][0], t[k][1], t[k][2], 0.f);
    }
}

// One term (h + l)(xh + xl + xr) of a true residual, added to a three-level
// sum (S, C, D): S the leading sum, C the next order, D the rest.  The
// products h xh, h xl and l xh are split exactly (FMA) and every rounding
// error of S and C goes one level down, so only D rounds, at 2^-24 of a
// 2^-48-sized quantity: the sum keeps about 70 bits, where the CG product's
// two levels keep 48 (enough for a search direction, not for f - A x, whose
// terms are 10^4 times |f| on a point-loaded cantilever).
__device__ __forceinline__ void res_term(float h, float l, float xh, float xl, float xr, float& S, float& C,
                                         float& D) {
    const float p1 = __fmul_rn(h, xh), e1 = __fmaf_rn(h, xh, -p1);
    const float p2 = __fmul_rn(h, xl), e2 = __fmaf_rn(h, xl, -p2);
    const float p3 = __fmul_rn(l, xh), e3 = __fmaf_rn(l, xh, -p3);
    const F2 s0 = two_sum(S, p1);
    S = s0.h;
    const F2 c1 = two_sum(C, s0.l);
    const F2 c2 = two_sum(c1.h, e1);
    const F2 c3 = two_sum(c2.h, p2);
    const F2 c4 = two_sum(c3.h, p3);
    C = c4.h;
    D = __fadd_rn(D, __fadd_rn(__fadd_rn(c1.l, c2.l), __fadd_rn(c3.l, c4.l)));
    D = __fadd_rn(D, __fadd_rn(e2, e3));
    D = __fmaf_rn(h, xr, __fmaf_rn(l, xl, D));
}

// True residual r = f - A x from the operator's hi / lo values (split-only
// assembly: no FP64 values) and the three FP32 parts of x written by the
// fold, each term by res_term.
__global__ void __launch_bounds__(kThreads) k_mg_residual_split(MgPcg M, int init, double tol2) {
    pdl_begin();
    const PcgArgs& A = M.a;
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (!init && !S[0].replace) return;
    F2 rr{0.f, 0.f};
    double ff = 0.0;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n_rows; row += gridDim.x * blockDim.x) {
        const int lane = row & 31;
        float Sm[3] = {0.f, 0.f, 0.f}, Cc[3] = {0.f, 0.f, 0.f}, Dd[3] = {0.f, 0.f, 0.f};
        const int64_t g0 = A.slice_off[row >> 5];
        const int len = A.row_len[row];
        for (int j = 0; j < len; ++j) {
            const int64_t g = g0 + j;
            const int c = A.col[g * 32 + lane];
            const float4 xh = M.xt[3 * (size_t)c], xl = M.xt[3 * (size_t)c + 1], xr = M.xt[3 * (size_t)c + 2];
            const float* hv = A.v32 + (g * 9) * 32 + lane;
            const float* lv = A.v32lo + (g * 9) * 32 + lane;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                res_term(hv[(3 * a) * 32], lv[(3 * a) * 32], xh.x, xl.x, xr.x, Sm[a], Cc[a], Dd[a]);
                res_term(hv[(3 * a + 1) * 32], lv[(3 * a + 1) * 32], xh.y, xl.y, xr.y, Sm[a], Cc[a], Dd[a]);
                res_term(hv[(3 * a + 2) * 32], lv[(3 * a + 2) * 32], xh.z, xl.z, xr.z, Sm[a], Cc[a], Dd[a]);
            }
        }
        float2* r = reinterpret_cast<float2*>(A.r);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const size_t o = 3 * (size_t)row + a;
            const double f = A.f[o];
            // f - (S + C + D): the leading cancellation against f is exact in
            // the pairs' TwoSum; C and D enter below it
            const F2 y = f2_add(two_sum(Sm[a], Cc[a]), F2{Dd[a], 0.f});
            const F2 rv = f2_add(f2_of(f), f2_neg(y));
            st_pair(r, o, rv);
            M.b0[o] = rv.h;
            rr = f2_add(rr, f2_mul(rv, rv));
            if (init) ff += f * f;
        }
    }
    double d[1][2] = {{f2_dbl(rr), ff}};
    double tot[1][2];
    if (last_block_reduce<1, 2>(A, d, 3, tot) && threadIdx.x == 0) {
        RhsScalars& s = S[0];
        s.rr = tot[0][0];
        s.rr_last_true = tot[0][0];
        if (init) {
            s.bb = tot[0][1];
            s.target = tol2 * s.bb;
            s.iter = 0;
            s.beta = 0.0;
            s.restart = 1;
        }
        s.replace = 0;
        s.refresh = 1;
        s.nonfinite = isfinite(s.rr) ? 0 : 1;
        s.finished = (s.rr <= s.target) || s.nonfinite;
        s.done = s.finished;
    }
}

// e += alpha p, r -= alpha A p, b0 = r (FP32), |r|^2, and the level-0 first
// smoothing sweep.
__global__ void __launch_bounds__(kThreads) k_mg_update_xr_pair(MgPcg M) {
    pdl_begin();
    const PcgArgs& A = M.a;
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (cta_done<1>(A, S)) return;
    F2 rr{0.f, 0.f};
    const F2 alpha{S[0].alpha2[0], S[0].alpha2[1]};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n_rows; row += gridDim.x * blockDim.x) {
        F2 pv[3], xv[3];
        ld_pad_pair(A.p, row, pv);
        ld_pad_pair(M.xp, row, xv);
        const float2* ap = reinterpret_cast<const float2*>(A.ap);
        float2* r = reinterpret_cast<float2*>(A.r);
        float rf[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const size_t o = 3 * (size_t)row + q;
            xv[q] = f2_add(xv[q], f2_mul(alpha, pv[q]));
            const F2 rv = f2_add(ld_pair(r, o), f2_neg(f2_mul(alpha, ld_pair(ap, o))));
            st_pair(r, o, rv);
            M.b0[o] = rv.h;
            rf[q] = rv.h;
            rr = f2_add(rr, f2_mul(rv, rv));
        }
        st_pad_pair(M.xp, row, xv);
        const float* B = M.binv0 + 9 * (size_t)row;
        M.x40[row] = make_float4(B[0] * rf[0] + B[1] * rf[1] + B[2] * rf[2], B[3] * rf[0] + B[4] * rf[1] + B[5] * rf[2],
                                 B[6] * rf[0] + B[7] * rf[1] + B[8] * rf[2], 0.f);
    }
    double d[1][1] = {{f2_dbl(rr)}};
    double tot[1][1];
    if (last_block_reduce<1, 1>(A, d, 1, tot) && threadIdx.x == 0) {
        RhsScalars& s = S[0];
        s.rr = tot[0][0];
        s.iter += 1;
        if (!isfinite(s.rr)) {
            s.nonfinite = 1;
            s.done = 1;
        } else if (s.rr <= s.target) {
            s.done = 1;
            s.restart = 1;  // this iteration's p update is skipped
        }
        if (s.done) retire_instance(A);
    }
}

// r . z and (mode 0) A p . z in pairs, beta (Polak-Ribiere); mode 1: rz
// after a true-residual evaluation, and p = z on a restart.
__global__ void __launch_bounds__(kThreads) k_mg_rz_pair(MgPcg M, int mode) {
    pdl_begin();
    const PcgArgs& A = M.a;
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (mode == 0 && cta_done<1>(A, S)) return;
    if (mode == 1 && !S[0].refresh) return;
    const bool restart = mode == 1 && S[0].restart;
    F2 a0{0.f, 0.f}, a1{0.f, 0.f};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n_rows; row += gridDim.x * blockDim.x) {
        const float4 z = M.z[row];
        const float zz[3] = {z.x, z.y, z.z};
        const float2* r = reinterpret_cast<const float2*>(A.r);
        const float2* ap = reinterpret_cast<const float2*>(A.ap);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const size_t o = 3 * (size_t)row + q;
            a0 = f2_add(a0, f2_mul_f(ld_pair(r, o), zz[q]));
            if (mode == 0) a1 = f2_add(a1, f2_mul_f(ld_pair(ap, o), zz[q]));
        }
        if (restart) {
            const F2 pz[3] = {{zz[0], 0.f}, {zz[1], 0.f}, {zz[2], 0.f}};
            st_pad_pair(A.p, row, pz);
        }
    }
    double d[1][2] = {{f2_dbl(a0), f2_dbl(a1)}};
    double tot[1][2];
    if (last_block_reduce<1, 2>(A, d, 2, tot) && threadIdx.x == 0) {
        RhsScalars& s = S[0];
        if (mode == 0) {
            s.beta = -s.alpha * tot[0][1] / s.rz;
            const F2 b = f2_of(s.beta);
            s.beta2[0] = b.h;
            s.beta2[1] = b.l;
        }
        s.rz = tot[0][0];
        if (mode == 1) {
            s.refresh = 0;
            s.restart = 0;
        }
        if (!isfinite(s.rz)) {
            s.nonfinite = 1;
            if (!s.done) {
                s.done = 1;
                if (mode == 0) retire_instance(A);
            }
            s.finished = 1;
        }
    }
}

// p = z + beta p in pairs
__global__ void __launch_bounds__(kThreads) k_mg_update_p_pair(MgPcg M) {
    pdl_begin();
    const PcgArgs& A = M.a;
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (cta_done<1>(A, S)) return;
    const F2 beta{S[0].beta2[0], S[0].beta2[1]};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n_rows; row += gridDim.x * blockDim.x) {
        const float4 z = M.z[row];
        F2 pv[3];
        ld_pad_pair(A.p, row, pv);
        pv[0] = f2_add(f2_mul(beta, pv[0]), F2{z.x, 0.f});
        pv[1] = f2_add(f2_mul(beta, pv[1]), F2{z.y, 0.f});
        pv[2] = f2_add(f2_mul(beta, pv[2]), F2{z.z, 0.f});
        st_pad_pair(A.p, row, pv);
    }
}

// The split product with its values and columns staged through shared memory
// by bulk copies (spmv_row_split_staged): same rows per CTA, same results and
// the same pair epilogue and p.Ap reduction as k_mg_spmv_dot_pair.  A warp whose
// copies time out makes its rows' contribution NaN, which the solve reports
// as a non-finite breakdown.
template <int G, int S>
__global__ void __launch_bounds__(kThreads) k_mg_spmv_dot_staged(MgPcg M) {
    pdl_begin();
    extern __shared__ __align__(128) unsigned char st_smem[];
    const PcgArgs& A = M.a;
    RhsScalars* Sc = A.sc + cta_instance(A) * kMaxRhs;
    if (cta_done<1>(A, Sc)) return;
    F2 acc{0.f, 0.f};
    const bool ok = split_staged_slices<G, S>(
        A, A.p, st_smem, [&](int row, const F2 (&y)[3]) { acc = f2_add(acc, pair_ap_dot(A, row, y)); });
    double d[1][1] = {{f2_dbl(acc)}};
    if (!ok) d[0][0] = __longlong_as_double(0x7ff8000000000000ll);
    double tot[1][1];
    if (last_block_reduce<1, 1>(A, d, 0, tot) && threadIdx.x == 0) set_alpha(Sc[0], tot[0][0]);
}

// Launch of the split outer product in one of its shapes (ASEND_PRODUCT_*):
// register-fed, or staged with G groups per stage and S stages per warp.
template <int G, int S>
void launch_staged(const Ctx& c, const MgPcg& M, int grid) {
    launch_k(c, k_mg_spmv_dot_staged<G, S>, grid, kThreads, SplitStage<G, S>::smem(kThreads), M);
}

// Opt the staged shapes into their dynamic shared memory (above the 48 KB
// default) on the current device; called outside stream capture.
template <int G, int S>
void staged_attr() {
    ASEND_CUDA(cudaFuncSetAttribute(k_mg_spmv_dot_staged<G, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    SplitStage<G, S>::smem(kThreads)));
}
void product_attrs() {
    static bool done[64] = {};
    int dev = 0;
    ASEND_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && done[dev]) return;
    staged_attr<2, 3>();
    staged_attr<3, 2>();
    staged_attr<2, 2>();
    staged_attr<4, 2>();
    if (dev >= 0 && dev < 64) done[dev] = true;
}

void launch_split_product(const Ctx& c, const MgPcg& M, int grid) {
    switch (c.product_variant) {
        case ASEND_PRODUCT_REGISTERS: launch_k(c, k_mg_spmv_dot_pair, grid, kThreads, 0, M); break;
        case ASEND_PRODUCT_STAGED_3x2: launch_staged<3, 2>(c, M, grid); break;
        case ASEND_PRODUCT_STAGED_2x2: launch_staged<2, 2>(c, M, grid); break;
        case ASEND_PRODUCT_STAGED_4x2: launch_staged<4, 2>(c, M, grid); break;
        default: launch_staged<2, 3>(c, M, grid); break;  // ASEND_PRODUCT_DEFAULT, ASEND_PRODUCT_STAGED_2x3
    }
}

template <typename TP>
__global__ void __launch_bounds__(kThreads) k_mg_update_xr(MgPcg M) {
    using PV = typename ApOf<TP>::T;
    const PcgArgs& A = M.a;
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (cta_done<1>(A, S)) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    double d[1][1] = {{0.0}};
    if (row < A.n_rows) {
        const double alpha = S[0].alpha;
        PV pv[3];
        PadVec<TP>::load(A.p, row, pv);
        const PV* ap = reinterpret_cast<const PV*>(A.ap) + 3 * (size_t)row;
        double rr[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const size_t o = 3 * (size_t)row + q;
            A.x[o] += alpha * (double)pv[q];
            const double rv = A.r[o] - alpha * (double)ap[q];
            A.r[o] = rv;
            M.b0[o] = (float)rv;
            rr[q] = rv;
            d[0][0] += rv * rv;
        }
        fused_smooth0(M, row, rr);
    }
    double tot[1][1];
    if (last_block_reduce<1, 1>(A, d, 1, tot) && threadIdx.x == 0) {
        RhsScalars& s = S[0];
        s.rr = tot[0][0];
        s.iter += 1;
        if (!isfinite(s.rr)) {
            s.nonfinite = 1;
            s.done = 1;
        } else if (s.rr <= s.target) {
            s.done = 1;
            s.restart = 1;  // this iteration's p update is skipped
        }
        if (s.done) retire_instance(A);
    }
}

// mode 0: after an iteration's V-cycle -> beta (Polak-Ribiere), rz
// mode 1: start of the solve, or after a true-residual evaluation: for every
//         instance whose refresh flag is set, rz, and p = z when its restart
//         flag is set (initialisation, or convergence of the recurrence)
template <typename TP>
__global__ void __launch_bounds__(kThreads) k_mg_rz(MgPcg M, int mode) {
    using PV = typename ApOf<TP>::T;
    const PcgArgs& A = M.a;
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (mode == 0 && cta_done<1>(A, S)) return;
    if (mode == 1 && !S[0].refresh) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    double d[1][2] = {{0.0, 0.0}};
    if (row < A.n_rows) {
        const float4 z = M.z[row];
        const double zz[3] = {z.x, z.y, z.z};
        const PV* ap = reinterpret_cast<const PV*>(A.ap) + 3 * (size_t)row;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            d[0][0] += zz[q] * A.r[3 * (size_t)row + q];
            if (mode == 0) d[0][1] += zz[q] * (double)ap[q];
        }
        if (mode == 1 && S[0].restart) PadVec<TP>::store(A.p, row, zz);
    }
    double tot[1][2];
    if (last_block_reduce<1, 2>(A, d, 2, tot) && threadIdx.x == 0) {
        RhsScalars& s = S[0];
        if (mode == 0) s.beta = -s.alpha * tot[0][1] / s.rz;
        s.rz = tot[0][0];
        if (mode == 1) {
            s.refresh = 0;
            s.restart = 0;
        }
        if (!isfinite(s.rz)) {
            s.nonfinite = 1;
            if (!s.done) {
                s.done = 1;
                if (mode == 0) retire_instance(A);
            }
            s.finished = 1;
        }
    }
}

template <typename TP>
__global__ void __launch_bounds__(kThreads) k_mg_update_p(MgPcg M) {
    using PV = typename ApOf<TP>::T;
    const PcgArgs& A = M.a;
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (cta_done<1>(A, S)) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= A.n_rows) return;
    const double beta = S[0].beta;
    const float4 z = M.z[row];
    PV pv[3];
    PadVec<TP>::load(A.p, row, pv);
    const double pn[3] = {z.x + beta * (double)pv[0], z.y + beta * (double)pv[1], z.z + beta * (double)pv[2]};
    PadVec<TP>::store(A.p, row, pn);
}

// FP64 true residual r = f - A64 x, b0 = float(r) for every instance
// (init = 1: also |f|^2, the target and fresh recurrence state) or for the
// instances whose replace flag is set (init = 0).  Marks them for the rz /
// direction refresh that follows the next V-cycle.
template <bool PAIR_R>
__global__ void __launch_bounds__(kThreads) k_mg_residual(MgPcg M, int init, double tol2) {
    pdl_begin();
    const PcgArgs& A = M.a;
    RhsScalars* S = A.sc + cta_instance(A) * kMaxRhs;
    if (!init && !S[0].replace) return;
    double d[1][2] = {{0.0, 0.0}};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n_rows; row += gridDim.x * blockDim.x) {
        const int lane = row & 31;
        double y[3] = {0, 0, 0};
        const int64_t g0 = A.slice_off[row >> 5];
        const int len = A.row_len[row];
        for (int j = 0; j < len; ++j) {
            const int64_t g = g0 + j;
            const int c = A.col[g * 32 + lane];
            const double* v = A.v64 + (g * 9) * 32 + lane;
            const double x0 = A.x[3 * (size_t)c], x1 = A.x[3 * (size_t)c + 1], x2 = A.x[3 * (size_t)c + 2];
#pragma unroll
            for (int a = 0; a < 3; ++a) y[a] = fma(v[(a * 3) * 32], x0, fma(v[(a * 3 + 1) * 32], x1, fma(v[(a * 3 + 2) * 32], x2, y[a])));
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const size_t o = 3 * (size_t)row + a;
            const double rv = A.f[o] - y[a];
            if constexpr (PAIR_R) st_pair(reinterpret_cast<float2*>(A.r), o, f2_of(rv));  // split method
            else A.r[o] = rv;
            M.b0[o] = (float)rv;
            d[0][0] += rv * rv;
            d[0][1] += A.f[o] * A.f[o];
        }
    }
    double tot[1][2];
    if (last_block_reduce<1, 2>(A, d, 3, tot) && threadIdx.x == 0) {
        RhsScalars& s = S[0];
        s.rr = tot[0][0];
        s.rr_last_true = tot[0][0];
        if (init) {
            s.bb = tot[0][1];
            s.target = tol2 * s.bb;
            s.iter = 0;
            s.beta = 0.0;
            s.restart = 1;
        }
        s.replace = 0;
        s.refresh = 1;
        s.nonfinite = isfinite(s.rr) ? 0 : 1;
        s.finished = (s.rr <= s.target) || s.nonfinite;
        s.done = s.finished;
    }
}

// ---------------------------------------------------------------------------
// host: hierarchy construction
// ---------------------------------------------------------------------------
// Coarse-node positions on one axis: every second fine node (the last cell
// of an odd count is merged into its neighbour), or all of them when the axis
// is not coarsened at this level (semi-coarsening).
MgAxis make_axis(int n_f, bool coarsen) {
    MgAxis a;
    a.n_f = n_f;
    const int step = coarsen ? 2 : 1;
    for (int i = 0; i <= n_f; i += step) a.xs.push_back(i);
    if (a.xs.back() != n_f) a.xs.push_back(n_f);
    a.n_c = (int)a.xs.size() - 1;
    a.lo.assign(n_f + 1, 0);
    a.w.assign(n_f + 1, 0.f);
    for (int i = 0; i <= n_f; ++i) {
        const int m = (int)(std::upper_bound(a.xs.begin(), a.xs.end(), i) - a.xs.begin()) - 1;
        a.lo[i] = m;  // i == xs[m] gives weight 0 for m + 1 (never read)
        a.w[i] = (m < a.n_c) ? (float)(i - a.xs[m]) / (float)(a.xs[m + 1] - a.xs[m]) : 0.f;
    }
    return a;
}

// SBELL pattern, element connectivity, slot map and parity colouring of a
// level made of the blocks L.blk (nodes and elements numbered block by block;
// elements of different blocks share no node).
void level_pattern(Ctx& c, MgLevel& L) {
    const int N = L.n_nodes;
    std::vector<std::vector<int32_t>> adj(N);
    for (const MgBlk& B : L.blk) {
        auto id = [&](int i, int j, int k) { return B.node0 + (i * (B.ny + 1) + j) * (B.nz + 1) + k; };
        for (int i = 0; i <= B.nx; ++i)
            for (int j = 0; j <= B.ny; ++j)
                for (int k = 0; k <= B.nz; ++k) {
                    auto& v = adj[id(i, j, k)];
                    for (int di = -1; di <= 1; ++di)
                        for (int dj = -1; dj <= 1; ++dj)
                            for (int dk = -1; dk <= 1; ++dk) {
                                const int a = i + di, b = j + dj, q = k + dk;
                                if (a < 0 || b < 0 || q < 0 || a > B.nx || b > B.ny || q > B.nz) continue;
                                v.push_back(id(a, b, q));
                            }
                    std::sort(v.begin(), v.end());
                }
    }
    Sbell& A = L.own;
    A.b = 3;
    A.n_rows = N;
    A.n_slices = (N + kSlice - 1) / kSlice;
    A.h_slice_off.assign(A.n_slices + 1, 0);
    A.h_row_len.assign(N, 0);
    A.h_diag.assign(N, 0);
    for (int s = 0; s < A.n_slices; ++s) {
        size_t w = 0;
        for (int r = s * kSlice; r < std::min(N, (s + 1) * kSlice); ++r) w = std::max(w, adj[r].size());
        A.h_slice_off[s + 1] = A.h_slice_off[s] + (int64_t)w;
    }
    A.n_groups = A.h_slice_off[A.n_slices];
    A.h_col.assign((size_t)A.n_groups * kSlice, 0);
    for (int r = 0; r < N; ++r) {
        const int s = r / kSlice, lane = r % kSlice;
        const int64_t w = A.h_slice_off[s + 1] - A.h_slice_off[s];
        A.h_row_len[r] = (uint8_t)adj[r].size();
        for (int64_t j = 0; j < w; ++j) {
            const int col = (j < (int64_t)adj[r].size()) ? adj[r][j] : r;
            A.h_col[(size_t)(A.h_slice_off[s] + j) * kSlice + lane] = col;
            if (j < (int64_t)adj[r].size() && adj[r][j] == r) A.h_diag[r] = (uint8_t)j;
        }
    }
    // elements, slot map, parity colouring
    std::vector<int32_t> conn((size_t)L.n_el * 8), slot((size_t)L.n_el * 64);
    const int co[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    std::vector<std::vector<int32_t>> colour(8);
    for (const MgBlk& B : L.blk) {
        auto id = [&](int i, int j, int k) { return B.node0 + (i * (B.ny + 1) + j) * (B.nz + 1) + k; };
        for (int i = 0; i < B.nx; ++i)
            for (int j = 0; j < B.ny; ++j)
                for (int k = 0; k < B.nz; ++k) {
                    const int e = B.el0 + (i * B.ny + j) * B.nz + k;
                    for (int a = 0; a < 8; ++a)
                        conn[(size_t)e * 8 + a] = id(i + co[a][0], j + co[a][1], k + co[a][2]);
                    for (int a = 0; a < 8; ++a) {
                        const int ra = conn[(size_t)e * 8 + a];
                        for (int b = 0; b < 8; ++b) {
                            const int cb = conn[(size_t)e * 8 + b];
                            const auto& v = adj[ra];
                            const int p = (int)(std::lower_bound(v.begin(), v.end(), cb) - v.begin());
                            slot[(size_t)e * 64 + a * 8 + b] = (int32_t)A.slot(ra, p);
                        }
                    }
                    colour[(i & 1) * 4 + (j & 1) * 2 + (k & 1)].push_back(e);
                }
    }
    std::vector<int32_t> ce;
    L.colour_ptr.assign(1, 0);
    for (auto& cl : colour) {
        ce.insert(ce.end(), cl.begin(), cl.end());
        L.colour_ptr.push_back((int32_t)ce.size());
    }
    A.slice_off.upload(A.h_slice_off, c.stream);
    A.col.upload(A.h_col, c.stream);
    A.row_len.upload(A.h_row_len, c.stream);
    A.diag.upload(A.h_diag, c.stream);
    A.v32.alloc((size_t)A.n_groups * 9 * kSlice);
    L.conn.upload(conn, c.stream);
    L.slot_map.upload(slot, c.stream);
    L.colour_elems.upload(ce, c.stream);
    L.A = &L.own;
}

// Device block descriptors and per-block start tables of level l (levels
// >= 1 also describe the finer level's blocks).
void level_tables(Ctx& c, MgHierarchy& H, int l) {
    MgLevel& L = *H.L[l];
    const MgLevel* F = l > 0 ? H.L[l - 1].get() : nullptr;
    const int nb = (int)L.blk.size();
    std::vector<BlkDev> dv(nb);
    std::vector<int32_t> pn(nb + 1), pe(nb + 1);
    for (int b = 0; b < nb; ++b) {
        const MgBlk& B = L.blk[b];
        BlkDev& d = dv[b];
        std::memset(&d, 0, sizeof(d));
        d.nx = B.nx;
        d.ny = B.ny;
        d.nz = B.nz;
        d.node0 = B.node0;
        d.el0 = B.el0;
        if (F) {
            const MgBlk& P = F->blk[b];
            d.fnx = P.nx;
            d.fny = P.ny;
            d.fnz = P.nz;
            d.fnode0 = P.node0;
            d.fel0 = P.el0;
        }
        d.ox0 = B.ox[0];
        d.ox1 = B.ox[1];
        d.ox2 = B.ox[2];
        d.ol0 = B.ol[0];
        d.ol1 = B.ol[1];
        d.ol2 = B.ol[2];
        d.dense0 = (l + 1 == (int)H.L.size() && !H.h_dense0.empty()) ? H.h_dense0[b] : 0;
        pn[b] = B.node0;
        pe[b] = B.el0;
    }
    pn[nb] = L.n_nodes;
    pe[nb] = L.n_el;
    L.d_blk.upload(dv, c.stream);
    L.pre_node.upload(pn, c.stream);
    L.pre_el.upload(pe, c.stream);
}

LevelView view_of(const MgLevel& L) {
    LevelView v{};
    v.n_blk = (int)L.blk.size();
    v.blk = L.d_blk.p;
    v.xs = L.d_xs.p;
    v.lo = L.d_lo.p;
    v.w = L.d_w.p;
    return v;
}

SbView sbview(const MgLevel& L) {
    return SbView{L.A->n_rows, L.A->slice_off.p, L.A->row_len.p, L.A->col.p, L.A->v32.p};
}

// Level-0 blocks: the declared structured block, or one block per instance
// of a batched stack (asend_set_instance_blocks).
std::vector<MgBlk> level0_blocks(const Ctx& c) {
    std::vector<MgBlk> out;
    auto spacing = [&](MgBlk& B) {
        const int n100 = (B.ny + 1) * (B.nz + 1), n010 = B.nz + 1, n001 = 1;
        const int nb[3] = {n100, n010, n001};
        for (int ax = 0; ax < 3; ++ax) {
            double d2 = 0.0;
            for (int j = 0; j < 3; ++j) {
                const double d = c.xyz[3 * (size_t)(B.node0 + nb[ax]) + j] - c.xyz[3 * (size_t)B.node0 + j];
                d2 += d * d;
            }
            B.h[ax] = std::sqrt(d2);
        }
    };
    if (!c.inst_dims.empty()) {
        int el0 = 0;
        for (int i = 0; i < c.n_inst; ++i) {
            MgBlk B;
            B.nx = c.inst_dims[3 * i];
            B.ny = c.inst_dims[3 * i + 1];
            B.nz = c.inst_dims[3 * i + 2];
            B.node0 = c.inst_node_ptr[i];
            B.el0 = el0;
            el0 += B.n_el();
            spacing(B);
            out.push_back(B);
        }
    } else if (c.bx > 0) {
        MgBlk B;
        B.nx = c.bx;
        B.ny = c.by;
        B.nz = c.bz;
        spacing(B);
        out.push_back(B);
    }
    return out;
}

void build_hierarchy(Ctx& c) {
    if (c.type != 8 && c.type != 81)
        throw InputError("multigrid needs structured hex8 / brickIM blocks (asend_set_block_structure or "
                         "asend_set_instance_blocks)");
    std::vector<MgBlk> b0 = level0_blocks(c);
    if (b0.empty())
        throw InputError("multigrid needs structured hex8 / brickIM blocks (asend_set_block_structure or "
                         "asend_set_instance_blocks)");
    auto H = std::make_shared<MgHierarchy>();
    H->n_blk = (int)b0.size();
    auto L0 = std::make_unique<MgLevel>();
    L0->n_nodes = c.n_nodes;
    L0->n_el = c.n_el;
    L0->n_dof = c.n_dof;
    L0->blk = b0;
    L0->A = &c.A;
    // level-0 lumped penalty (coef^2 per constrained DOF, in units of the instance's scale)
    L0->h_pen.assign(c.n_dof, 0.f);
    for (size_t r = 0; r + 1 < c.c_ptr.size(); ++r)
        for (int k = c.c_ptr[r]; k < c.c_ptr[r + 1]; ++k) L0->h_pen[c.c_dof[k]] += (float)(c.c_coef[k] * c.c_coef[k]);
    H->L.push_back(std::move(L0));
    for (;;) {
        MgLevel& F = *H->L.back();
        // Per block: the coarsest grid is solved directly (<= 256 DOF);
        // semi-coarsening coarsens only the axes whose spacing is within a
        // factor sqrt(2) of the smallest (the strongly coupled directions of
        // stretched elements), the others wait until the cells are
        // isotropic.  An axis two cells thick is coarsened to one cell only
        // once every axis is that thin: a one-cell-thick coarse grid of a
        // deep bar is a poor coarse space.  A block that is done is carried
        // down unchanged while other blocks still coarsen.
        const int nb = (int)F.blk.size();
        std::vector<std::array<bool, 3>> co(nb);
        bool any_block = false;
        for (int b = 0; b < nb; ++b) {
            const MgBlk& P = F.blk[b];
            co[b] = {false, false, false};
            if (P.done || 3 * P.n_nodes() <= 256 || (P.nx <= 1 && P.ny <= 1 && P.nz <= 1)) continue;
            const int nf[3] = {P.nx, P.ny, P.nz};
            const bool all_thin = nf[0] <= 2 && nf[1] <= 2 && nf[2] <= 2;
            auto eligible = [&](int ax) { return nf[ax] >= 2 && (nf[ax] > 2 || all_thin); };
            double hmin = 1e300;
            for (int ax = 0; ax < 3; ++ax)
                if (eligible(ax)) hmin = std::min(hmin, P.h[ax]);
            for (int ax = 0; ax < 3; ++ax) {
                co[b][ax] = eligible(ax) && P.h[ax] <= 1.4142135623730951 * hmin;
                any_block |= co[b][ax];
            }
        }
        if (!any_block) break;
        auto L = std::make_unique<MgLevel>();
        std::vector<int32_t> xs, lo;
        std::vector<float> w;
        int node0 = 0, el0 = 0;
        for (int b = 0; b < nb; ++b) {
            const MgBlk& P = F.blk[b];
            MgBlk B;
            const int nf[3] = {P.nx, P.ny, P.nz};
            bool any = false;
            for (int ax = 0; ax < 3; ++ax) {
                B.ax[ax] = make_axis(nf[ax], co[b][ax]);
                B.h[ax] = P.h[ax] * (double)nf[ax] / (double)B.ax[ax].n_c;
                any |= co[b][ax];
            }
            B.done = !any;
            B.nx = B.ax[0].n_c;
            B.ny = B.ax[1].n_c;
            B.nz = B.ax[2].n_c;
            B.node0 = node0;
            B.el0 = el0;
            node0 += B.n_nodes();
            el0 += B.n_el();
            for (int ax = 0; ax < 3; ++ax) {
                B.ox[ax] = (int)xs.size();
                B.ol[ax] = (int)lo.size();
                xs.insert(xs.end(), B.ax[ax].xs.begin(), B.ax[ax].xs.end());
                lo.insert(lo.end(), B.ax[ax].lo.begin(), B.ax[ax].lo.end());
                w.insert(w.end(), B.ax[ax].w.begin(), B.ax[ax].w.end());
            }
            L->blk.push_back(B);
        }
        L->n_nodes = node0;
        L->n_el = el0;
        L->n_dof = 3 * node0;
        L->d_xs.upload(xs, c.stream);
        L->d_lo.upload(lo, c.stream);
        L->d_w.upload(w, c.stream);
        // lumped Galerkin penalty: pen_c[I] = sum_i w_iI pen_f[i]
        L->h_pen.assign(L->n_dof, 0.f);
        for (int b = 0; b < nb; ++b) {
            const MgBlk& P = F.blk[b];
            const MgBlk& B = L->blk[b];
            for (int i = 0; i <= P.nx; ++i)
                for (int j = 0; j <= P.ny; ++j)
                    for (int k = 0; k <= P.nz; ++k) {
                        const int f = P.node0 + (i * (P.ny + 1) + j) * (P.nz + 1) + k;
                        const float p0 = F.h_pen[3 * f], p1 = F.h_pen[3 * f + 1], p2 = F.h_pen[3 * f + 2];
                        if (p0 == 0.f && p1 == 0.f && p2 == 0.f) continue;
                        const int li[3] = {B.ax[0].lo[i], B.ax[1].lo[j], B.ax[2].lo[k]};
                        const float wi[3] = {B.ax[0].w[i], B.ax[1].w[j], B.ax[2].w[k]};
                        for (int d0 = 0; d0 < 2; ++d0)
                            for (int d1 = 0; d1 < 2; ++d1)
                                for (int d2 = 0; d2 < 2; ++d2) {
                                    const float ww = (d0 ? wi[0] : 1 - wi[0]) * (d1 ? wi[1] : 1 - wi[1]) *
                                                     (d2 ? wi[2] : 1 - wi[2]);
                                    if (ww == 0.f) continue;
                                    const int I = B.node0 +
                                                  ((li[0] + d0) * (B.ny + 1) + (li[1] + d1)) * (B.nz + 1) + (li[2] + d2);
                                    L->h_pen[3 * I] += ww * p0;
                                    L->h_pen[3 * I + 1] += ww * p1;
                                    L->h_pen[3 * I + 2] += ww * p2;
                                }
                    }
        }
        level_pattern(c, *L);
        L->Ke.alloc((size_t)L->n_el * 576);
        H->L.push_back(std::move(L));
    }
    for (auto& Lp : H->L) {
        MgLevel& L = *Lp;
        L.pen.upload(L.h_pen, c.stream);
        L.binv.alloc((size_t)9 * L.n_nodes);
        L.b.alloc(L.n_dof);
        L.r.alloc(L.n_dof);
        L.x4.alloc((size_t)4 * L.n_nodes);
        L.y4.alloc((size_t)4 * L.n_nodes);
    }
    // coarsest level: one dense block per instance
    MgLevel& Lc = *H->L.back();
    H->h_dense0.assign(H->n_blk, 0);
    size_t dense_tot = 0;
    H->n_coarse = 0;
    for (int b = 0; b < H->n_blk; ++b) {
        const int nd = 3 * Lc.blk[b].n_nodes();
        H->h_dense0[b] = (int32_t)dense_tot;
        dense_tot += (size_t)nd * nd;
        H->n_coarse = std::max(H->n_coarse, nd);
    }
    if (H->n_coarse > 1020) throw InputError("multigrid coarsest level too large");
    if (dense_tot > (size_t)INT32_MAX) throw InputError("multigrid coarsest blocks too large");
    H->dense.alloc(dense_tot);
    for (int l = 0; l < (int)H->L.size(); ++l) level_tables(c, *H, l);
    // fused tail: the deepest levels whose every block has <= kTailNodes
    // nodes, if there are at least two (one besides the coarsest)
    {
        const int nl = (int)H->L.size();
        int lt = nl;
        for (int l = nl - 1; l >= 1; --l) {
            int mx = 0;
            for (const MgBlk& B : H->L[l]->blk) mx = std::max(mx, B.n_nodes());
            if (mx > kTailNodes) break;
            lt = l;
        }
        // only for stacks of many instances: one CTA cannot carry a lone
        // block's small levels as fast as the grid-wide launches do
        H->tail = (H->n_blk >= kTailMinBlocks && nl - lt >= 2 && nl - lt <= kMaxTail) ? lt : 0;
    }
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    c.mg = H;
}

void damp_smoother(Ctx& c, int l) {
    MgHierarchy& H = *c.mg;
    MgLevel& L = *H.L[l];
    float* nrm = H.pow_nrm.p + (size_t)l * (kPowSteps + 1);
    uint32_t* tk = H.pow_ticket.p + (size_t)l * kPowSteps;
    float4* xa = reinterpret_cast<float4*>(L.x4.p);
    float4* xb = reinterpret_cast<float4*>(L.y4.p);
    const int g = grid_of(L.n_nodes);
    // later assemblies start from the previous dominant vector (the operator
    // changes little between assemblies of one hierarchy): fewer steps
    const bool warm = L.pow_warm;
    const int steps = warm ? kPowWarmSteps : kPowSteps;
    if (L.pow_vec.n != (size_t)4 * L.n_nodes) L.pow_vec.alloc((size_t)4 * L.n_nodes);
    ASEND_CUDA(cudaMemsetAsync(tk, 0, sizeof(uint32_t) * kPowSteps, c.stream));
    ASEND_CUDA(cudaMemsetAsync(H.pow_bound.p + l, 0, sizeof(unsigned int), c.stream));
    if (warm)
        ASEND_CUDA(cudaMemcpyAsync(xa, L.pow_vec.p, sizeof(float) * 4 * L.n_nodes, cudaMemcpyDeviceToDevice,
                                   c.stream));
    k_pow_init<<<g, kT, 0, c.stream>>>(L.n_nodes, xa, nrm, warm ? 0 : 1);
    for (int k = 0; k < steps; ++k) {
        k_pow_step<<<g, kT, 0, c.stream>>>(sbview(L), L.binv.p, xa, xb, nrm, k, H.pow_part.p, tk);
        std::swap(xa, xb);
    }
    ASEND_CUDA(cudaMemcpyAsync(L.pow_vec.p, xa, sizeof(float) * 4 * L.n_nodes, cudaMemcpyDeviceToDevice, c.stream));
    L.pow_warm = true;
    L.pow_steps = steps;
    unsigned int* bound = H.pow_bound.p + l;
    k_inf_bound<<<g, kT, 0, c.stream>>>(sbview(L), L.binv.p, bound);
    k_scale_blocks<<<(9 * L.n_nodes + 255) / 256, 256, 0, c.stream>>>(L.n_nodes, L.binv.p, nrm, steps, bound,
                                                                       H.safe_damping ? 1 : 0, c.mg_damping,
                                                                       H.pow_omega.p + l);
    c.launches += steps + 3;
}

// per-assembly values: Galerkin element matrices, level operators, penalty,
// smoother blocks, coarsest inverses
// Level-0 smoother blocks (undamped D_n^-1) from the FP64 values, or from the
// FP32 values after a split-only assembly (the smoother is FP32 either way).
void level0_smoother_blocks(Ctx& c, MgLevel& L0) {
    if (c.v64_valid)
        k_smoother_blocks<double><<<grid_of(L0.n_nodes), kT, 0, c.stream>>>(L0.n_nodes, c.A.slice_off.p, c.A.diag.p,
                                                                            c.A.v64.p, 1.f, L0.binv.p);
    else
        k_smoother_blocks<float><<<grid_of(L0.n_nodes), kT, 0, c.stream>>>(L0.n_nodes, c.A.slice_off.p, c.A.diag.p,
                                                                           c.A.v32.p, 1.f, L0.binv.p);
}

// Per-assembly multigrid values.  skip_l0: the solve takes its finest-level
// smoother blocks from the learned model, so the finest level's eigenvalue
// estimate (its power iteration, the largest of the set-up) is not made.
void setup_values(Ctx& c, bool skip_l0) {
    MgHierarchy& H = *c.mg;
    const int n_lev = (int)H.L.size();
    H.pow_nrm.alloc((size_t)n_lev * (kPowSteps + 1));
    H.pow_bound.alloc((size_t)n_lev);
    H.pow_omega.alloc((size_t)n_lev);
    H.pow_bound.zero(c.stream);
    H.pow_omega.zero(c.stream);
    H.pow_ticket.alloc((size_t)n_lev * kPowSteps);
    H.pow_part.alloc((size_t)grid_of(H.L[0]->n_nodes));
    {
        std::vector<double> sf(H.n_blk, c.sf);
        if (c.n_inst > 1 && (int)c.sf_inst.size() == H.n_blk) sf = c.sf_inst;
        H.blk_sf.upload(sf, c.stream);
    }
    if (!skip_l0) {
        MgLevel& L0 = *H.L[0];
        level0_smoother_blocks(c, L0);
        ++c.launches;
        if (n_lev > 1) damp_smoother(c, 0);
    }
    H.l0_damped = !skip_l0;
    for (size_t l = 1; l < H.L.size(); ++l) {
        MgLevel& L = *H.L[l];
        MgLevel& F = *H.L[l - 1];
        const float* fine_ke = F.Ke.p;
        const float* cls_ke = nullptr;
        const int32_t* cls_of = nullptr;
        if (l == 1) {
            // level 0: K_e = E_e * (unit-modulus matrix of its geometry class)
            // when the assembly keeps classes; otherwise hex8 matrices are
            // integrated inside k_coarsen and brickIM ones (condensed
            // incompatible modes) are computed first
            fine_ke = nullptr;
            if (c.cls_ke32.n && c.cls_type == c.type && c.ortho.empty()) {
                cls_ke = c.cls_ke32.p;
                cls_of = c.d_cls_of.p;
            } else if (c.type == 81) {
                F.Ke.alloc((size_t)c.n_el * 576);
                brickim_element_ke32(c, F.Ke.p);
                fine_ke = F.Ke.p;
            }
        }
        if (l == 1 && cls_ke && c.n_cls <= kMaxChildClasses) {
            if (!H.child_ready) {
                H.child.alloc((size_t)c.n_cls * 27 * 576);
                k_child_mats<<<dim3(27, c.n_cls), 256, 0, c.stream>>>(c.cls_ke.p, H.child.p);
                ++c.launches;
                H.child_ready = true;
            }
            k_coarsen_lin<<<L.n_el, 144, 0, c.stream>>>(view_of(L), L.pre_el.p, c.d_E.p, cls_of, H.child.p, L.Ke.p);
        } else {
            k_coarsen<<<L.n_el, 512, 0, c.stream>>>(view_of(L), L.pre_el.p, fine_ke, cls_ke, cls_of, c.d_xyz.p,
                                                    c.d_conn.p, c.d_E.p, c.d_nu.p, L.Ke.p);
        }
        L.own.v32.zero(c.stream);
        for (size_t k = 0; k + 1 < L.colour_ptr.size(); ++k) {
            const int n = L.colour_ptr[k + 1] - L.colour_ptr[k];
            if (!n) continue;
            k_scatter_ke<<<(n * 64 + 255) / 256, 256, 0, c.stream>>>(n, L.colour_elems.p + L.colour_ptr[k], L.slot_map.p,
                                                                     L.Ke.p, L.own.v32.p);
            ++c.launches;
        }
        k_add_pen<<<grid_of(L.n_nodes), kT, 0, c.stream>>>(L.n_nodes, L.own.slice_off.p, L.own.diag.p, L.pen.p,
                                                           L.pre_node.p, (int)L.blk.size(), H.blk_sf.p, L.own.v32.p);
        k_smoother_blocks<float><<<grid_of(L.n_nodes), kT, 0, c.stream>>>(L.n_nodes, L.own.slice_off.p, L.own.diag.p,
                                                                          L.own.v32.p, 1.f, L.binv.p);
        c.launches += 3;
        if (l + 1 < H.L.size()) damp_smoother(c, (int)l);  // the coarsest level is solved directly
    }
    MgLevel& Lc = *H.L.back();
    k_dense_build<<<Lc.n_nodes, 128, 0, c.stream>>>(Lc.n_nodes, Lc.A->slice_off.p, Lc.A->row_len.p, Lc.A->col.p,
                                                    Lc.A->v32.p, view_of(Lc), Lc.pre_node.p, H.dense.p);
    const int ld = (H.n_coarse + 3) & ~3;
    const size_t blk_smem = sizeof(float) * (size_t)H.n_coarse * ld;
    if (blk_smem <= kGjSmem) {  // blocked elimination in shared memory
        ASEND_CUDA(cudaFuncSetAttribute(k_gauss_jordan_blk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)blk_smem));
        k_gauss_jordan_blk<<<H.n_blk, 1024, blk_smem, c.stream>>>(view_of(Lc), H.dense.p, ld);
    } else {  // larger coarsest blocks: column-by-column elimination in global memory
        k_gauss_jordan<<<H.n_blk, 1024, 0, c.stream>>>(view_of(Lc), H.dense.p, 0);
    }
    c.launches += 2;
    ASEND_CUDA(cudaGetLastError());
    H.epoch = c.assembly_epoch;
}

// Restriction of level l's residual r to level l + 1's right-hand side b (and
// its first smoothing sweep, unless l + 1 is the coarsest level).
void restrict_to(Ctx& c, int l, const Control* ctl) {
    MgHierarchy& H = *c.mg;
    MgLevel& L = *H.L[l];
    MgLevel& C = *H.L[l + 1];
    const bool last = (l + 2 == (int)H.L.size());  // the coarsest level is solved directly: no sweep
    launch_k(c, k_vc_restrict, grid_of(C.n_nodes), kT, 0, view_of(C), C.pre_node.p, C.n_nodes, L.r.p, C.b.p,
                                                           last ? nullptr : C.binv.p,
                                                           reinterpret_cast<float4*>(C.x4.p), ctl);
}

void coarsest_solve(Ctx& c, const Control* ctl) {
    MgHierarchy& H = *c.mg;
    MgLevel& Lc = *H.L.back();
    launch_k(c, k_vc_dense, H.n_blk, 1024, 0, view_of(Lc), H.dense.p, Lc.b.p, Lc.y4.p, ctl);
}

void prolong_from(Ctx& c, int l, const Control* ctl) {
    MgHierarchy& H = *c.mg;
    MgLevel& L = *H.L[l];
    MgLevel& C = *H.L[l + 1];
    launch_k(c, k_vc_prolong, grid_of(L.n_nodes), kT, 0, view_of(C), L.pre_node.p, L.n_nodes,
                                                          reinterpret_cast<const float4*>(C.y4.p),
                                                          reinterpret_cast<float4*>(L.x4.p), ctl);
}

// One V(1,1) cycle on level 0's b.  With fused0, the caller has already
// written level 0's first sweep x4 = B^-1 b (fused into the PCG update).
// Lanes per row of a level's products: one per row while the rows alone
// fill the GPU (about 152 SMs x 1024 threads), else the smallest power of two
// up to 16 that does.
int lanes_for(int n_rows) {
    constexpr int kFill = 152 * 1024;
    int t = 1;
    while (t < 16 && (int64_t)n_rows * t < kFill) t *= 2;
    return t;
}

// Levels with at least this many node rows run the staged (bulk-copy) row
// products, one row per lane; smaller ones split each row over T lanes.
constexpr int kStagedRows = 8192;

void level_resid(Ctx& c, MgLevel& L, const Control* ctl) {
    const int t = L.n_nodes >= kStagedRows ? 1 : lanes_for(L.n_nodes);
    const SbView A = sbview(L);
    const float4* x = reinterpret_cast<const float4*>(L.x4.p);
    const int g = (int)(((int64_t)L.n_nodes * t + kT - 1) / kT);
    switch (t) {
        case 1:
            launch_k(c, k_vc_resid_staged, std::min(grid_of(L.n_nodes), kPersistCtas), kT,
                     (size_t)F32Stage<kVcG, kVcS>::smem(kT), A, L.b.p, x, L.r.p, ctl);
            break;
        case 2: launch_k(c, k_vc_resid_t<2>, g, kT, 0, A, L.b.p, x, L.r.p, ctl); break;
        case 4: launch_k(c, k_vc_resid_t<4>, g, kT, 0, A, L.b.p, x, L.r.p, ctl); break;
        case 8: launch_k(c, k_vc_resid_t<8>, g, kT, 0, A, L.b.p, x, L.r.p, ctl); break;
        default: launch_k(c, k_vc_resid_t<16>, g, kT, 0, A, L.b.p, x, L.r.p, ctl); break;
    }
}

void level_post(Ctx& c, MgLevel& L, const Control* ctl);
void level_resid_or_post(Ctx& c, MgLevel& L, bool post, const Control* ctl) {
    if (post) level_post(c, L, ctl);
    else level_resid(c, L, ctl);
}

void level_post(Ctx& c, MgLevel& L, const Control* ctl) {
    const int t = L.n_nodes >= kStagedRows ? 1 : lanes_for(L.n_nodes);
    const SbView A = sbview(L);
    const float4* x = reinterpret_cast<const float4*>(L.x4.p);
    float4* y = reinterpret_cast<float4*>(L.y4.p);
    const int g = (int)(((int64_t)L.n_nodes * t + kT - 1) / kT);
    switch (t) {
        case 1:
            launch_k(c, k_vc_post_staged, std::min(grid_of(L.n_nodes), kPersistCtas), kT,
                     (size_t)F32Stage<kVcG, kVcS>::smem(kT), A, L.binv.p, L.b.p, x, y, ctl);
            break;
        case 2: launch_k(c, k_vc_post_t<2>, g, kT, 0, A, L.binv.p, L.b.p, x, y, ctl); break;
        case 4: launch_k(c, k_vc_post_t<4>, g, kT, 0, A, L.binv.p, L.b.p, x, y, ctl); break;
        case 8: launch_k(c, k_vc_post_t<8>, g, kT, 0, A, L.binv.p, L.b.p, x, y, ctl); break;
        default: launch_k(c, k_vc_post_t<16>, g, kT, 0, A, L.binv.p, L.b.p, x, y, ctl); break;
    }
}

// First level of the fused coarse tail in use (nl - 1: no tail, the
// coarsest level alone is solved by its own launch).
int tail_level(const Ctx& c) {
    const MgHierarchy& H = *c.mg;
    const int nl = (int)H.L.size();
    return (c.mg_tail && H.tail > 0) ? H.tail : nl - 1;
}

// Levels lt .. nl - 1 in one launch of k_vc_tail (one CTA per block).
void launch_tail(Ctx& c, int lt, const Control* ctl) {
    MgHierarchy& H = *c.mg;
    TailArgs ta;
    std::memset(&ta, 0, sizeof(ta));
    ta.n_lev = (int)H.L.size() - lt;
    for (int i = 0; i < ta.n_lev; ++i) {
        MgLevel& L = *H.L[lt + i];
        TailLevel& T = ta.L[i];
        T.A = sbview(L);
        T.V = view_of(L);
        T.binv = L.binv.p;
        T.b = L.b.p;
        T.r = L.r.p;
        T.x4 = reinterpret_cast<float4*>(L.x4.p);
        T.y4 = reinterpret_cast<float4*>(L.y4.p);
        T.lanes = lanes_for(L.n_nodes);
    }
    ta.ainv = H.dense.p;
    launch_k(c, k_vc_tail, H.n_blk, kTailThreads, 0, ta, ctl);
}

void vcycle(Ctx& c, const Control* ctl, bool fused0) {
    MgHierarchy& H = *c.mg;
    const int nl = (int)H.L.size();
    const int lt = tail_level(c);
    if (!fused0 && nl > 1) {
        MgLevel& L = *H.L[0];
        launch_k(c, k_vc_smooth0, grid_of(L.n_nodes), kT, 0, L.n_nodes, L.binv.p, L.b.p,
                                                              reinterpret_cast<float4*>(L.x4.p), ctl);
    }
    for (int l = 0; l < lt; ++l) {
        level_resid(c, *H.L[l], ctl);
        restrict_to(c, l, ctl);
    }
    if (lt < nl - 1) launch_tail(c, lt, ctl);
    else coarsest_solve(c, ctl);
    for (int l = lt - 1; l >= 0; --l) {
        prolong_from(c, l, ctl);
        level_post(c, *H.L[l], ctl);
    }
}

int vcycle_launches(const Ctx& c) { return 4 * tail_level(c) + 1; }

// L0.x4 = P C R (L0.r): the coarse-grid correction of one V-cycle alone
// (restriction of level 0's r, the V-cycle of the coarser levels, and the
// prolongation into a zeroed level-0 vector; no level-0 smoothing).
void coarse_correction(Ctx& c) {
    MgHierarchy& H = *c.mg;
    const int nl = (int)H.L.size();
    MgLevel& L0 = *H.L[0];
    for (int l = 0; l < nl - 1; ++l) {
        MgLevel& L = *H.L[l];
        if (l > 0)
            launch_k(c, k_vc_resid, grid_of(L.n_nodes), kT, 0, sbview(L), L.b.p, reinterpret_cast<float4*>(L.x4.p),
                                                                L.r.p, nullptr);
        restrict_to(c, l, nullptr);
    }
    coarsest_solve(c, nullptr);
    ASEND_CUDA(cudaMemsetAsync(L0.x4.p, 0, sizeof(float) * 4 * L0.n_nodes, c.stream));
    for (int l = nl - 2; l >= 0; --l) {
        MgLevel& L = *H.L[l];
        prolong_from(c, l, nullptr);
        if (l > 0)
            launch_k(c, k_vc_post, grid_of(L.n_nodes), kT, 0, sbview(L), L.binv.p, L.b.p,
                                                               reinterpret_cast<const float4*>(L.x4.p),
                                                               reinterpret_cast<float4*>(L.y4.p), nullptr);
    }
    c.launches += 6 * (nl - 1) - 1;
}


}  // namespace

void mg_invalidate_values(Ctx& c) {
    if (c.mg) c.mg->epoch = -1;
}

void mg_prepare(Ctx& c, bool learned) {
    product_attrs();
    if (!c.mg) build_hierarchy(c);
    if (c.mg->epoch != c.assembly_epoch) {
        setup_values(c, learned);
        c.mg->l0_learned = false;
    }
}

// Finest-level smoother blocks: damped block Jacobi (omega D_n^-1, omega from
// the eigenvalue estimate), or the
// learned nodal blocks M_n (recomputed on every request, since the weights
// may have changed since the last one).
void mg_select_smoother(Ctx& c, bool learned) {
    MgHierarchy& H = *c.mg;
    MgLevel& L0 = *H.L[0];
    if (learned) {
        learned_blocks(c, L0.binv.p, true);
        H.l0_learned = true;
    } else if (H.l0_learned || !H.l0_damped) {
        level0_smoother_blocks(c, L0);
        ++c.launches;
        if (H.L.size() > 1) damp_smoother(c, 0);
        H.l0_learned = false;
        H.l0_damped = true;
    }
}

void mg_apply(Ctx& c, const float* d_b, float* d_z4) {
    mg_prepare(c);
    mg_select_smoother(c, false);
    MgLevel& L0 = *c.mg->L[0];
    ASEND_CUDA(cudaMemcpyAsync(L0.b.p, d_b, sizeof(float) * c.n_dof, cudaMemcpyDeviceToDevice, c.stream));
    vcycle(c, nullptr, false);
    ASEND_CUDA(cudaMemcpyAsync(d_z4, L0.y4.p, sizeof(float) * 4 * c.n_nodes, cudaMemcpyDeviceToDevice, c.stream));
    c.launches += vcycle_launches(c);
}

int mg_levels(const Ctx& c) { return c.mg ? (int)c.mg->L.size() : 0; }

// Mean device time of n_launch back-to-back launches of one kernel of the
// multigrid CG (0: outer product + p.Ap in the method's value format; 1:
// level-0 V-cycle residual; 2: level-0 post-smoothing) and its algorithmic
// bytes per launch.  Scratch scalars keep the kernels from exiting early.
double mg_time_kernel(Ctx& c, int kernel, int method, int n_launch, double* bytes) {
    ensure_v64(c);
    mg_prepare(c);
    mg_select_smoother(c, false);
    MgHierarchy& H = *c.mg;
    MgLevel& L0 = *H.L[0];
    const int n = c.A.n_rows, nd = c.n_dof;
    const int grid = (method == ASEND_METHOD_SPLIT && kernel == 0) ? std::min(grid_of(n), kPersistCtas) : grid_of(n);
    const double blocks = (double)(c.A.nnz_scalar() / 9);
    if (kernel != 0 && H.L.size() < 2) throw InputError("multigrid hierarchy has a single level");
    DArr<RhsScalars> sc;
    DArr<Control> ctl;
    DArr<double> part, p, ap;
    sc.alloc(1);
    ctl.alloc(1);
    sc.zero(c.stream);
    ctl.zero(c.stream);
    part.alloc((size_t)grid * kMaxRhs * 3);
    p.alloc((size_t)4 * n);
    ap.alloc(nd);
    MgPcg M;
    std::memset(&M, 0, sizeof(M));
    PcgArgs& a = M.a;
    a.n_rows = n;
    a.nrhs = 1;
    a.n_dof = nd;
    a.slice_off = c.A.slice_off.p;
    a.row_len = c.A.row_len.p;
    a.col = c.A.col.p;
    a.v32 = c.A.v32.p;
    a.v32lo = c.A.v32lo.p;
    a.v64 = c.A.v64.p;
    a.p = p.p;
    a.ap = ap.p;
    a.partials = part.p;
    a.sc = sc.p;
    a.ctl = ctl.p;
    M.n_inst = 1;
    // the direction's values do not change the kernels' work: zeros
    ASEND_CUDA(cudaMemsetAsync(p.p, 0, sizeof(double) * 4 * n, c.stream));
    auto launch = [&]() {
        if (kernel == 0) {
            if (method == ASEND_METHOD_MIXED) k_mg_spmv_dot<float, float><<<grid, kThreads, 0, c.stream>>>(M);
            else if (method == ASEND_METHOD_SPLIT) launch_split_product(c, M, grid);
            else k_mg_spmv_dot<double, double><<<grid, kThreads, 0, c.stream>>>(M);
        } else {  // the finest level's products as the V-cycle runs them
            level_resid_or_post(c, L0, kernel == 2, nullptr);
        }
    };
    const double ps = (method == ASEND_METHOD_MIXED) ? 4.0 : 8.0;  // bytes per value / direction entry
    if (kernel == 0) *bytes = blocks * (9.0 * ps + 4.0) + (double)n * 4.0 * ps + (double)nd * ps;
    else if (kernel == 1) *bytes = blocks * 40.0 + (double)n * 16.0 + (double)nd * 8.0;
    else *bytes = blocks * 40.0 + (double)n * (16.0 + 36.0 + 16.0) + (double)nd * 4.0;
    for (int w = 0; w < 3; ++w) launch();
    ASEND_CUDA(cudaEventRecord(c.ev0, c.stream));
    for (int i = 0; i < n_launch; ++i) launch();
    ASEND_CUDA(cudaEventRecord(c.ev1, c.stream));
    ASEND_CUDA(cudaEventSynchronize(c.ev1));
    ASEND_CUDA(cudaGetLastError());
    float ms = 0.f;
    ASEND_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.launches += n_launch + 3;
    return ms / n_launch;
}

// per-level diagnostics: dims (nx, ny, nz), power estimate and guaranteed
// bound of lambda_max(D^-1 A), damping in use (the coarsest level: zeros)
void mg_level_info(Ctx& c, int level, int32_t* dims, double* lam_est, double* lam_bound, double* omega) {
    if (!c.mg || level < 0 || level >= (int)c.mg->L.size()) throw InputError("no such multigrid level");
    MgHierarchy& H = *c.mg;
    MgLevel& L = *H.L[level];
    if (dims) {  // the first block (instance 0)
        dims[0] = L.blk[0].nx;
        dims[1] = L.blk[0].ny;
        dims[2] = L.blk[0].nz;
    }
    float nrm = 0.f, om = 0.f;
    unsigned int bb = 0;
    if (H.pow_nrm.n) {
        ASEND_CUDA(cudaMemcpyAsync(&nrm, H.pow_nrm.p + (size_t)level * (kPowSteps + 1) + L.pow_steps, sizeof(float),
                                   cudaMemcpyDeviceToHost, c.stream));
        ASEND_CUDA(cudaMemcpyAsync(&bb, H.pow_bound.p + level, sizeof(unsigned int), cudaMemcpyDeviceToHost, c.stream));
        ASEND_CUDA(cudaMemcpyAsync(&om, H.pow_omega.p + level, sizeof(float), cudaMemcpyDeviceToHost, c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
    }
    float bf;
    std::memcpy(&bf, &bb, sizeof(float));
    if (lam_est) *lam_est = nrm;
    if (lam_bound) *lam_bound = bf;
    if (omega) *omega = om;
}

// z = V(b) with the current finest-level smoother, host FP32 vectors [n_dof]
void mg_vcycle_host(Ctx& c, const float* b, float* z) {
    mg_prepare(c);
    MgHierarchy& H = *c.mg;
    MgLevel& L0 = *H.L[0];
    if (H.L.size() < 2) throw InputError("multigrid hierarchy has a single level");
    ASEND_CUDA(cudaMemcpyAsync(L0.b.p, b, sizeof(float) * c.n_dof, cudaMemcpyHostToDevice, c.stream));
    vcycle(c, nullptr, false);
    c.launches += vcycle_launches(c);
    std::vector<float> y4((size_t)4 * c.n_nodes);
    ASEND_CUDA(cudaMemcpyAsync(y4.data(), L0.y4.p, sizeof(float) * y4.size(), cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    for (int i = 0; i < c.n_nodes; ++i)
        for (int a = 0; a < 3; ++a) z[3 * (size_t)i + a] = y4[4 * (size_t)i + a];
}

// r := (I - A V)^k r on a host FP32 vector [n_dof] with the finest-level
// smoother in force (learned or damped): the residual after k stationary
// V-cycle iterations, dominated by the modes the V-cycle reduces slowest.
void mg_stationary_residual(Ctx& c, float* r_host, int k, bool learned_smoother) {
    mg_prepare(c);
    mg_select_smoother(c, learned_smoother);
    MgHierarchy& H = *c.mg;
    MgLevel& L0 = *H.L[0];
    if (H.L.size() < 2) throw InputError("multigrid hierarchy has a single level");
    if (H.vl_w.n != (size_t)c.n_dof) H.vl_w.alloc(c.n_dof);
    ASEND_CUDA(cudaMemcpyAsync(H.vl_w.p, r_host, sizeof(float) * c.n_dof, cudaMemcpyHostToDevice, c.stream));
    const int g = grid_of(L0.n_nodes);
    for (int i = 0; i < k; ++i) {
        ASEND_CUDA(cudaMemcpyAsync(L0.b.p, H.vl_w.p, sizeof(float) * c.n_dof, cudaMemcpyDeviceToDevice, c.stream));
        vcycle(c, nullptr, false);
        k_vl_rstep<<<g, kT, 0, c.stream>>>(sbview(L0), reinterpret_cast<const float4*>(L0.y4.p), H.vl_w.p);
        c.launches += vcycle_launches(c) + 1;
    }
    ASEND_CUDA(cudaMemcpyAsync(r_host, H.vl_w.p, sizeof(float) * c.n_dof, cudaMemcpyDeviceToHost, c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
}

// Loss sum_s ||b_s - A V(b_s)||^2 over the samples (FP32, unit-norm b_s) with
// the learned finest-level smoother blocks, added to *d_loss; the block
// gradient (summed over samples) is added to gblk [n_nodes][6].  The caller
// has installed the learned blocks (mg_select_smoother(c, true)).
void mg_learned_loss_grad(Ctx& c, const float* samples, int n_samples, float* gblk, double* d_loss) {
    MgHierarchy& H = *c.mg;
    MgLevel& L0 = *H.L[0];
    const int n = L0.n_nodes, nd = 3 * n;
    if (H.L.size() < 2) throw InputError("multigrid hierarchy has a single level");
    if (H.vl_q.n != (size_t)4 * n) {
        H.vl_q.alloc((size_t)4 * n);
        H.vl_mw.alloc((size_t)4 * n);
        H.vl_t4.alloc((size_t)4 * n);
        H.vl_r2.alloc(nd);
        H.vl_w.alloc(nd);
    }
    float4* q = reinterpret_cast<float4*>(H.vl_q.p);
    float4* mw = reinterpret_cast<float4*>(H.vl_mw.p);
    float4* t4 = reinterpret_cast<float4*>(H.vl_t4.p);
    const int g = grid_of(n);
    for (int s = 0; s < n_samples; ++s) {
        const float* b = samples + (size_t)s * nd;
        ASEND_CUDA(cudaMemcpyAsync(L0.b.p, b, sizeof(float) * nd, cudaMemcpyDeviceToDevice, c.stream));
        vcycle(c, nullptr, false);  // z in L0.y4, x2 in L0.x4
        k_vl_resid<<<g, kT, 0, c.stream>>>(sbview(L0), b, reinterpret_cast<const float4*>(L0.y4.p),
                                          reinterpret_cast<const float4*>(L0.x4.p), q, H.vl_r2.p, d_loss);
        k_vl_w<<<g, kT, 0, c.stream>>>(sbview(L0), L0.binv.p, q, H.vl_w.p, mw);
        k_vl_t<<<g, kT, 0, c.stream>>>(sbview(L0), H.vl_w.p, mw, L0.r.p, t4);
        coarse_correction(c);  // L0.x4 = P C R t
        k_vl_grad<<<g, kT, 0, c.stream>>>(sbview(L0), t4, reinterpret_cast<const float4*>(L0.x4.p), b, H.vl_w.p,
                                         H.vl_r2.p, gblk);
        c.launches += vcycle_launches(c) + 4;
    }
    ASEND_CUDA(cudaGetLastError());
}


namespace {
int pcg_solve_mg_once(Ctx& c, const asend_solve_opts& o, asend_solve_stats* st, bool warm, const double* d_f,
                      double* d_x, int nrhs_all);
}

// Multigrid-preconditioned flexible CG, one right-hand side at a time.  A
// solve that turns non-finite (a smoother damped from an eigenvalue estimate
// that fell short of a localised top mode) is repeated from zero with every
// level's damping taken from the guaranteed bound ||D^-1 A||_inf, which then
// stays in force for this hierarchy.
int pcg_solve_mg(Ctx& c, const asend_solve_opts& o, asend_solve_stats* st, bool warm, const double* d_f, double* d_x,
                 int nrhs_all) {
    const int rc = pcg_solve_mg_once(c, o, st, warm, d_f, d_x, nrhs_all);
    if (rc != ASEND_NONFINITE || !c.mg || c.mg->safe_damping) return rc;
    c.mg->safe_damping = true;
    mg_invalidate_values(c);
    return pcg_solve_mg_once(c, o, st, false, d_f, d_x, nrhs_all);
}

namespace {
int pcg_solve_mg_once(Ctx& c, const asend_solve_opts& o, asend_solve_stats* st, bool warm, const double* d_f,
                      double* d_x, int nrhs_all) {
    const bool mixed = o.method == ASEND_METHOD_MIXED;
    const bool split = o.method == ASEND_METHOD_SPLIT;
    if (!split) ensure_v64(c);  // the split method runs on the hi / lo values alone
    const bool split_only = split && !c.v64_valid;  // the true residual from the pairs too
    mg_prepare(c, o.precond == ASEND_PC_MG_LEARNED);
    mg_select_smoother(c, o.precond == ASEND_PC_MG_LEARNED);
    MgHierarchy& H = *c.mg;
    const int n = c.A.n_rows, nd = c.n_dof;
    const int max_it = o.max_iter > 0 ? o.max_iter : nd;
    const int G = o.graph_iters > 0 ? o.graph_iters : 8;
    if (!warm) ASEND_CUDA(cudaMemsetAsync(d_x, 0, (size_t)nrhs_all * nd * sizeof(double), c.stream));
    c.d_r.alloc(std::max(c.d_r.n, (size_t)nrhs_all * nd));
    const int grid = grid_of(n);
    c.d_partials.alloc(std::max(c.d_partials.n, (size_t)grid * kMaxRhs * 3));
    if (mixed) {
        c.d_p32.alloc(std::max(c.d_p32.n, (size_t)kMaxRhs * 4 * n));
        c.d_ap32.alloc(std::max(c.d_ap32.n, (size_t)kMaxRhs * nd));
    } else {  // FP64: 2 x double2 per node; split: hi + lo float4 per node (same bytes)
        c.d_p64.alloc(std::max(c.d_p64.n, (size_t)kMaxRhs * 4 * n));
        c.d_ap64.alloc(std::max(c.d_ap64.n, (size_t)kMaxRhs * nd));
    }
    if (split) c.d_xpair.alloc(std::max(c.d_xpair.n, (size_t)2 * n));
    if (split_only) c.d_xtrip.alloc(std::max(c.d_xtrip.n, (size_t)3 * n));
    // one scalar set per instance (slot 0 of kMaxRhs), persistent so the
    // captured iteration graphs stay valid across solves
    const int NI = c.n_inst > 1 ? c.n_inst : 1;
    // a batched stack keeps one CTA per 128 rows (its reductions are per instance)
    const int grid_cg = (split && NI == 1) ? std::min(grid, kPersistCtas) : grid;
    const size_t sc_need = sizeof(RhsScalars) * NI * kMaxRhs, tk_need = sizeof(uint32_t) * NI * 4;
    if (c.pcg_sc.n < sc_need) c.pcg_sc.alloc(sc_need);
    if (c.pcg_ctl.n < sizeof(Control)) c.pcg_ctl.alloc(sizeof(Control));
    if (NI > 1 && c.pcg_tk.n < tk_need) c.pcg_tk.alloc(tk_need);
    RhsScalars* d_sc = reinterpret_cast<RhsScalars*>(c.pcg_sc.p);
    Control* d_ctl = reinterpret_cast<Control*>(c.pcg_ctl.p);
    ensure_pinned_scalars(c, sc_need);
    RhsScalars* h = reinterpret_cast<RhsScalars*>(c.h_sc);
    int iters_max = 0, repl = 0, status = 0;
    double relmax = 0.0;
    MgLevel& L0 = *H.L[0];
    ASEND_CUDA(cudaEventRecord(c.ev0, c.stream));
    for (int r0 = 0; r0 < nrhs_all; ++r0) {
        MgPcg M;
        std::memset(&M, 0, sizeof(M));  // padding too: the bytes key the cached graph
        PcgArgs& a = M.a;
        a.n_rows = n;
        a.nrhs = 1;
        a.n_dof = nd;
        a.slice_off = c.A.slice_off.p;
        a.row_len = c.A.row_len.p;
        a.col = c.A.col.p;
        a.v32 = c.A.v32.p;
        a.v32lo = c.A.v32lo.p;
        a.v64 = c.A.v64.p;
        a.f = d_f + (size_t)r0 * nd;
        a.x = d_x + (size_t)r0 * nd;
        a.r = c.d_r.p + (size_t)r0 * nd;
        a.p = mixed ? (void*)c.d_p32.p : (void*)c.d_p64.p;
        a.ap = mixed ? (void*)c.d_ap32.p : (void*)c.d_ap64.p;
        a.partials = c.d_partials.p;
        a.sc = d_sc;
        a.ctl = d_ctl;
        if (NI > 1) {
            a.cta_inst = c.d_cta_inst.p;
            a.inst_cta0 = c.d_inst_cta0.p;
            a.inst_ncta = c.d_inst_ncta.p;
            a.tickets = reinterpret_cast<uint32_t*>(c.pcg_tk.p);
            ASEND_CUDA(cudaMemsetAsync(c.pcg_tk.p, 0, tk_need, c.stream));
        }
        M.b0 = L0.b.p;
        M.z = reinterpret_cast<const float4*>(L0.y4.p);
        M.binv0 = L0.binv.p;
        M.x40 = reinterpret_cast<float4*>(L0.x4.p);
        M.n_inst = NI;
        if (split) {  // the split method's correction e (FP32 pairs) starts at zero
            M.xp = c.d_xpair.p;
            M.xt = split_only ? c.d_xtrip.p : nullptr;
            k_zero_pairs<<<(2 * n + kThreads - 1) / kThreads, kThreads, 0, c.stream>>>(n, M.xp);
            ++c.launches;
        }
        ASEND_CUDA(cudaMemsetAsync(d_sc, 0, sc_need, c.stream));
        ASEND_CUDA(cudaMemsetAsync(d_ctl, 0, sizeof(Control), c.stream));
        auto launch_residual = [&](int init) {
            if (split) {  // x64 += e first (the instances being replaced), then r = f - A64 x64
                launch_k(c, k_fold_pairs, grid_cg, kThreads, 0, M, init);
                if (split_only)
                    launch_k(c, k_mg_residual_split, grid, kThreads, 0, M, init, o.rel_tol * o.rel_tol);
                else  // FP64-pipe bound: all 4 warps of every row tile in flight
                    launch_k(c, k_mg_residual<true>, grid, kThreads, 0, M, init, o.rel_tol * o.rel_tol);
                c.launches += 2;
            } else {
                launch_k(c, k_mg_residual<false>, grid, kThreads, 0, M, init, o.rel_tol * o.rel_tol);
                ++c.launches;
            }
        };
        auto launch_iteration = [&]() {
            if (mixed) {
                k_mg_spmv_dot<float, float><<<grid, kThreads, 0, c.stream>>>(M);
                k_mg_update_xr<float><<<grid, kThreads, 0, c.stream>>>(M);
            } else if (split) {
                launch_split_product(c, M, grid_cg);
                launch_k(c, k_mg_update_xr_pair, grid_cg, kThreads, 0, M);
            } else {
                k_mg_spmv_dot<double, double><<<grid, kThreads, 0, c.stream>>>(M);
                k_mg_update_xr<double><<<grid, kThreads, 0, c.stream>>>(M);
            }
            vcycle(c, a.ctl, true);
            if (mixed) {
                k_mg_rz<float><<<grid, kThreads, 0, c.stream>>>(M, 0);
                k_mg_update_p<float><<<grid, kThreads, 0, c.stream>>>(M);
            } else if (split) {
                launch_k(c, k_mg_rz_pair, grid_cg, kThreads, 0, M, 0);
                launch_k(c, k_mg_update_p_pair, grid_cg, kThreads, 0, M);
            } else {
                k_mg_rz<double><<<grid, kThreads, 0, c.stream>>>(M, 0);
                k_mg_update_p<double><<<grid, kThreads, 0, c.stream>>>(M);
            }
        };
        // V-cycle of every instance's current b0, then rz (and p = z on a
        // restart) for the instances the residual kernel marked
        auto launch_start = [&]() {
            vcycle(c, nullptr, false);
            if (mixed) k_mg_rz<float><<<grid, kThreads, 0, c.stream>>>(M, 1);
            else if (split) launch_k(c, k_mg_rz_pair, grid_cg, kThreads, 0, M, 1);
            else k_mg_rz<double><<<grid, kThreads, 0, c.stream>>>(M, 1);
            c.launches += vcycle_launches(c) + 2;
        };
        launch_residual(1);
        launch_start();
        ASEND_CUDA(cudaGetLastError());
        // G iterations as one graph, kept with the hierarchy and reused while
        // the launch arguments are the same (they fully define the graph)
        // (with everything else that changes the captured sequence: the
        // method, the chunk length, the product shape, the tail switch and
        // the launch overlap)
        std::vector<uint8_t> key(sizeof(MgPcg) + 4 * sizeof(int));
        std::memcpy(key.data(), &M, sizeof(MgPcg));
        const int extra[4] = {o.method, G, c.product_variant, (c.mg_tail ? 1 : 0) | (c.pdl ? 2 : 0)};
        std::memcpy(key.data() + sizeof(MgPcg), extra, sizeof(extra));
        cudaGraphExec_t exec = nullptr;
        for (auto& g : H.graphs)
            if (g.first == key) exec = g.second;
        if (!exec) {
            cudaGraph_t graph;
            ASEND_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            launch_k(c, k_mg_count_active, 1, 32, 0, M);
            for (int i = 0; i < G; ++i) launch_iteration();
            ASEND_CUDA(cudaStreamEndCapture(c.stream, &graph));
            ASEND_CUDA(cudaGraphInstantiate(&exec, graph, 0));
            ASEND_CUDA(cudaGraphDestroy(graph));
            if (H.graphs.size() >= 8) {
                ASEND_CUDA(cudaGraphExecDestroy(H.graphs.front().second));
                H.graphs.erase(H.graphs.begin());
            }
            H.graphs.emplace_back(key, exec);
        }
        const int per_iter = 4 + vcycle_launches(c);
        const size_t sc_bytes = sizeof(RhsScalars) * NI * kMaxRhs;
        int since_repl = 0;
        for (;;) {
            ASEND_CUDA(cudaMemcpyAsync(h, d_sc, sc_bytes, cudaMemcpyDeviceToHost, c.stream));
            ASEND_CUDA(cudaStreamSynchronize(c.stream));
            bool all_finished = true, any_replace = false, any_nonfinite = false;
            int it_now = 0;
            for (int i = 0; i < NI; ++i) {
                RhsScalars& s = h[(size_t)i * kMaxRhs];
                it_now = std::max(it_now, (int)s.iter);
                if (s.nonfinite) { any_nonfinite = true; continue; }
                if (s.finished) continue;
                all_finished = false;
                const bool drop = mixed && s.rr < 1e-4 * s.rr_last_true;
                const bool periodic = o.replace_every > 0 && since_repl >= o.replace_every;
                if (s.done || drop || periodic) {
                    s.replace = 1;
                    any_replace = true;
                }
            }
            if (any_nonfinite) { status = ASEND_NONFINITE; break; }
            if (all_finished) break;
            if (it_now >= max_it) { status = std::max(status, (int)ASEND_MAX_ITER); break; }
            if (any_replace) {
                // after convergence of the recurrence the last p update was
                // skipped: the instance restarts its direction (p = z);
                // otherwise p is kept
                ASEND_CUDA(cudaMemcpyAsync(d_sc, h, sc_bytes, cudaMemcpyHostToDevice, c.stream));
                launch_residual(0);
                launch_start();
                ++repl;
                since_repl = 0;
                continue;
            }
            ASEND_CUDA(cudaGraphLaunch(exec, c.stream));
            c.launches += (int64_t)per_iter * G + 1;
            since_repl += G;
        }
        if (split) {  // the solution: x64 + e
            launch_k(c, k_fold_pairs, grid_cg, kThreads, 0, M, 1);
            ++c.launches;
        }
        ASEND_CUDA(cudaMemcpyAsync(h, d_sc, sc_bytes, cudaMemcpyDeviceToHost, c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        for (int i = 0; i < NI; ++i) {
            const RhsScalars& s = h[(size_t)i * kMaxRhs];
            iters_max = std::max(iters_max, (int)s.iter);
            if (s.nonfinite) status = ASEND_NONFINITE;
            else if (!s.finished) status = std::max(status, (int)ASEND_MAX_ITER);
            if (s.bb == 0.0) continue;  // empty load case of this instance
            relmax = std::max(relmax, std::sqrt(s.rr_last_true / s.bb));
        }
    }
    ASEND_CUDA(cudaEventRecord(c.ev1, c.stream));
    ASEND_CUDA(cudaEventSynchronize(c.ev1));
    ASEND_CUDA(cudaGetLastError());
    float ms = 0.f;
    ASEND_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.last_method = o.method;
    if (st) {
        st->iterations = iters_max;
        st->status = status;
        st->replacements = repl;
        st->n_rhs = nrhs_all;
        st->rel_residual = relmax;
        st->ms_solve = ms;
        st->ms_assemble = c.last_assemble_ms;
        st->penalty_scale = c.sf;
    }
    return status;
}

}  // namespace

}  // namespace asend
