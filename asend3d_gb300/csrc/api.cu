// api.cu -- C ABI entry points and the host-side model (C++).
//
// The host side restates the reference's model container and input semantics
// (solverSrc/asend_run_job/src/model_input.rs, model_prep.rs, const_meth.rs,
// model_analysis.rs load building) and drives the CUDA kernels of
// k_assemble.cu, k_pcg.cu, k_adjoint.cu and k_newmark.cu.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <exception>
#include <numeric>

#include "common.cuh"
#include <nvtx3/nvToolsExt.h>

namespace {
// NVTX range over one ABI call (named phases in Nsight timelines; a no-op
// without a profiler attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};
}  // namespace

using namespace asend;

namespace {

constexpr double kPi = 3.14159265358979323846;

int nodes_per_elem(int type) {
    switch (type) {
        case 8: return 8;
        case 81: return 8;
        case 4: return 4;
        case 10: return 10;
        case 41: return 4;
        case 2: return 2;
        default: return 0;
    }
}

template <typename F>
int guarded(asend_ctx* ctx, F&& fn) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c) return ASEND_EINVAL;
    try {
        c->err.clear();
        return fn(*c);
    } catch (const InputError& e) {
        c->err = e.msg;
        return ASEND_EINVAL;
    } catch (const CudaError& e) {
        c->err = e.msg;
        return ASEND_ECUDA;
    } catch (const std::exception& e) {
        c->err = e.what();
        return ASEND_ECUDA;
    }
}

void require(bool ok, const char* msg) {
    if (!ok) throw InputError(msg);
}

// Hex8 / tet4 face tables (local node lists, element_meth.rs:525-591 and
// :460-490) used by the surface-traction load builder.
const int kHexFaces[6][4] = {{3, 2, 1, 0}, {4, 5, 6, 7}, {0, 1, 5, 4},
                             {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
const int kTetFaces[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {0, 3, 2}};

// Consistent unit-density mass image of a face traction, restricted to the
// face nodes and rescaled to area*|t| (element_equations.rs:1970-2043).  For
// the trilinear hex / linear tet the restriction of N_a N_b over the element
// is evaluated with the element's own Gauss rule on the host.
void face_load(const Ctx& c, int e, const int* ln, int fnn, const double* trac, double* el_ld) {
    const int nn = c.nn, tot = 3 * nn;
    double xyz[24];
    for (int a = 0; a < nn; ++a)
        for (int j = 0; j < 3; ++j) xyz[3 * a + j] = c.xyz[3 * (size_t)c.conn[(size_t)e * nn + a] + j];
    // Gauss data
    const double g = 0.5773502691896257;
    double pts[8][3];
    double wts[8];
    int np;
    if (c.nn == 8) {  // hex8 / brickIM: the node shape functions
        np = 8;
        int k = 0;
        for (int zc = 0; zc < 2; ++zc)
            for (int yc = 0; yc < 2; ++yc)
                for (int xc = 0; xc < 2; ++xc) {
                    pts[k][0] = xc ? g : -g;
                    pts[k][1] = yc ? g : -g;
                    pts[k][2] = zc ? g : -g;
                    wts[k] = 1.0;
                    ++k;
                }
    } else {
        np = 1;
        pts[0][0] = pts[0][1] = pts[0][2] = 0.25;
        wts[0] = 1.0 / 6.0;
    }
    double acc[24] = {0};
    for (int q = 0; q < fnn; ++q)
        for (int i = 0; i < 3; ++i) acc[3 * ln[q] + i] = trac[i];
    double ld[24] = {0};
    for (int p = 0; p < np; ++p) {
        double N[8], dN[8][3];
        const double* s = pts[p];
        if (c.nn == 8) {
            const double sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                     {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
            for (int a = 0; a < 8; ++a) {
                const double f0 = 1 + sg[a][0] * s[0], f1 = 1 + sg[a][1] * s[1], f2 = 1 + sg[a][2] * s[2];
                N[a] = 0.125 * f0 * f1 * f2;
                dN[a][0] = 0.125 * sg[a][0] * f1 * f2;
                dN[a][1] = 0.125 * sg[a][1] * f0 * f2;
                dN[a][2] = 0.125 * sg[a][2] * f0 * f1;
            }
        } else {
            N[0] = 1 - s[0] - s[1] - s[2]; N[1] = s[0]; N[2] = s[1]; N[3] = s[2];
            const double d[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
            std::memcpy(dN, d, sizeof(d));
        }
        double J[3][3] = {{0}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int a = 0; a < nn; ++a) J[i][j] += xyz[3 * a + i] * dN[a][j];
        const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                           J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        const double w = det * wts[p];
        for (int i = 0; i < tot; ++i) {
            double a = 0;
            for (int b = 0; b < nn; ++b) a += N[i / 3] * N[b] * acc[3 * b + i % 3];
            ld[i] += a * w;
        }
    }
    double tf[3] = {0, 0, 0};
    for (int i = 0; i < tot; ++i) {
        bool in_face = false;
        for (int q = 0; q < fnn; ++q) in_face |= (ln[q] == i / 3);
        el_ld[i] = in_face ? ld[i] : 0.0;
        tf[i % 3] += el_ld[i];
    }
    // area and scale
    double v1[3], v2[3], nr[3];
    for (int i = 0; i < 3; ++i) {
        if (fnn == 4) {
            v1[i] = xyz[3 * ln[2] + i] - xyz[3 * ln[0] + i];
            v2[i] = xyz[3 * ln[3] + i] - xyz[3 * ln[1] + i];
        } else {
            v1[i] = xyz[3 * ln[1] + i] - xyz[3 * ln[0] + i];
            v2[i] = xyz[3 * ln[2] + i] - xyz[3 * ln[0] + i];
        }
    }
    nr[0] = v1[1] * v2[2] - v1[2] * v2[1];
    nr[1] = v1[2] * v2[0] - v1[0] * v2[2];
    nr[2] = v1[0] * v2[1] - v1[1] * v2[0];
    const double area = 0.5 * std::sqrt(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]);
    const double vmag = std::sqrt(tf[0] * tf[0] + tf[1] * tf[1] + tf[2] * tf[2]);
    const double imag = std::sqrt(trac[0] * trac[0] + trac[1] * trac[1] + trac[2] * trac[2]);
    const double scale = area * imag / vmag;
    for (int i = 0; i < tot; ++i) el_ld[i] *= scale;
}

void ensure_case(Ctx& c, int rhs) {
    require(rhs >= 0 && rhs < 4096, "load case index out of range");
    require(c.n_dof > 0, "set the mesh before adding loads");
    while ((int)c.loads.size() <= rhs) c.loads.emplace_back(c.n_dof, 0.0);
    ++c.loads_version;  // every caller modifies the load case next
}

}  // namespace

namespace asend {

// Pattern: node adjacency from elements plus constraint couplings; sliced
// block-ELL layout; element slot map; greedy element colouring; penalty
// entry list.
void build_pattern(Ctx& c) {
    const int N = c.n_nodes, nn = c.nn, b = c.dpn, b2 = b * b;
    std::vector<std::vector<int32_t>> adj(N);
    for (int e = 0; e < c.n_el; ++e)
        for (int a = 0; a < nn; ++a)
            for (int q = 0; q < nn; ++q) adj[c.conn[(size_t)e * nn + a]].push_back(c.conn[(size_t)e * nn + q]);
    const int nrow_c = (int)c.c_rhs.size();
    for (int r = 0; r < nrow_c; ++r)
        for (int k = c.c_ptr[r]; k < c.c_ptr[r + 1]; ++k)
            for (int k2 = c.c_ptr[r]; k2 < c.c_ptr[r + 1]; ++k2)
                adj[c.c_dof[k] / b].push_back(c.c_dof[k2] / b);
    std::vector<int32_t> isolated;
    for (int i = 0; i < N; ++i) {
        auto& v = adj[i];
        if (v.empty()) {  // node without elements or constraints (e.g. instance padding)
            v.push_back(i);
            isolated.push_back(i);
        }
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        require(v.size() <= 255, "a node has more than 255 neighbouring nodes");
    }
    Sbell& A = c.A;
    A.b = b;
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
    auto pos = [&](int row, int col) -> int {
        const auto& v = adj[row];
        auto it = std::lower_bound(v.begin(), v.end(), col);
        return (int)(it - v.begin());
    };
    // element slot map
    std::vector<int32_t> slot_map((size_t)c.n_el * nn * nn);
    for (int e = 0; e < c.n_el; ++e)
        for (int a = 0; a < nn; ++a) {
            const int ra = c.conn[(size_t)e * nn + a];
            for (int q = 0; q < nn; ++q) {
                const int cb = c.conn[(size_t)e * nn + q];
                slot_map[((size_t)e * nn + a) * nn + q] = (int32_t)A.slot(ra, pos(ra, cb));
            }
        }
    // penalty entries: value index of (dof_i, dof_j) for every term pair
    std::vector<int64_t> pen_idx;
    std::vector<double> pen_coef;
    std::vector<int32_t> pen_dof;
    for (int r = 0; r < nrow_c; ++r)
        for (int k = c.c_ptr[r]; k < c.c_ptr[r + 1]; ++k)
            for (int k2 = c.c_ptr[r]; k2 < c.c_ptr[r + 1]; ++k2) {
                const int di = c.c_dof[k], dj = c.c_dof[k2];
                const int ni = di / b, ai = di % b, nj = dj / b, aj = dj % b;
                const int64_t slot = A.slot(ni, pos(ni, nj));
                const int64_t g = slot / kSlice, lane = slot % kSlice;
                pen_idx.push_back((g * b2 + ai * b + aj) * kSlice + lane);
                pen_coef.push_back(c.c_coef[k] * c.c_coef[k2]);
                pen_dof.push_back(di);
            }
    // greedy colouring with per-node colour masks
    std::vector<uint64_t> mask(N, 0);
    c.colour_of.assign(c.n_el, 0);
    int n_col = 0;
    for (int e = 0; e < c.n_el; ++e) {
        uint64_t used = 0;
        for (int a = 0; a < nn; ++a) used |= mask[c.conn[(size_t)e * nn + a]];
        require(~used != 0, "element colouring needs more than 64 colours");
        int col = 0;
        while (used & (1ull << col)) ++col;
        c.colour_of[e] = col;
        n_col = std::max(n_col, col + 1);
        for (int a = 0; a < nn; ++a) mask[c.conn[(size_t)e * nn + a]] |= (1ull << col);
    }
    c.colour_ptr.assign(n_col + 1, 0);
    for (int e = 0; e < c.n_el; ++e) c.colour_ptr[c.colour_of[e] + 1]++;
    for (int k = 0; k < n_col; ++k) c.colour_ptr[k + 1] += c.colour_ptr[k];
    c.colour_elems.assign(c.n_el, 0);
    {
        std::vector<int32_t> fill(c.colour_ptr.begin(), c.colour_ptr.end() - 1);
        for (int e = 0; e < c.n_el; ++e) c.colour_elems[fill[c.colour_of[e]]++] = e;
    }
    // unit diagonal for isolated nodes (their DOFs decouple: x = f)
    std::vector<int64_t> unit_idx;
    for (int nd : isolated) {
        const int64_t slot = A.slot(nd, pos(nd, nd));
        const int64_t g = slot / kSlice, lane = slot % kSlice;
        for (int a = 0; a < b; ++a) unit_idx.push_back((g * b2 + a * b + a) * kSlice + lane);
    }
    // uploads
    cudaStream_t s = c.stream;
    c.d_unit_idx.upload(unit_idx, s);
    A.slice_off.upload(A.h_slice_off, s);
    A.col.upload(A.h_col, s);
    A.row_len.upload(A.h_row_len, s);
    A.diag.upload(A.h_diag, s);
    c.d_slot_map.upload(slot_map, s);
    c.d_colour_elems.upload(c.colour_elems, s);
    c.d_pen_idx.upload(pen_idx, s);
    c.d_pen_coef.upload(pen_coef, s);
    c.pen_dof = pen_dof;
    c.pen_coef_host = pen_coef;
    ASEND_CUDA(cudaStreamSynchronize(s));
    build_classes(c, slot_map);
    c.pattern_ready = true;
}

// 6x6 solid stiffness (Voigt 11,22,33,12,13,23, engineering shear) from
// engineering constants p = E1 E2 E3 nu12 nu13 nu23 G12 G13 G23 by inverting
// the compliance, as get_solid_stiff (element_properties.rs:648-764) does:
// S11 = 1/E1, S12 = -nu12/E1, S13 = -nu13/E1, S22 = 1/E2, S23 = -nu23/E2,
// S33 = 1/E3, S44 = 1/G12, S55 = 1/G13, S66 = 1/G23.  Returns false when the
// normal block is not positive definite.
bool orthotropic_cmat(const double* p, double* C) {
    for (int i = 0; i < 9; ++i)
        if (!std::isfinite(p[i])) return false;
    if (!(p[0] > 0 && p[1] > 0 && p[2] > 0 && p[6] > 0 && p[7] > 0 && p[8] > 0)) return false;
    double S[3][3] = {{1.0 / p[0], -p[3] / p[0], -p[4] / p[0]},
                      {-p[3] / p[0], 1.0 / p[1], -p[5] / p[1]},
                      {-p[4] / p[0], -p[5] / p[1], 1.0 / p[2]}};
    const double c00 = S[1][1] * S[2][2] - S[1][2] * S[2][1];
    const double c01 = S[1][2] * S[2][0] - S[1][0] * S[2][2];
    const double c02 = S[1][0] * S[2][1] - S[1][1] * S[2][0];
    const double det = S[0][0] * c00 + S[0][1] * c01 + S[0][2] * c02;
    if (!(det > 0.0) || !(S[0][0] > 0.0) || !(S[0][0] * S[1][1] - S[0][1] * S[1][0] > 0.0)) return false;
    const double inv[3][3] = {{c00 / det, (S[0][2] * S[2][1] - S[0][1] * S[2][2]) / det,
                               (S[0][1] * S[1][2] - S[0][2] * S[1][1]) / det},
                              {c01 / det, (S[0][0] * S[2][2] - S[0][2] * S[2][0]) / det,
                               (S[0][2] * S[1][0] - S[0][0] * S[1][2]) / det},
                              {c02 / det, (S[0][1] * S[2][0] - S[0][0] * S[2][1]) / det,
                               (S[0][0] * S[1][1] - S[0][1] * S[1][0]) / det}};
    for (int i = 0; i < 36; ++i) C[i] = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C[6 * i + j] = inv[i][j];
    C[21] = p[6];
    C[28] = p[7];
    C[35] = p[8];
    return true;
}

int instance_of_node(const Ctx& c, int node) {
    if (c.n_inst <= 1) return 0;
    return (int)(std::upper_bound(c.inst_node_ptr.begin(), c.inst_node_ptr.end(), node) - c.inst_node_ptr.begin()) - 1;
}

// Penalty scale of constraint row `row`: per instance in a batched stack
// (each instance is its own model, as the reference scales per model).
double row_penalty_scale(const Ctx& c, int row) {
    if (c.n_inst <= 1 || c.sf_inst.empty()) return c.sf;
    return c.sf_inst[instance_of_node(c, c.c_dof[c.c_ptr[row]] / c.dpn)];
}

// Pinned host mirror of the PCG scalars, grown on demand.
void ensure_pinned_scalars(Ctx& c, size_t bytes) {
    if (bytes <= c.h_sc_bytes) return;
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    if (c.h_sc) cudaFreeHost(c.h_sc);
    c.h_sc = nullptr;
    c.h_sc_bytes = 0;
    ASEND_CUDA(cudaMallocHost(&c.h_sc, bytes));
    c.h_sc_bytes = bytes;
}

// Load vectors incl. the penalty right-hand side -sf C^T (C*0 - q) = sf C^T q
// (const_meth.rs:105-119 at u = 0) to the device.
void upload_rhs(Ctx& c) {
    if (c.loads.empty()) {
        c.loads.emplace_back(c.n_dof, 0.0);
        ++c.loads_version;
    }
    const int nr = (int)c.loads.size();
    if (c.rhs_version == c.loads_version && c.rhs_sf == c.sf && c.d_f.n == (size_t)nr * c.n_dof &&
        c.n_inst <= 1)
        return;
    c.rhs_version = c.loads_version;
    c.rhs_sf = c.sf;
    std::vector<double> f((size_t)nr * c.n_dof);
    for (int r = 0; r < nr; ++r) {
        double* fr = &f[(size_t)r * c.n_dof];
        std::copy(c.loads[r].begin(), c.loads[r].end(), fr);
        const int nrow_c = (int)c.c_rhs.size();
        for (int q = 0; q < nrow_c; ++q) {
            const double qq = row_penalty_scale(c, q) * c.c_rhs[q];
            for (int k = c.c_ptr[q]; k < c.c_ptr[q + 1]; ++k) fr[c.c_dof[k]] += c.c_coef[k] * qq;
        }
    }
    c.nrhs = nr;
    c.d_f.upload(f, c.stream);
}

}  // namespace asend

extern "C" {

const char* asend_version(void) {
    return "asend_gpu 0.1 (sm_103a; sliced block-ELL; mixed FP32/FP64 PCG)";
}

asend_ctx* asend_create(int32_t device) {
    Ctx* c = new Ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return nullptr;
    }
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    c->h_sc_bytes = sizeof(PcgScalars) * 64;
    if (cudaMallocHost(&c->h_sc, c->h_sc_bytes) != cudaSuccess) {
        delete c;
        return nullptr;
    }
    return reinterpret_cast<asend_ctx*>(c);
}

void asend_destroy(asend_ctx* ctx) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    if (c->h_sc) cudaFreeHost(c->h_sc);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
    delete c;
}

const char* asend_last_error(const asend_ctx* ctx) {
    const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
    return c ? c->err.c_str() : "null context";
}

void* asend_stream(const asend_ctx* ctx) {
    const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
    return c ? reinterpret_cast<void*>(c->stream) : nullptr;
}

int64_t asend_kernel_launches(const asend_ctx* ctx) {
    const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
    return c ? c->launches : -1;
}

int asend_set_mesh(asend_ctx* ctx, int32_t elem_type, int32_t n_nodes, const double* coords,
                   int32_t n_elems, const int32_t* conn, const double* E, const double* nu,
                   const double* rho, const double* thickness) {
    return guarded(ctx, [&](Ctx& c) {
        const int nn = nodes_per_elem(elem_type);
        require(nn > 0,
                "unsupported element type (supported: 8 hex8, 81 brickIM, 4 tet4, 10 tet10, 41 shell4, 2 beam2)");
        require(n_nodes > 0 && n_elems > 0 && coords && conn && E && nu, "empty or null mesh input");
        for (int64_t k = 0; k < (int64_t)n_elems * nn; ++k)
            require(conn[k] >= 0 && conn[k] < n_nodes, "connectivity refers to a node out of range");
        for (int e = 0; e < n_elems; ++e) {
            require(std::isfinite(E[e]) && E[e] > 0.0, "element modulus must be positive and finite");
            require(nu[e] > -1.0 && nu[e] < 0.5, "Poisson ratio out of range (-1, 0.5)");
        }
        const bool shell = elem_type == 41, beam = elem_type == 2;
        if (beam) {
            require(n_nodes <= (1 << 29), "too many beam nodes");
            for (int e = 0; e < n_elems; ++e) {
                const double* x0 = coords + 3 * (size_t)conn[2 * (size_t)e];
                const double* x1 = coords + 3 * (size_t)conn[2 * (size_t)e + 1];
                require(x0[0] != x1[0] || x0[1] != x1[1] || x0[2] != x1[2], "beam2 element of zero length");
            }
        }
        if (shell) {
            require(n_nodes <= (1 << 29), "too many shell nodes");
            require(thickness != nullptr, "shell4 elements need a thickness per element");
            for (int e = 0; e < n_elems; ++e) {
                require(std::isfinite(thickness[e]) && thickness[e] > 0.0, "shell thickness must be positive");
                for (int a = 1; a < 4; ++a)
                    require(coords[3 * (size_t)conn[4 * (size_t)e + a] + 2] == coords[3 * (size_t)conn[4 * (size_t)e] + 2],
                            "shell4 elements must be flat in a plane z = const");
            }
        }
        ASEND_CUDA(cudaSetDevice(c.device));
        c.type = elem_type;
        c.dpn = 3;
        c.n_unodes = n_nodes;
        c.n_el = n_elems;
        if (shell || beam) {
            // two internal 3-DOF nodes per shell / beam node: DOF 6 n + c stays
            // the caller's numbering
            const int np = shell ? 4 : 2;  // physical nodes per element
            c.nn = 2 * np;
            c.udpn = 6;
            c.nip = shell ? 4 : 2;
            c.n_nodes = 2 * n_nodes;
            c.xyz.resize((size_t)6 * n_nodes);
            for (int i = 0; i < n_nodes; ++i)
                for (int j = 0; j < 3; ++j)
                    c.xyz[6 * (size_t)i + j] = c.xyz[6 * (size_t)i + 3 + j] = coords[3 * (size_t)i + j];
            c.conn.resize((size_t)n_elems * 2 * np);
            for (size_t k = 0; k < (size_t)n_elems * np; ++k) {
                c.conn[2 * k] = 2 * conn[k];
                c.conn[2 * k + 1] = 2 * conn[k] + 1;
            }
            std::vector<int32_t> c4(conn, conn + (size_t)n_elems * np);
            std::vector<double> x3(coords, coords + (size_t)3 * n_nodes);
            c.d_shell_conn.upload(c4, c.stream);
            c.d_shell_xyz.upload(x3, c.stream);
            ASEND_CUDA(cudaStreamSynchronize(c.stream));
        } else {
            c.nn = nn;
            c.udpn = 3;
            c.nip = (nn == 8) ? 8 : (nn == 10 ? 4 : 1);
            c.n_nodes = n_nodes;
            c.xyz.assign(coords, coords + (size_t)3 * n_nodes);
            c.conn.assign(conn, conn + (size_t)n_elems * nn);
            c.d_shell_conn.release();
            c.d_shell_xyz.release();
        }
        c.n_dof = c.n_nodes * c.dpn;
        c.E.assign(E, E + n_elems);
        c.nu.assign(nu, nu + n_elems);
        c.rho.assign(n_elems, 0.0);
        if (rho) c.rho.assign(rho, rho + n_elems);
        c.thk.clear();
        if (thickness) c.thk.assign(thickness, thickness + n_elems);
        c.node_sets.clear();
        c.elem_sets.clear();
        c.c_ptr.assign(1, 0);
        c.c_dof.clear();
        c.c_coef.clear();
        c.c_rhs.clear();
        c.loads.clear();
        ++c.loads_version;
        c.dv_ptr.assign(1, 0);
        c.dv_el.clear();
        c.dv_coef.clear();
        c.pattern_ready = c.assembled = c.solved = false;
        c.bx = c.by = c.bz = 0;
        c.mg.reset();
        learned_mesh_changed(c);
        c.n_inst = 0;
        c.inst_node_ptr.clear();
        c.inst_dims.clear();
        c.shell_layered = false;
        c.d_shell_abd.release();
        c.d_shell_msec.release();
        c.beam_sec.clear();
        c.beam_cm.clear();
        c.d_beam_sec.release();
        c.d_xyz.upload(c.xyz, c.stream);
        c.d_conn.upload(c.conn, c.stream);
        c.d_E.upload(c.E, c.stream);
        c.d_nu.upload(c.nu, c.stream);
        c.d_rho.upload(c.rho, c.stream);
        if (!c.thk.empty()) c.d_thk.upload(c.thk, c.stream);
        else c.d_thk.release();
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        return ASEND_OK;
    });
}

// Declares the mesh to be the structured block produced by the reference's
// swept hex meshing: node (i,j,k) = (i*(ny+1)+j)*(nz+1)+k, element (i,j,k) =
// (i*ny+j)*nz+k with corners in the hex8 order.  Enables ASEND_PC_MG.
int asend_set_block_structure(asend_ctx* ctx, int32_t nx, int32_t ny, int32_t nz) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.type == 8 || c.type == 81, "block structure needs a hex8 / brickIM mesh");
        require(nx > 0 && ny > 0 && nz > 0 && (int64_t)nx * ny * nz == c.n_el &&
                    (int64_t)(nx + 1) * (ny + 1) * (nz + 1) == c.n_nodes,
                "block dimensions do not match the mesh");
        const int co[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j)
                for (int k = 0; k < nz; ++k) {
                    const size_t e = ((size_t)i * ny + j) * nz + k;
                    for (int a = 0; a < 8; ++a) {
                        const int expect = ((i + co[a][0]) * (ny + 1) + (j + co[a][1])) * (nz + 1) + (k + co[a][2]);
                        require(c.conn[e * 8 + a] == expect, "connectivity does not follow the block numbering");
                    }
                }
        c.bx = nx;
        c.by = ny;
        c.bz = nz;
        c.mg.reset();
        return ASEND_OK;
    });
}

// Declares the mesh a stack of independent sub-systems (e.g. a batch of UQ /
// design instances): instance i owns nodes [node_ptr[i], node_ptr[i+1]) and
// every element and constraint lies inside one instance.  Each instance must
// start on a multiple of 128 nodes (pad with unused nodes), so every CTA of
// the PCG kernels belongs to one instance; convergence, step lengths and
// stopping are then per instance and load case.
int asend_set_instances(asend_ctx* ctx, int32_t n_inst, const int32_t* node_ptr) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.n_nodes > 0, "set the mesh first");
        require(c.type != 41 && c.type != 2, "batched instances take solid meshes");
        require(n_inst >= 1 && node_ptr, "need at least one instance");
        require(node_ptr[0] == 0 && node_ptr[n_inst] == c.n_nodes, "node_ptr must span all nodes");
        for (int i = 0; i < n_inst; ++i) {
            require(node_ptr[i + 1] > node_ptr[i], "empty instance");
            require(node_ptr[i] % 128 == 0, "each instance must start at a multiple of 128 nodes");
        }
        std::vector<int32_t> inst_of(c.n_nodes);
        for (int i = 0; i < n_inst; ++i)
            for (int v = node_ptr[i]; v < node_ptr[i + 1]; ++v) inst_of[v] = i;
        for (int e = 0; e < c.n_el; ++e)
            for (int a = 1; a < c.nn; ++a)
                require(inst_of[c.conn[(size_t)e * c.nn + a]] == inst_of[c.conn[(size_t)e * c.nn]],
                        "an element spans two instances");
        for (size_t r = 0; r + 1 < c.c_ptr.size(); ++r)
            for (int k = c.c_ptr[r] + 1; k < c.c_ptr[r + 1]; ++k)
                require(inst_of[c.c_dof[k] / c.dpn] == inst_of[c.c_dof[c.c_ptr[r]] / c.dpn],
                        "a constraint spans two instances");
        const int n_cta = (c.n_nodes + 127) / 128;
        std::vector<int32_t> cta_inst(n_cta), cta0(n_inst), ncta(n_inst, 0);
        for (int b = 0; b < n_cta; ++b) cta_inst[b] = inst_of[b * 128];
        for (int b = n_cta - 1; b >= 0; --b) {
            cta0[cta_inst[b]] = b;
            ncta[cta_inst[b]]++;
        }
        c.n_inst = n_inst;
        c.inst_node_ptr.assign(node_ptr, node_ptr + n_inst + 1);
        c.inst_dims.clear();
        c.mg.reset();
        c.d_cta_inst.upload(cta_inst, c.stream);
        c.d_inst_cta0.upload(cta0, c.stream);
        c.d_inst_ncta.upload(ncta, c.stream);
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        return ASEND_OK;
    });
}

// Declares every instance of a batched stack a structured block in the
// numbering of asend_set_block_structure, relative to the instance's first
// node: instance i's elements are the next nx*ny*nz elements (instances in
// order).  Enables ASEND_PC_MG on the whole stack: one V-cycle over every
// instance's hierarchy at once.
int asend_set_instance_blocks(asend_ctx* ctx, int32_t n_inst, const int32_t* dims) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.type == 8 || c.type == 81, "instance blocks need a hex8 / brickIM mesh");
        require(c.n_inst >= 1 && n_inst == c.n_inst && dims, "declare the instances first (asend_set_instances)");
        const int co[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
        int64_t el0 = 0;
        for (int q = 0; q < n_inst; ++q) {
            const int nx = dims[3 * q], ny = dims[3 * q + 1], nz = dims[3 * q + 2];
            require(nx > 0 && ny > 0 && nz > 0, "block dimensions must be positive");
            const int node0 = c.inst_node_ptr[q];
            require((int64_t)(nx + 1) * (ny + 1) * (nz + 1) <= (int64_t)c.inst_node_ptr[q + 1] - node0,
                    "block does not fit the instance's nodes");
            require(el0 + (int64_t)nx * ny * nz <= c.n_el, "block dimensions exceed the element count");
            for (int i = 0; i < nx; ++i)
                for (int j = 0; j < ny; ++j)
                    for (int k = 0; k < nz; ++k) {
                        const size_t e = (size_t)el0 + ((size_t)i * ny + j) * nz + k;
                        for (int a = 0; a < 8; ++a) {
                            const int expect =
                                node0 + ((i + co[a][0]) * (ny + 1) + (j + co[a][1])) * (nz + 1) + (k + co[a][2]);
                            require(c.conn[e * 8 + a] == expect,
                                    "connectivity does not follow the block numbering of its instance");
                        }
                    }
            el0 += (int64_t)nx * ny * nz;
        }
        require(el0 == c.n_el, "the instance blocks do not cover every element");
        c.inst_dims.assign(dims, dims + 3 * n_inst);
        c.mg.reset();
        return ASEND_OK;
    });
}

int asend_mg_set_damping(asend_ctx* ctx, double factor) {
    return guarded(ctx, [&](Ctx& c) {
        require(std::isfinite(factor) && factor > 0.0 && factor < 2.0, "damping factor must be in (0, 2)");
        c.mg_damping = (float)factor;
        mg_invalidate_values(c);  // recompute the smoothers at the next solve
        return ASEND_OK;
    });
}

int asend_set_product_variant(asend_ctx* ctx, int32_t variant) {
    return guarded(ctx, [&](Ctx& c) {
        require(variant >= ASEND_PRODUCT_DEFAULT && variant <= ASEND_PRODUCT_STAGED_4x2,
                "unknown product variant");
        c.product_variant = variant;
        return ASEND_OK;
    });
}

int asend_mg_set_fused_tail(asend_ctx* ctx, int32_t enable) {
    return guarded(ctx, [&](Ctx& c) {
        require(enable == 0 || enable == 1, "enable must be 0 or 1");
        c.mg_tail = enable != 0;
        return ASEND_OK;
    });
}

int asend_set_launch_overlap(asend_ctx* ctx, int32_t enable) {
    return guarded(ctx, [&](Ctx& c) {
        require(enable == 0 || enable == 1, "enable must be 0 or 1");
        c.pdl = enable != 0;
        return ASEND_OK;
    });
}

int asend_mg_levels(const asend_ctx* ctx) {
    const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
    return c ? mg_levels(*c) : ASEND_EINVAL;
}

int asend_mg_level_info(asend_ctx* ctx, int32_t level, int32_t* dims, double* lambda_est, double* lambda_bound,
                        double* omega) {
    return guarded(ctx, [&](Ctx& c) {
        mg_level_info(c, level, dims, lambda_est, lambda_bound, omega);
        return ASEND_OK;
    });
}

int asend_mg_vcycle(asend_ctx* ctx, const float* b, float* z) {
    return guarded(ctx, [&](Ctx& c) {
        require(b && z, "null vector");
        require(c.assembled, "assemble first");
        mg_vcycle_host(c, b, z);
        return ASEND_OK;
    });
}

int asend_set_modulus(asend_ctx* ctx, const double* E) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.n_el > 0 && E, "set the mesh first");
        for (int e = 0; e < c.n_el; ++e)
            require(std::isfinite(E[e]) && E[e] > 0.0, "element modulus must be positive and finite");
        c.E.assign(E, E + c.n_el);
        c.d_E.upload(c.E, c.stream);
        c.assembled = c.solved = false;
        return ASEND_OK;
    });
}

int asend_orthotropic_cmat(const double* props, double* C_out) {
    if (!props || !C_out) return ASEND_EINVAL;
    return orthotropic_cmat(props, C_out) ? ASEND_OK : ASEND_EINVAL;
}

// Layered shell section: layers bottom to top from z = -t (1 + z_offset) / 2;
// each layer's plane-stress stiffness Q = S^-1 (S from E1, E2, nu12, G12) is
// turned to the section axes as Qbar = Ts Q Te^-1 with the stress and strain
// rotations of its angle, and integrated through its thickness into A (z^0),
// B (z^1) and D (z^2); the section mass integrates the layer density the
// same way (translation 1, coupling +-z, rotation z^2).
static bool shell_section(int n_lay, const double* L, double z_offset, double* C, double* M) {
    std::fill(C, C + 81, 0.0);
    std::fill(M, M + 36, 0.0);
    double tot = 0.0;
    for (int k = 0; k < n_lay; ++k) {
        const double* p = L + 7 * k;
        for (int i = 0; i < 7; ++i)
            if (!std::isfinite(p[i])) return false;
        if (!(p[0] > 0 && p[1] > 0 && p[3] > 0 && p[5] > 0 && p[4] >= 0)) return false;
        tot += p[5];
    }
    double z0 = -0.5 * tot * (1.0 + z_offset);
    for (int k = 0; k < n_lay; ++k) {
        const double* p = L + 7 * k;
        const double E1 = p[0], E2 = p[1], n12 = p[2], G12 = p[3], rho = p[4], th = p[5];
        const double z1 = z0 + th;
        // Q = inverse of [[1/E1, -n12/E1, 0], [-n12/E1, 1/E2, 0], [0, 0, 1/G12]]
        const double det = 1.0 / (E1 * E2) - n12 * n12 / (E1 * E1);
        if (!(det > 0.0)) return false;
        double Q[3][3] = {{1.0 / E2 / det, n12 / E1 / det, 0.0}, {n12 / E1 / det, 1.0 / E1 / det, 0.0},
                          {0.0, 0.0, G12}};
        const double a = p[6] * (M_PI / 180.0), c = std::cos(a), s = std::sin(a);
        const double Ts[3][3] = {{c * c, s * s, -2.0 * c * s}, {s * s, c * c, 2.0 * c * s}, {c * s, -s * c, c * c - s * s}};
        double Te[3][3] = {{c * c, s * s, -c * s}, {s * s, c * c, c * s}, {2.0 * c * s, -2.0 * s * c, c * c - s * s}};
        // Te^-1 by the adjugate
        double Ti[3][3];
        const double dT = Te[0][0] * (Te[1][1] * Te[2][2] - Te[1][2] * Te[2][1]) -
                          Te[0][1] * (Te[1][0] * Te[2][2] - Te[1][2] * Te[2][0]) +
                          Te[0][2] * (Te[1][0] * Te[2][1] - Te[1][1] * Te[2][0]);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                const int i1 = (j + 1) % 3, i2 = (j + 2) % 3, j1 = (i + 1) % 3, j2 = (i + 2) % 3;
                Ti[i][j] = (Te[i1][j1] * Te[i2][j2] - Te[i1][j2] * Te[i2][j1]) / dT;
            }
        double Qb[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double acc = 0.0;
                for (int l = 0; l < 3; ++l)
                    for (int m = 0; m < 3; ++m) acc += Ts[i][l] * Q[l][m] * Ti[m][j];
                Qb[i][j] = acc;
            }
        const double fa = z1 - z0, fb = 0.5 * (z1 * z1 - z0 * z0), fd = (z1 * z1 * z1 - z0 * z0 * z0) / 3.0;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                C[9 * i + j] += fa * Qb[i][j];
                C[9 * i + j + 3] += fb * Qb[i][j];
                C[9 * (i + 3) + j] += fb * Qb[i][j];
                C[9 * (i + 3) + j + 3] += fd * Qb[i][j];
            }
        for (int i = 0; i < 3; ++i) {
            M[7 * i] += rho * fa;
            M[7 * (i + 3)] += rho * fd;
        }
        // translation-rotation coupling: u with theta_y (+), v with theta_x (-)
        M[0 * 6 + 4] += rho * fb;
        M[4 * 6 + 0] += rho * fb;
        M[1 * 6 + 3] -= rho * fb;
        M[3 * 6 + 1] -= rho * fb;
        z0 = z1;
    }
    C[60] = C[70] = C[80] = C[20];
    return true;
}

int asend_shell_section(int32_t n_layers, const double* layers, double z_offset, double* abd_out,
                        double* msec_out) {
    if (n_layers < 1 || !layers || !abd_out || !msec_out || !std::isfinite(z_offset)) return ASEND_EINVAL;
    return shell_section(n_layers, layers, z_offset, abd_out, msec_out) ? ASEND_OK : ASEND_EINVAL;
}

int asend_set_shell_sections(asend_ctx* ctx, const double* abd, const double* msec) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.type == 41, "layered sections take shell4 meshes");
        if (!abd) {
            c.shell_layered = false;
            c.d_shell_abd.release();
            c.d_shell_msec.release();
        } else {
            require(msec != nullptr, "layered sections need their section mass");
            const size_t n = (size_t)c.n_el;
            for (size_t i = 0; i < n * 81; ++i) require(std::isfinite(abd[i]), "non-finite ABD entry");
            for (size_t i = 0; i < n * 36; ++i) require(std::isfinite(msec[i]), "non-finite section mass entry");
            c.d_shell_abd.upload(abd, n * 81, c.stream);
            c.d_shell_msec.upload(msec, n * 36, c.stream);
            ASEND_CUDA(cudaStreamSynchronize(c.stream));
            c.shell_layered = true;
        }
        c.assembled = c.solved = false;
        return ASEND_OK;
    });
}

int asend_set_beam_sections(asend_ctx* ctx, const double* sections) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.type == 2, "beam sections take beam2 meshes");
        require(sections != nullptr, "null section table");
        for (int e = 0; e < c.n_el; ++e) {
            const double* s = sections + (size_t)e * 10;
            for (int k = 0; k < 10; ++k) require(std::isfinite(s[k]), "beam section values must be finite");
            require(s[0] > 0.0 && s[3] > 0.0 && s[4] > 0.0 && s[6] > 0.0,
                    "beam section: area, I3, I4 and J must be positive");
            // the frame: v must not lie along the element axis
            const int n0 = c.conn[(size_t)e * 4], n1 = c.conn[(size_t)e * 4 + 2];
            double d[3], cr[3];
            for (int j = 0; j < 3; ++j) d[j] = c.xyz[3 * (size_t)n1 + j] - c.xyz[3 * (size_t)n0 + j];
            const double* v = s + 7;
            cr[0] = d[1] * v[2] - d[2] * v[1];
            cr[1] = d[2] * v[0] - d[0] * v[2];
            cr[2] = d[0] * v[1] - d[1] * v[0];
            const double nc = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
            const double nd = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            const double nv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            require(nc > 1e-9 * nd * nv, "beam section direction v lies along the element axis");
        }
        c.beam_sec.assign(sections, sections + (size_t)c.n_el * 10);
        c.d_beam_sec.upload(beam_device_table(c), c.stream);
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        c.assembled = c.solved = false;
        return ASEND_OK;
    });
}

int asend_set_beam_section_matrices(asend_ctx* ctx, const double* stiffness, const double* mass) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.type == 2, "beam section matrices take beam2 meshes");
        require(c.beam_sec.size() == (size_t)c.n_el * 10, "set the beam sections first");
        if (!stiffness && !mass) {
            c.beam_cm.clear();
        } else {
            c.beam_cm.assign((size_t)c.n_el * 72, 0.0);
            for (int e = 0; e < c.n_el; ++e)
                for (int k = 0; k < 36; ++k) {
                    const double cv = stiffness ? stiffness[(size_t)e * 36 + k] : 0.0;
                    const double mv = mass ? mass[(size_t)e * 36 + k] : 0.0;
                    require(std::isfinite(cv) && std::isfinite(mv), "beam section matrices must be finite");
                    c.beam_cm[(size_t)e * 72 + k] = cv;
                    c.beam_cm[(size_t)e * 72 + 36 + k] = mv;
                }
        }
        c.d_beam_sec.upload(beam_device_table(c), c.stream);
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        c.assembled = c.solved = false;
        return ASEND_OK;
    });
}

int asend_set_orthotropic(asend_ctx* ctx, const double* props) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.n_el > 0, "set the mesh first");
        if (!props) {
            c.ortho.clear();
            c.d_cmat.release();
        } else {
            require(c.type == 8 || c.type == 4 || c.type == 10,
                    "orthotropic materials take hex8 / tet4 / tet10 meshes (elements without condensed internal DOF)");
            std::vector<double> C((size_t)c.n_el * 36);
            for (int e = 0; e < c.n_el; ++e)
                require(orthotropic_cmat(props + (size_t)e * 9, &C[(size_t)e * 36]),
                        "orthotropic constants give no positive definite stiffness");
            c.ortho.assign(props, props + (size_t)c.n_el * 9);
            c.d_cmat.upload(C, c.stream);
            ASEND_CUDA(cudaStreamSynchronize(c.stream));
        }
        c.assembled = c.solved = false;
        return ASEND_OK;
    });
}

int asend_set_damping(asend_ctx* ctx, double rayleigh_cm, double rayleigh_ck, const double* D) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.n_el > 0, "set the mesh first");
        require(std::isfinite(rayleigh_cm) && std::isfinite(rayleigh_ck) && rayleigh_cm >= 0.0 && rayleigh_ck >= 0.0,
                "Rayleigh coefficients must be finite and non-negative");
        require(!(rayleigh_ck != 0.0 || D) || c.type == 8 || c.type == 4 || c.type == 10,
                "stiffness-proportional and material damping take hex8 / tet4 / tet10 meshes (elements without "
                "condensed internal DOF)");
        c.ray_cm = rayleigh_cm;
        c.ray_ck = rayleigh_ck;
        if (D) {
            c.dmat.assign(D, D + (size_t)c.n_el * 36);
            c.d_dmat.upload(c.dmat, c.stream);
            ASEND_CUDA(cudaStreamSynchronize(c.stream));
        } else {
            c.dmat.clear();
            c.d_dmat.release();
        }
        c.assembled = c.solved = false;
        return ASEND_OK;
    });
}

int asend_set_lumped_mass(asend_ctx* ctx, int32_t on) {
    return guarded(ctx, [&](Ctx& c) {
        c.lump = on != 0;
        c.assembled = c.solved = false;
        return ASEND_OK;
    });
}

int asend_add_node_set(asend_ctx* ctx, int32_t n, const int32_t* nodes) {
    return guarded(ctx, [&](Ctx& c) {
        require(n >= 1 && nodes, "empty node set");
        for (int i = 0; i < n; ++i) require(nodes[i] >= 0 && nodes[i] < c.n_unodes, "node set entry out of range");
        c.node_sets.emplace_back(nodes, nodes + n);
        return (int)c.node_sets.size() - 1;
    });
}

int asend_add_element_set(asend_ctx* ctx, int32_t n, const int32_t* elems) {
    return guarded(ctx, [&](Ctx& c) {
        require(n >= 1 && elems, "empty element set");
        for (int i = 0; i < n; ++i) require(elems[i] >= 0 && elems[i] < c.n_el, "element set entry out of range");
        c.elem_sets.emplace_back(elems, elems + n);
        return (int)c.elem_sets.size() - 1;
    });
}

// const_meth.rs:30-90 (Constraint::build_mat): the row count is the largest
// term-set size; a term over a one-node set adds that DOF to every row, a term
// over an n-node set adds its k-th node to row k.
int asend_add_constraint(asend_ctx* ctx, int32_t n_terms, const int32_t* node_set,
                         const int32_t* comp, const double* coef, double rhs) {
    return guarded(ctx, [&](Ctx& c) {
        require(n_terms >= 1 && node_set && comp && coef, "constraint needs at least one term");
        size_t rows = 1;
        for (int t = 0; t < n_terms; ++t) {
            require(node_set[t] >= 0 && node_set[t] < (int)c.node_sets.size(), "unknown node set");
            require(comp[t] >= 1 && comp[t] <= c.udpn, "constraint component out of range");
            rows = std::max(rows, c.node_sets[node_set[t]].size());
        }
        for (int t = 0; t < n_terms; ++t) {
            const size_t len = c.node_sets[node_set[t]].size();
            require(len == 1 || len == rows, "constraint term sets of mismatched size");
        }
        for (size_t r = 0; r < rows; ++r) {
            for (int t = 0; t < n_terms; ++t) {
                const auto& set = c.node_sets[node_set[t]];
                const int nd = (set.size() == 1) ? set[0] : set[r];
                c.c_dof.push_back(nd * c.udpn + comp[t] - 1);
                c.c_coef.push_back(coef[t]);
            }
            c.c_ptr.push_back((int32_t)c.c_dof.size());
            c.c_rhs.push_back(rhs);
        }
        ++c.loads_version;  // the penalty right-hand side changes with the rows
        c.mg.reset();
        c.pattern_ready = c.assembled = c.solved = false;
        return ASEND_OK;
    });
}

// build_elastic_app_load nodalForce branch (model_analysis.rs:37-46).
int asend_add_nodal_force(asend_ctx* ctx, int32_t rhs, int32_t node_set, const double* load6) {
    return guarded(ctx, [&](Ctx& c) {
        ensure_case(c, rhs);
        require(node_set >= 0 && node_set < (int)c.node_sets.size() && load6, "unknown node set");
        for (int nd : c.node_sets[node_set])
            for (int k = 0; k < c.udpn; ++k) c.loads[rhs][(size_t)nd * c.udpn + k] += load6[k];
        return ASEND_OK;
    });
}

// surfaceTraction (element_equations.rs:1970-2043); surface faces are faces
// owned by one element only (model_prep.rs:510-554).
// Surface traction (traction given) or pressure (traction = -p n on each
// loaded face, n its outward unit normal): get_app_load_dfd0,
// element_equations.rs:1970-2043.
static void surface_load(Ctx& c, int32_t rhs, int32_t elem_set, const double* norm_dir, double norm_tol_deg,
                         const double* traction, double pressure) {
    require(c.type == 8 || c.type == 81 || c.type == 4, "surface loads apply to solid element faces");
    ensure_case(c, rhs);
    require(elem_set >= 0 && elem_set < (int)c.elem_sets.size() && norm_dir, "unknown element set");
    const int nf = (c.nn == 8) ? 6 : 4, fnn = (c.nn == 8) ? 4 : 3;
    auto face_nodes = [&](int fi) -> const int* { return c.nn == 8 ? kHexFaces[fi] : kTetFaces[fi]; };
    auto key = [&](int e, int fi) {
        std::array<int32_t, 4> k{-1, -1, -1, -1};
        const int* ln = face_nodes(fi);
        for (int q = 0; q < fnn; ++q) k[q] = c.conn[(size_t)e * c.nn + ln[q]];
        for (int i = 1; i < fnn; ++i)
            for (int j = i; j > 0 && k[j - 1] > k[j]; --j) std::swap(k[j - 1], k[j]);
        return k;
    };
    std::vector<std::array<int32_t, 4>> all;
    all.reserve((size_t)c.n_el * nf);
    for (int e = 0; e < c.n_el; ++e)
        for (int fi = 0; fi < nf; ++fi) all.push_back(key(e, fi));
    std::sort(all.begin(), all.end());
    const double cos_tol = std::cos(kPi / 180.0 * norm_tol_deg);
    double el_ld[24], keep[24];
    for (int e : c.elem_sets[elem_set]) {
        bool any = false;
        for (int fi = 0; fi < nf; ++fi) {
            const auto k = key(e, fi);
            auto rg = std::equal_range(all.begin(), all.end(), k);
            if (rg.second - rg.first != 1) continue;
            const int* ln = face_nodes(fi);
            double v1[3], v2[3], nr[3];
            for (int i = 0; i < 3; ++i) {
                const double* x0 = &c.xyz[3 * (size_t)c.conn[(size_t)e * c.nn + ln[0]]];
                const double* x1 = &c.xyz[3 * (size_t)c.conn[(size_t)e * c.nn + ln[1]]];
                const double* x2 = &c.xyz[3 * (size_t)c.conn[(size_t)e * c.nn + ln[2]]];
                if (fnn == 4) {
                    const double* x3 = &c.xyz[3 * (size_t)c.conn[(size_t)e * c.nn + ln[3]]];
                    v1[i] = x2[i] - x0[i];
                    v2[i] = x3[i] - x1[i];
                } else {
                    v1[i] = x1[i] - x0[i];
                    v2[i] = x2[i] - x0[i];
                }
            }
            nr[0] = v1[1] * v2[2] - v1[2] * v2[1];
            nr[1] = v1[2] * v2[0] - v1[0] * v2[2];
            nr[2] = v1[0] * v2[1] - v1[1] * v2[0];
            const double l = std::sqrt(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]);
            const double dp = (norm_dir[0] * nr[0] + norm_dir[1] * nr[1] + norm_dir[2] * nr[2]) / l;
            if (!(dp > cos_tol)) continue;
            double tr[3];
            for (int i = 0; i < 3; ++i) tr[i] = traction ? traction[i] : -pressure * nr[i] / l;
            face_load(c, e, ln, fnn, tr, el_ld);
            std::copy(el_ld, el_ld + 3 * c.nn, keep);  // last loaded face survives
            any = true;
        }
        if (any)
            for (int i = 0; i < 3 * c.nn; ++i)
                c.loads[rhs][(size_t)c.conn[(size_t)e * c.nn + i / 3] * 3 + i % 3] += keep[i];
    }
}

int asend_add_surface_traction(asend_ctx* ctx, int32_t rhs, int32_t elem_set, const double* norm_dir,
                               double norm_tol_deg, const double* traction) {
    return guarded(ctx, [&](Ctx& c) {
        require(traction != nullptr, "null traction");
        surface_load(c, rhs, elem_set, norm_dir, norm_tol_deg, traction, 0.0);
        return ASEND_OK;
    });
}

int asend_add_surface_pressure(asend_ctx* ctx, int32_t rhs, int32_t elem_set, const double* norm_dir,
                               double norm_tol_deg, double pressure) {
    return guarded(ctx, [&](Ctx& c) {
        require(std::isfinite(pressure), "pressure must be finite");
        surface_load(c, rhs, elem_set, norm_dir, norm_tol_deg, nullptr, pressure);
        return ASEND_OK;
    });
}

// Integrals of the element's node shape functions, w_a = int N_a dV (shells:
// t int N_a dA), so that the inertial load of a uniform acceleration acc,
// M_e acc = rho_e w_a acc on the translational DOF (get_rum_dfd0 with a
// constant acceleration field, element_equations.rs:420-626), is formed
// without the mass matrix.  Returns the number of physical nodes; dof[a] is
// node a's first translational DOF; cent the mean of the node coordinates.
static int element_node_weights(const Ctx& c, int e, double* w, int64_t* dof, double* cent) {
    if (c.type == 2) {  // beam2: rho A L / 2 per node on the translations
        require(c.beam_sec.size() == (size_t)c.n_el * 10, "beam2 meshes need asend_set_beam_sections");
        const double* s = &c.beam_sec[(size_t)e * 10];
        require(s[1] == 0.0 && s[2] == 0.0,
                "body loads on beam sections with first moments (I1, I2 != 0) are not built");
        require(c.beam_cm.empty() || !(c.beam_cm[(size_t)e * 72 + 36] > 0.0),
                "body loads on beam sections with a given mass matrix are not built");
        double x[2][3], l2 = 0.0;
        for (int a = 0; a < 2; ++a) {
            const int pn = c.conn[(size_t)e * 4 + 2 * a];
            for (int j = 0; j < 3; ++j) x[a][j] = c.xyz[3 * (size_t)pn + j];
            dof[a] = (int64_t)(pn / 2) * 6;
        }
        for (int j = 0; j < 3; ++j) {
            l2 += (x[1][j] - x[0][j]) * (x[1][j] - x[0][j]);
            cent[j] = 0.5 * (x[0][j] + x[1][j]);
        }
        w[0] = w[1] = 0.5 * s[0] * std::sqrt(l2);
        return 2;
    }
    if (c.type == 41) {
        if (c.shell_layered) throw InputError("body loads on layered shell sections are not built");
        double x[4][3];
        for (int a = 0; a < 4; ++a) {
            const int pn = c.conn[(size_t)e * 8 + 2 * a];  // translational pseudo-node 2 n
            for (int j = 0; j < 3; ++j) x[a][j] = c.xyz[3 * (size_t)pn + j];
            dof[a] = (int64_t)(pn / 2) * 6;
        }
        const double g = 0.5773502691896257, sg[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
        for (int a = 0; a < 4; ++a) w[a] = 0.0;
        for (int p = 0; p < 4; ++p) {
            const double s = sg[p][0] * g, t = sg[p][1] * g;
            double J[2][2] = {{0, 0}, {0, 0}}, N[4];
            for (int a = 0; a < 4; ++a) {
                N[a] = 0.25 * (1 + sg[a][0] * s) * (1 + sg[a][1] * t);
                const double ds = 0.25 * sg[a][0] * (1 + sg[a][1] * t), dt = 0.25 * sg[a][1] * (1 + sg[a][0] * s);
                for (int j = 0; j < 2; ++j) {
                    J[j][0] += x[a][j] * ds;
                    J[j][1] += x[a][j] * dt;
                }
            }
            const double det = std::fabs(J[0][0] * J[1][1] - J[0][1] * J[1][0]);
            for (int a = 0; a < 4; ++a) w[a] += N[a] * det * c.thk[e];
        }
        for (int j = 0; j < 3; ++j) cent[j] = 0.25 * (x[0][j] + x[1][j] + x[2][j] + x[3][j]);
        return 4;
    }
    const int nn = c.nn;
    double x[10][3];
    for (int a = 0; a < nn; ++a) {
        const int nd = c.conn[(size_t)e * nn + a];
        for (int j = 0; j < 3; ++j) x[a][j] = c.xyz[3 * (size_t)nd + j];
        dof[a] = (int64_t)nd * 3;
    }
    for (int j = 0; j < 3; ++j) {
        cent[j] = 0.0;
        for (int a = 0; a < nn; ++a) cent[j] += x[a][j];
        cent[j] /= nn;
    }
    if (nn == 4) {  // linear tet: int N_a = V / 4
        double v1[3], v2[3], v3[3];
        for (int j = 0; j < 3; ++j) {
            v1[j] = x[1][j] - x[0][j];
            v2[j] = x[2][j] - x[0][j];
            v3[j] = x[3][j] - x[0][j];
        }
        const double det = v1[0] * (v2[1] * v3[2] - v2[2] * v3[1]) - v1[1] * (v2[0] * v3[2] - v2[2] * v3[0]) +
                           v1[2] * (v2[0] * v3[1] - v2[1] * v3[0]);
        for (int a = 0; a < 4; ++a) w[a] = std::fabs(det) / 24.0;
        return 4;
    }
    if (nn == 10) {  // quadratic tet: the 4-point rule, weights 1/24
        for (int a = 0; a < 10; ++a) w[a] = 0.0;
        for (int p = 0; p < 4; ++p) {
            double s[3], N[10], dn[10][3], J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            tet10_point(p, s);
            tet10_shape(s, N, dn);
            for (int a = 0; a < 10; ++a)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) J[i][j] += x[a][i] * dn[a][j];
            const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                               J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
            for (int a = 0; a < 10; ++a) w[a] += N[a] * det / 24.0;
        }
        return 10;
    }
    const double g = 0.5773502691896257;
    const double sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                             {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (int a = 0; a < 8; ++a) w[a] = 0.0;
    for (int p = 0; p < 8; ++p) {
        const double s[3] = {(p & 1) ? g : -g, (p & 2) ? g : -g, (p & 4) ? g : -g};
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, N[8];
        for (int a = 0; a < 8; ++a) {
            const double f0 = 1 + sg[a][0] * s[0], f1 = 1 + sg[a][1] * s[1], f2 = 1 + sg[a][2] * s[2];
            N[a] = 0.125 * f0 * f1 * f2;
            const double dn[3] = {0.125 * sg[a][0] * f1 * f2, 0.125 * sg[a][1] * f0 * f2, 0.125 * sg[a][2] * f0 * f1};
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) J[i][j] += x[a][i] * dn[j];
        }
        const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                           J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        for (int a = 0; a < 8; ++a) w[a] += N[a] * det;
    }
    return 8;
}

// Element loads of a uniform acceleration field over an element set
// (get_app_load_dfd0, element_equations.rs:1875-1968): body force (force per
// unit volume, unit density), gravity (acceleration, the element's density)
// and centrifugal (omega^2 times the distance of the element centroid from
// the axis through center, the element's density).
int asend_add_body_load(asend_ctx* ctx, int32_t rhs, int32_t elem_set, int32_t kind, const double* vec,
                        double omega, const double* center, const double* axis) {
    return guarded(ctx, [&](Ctx& c) {
        ensure_case(c, rhs);
        require(elem_set >= 0 && elem_set < (int)c.elem_sets.size(), "unknown element set");
        require(kind >= ASEND_LOAD_BODY_FORCE && kind <= ASEND_LOAD_CENTRIFUGAL, "unknown body load kind");
        require(kind == ASEND_LOAD_CENTRIFUGAL ? (center && axis && std::isfinite(omega)) : vec != nullptr,
                "body load without its data");
        require(kind == ASEND_LOAD_BODY_FORCE || !c.rho.empty(), "gravity and centrifugal loads need densities");
        double ax[3] = {0, 0, 0};
        if (kind == ASEND_LOAD_CENTRIFUGAL) {  // the axis is normalised on input (load_meth.rs:41-51)
            const double l = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
            require(l > 0.0, "centrifugal axis of zero length");
            for (int j = 0; j < 3; ++j) ax[j] = axis[j] / l;
        }
        double w[10], cent[3];
        int64_t dof[10];
        for (int e : c.elem_sets[elem_set]) {
            const int na = element_node_weights(c, e, w, dof, cent);
            double acc[3];
            double rho = (kind == ASEND_LOAD_BODY_FORCE) ? 1.0 : c.rho[e];
            if (kind == ASEND_LOAD_CENTRIFUGAL) {
                double d[3], dp = 0.0;
                for (int j = 0; j < 3; ++j) {
                    d[j] = cent[j] - center[j];
                    dp += ax[j] * d[j];
                }
                for (int j = 0; j < 3; ++j) acc[j] = omega * omega * (d[j] - ax[j] * dp);
            } else {
                for (int j = 0; j < 3; ++j) acc[j] = vec[j];
            }
            for (int a = 0; a < na; ++a)
                for (int j = 0; j < 3; ++j) c.loads[rhs][(size_t)dof[a] + j] += rho * w[a] * acc[j];
        }
        return ASEND_OK;
    });
}

int asend_add_load_vector(asend_ctx* ctx, int32_t rhs, const double* f) {
    return guarded(ctx, [&](Ctx& c) {
        ensure_case(c, rhs);
        require(f != nullptr, "null load vector");
        for (int i = 0; i < c.n_dof; ++i) c.loads[rhs][i] += f[i];
        return ASEND_OK;
    });
}

int asend_clear_loads(asend_ctx* ctx) {
    return guarded(ctx, [&](Ctx& c) {
        c.loads.clear();
        ++c.loads_version;
        c.solved = false;
        return ASEND_OK;
    });
}

int asend_n_dof(const asend_ctx* ctx) {
    const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
    return c ? c->n_dof : ASEND_EINVAL;
}
int asend_n_load_cases(const asend_ctx* ctx) {
    const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
    return c ? (int)c->loads.size() : ASEND_EINVAL;
}

int asend_get_load_vector(asend_ctx* ctx, int32_t rhs, double* f_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(rhs >= 0 && rhs < (int)c.loads.size() && f_out, "bad load case");
        std::copy(c.loads[rhs].begin(), c.loads[rhs].end(), f_out);
        if (c.assembled) {
            const int nrow_c = (int)c.c_rhs.size();
            for (int q = 0; q < nrow_c; ++q)
                for (int k = c.c_ptr[q]; k < c.c_ptr[q + 1]; ++k)
                    f_out[c.c_dof[k]] += c.c_coef[k] * row_penalty_scale(c, q) * c.c_rhs[q];
        }
        return ASEND_OK;
    });
}

int asend_assemble(asend_ctx* ctx, int32_t precision, int32_t dynamic, double dt, double beta,
                   double gamma) {
    return guarded(ctx, [&](Ctx& c) {
        NvtxRange nvtx_range("asend_assemble");
        require(c.n_el > 0, "set the mesh first");
        require(precision == 32 || precision == 48 || precision == 64, "precision must be 32, 48 or 64");
        require(dynamic >= 0 && dynamic <= 2, "dynamic must be 0, 1 or 2");
        if (dynamic == 1) require(dt > 0.0 && beta != gamma, "Newmark needs dt > 0 and beta != gamma");
        if (dynamic) for (double r : c.rho) require(r > 0.0, "dynamic / modal assembly needs positive densities");
        ASEND_CUDA(cudaSetDevice(c.device));
        c.dynamic = dynamic != 0;
        c.modal = dynamic == 2;
        c.dt = dt;
        c.beta = beta;
        c.gamma = gamma;
        c.cM = dynamic == 1 ? -1.0 / (dt * dt * (beta - gamma)) : 0.0;
        if (!c.pattern_ready) build_pattern(c);
        assemble_operator(c, precision);
        c.assembled = true;
        c.solved = false;
        return ASEND_OK;
    });
}

int asend_get_coloring(asend_ctx* ctx, int32_t* colour_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.pattern_ready, "assemble first");
        if (colour_out) std::copy(c.colour_of.begin(), c.colour_of.end(), colour_out);
        return (int)c.colour_ptr.size() - 1;
    });
}

// Scalar CSR view (sorted columns) of the assembled operator; which 0 = the
// operator with penalty, 1 = the mass matrix, 2 = the operator without the
// penalty terms.
int asend_get_csr(asend_ctx* ctx, int32_t which, int64_t* nnz_out, int64_t* row_ptr, int32_t* col,
                  double* val) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.assembled, "assemble first");
        require(which >= 0 && which <= 3, "which must be 0, 1, 2 or 3");
        require(which != 1 || c.dynamic, "no mass matrix (static assembly)");
        require(which != 3 || c.A.d64.n, "no damping matrix (assembly without damping)");
        const Sbell& A = c.A;
        const int b = A.b, b2 = b * b;
        const int64_t nnz = A.nnz_scalar();
        if (nnz_out) *nnz_out = nnz;
        if (!row_ptr && !col && !val) return ASEND_OK;
        std::vector<double> h;
        if (val) {
            if (which != 1 && which != 3) ensure_v64(c);
            const DArr<double>& src = (which == 1) ? A.m64 : (which == 3) ? A.d64 : A.v64;
            h.resize(src.n);
            ASEND_CUDA(cudaMemcpyAsync(h.data(), src.p, src.n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            ASEND_CUDA(cudaStreamSynchronize(c.stream));
            if (which == 2) {
                std::vector<int64_t> pi(c.d_pen_idx.n);
                std::vector<double> pc(c.d_pen_coef.n);
                ASEND_CUDA(cudaMemcpy(pi.data(), c.d_pen_idx.p, pi.size() * sizeof(int64_t), cudaMemcpyDeviceToHost));
                ASEND_CUDA(cudaMemcpy(pc.data(), c.d_pen_coef.p, pc.size() * sizeof(double), cudaMemcpyDeviceToHost));
                for (size_t k = 0; k < pi.size(); ++k) h[pi[k]] -= c.sf * pc[k];
            }
        }
        int64_t k = 0;
        if (row_ptr) row_ptr[0] = 0;
        for (int r = 0; r < A.n_rows; ++r) {
            const int s = r / kSlice, lane = r % kSlice;
            for (int a = 0; a < b; ++a) {
                for (int j = 0; j < A.h_row_len[r]; ++j) {
                    const int64_t g = A.h_slice_off[s] + j;
                    const int cn = A.h_col[(size_t)g * kSlice + lane];
                    for (int cc = 0; cc < b; ++cc) {
                        if (col) col[k] = cn * b + cc;
                        if (val) val[k] = h[(size_t)(g * b2 + a * b + cc) * kSlice + lane];
                        ++k;
                    }
                }
                if (row_ptr) row_ptr[r * b + a + 1] = k;
            }
        }
        return ASEND_OK;
    });
}

int asend_apply_operator(asend_ctx* ctx, int32_t precision, const double* x, double* y) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.assembled, "assemble first");
        require(x && y, "null vector");
        require(precision == 32 || precision == 48 || precision == 64, "precision must be 32, 48 or 64");
        DArr<double> dx, dy;
        dx.upload(x, c.n_dof, c.stream);
        dy.alloc(c.n_dof);
        apply_operator_device(c, precision, dx.p, dy.p);
        ASEND_CUDA(cudaMemcpyAsync(y, dy.p, c.n_dof * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        return ASEND_OK;
    });
}

int asend_time_spmv(asend_ctx* ctx, int32_t precision, int32_t n_launch, double* ms_per_launch,
                    double* bytes_per_launch) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.assembled, "assemble first");
        require(n_launch > 0, "n_launch must be positive");
        require(precision == 32 || precision == 48 || precision == 64, "precision must be 32, 48 or 64");
        double bytes = 0.0;
        const double ms = time_spmv(c, precision, n_launch, &bytes);
        if (ms_per_launch) *ms_per_launch = ms;
        if (bytes_per_launch) *bytes_per_launch = bytes;
        return ASEND_OK;
    });
}

int asend_time_mg_kernel(asend_ctx* ctx, int32_t kernel, int32_t method, int32_t n_launch, double* ms_per_launch,
                         double* bytes_per_launch) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.assembled, "assemble first");
        require(n_launch > 0, "n_launch must be positive");
        require(kernel >= 0 && kernel <= 2, "kernel must be 0, 1 or 2");
        require(method == ASEND_METHOD_FP64 || method == ASEND_METHOD_MIXED || method == ASEND_METHOD_SPLIT,
                "unknown method");
        double bytes = 0.0;
        const double ms = mg_time_kernel(c, kernel, method, n_launch, &bytes);
        if (ms_per_launch) *ms_per_launch = ms;
        if (bytes_per_launch) *bytes_per_launch = bytes;
        return ASEND_OK;
    });
}

int asend_static_solve_device(asend_ctx* ctx, const asend_solve_opts* opts, asend_solve_stats* stats) {
    return guarded(ctx, [&](Ctx& c) {
        NvtxRange nvtx_range("asend_static_solve_device");
        require(opts != nullptr, "null options");
        require(c.assembled, "assemble first");
        upload_rhs(c);
        c.d_x.alloc((size_t)c.nrhs * c.n_dof);
        const int rc = pcg_solve(c, *opts, stats, false, c.d_f.p, c.d_x.p, c.nrhs);
        c.solved = true;
        return rc;
    });
}

int asend_static_solve(asend_ctx* ctx, const asend_solve_opts* opts, double* u_io, asend_solve_stats* stats) {
    return guarded(ctx, [&](Ctx& c) {
        NvtxRange nvtx_range("asend_static_solve");
        require(opts != nullptr && u_io != nullptr, "null argument");
        require(c.assembled, "assemble first");
        upload_rhs(c);
        const size_t n = (size_t)c.nrhs * c.n_dof;
        if (opts->warm_start) c.d_x.upload(u_io, n, c.stream);
        else c.d_x.alloc(n);
        const int rc = pcg_solve(c, *opts, stats, opts->warm_start != 0, c.d_f.p, c.d_x.p, c.nrhs);
        c.solved = true;
        ASEND_CUDA(cudaMemcpyAsync(u_io, c.d_x.p, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        return rc;
    });
}

int asend_get_solution(asend_ctx* ctx, int32_t rhs, double* u_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.solved, "no solution available");
        require(rhs >= 0 && rhs < c.nrhs && u_out, "bad load case");
        ASEND_CUDA(cudaMemcpyAsync(u_out, c.d_x.p + (size_t)rhs * c.n_dof, c.n_dof * sizeof(double),
                                   cudaMemcpyDeviceToHost, c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        return ASEND_OK;
    });
}

int asend_set_objective(asend_ctx* ctx, int32_t kind, int32_t node_set, int32_t comp, double coef) {
    return guarded(ctx, [&](Ctx& c) {
        require(kind == ASEND_OBJ_DISPLACEMENT || kind == ASEND_OBJ_COMPLIANCE, "unknown objective kind "
                "(element-category terms are set by asend_set_element_objective)");
        if (kind == ASEND_OBJ_DISPLACEMENT) {
            require(node_set >= 0 && node_set < (int)c.node_sets.size(), "unknown node set");
            require(comp >= 1 && comp <= c.udpn, "objective component out of range");
        }
        c.obj_kind = kind;
        c.obj_set = node_set;
        c.obj_comp = comp;
        c.obj_coef = coef;
        return ASEND_OK;
    });
}

int asend_set_element_objective(asend_ctx* ctx, const double* w_stress, const double* w_strain) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.n_el > 0, "set the mesh first");
        require(c.type == 8 || c.type == 81 || c.type == 4 || c.type == 10,
                "element-category objectives are built for hex8, brickIM, tet4 and tet10 meshes");
        const size_t m = (size_t)c.n_el * 6;
        for (const double* w : {w_stress, w_strain})
            if (w)
                for (size_t i = 0; i < m; ++i) require(std::isfinite(w[i]), "non-finite objective weight");
        std::vector<double> zero;
        if (!w_stress || !w_strain) zero.assign(m, 0.0);
        c.d_obj_wa.upload(w_stress ? w_stress : zero.data(), m, c.stream);
        c.d_obj_wb.upload(w_strain ? w_strain : zero.data(), m, c.stream);
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        c.obj_kind = ASEND_OBJ_ELEMENT;
        c.obj_set = -1;
        return ASEND_OK;
    });
}

int asend_element_fields(asend_ctx* ctx, int32_t rhs, double* eps_out, double* sig_out, double* vol_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.solved, "run a static solve first");
        require(rhs >= 0 && rhs < c.nrhs, "load case out of range");
        const size_t m = (size_t)c.n_el;
        DArr<double> eps, sig, vol;
        if (eps_out) eps.alloc(m * 6);
        if (sig_out) sig.alloc(m * 6);
        if (vol_out) vol.alloc(m);
        element_fields(c, c.d_x.p + (size_t)rhs * c.n_dof, eps.p, sig.p, vol.p);
        if (eps_out) ASEND_CUDA(cudaMemcpyAsync(eps_out, eps.p, sizeof(double) * m * 6, cudaMemcpyDeviceToHost, c.stream));
        if (sig_out) ASEND_CUDA(cudaMemcpyAsync(sig_out, sig.p, sizeof(double) * m * 6, cudaMemcpyDeviceToHost, c.stream));
        if (vol_out) ASEND_CUDA(cudaMemcpyAsync(vol_out, vol.p, sizeof(double) * m, cudaMemcpyDeviceToHost, c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        return ASEND_OK;
    });
}

// Static adjoint gradient w.r.t. per-element modulus (get_obj_gradient static
// branch, model_analysis.rs:1632-1704; solve_for_adjoint :1065-1126).
int asend_adjoint_gradient(asend_ctx* ctx, const asend_solve_opts* opts, double* L_out, double* dLdE_out,
                           asend_solve_stats* stats) {
    return guarded(ctx, [&](Ctx& c) {
        NvtxRange nvtx_range("asend_adjoint_gradient");
        require(opts != nullptr, "null options");
        require(c.solved, "run a static solve before the adjoint gradient");
        // the per-element modulus gradient scales an isotropic element; with
        // orthotropic constants the gradient goes through the strain pairs
        // (asend_material_dv_gradient)
        const bool iso = c.ortho.empty() && !c.shell_layered && !c.beam_given_stiffness();
        require(iso || !dLdE_out,
                "per-element modulus gradients need isotropic elements; use asend_material_dv_gradient");
        const size_t n = c.n_dof;
        c.d_gE.alloc(c.n_el);
        DArr<double> part, scal;
        part.alloc(256);
        scal.alloc(1);
        double L = 0.0;
        int rc = ASEND_OK;
        asend_solve_stats ast{};
        float ms_solve = 0.f;
        ASEND_CUDA(cudaEventRecord(c.ev0, c.stream));
        if (c.obj_kind == ASEND_OBJ_COMPLIANCE) {
            // L = sum_r b_r^T u_r, self-adjoint: lambda_r = u_r
            for (int r = 0; r < c.nrhs; ++r) {
                device_dot(c, n, c.d_f.p + r * n, c.d_x.p + r * n, scal.p, part.p);
                double v = 0.0;
                ASEND_CUDA(cudaMemcpyAsync(&v, scal.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
                ASEND_CUDA(cudaStreamSynchronize(c.stream));
                L += v;
                if (iso) adjoint_contract(c, c.d_x.p + r * n, c.d_x.p + r * n, c.d_gE.p, r > 0);
            }
        } else {
            DArr<double> d_dldu;
            DArr<double>& d_usum = c.d_adj_b;
            d_usum.alloc(n);
            d_usum.zero(c.stream);
            if (c.obj_kind == ASEND_OBJ_ELEMENT) {
                // element-category term: adjoint load sum_e B_c^T (b_e + C_e a_e)
                // from the caller's weights; L is evaluated by the caller
                require(c.nrhs == 1, "element-category objectives take a single load case");
                d_dldu.alloc(n);
                d_dldu.zero(c.stream);
                element_objective_rhs(c, d_dldu.p);
                device_axpy(c, n, 1.0, c.d_x.p, d_usum.p);
            } else {
                // L = coef * sum_r sum_{node in set} u_r[node, comp]  ('powerNorm', exponent 1)
                const auto& set = c.node_sets[c.obj_set];
                std::vector<double> dldu(n, 0.0);
                for (int nd : set) dldu[(size_t)nd * c.udpn + c.obj_comp - 1] += c.obj_coef;
                d_dldu.upload(dldu, c.stream);
                for (int r = 0; r < c.nrhs; ++r) {
                    device_dot(c, n, d_dldu.p, c.d_x.p + r * n, scal.p, part.p);
                    double v = 0.0;
                    ASEND_CUDA(cudaMemcpyAsync(&v, scal.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
                    ASEND_CUDA(cudaStreamSynchronize(c.stream));
                    L += v;
                    device_axpy(c, n, 1.0, c.d_x.p + r * n, d_usum.p);
                }
            }
            c.d_lam.alloc(n);
            rc = pcg_solve(c, *opts, &ast, false, d_dldu.p, c.d_lam.p, 1);
            ms_solve = (float)ast.ms_solve;
            cudaEvent_t e0, e1;
            ASEND_CUDA(cudaEventCreate(&e0));
            ASEND_CUDA(cudaEventCreate(&e1));
            ASEND_CUDA(cudaEventRecord(e0, c.stream));
            if (iso) adjoint_contract(c, c.d_lam.p, d_usum.p, c.d_gE.p, false);
            if (iso && c.obj_kind == ASEND_OBJ_ELEMENT) element_objective_explicit(c, d_usum.p, c.d_gE.p, nullptr);
            ASEND_CUDA(cudaEventRecord(e1, c.stream));
            ASEND_CUDA(cudaEventSynchronize(e1));
            float mc = 0.f;
            ASEND_CUDA(cudaEventElapsedTime(&mc, e0, e1));
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            ast.ms_adjoint = mc;
        }
        ASEND_CUDA(cudaEventRecord(c.ev1, c.stream));
        c.adj_kind = c.obj_kind;
        ++c.adj_serial;
        if (dLdE_out)
            ASEND_CUDA(cudaMemcpyAsync(dLdE_out, c.d_gE.p, sizeof(double) * c.n_el, cudaMemcpyDeviceToHost, c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        float ms = 0.f;
        ASEND_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
        if (L_out) *L_out = L;
        if (stats) {
            *stats = ast;
            stats->ms_solve = ms_solve;
            stats->ms_adjoint = (c.obj_kind == ASEND_OBJ_COMPLIANCE) ? ms : ast.ms_adjoint;
            stats->penalty_scale = c.sf;
        }
        return rc;
    });
}

int asend_newmark_run(asend_ctx* ctx, const asend_solve_opts* opts, int32_t n_steps, const double* amp,
                      int32_t probe_dof, double* probe_hist, double* u_final, asend_solve_stats* stats) {
    return guarded(ctx, [&](Ctx& c) {
        NvtxRange nvtx_range("asend_newmark_run");
        require(opts && amp && n_steps > 0, "bad Newmark arguments");
        require(c.assembled && c.dynamic && !c.modal, "assemble with dynamic=1 first");
        require(probe_dof < c.n_dof, "probe DOF out of range");
        return newmark_run(c, *opts, n_steps, amp, probe_dof, probe_hist, u_final, stats);
    });
}

int asend_newmark_keep_history(asend_ctx* ctx, int32_t fields) {
    return guarded(ctx, [&](Ctx& c) {
        require(fields == 0 || fields == 1 || fields == 3, "fields must be 0, 1 or 3");
        c.hist_fields = fields;
        if (!fields) {
            c.d_hist.release();
            c.hist_steps = 0;
        }
        return ASEND_OK;
    });
}

int asend_newmark_step_state(asend_ctx* ctx, int32_t step, double* u_out, double* v_out, double* a_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.hist_fields > 0 && c.hist_steps > 0, "no stored Newmark history (asend_newmark_keep_history)");
        require(step >= 1 && step <= c.hist_steps, "step out of range 1..n_steps");
        require(c.hist_fields == 3 || (!v_out && !a_out), "velocities and accelerations need fields = 3");
        const size_t n = c.n_dof;
        const double* h = c.d_hist.p + (size_t)(step - 1) * c.hist_fields * n;
        if (u_out) ASEND_CUDA(cudaMemcpy(u_out, h, sizeof(double) * n, cudaMemcpyDeviceToHost));
        if (v_out) ASEND_CUDA(cudaMemcpy(v_out, h + n, sizeof(double) * n, cudaMemcpyDeviceToHost));
        if (a_out) ASEND_CUDA(cudaMemcpy(a_out, h + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost));
        return ASEND_OK;
    });
}

int asend_newmark_adjoint(asend_ctx* ctx, const asend_solve_opts* opts, int32_t n_obj, const int32_t* obj_dof,
                          const double* obj_w, double* L_out, double* dLdE_out, asend_solve_stats* stats) {
    return guarded(ctx, [&](Ctx& c) {
        NvtxRange nvtx_range("asend_newmark_adjoint");
        require(opts && n_obj >= 1 && obj_dof && obj_w, "bad objective");
        require(c.assembled && c.dynamic && !c.modal, "assemble with dynamic=1 first");
        require(c.hist_fields > 0 && c.hist_steps > 0, "run asend_newmark_run with a kept history first");
        require(!c.A.d64.n && !c.lump && c.ortho.empty() && c.n_inst <= 1,
                "the transient adjoint takes undamped, consistent-mass, isotropic single models");
        for (int k = 0; k < n_obj; ++k) require(obj_dof[k] >= 0 && obj_dof[k] < c.n_dof, "objective DOF out of range");
        return newmark_adjoint(c, *opts, n_obj, obj_dof, obj_w, L_out, dLdE_out, stats);
    });
}

int asend_eigen_solve(asend_ctx* ctx, const asend_eigen_opts* opts, double* eig_out, double* freq_out,
                      double* modes_out, double* diag_mass_out, asend_eigen_stats* stats) {
    return guarded(ctx, [&](Ctx& c) {
        NvtxRange nvtx_range("asend_eigen_solve");
        require(opts != nullptr, "null options");
        require(c.n_el > 0, "set the mesh first");
        require(c.n_inst <= 1, "modal analysis takes one model, not a batch of instances");
        for (double r : c.rho) require(r > 0.0, "modal analysis needs positive densities");
        ASEND_CUDA(cudaSetDevice(c.device));
        if (!(c.assembled && c.modal)) {
            c.dynamic = true;
            c.modal = true;
            c.cM = 0.0;
            if (!c.pattern_ready) build_pattern(c);
            assemble_operator(c, 64);
            c.assembled = true;
            c.solved = false;
        }
        return eigen_solve(c, *opts, eig_out, freq_out, modes_out, diag_mass_out, stats);
    });
}

int asend_dense_sym_eigen(int32_t m, const double* a, double* vals, double* vecs) {
    if (m < 0 || (m > 0 && (!a || !vals))) return ASEND_EINVAL;
    return sym_eigen_dense(m, a, vals, vecs) == 0 ? ASEND_OK : ASEND_MAX_ITER;
}

int asend_add_modulus_design_var(asend_ctx* ctx, int32_t elem_set, int32_t n_coef, const double* coefs) {
    return guarded(ctx, [&](Ctx& c) {
        require(elem_set >= 0 && elem_set < (int)c.elem_sets.size(), "unknown element set");
        const auto& set = c.elem_sets[elem_set];
        require(n_coef <= 1 || (size_t)n_coef == set.size(),
                "coefficient list does not match the length of the element set");
        for (size_t k = 0; k < set.size(); ++k) {
            c.dv_el.push_back(set[k]);
            c.dv_coef.push_back(n_coef == 0 ? 1.0 : (n_coef == 1 ? coefs[0] : coefs[k]));
        }
        c.dv_ptr.push_back((int32_t)c.dv_el.size());
        return (int)c.dv_ptr.size() - 2;
    });
}

int asend_design_var_gradient(asend_ctx* ctx, const double* dLdE, double* dLdD_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(dLdE && dLdD_out, "null argument");
        const int ndv = (int)c.dv_ptr.size() - 1;
        for (int i = 0; i < ndv; ++i) {
            double s = 0.0;
            for (int k = c.dv_ptr[i]; k < c.dv_ptr[i + 1]; ++k) s += c.dv_coef[k] * dLdE[c.dv_el[k]];
            dLdD_out[i] = s;
        }
        return ndv;
    });
}

// dC/dD for a DV on one component of the reference's compliance S
// (element_properties.rs:648-764: S00 = 1/E1, S01 = -nu12/E1, S02 = -nu13/E1,
// S11 = 1/E2, S12 = -nu23/E2, S22 = 1/E3, S33..S55 = 1/G12, 1/G13, 1/G23;
// C = S^-1) at engineering constants p = E1 E2 E3 nu12 nu13 nu23 G12 G13 G23:
// dC = -C dS C.
static void material_dC_props(int category, int component, const double* p, double* dC) {
    const int k = component - 1;
    double C[36];
    orthotropic_cmat(p, C);
    double dS[36] = {0};
    if (category == ASEND_DV_MODULUS) {
        const double Ek = p[k];
        dS[7 * k] = -1.0 / (Ek * Ek);
        if (k == 0) {
            dS[1] = dS[6] = p[3] / (Ek * Ek);
            dS[2] = dS[12] = p[4] / (Ek * Ek);
        }
        if (k == 1) dS[8] = dS[13] = p[5] / (Ek * Ek);
    } else if (category == ASEND_DV_SHEAR_MODULUS) {
        const double Gk = p[6 + k];
        dS[7 * (3 + k)] = -1.0 / (Gk * Gk);
    } else {
        const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}};
        const int a = pr[k][0], b = pr[k][1];
        dS[6 * a + b] = dS[6 * b + a] = -1.0 / p[a];
    }
    double T[36];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double s = 0.0;
            for (int l = 0; l < 6; ++l) s += dS[6 * i + l] * C[6 * l + j];
            T[6 * i + j] = s;
        }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double s = 0.0;
            for (int l = 0; l < 6; ++l) s += C[6 * i + l] * T[6 * l + j];
            dC[6 * i + j] = -s;
        }
}

// The isotropic element (E, nu, G = E / (2 (1 + nu))) as constants.
static void iso_props(double E, double nu, double* p) {
    const double G = E / (2.0 * (1.0 + nu));
    const double q[9] = {E, E, E, nu, nu, nu, G, G, G};
    std::copy(q, q + 9, p);
}

static void material_dC(int category, int component, double E, double nu, double* dC) {
    double p[9];
    iso_props(E, nu, p);
    material_dC_props(category, component, p, dC);
}

int asend_material_dC(int32_t category, int32_t component, double E, double nu, double* dC_out) {
    if (category < ASEND_DV_MODULUS || category > ASEND_DV_POISSON_RATIO || component < 1 || component > 3 ||
        !dC_out || !(E > 0.0) || !(nu > -1.0 && nu < 0.5))
        return ASEND_EINVAL;
    material_dC(category, component, E, nu, dC_out);
    return ASEND_OK;
}

// Strain-pair tensors of the last adjoint gradient, P_e = sum_gp w detJ
// eps(lambda) eps(u)^T (compliance: sum over load cases of the u_r pairs).
static void ensure_pairs(Ctx& c) {
    require(c.adj_kind >= 0, "run asend_adjoint_gradient first");
    if (c.pairs_serial == c.adj_serial) return;
    const size_t n = c.n_dof;
    DArr<double> P;
    P.alloc((size_t)c.n_el * 36);
    if (c.adj_kind == ASEND_OBJ_COMPLIANCE) {
        for (int r = 0; r < c.nrhs; ++r) adjoint_pairs(c, c.d_x.p + r * n, c.d_x.p + r * n, P.p, r > 0);
    } else {
        adjoint_pairs(c, c.d_lam.p, c.d_adj_b.p, P.p, false);
        if (c.adj_kind == ASEND_OBJ_ELEMENT) element_objective_explicit(c, c.d_adj_b.p, nullptr, P.p);
    }
    c.h_pairs.resize((size_t)c.n_el * 36);
    ASEND_CUDA(cudaMemcpyAsync(c.h_pairs.data(), P.p, sizeof(double) * c.h_pairs.size(), cudaMemcpyDeviceToHost,
                               c.stream));
    ASEND_CUDA(cudaStreamSynchronize(c.stream));
    c.pairs_serial = c.adj_serial;
}

int asend_adjoint_strain_pairs(asend_ctx* ctx, double* pairs_out) {
    return guarded(ctx, [&](Ctx& c) {
        ensure_pairs(c);
        if (pairs_out) std::copy(c.h_pairs.begin(), c.h_pairs.end(), pairs_out);
        return ASEND_OK;
    });
}

// dL/dD for a material design variable over an element set
// (model_analysis.rs:1692-1700 with d_relasticd_d :1379-1457): the element
// stiffness C = S^-1 from the compliance S(E1..3, nu12, nu13, nu23,
// G12, G13, G23) of get_solid_stiff (element_properties.rs:648-764), per
// element orthotropic (asend_set_orthotropic) or isotropic (E_e, nu_e,
// G = E_e / (2 (1 + nu_e))); the DV adds
// coef * D to its component, so dC/dD = -coef C (dS/dE_k | dS/dG_k |
// dS/dnu_k) C and dL/dD = -sum_e sum_ij (dC/dD)_ij P_e[i][j].
int asend_material_dv_gradient(asend_ctx* ctx, int32_t category, int32_t component, int32_t elem_set,
                               int32_t n_coef, const double* coefs, double* grad_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(category >= ASEND_DV_MODULUS && category <= ASEND_DV_POLAR_MOMENT, "unknown DV category");
        require(category <= ASEND_DV_POISSON_RATIO || c.type == 2, "area / areaMoment / polarMoment DVs take beam2 meshes");
        if (category == ASEND_DV_AREA_MOMENT) require(component >= 1 && component <= 5, "areaMoment component must be 1-5");
        else if (category <= ASEND_DV_POISSON_RATIO) require(component >= 1 && component <= 3, "component must be 1, 2 or 3");
        require(elem_set >= 0 && elem_set < (int)c.elem_sets.size(), "unknown element set");
        require(grad_out, "null output");
        const auto& set = c.elem_sets[elem_set];
        require(n_coef <= 1 || (size_t)n_coef == set.size(), "coefficient list does not match the element set");
        require(n_coef == 0 || coefs, "null coefficients");
        ensure_pairs(c);
        double g = 0.0;
        for (size_t q = 0; q < set.size(); ++q) {
            const int e = set[q];
            double dC[36];
            if (c.type == 2 && !c.beam_cm.empty() && c.beam_cm[(size_t)e * 72] > 0.0)
                std::fill(dC, dC + 36, 0.0);  // a given section stiffness: no E or G in it
            else if (c.type == 2) beam_section_dC(category, component, &c.beam_sec[(size_t)e * 10], c.E[e], c.nu[e], dC);
            else if (!c.ortho.empty()) material_dC_props(category, component, &c.ortho[(size_t)e * 9], dC);
            else material_dC(category, component, c.E[e], c.nu[e], dC);
            const double* P = &c.h_pairs[(size_t)e * 36];
            double s = 0.0;
            for (int i = 0; i < 36; ++i) s += dC[i] * P[i];
            const double cf = n_coef == 0 ? 1.0 : (n_coef == 1 ? coefs[0] : coefs[q]);
            g -= cf * s;
        }
        *grad_out = g;
        return ASEND_OK;
    });
}

int asend_element_matrices(asend_ctx* ctx, int32_t first, int32_t count, double* ke, double* me) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.type == 41 || c.type == 81 || c.type == 2,
                "element matrix export is available for shell4, brickIM and beam2 meshes");
        require(first >= 0 && count > 0 && (int64_t)first + count <= c.n_el && ke, "bad element range");
        if (c.type == 41) shell_element_matrices(c, first, count, ke, me);
        else if (c.type == 2) beam_element_matrices(c, first, count, ke, me);
        else brickim_element_matrices(c, first, count, ke, me);
        return ASEND_OK;
    });
}

// ---- learned nodal preconditioner blocks ----------------------------------
int32_t asend_learned_n_params(void) { return learned_n_params(); }

int asend_learned_init(asend_ctx* ctx, uint64_t seed) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.n_nodes > 0, "set the mesh first");
        learned_init(c, seed);
        return ASEND_OK;
    });
}

int asend_learned_set_params(asend_ctx* ctx, const float* params) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.n_nodes > 0, "set the mesh first");
        require(params != nullptr, "null params");
        for (int i = 0; i < learned_n_params(); ++i) require(std::isfinite(params[i]), "non-finite parameter");
        learned_set_params(c, params);
        return ASEND_OK;
    });
}

int asend_learned_get_params(asend_ctx* ctx, float* params) {
    return guarded(ctx, [&](Ctx& c) {
        require(params != nullptr, "null params");
        require(learned_ready(c), "no learned weights");
        learned_get_params(c, params);
        return ASEND_OK;
    });
}

int asend_learned_add_samples(asend_ctx* ctx, int32_t n_samples, const int32_t* iters, int32_t append,
                              uint64_t seed) {
    return guarded(ctx, [&](Ctx& c) {
        require(n_samples > 0 && iters != nullptr, "need at least one sample");
        require(c.assembled, "assemble first");
        bool stationary = false;
        for (int s = 0; s < n_samples; ++s) stationary |= iters[s] < 0;
        require(!stationary || ((c.type == 8 || c.type == 81) && c.bx > 0), "multigrid samples need a structured hex8 block");
        learned_add_samples(c, n_samples, iters, append != 0, seed);
        return ASEND_OK;
    });
}

int asend_learned_set_objective(asend_ctx* ctx, int32_t kind) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.n_nodes > 0, "set the mesh first");
        learned_set_objective(c, kind);
        return ASEND_OK;
    });
}

int asend_learned_set_samples(asend_ctx* ctx, int32_t n_samples, const float* samples) {
    return guarded(ctx, [&](Ctx& c) {
        require(n_samples > 0 && samples != nullptr, "need at least one sample");
        require(c.n_nodes > 0, "set the mesh first");
        learned_set_samples(c, n_samples, samples);
        return ASEND_OK;
    });
}

int asend_learned_train(asend_ctx* ctx, int32_t n_steps, float lr, double* loss_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(learned_ready(c), "no learned weights");
        require(c.assembled, "assemble first");
        require(n_steps >= 0 && std::isfinite(lr) && lr >= 0.f, "bad training arguments");
        const double loss = learned_train(c, n_steps, lr);
        if (loss_out) *loss_out = loss;
        return std::isfinite(loss) ? ASEND_OK : ASEND_NONFINITE;
    });
}

int asend_learned_loss_grad(asend_ctx* ctx, double* loss_out, float* grad_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(learned_ready(c), "no learned weights");
        require(c.assembled, "assemble first");
        const double loss = learned_loss_grad(c, grad_out != nullptr);
        if (loss_out) *loss_out = loss;
        if (grad_out) learned_get_grad(c, grad_out);
        return ASEND_OK;
    });
}

int asend_learned_features(asend_ctx* ctx, float* feat, float* chol, float* outputs) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.assembled, "assemble first");
        require(!outputs || learned_ready(c), "no learned weights");
        learned_get_features(c, feat, chol, outputs);
        return ASEND_OK;
    });
}

int asend_learned_blocks(asend_ctx* ctx, int32_t use_net, float* blocks_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(c.assembled, "assemble first");
        require(blocks_out != nullptr, "null output");
        require(!use_net || learned_ready(c), "no learned weights");
        DArr<float> b;
        b.alloc((size_t)9 * c.n_nodes);
        learned_blocks(c, b.p, use_net != 0);
        ASEND_CUDA(cudaMemcpyAsync(blocks_out, b.p, sizeof(float) * 9 * c.n_nodes, cudaMemcpyDeviceToHost, c.stream));
        ASEND_CUDA(cudaStreamSynchronize(c.stream));
        return ASEND_OK;
    });
}

int asend_learned_forward(asend_ctx* ctx, int32_t n, const float* feat, float* outputs) {
    return guarded(ctx, [&](Ctx& c) {
        require(n > 0 && feat && outputs, "bad arguments");
        require(learned_ready(c), "no learned weights");
        learned_forward_host(c, n, feat, outputs);
        return ASEND_OK;
    });
}

int asend_learned_backward(asend_ctx* ctx, int32_t n, const float* feat, const float* dy, float* grad_out) {
    return guarded(ctx, [&](Ctx& c) {
        require(n > 0 && feat && dy && grad_out, "bad arguments");
        require(learned_ready(c), "no learned weights");
        learned_backward_host(c, n, feat, dy, grad_out);
        return ASEND_OK;
    });
}

}  // extern "C"
