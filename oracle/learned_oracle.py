"""CPU restatement (numpy) of the learned nodal preconditioner blocks.

TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels in
asend3d_gb300/csrc/k_learned.cu.  Nothing on the product path imports it.

The reference has no learned part (its CG uses block LDL^T factors,
solverSrc/asend_run_job/src/lower_tri_mat_meth.rs:15-241); this file restates
the network the GPU library defines, so that its forward pass, backward pass,
features, block map and loss gradient can be checked:

  features f (16, 12 used) per node n with diagonal block D_n, t = tr(D_n)/3:
    D00/t D11/t D22/t D01/t D02/t D12/t, 0.1 (log t - mean_n log t),
    mean / std / range of (log E_e - mean_e log E_e) over adjacent elements,
    adjacent-element count / 8, [max diag > 1e3 min diag], 0 0 0 0
  y = W3 a2 + b3,  a2 = relu(W2 a1 + b2),  a1 = relu(W1 x + b1)
    (BF16 weights, features and activations; FP32 accumulation on the GPU)
  C_n = chol(D_n^-1),  U_n = [[e^y0,0,0],[y3,e^y1,0],[y4,y5,e^y2]]
  M_n = C_n U_n U_n^T C_n^T
  loss = mean_s || r_s - A M r_s ||^2
"""
from __future__ import annotations

import numpy as np

NF, NH, NO = 16, 64, 8
SHAPES = [("W1", (NH, NF)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NO, NH)), ("b3", (NO,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(x) -> np.ndarray:
    """Round float32 values to the nearest BF16 value (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out)


def unpack(params):
    out, o = {}, 0
    for name, shp in SHAPES:
        k = int(np.prod(shp))
        out[name] = np.asarray(params[o:o + k], dtype=np.float64).reshape(shp)
        o += k
    return out


def pack(parts) -> np.ndarray:
    return np.concatenate([np.asarray(parts[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def init_like_gpu_shapes(rng, last_scale=1e-3) -> np.ndarray:
    """Random parameters with the GPU initialiser's scales (not its stream)."""
    p = {"W1": rng.standard_normal((NH, NF)) * np.sqrt(2 / 12), "b1": np.zeros(NH),
         "W2": rng.standard_normal((NH, NH)) * np.sqrt(2 / NH), "b2": np.zeros(NH),
         "W3": rng.standard_normal((NO, NH)) * last_scale, "b3": np.zeros(NO)}
    return pack(p)


def forward(params, feat, emulate_bf16=True):
    """Network outputs [n, 8] and the cache for ``backward``."""
    P = unpack(params)
    rnd = bf16 if emulate_bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    W1, W2, W3 = (np.asarray(rnd(P[k]), dtype=np.float64) for k in ("W1", "W2", "W3"))
    x = np.asarray(rnd(feat), dtype=np.float64)
    h1 = x @ W1.T + P["b1"]
    a1 = np.asarray(rnd(np.maximum(h1, 0.0)), dtype=np.float64)
    h2 = a1 @ W2.T + P["b2"]
    a2 = np.asarray(rnd(np.maximum(h2, 0.0)), dtype=np.float64)
    y = a2 @ W3.T + P["b3"]
    return y, (x, a1, a2, W2, W3, h1, h2)


def backward(cache, dy) -> np.ndarray:
    """Parameter gradient of sum(y * dy) (activation rounding passed straight through)."""
    x, a1, a2, W2, W3, h1, h2 = cache
    dy = np.asarray(dy, dtype=np.float64)
    d2 = (dy @ W3) * (h2 > 0)
    d1 = (d2 @ W2) * (h1 > 0)
    return pack({"W1": d1.T @ x, "b1": d1.sum(0), "W2": d2.T @ a1, "b2": d2.sum(0),
                 "W3": dy.T @ a2, "b3": dy.sum(0)})


def diag_blocks(rp, col, val, n_nodes) -> np.ndarray:
    """3x3 diagonal blocks [n, 3, 3] of a node-interleaved CSR matrix."""
    D = np.zeros((n_nodes, 3, 3))
    for i in range(3 * n_nodes):
        n, a = divmod(i, 3)
        cs, vs = col[rp[i]:rp[i + 1]], val[rp[i]:rp[i + 1]]
        sel = (cs // 3) == n
        D[n, a, cs[sel] % 3] = vs[sel]
    return D


def features(D, conn, E, n_nodes) -> np.ndarray:
    t = np.trace(D, axis1=1, axis2=2) / 3.0
    f = np.zeros((n_nodes, NF))
    f[:, 0], f[:, 1], f[:, 2] = D[:, 0, 0] / t, D[:, 1, 1] / t, D[:, 2, 2] / t
    f[:, 3], f[:, 4], f[:, 5] = D[:, 0, 1] / t, D[:, 0, 2] / t, D[:, 1, 2] / t
    lt = np.log(t)
    f[:, 6] = 0.1 * (lt - lt.mean())
    le = np.log(E) - np.log(E).mean()
    adj = [[] for _ in range(n_nodes)]
    for e, row in enumerate(np.asarray(conn)):
        for nd in row:
            adj[nd].append(le[e])
    for n in range(n_nodes):
        v = np.array(adj[n])
        if len(v):
            f[n, 7] = v.mean()
            f[n, 8] = np.sqrt(max((v * v).mean() - v.mean() ** 2, 0.0))
            f[n, 9] = v.max() - v.min()
            f[n, 10] = len(v) / 8.0
    dg = np.stack([D[:, 0, 0], D[:, 1, 1], D[:, 2, 2]], 1)
    f[:, 11] = (dg.max(1) > 1e3 * dg.min(1)).astype(float)
    return f


def chol_of_inverse(D) -> np.ndarray:
    """[n, 6] = l00 l10 l11 l20 l21 l22 of chol(D_n^-1)."""
    L = np.linalg.cholesky(np.linalg.inv(D))
    return np.stack([L[:, 0, 0], L[:, 1, 0], L[:, 1, 1], L[:, 2, 0], L[:, 2, 1], L[:, 2, 2]], 1)


def _lower(c6):
    n = c6.shape[0]
    C = np.zeros((n, 3, 3))
    C[:, 0, 0], C[:, 1, 0], C[:, 1, 1] = c6[:, 0], c6[:, 1], c6[:, 2]
    C[:, 2, 0], C[:, 2, 1], C[:, 2, 2] = c6[:, 3], c6[:, 4], c6[:, 5]
    return C


def _u(y):
    n = y.shape[0]
    U = np.zeros((n, 3, 3))
    U[:, 0, 0], U[:, 1, 1], U[:, 2, 2] = np.exp(y[:, 0]), np.exp(y[:, 1]), np.exp(y[:, 2])
    U[:, 1, 0], U[:, 2, 0], U[:, 2, 1] = y[:, 3], y[:, 4], y[:, 5]
    return U


def blocks(y, c6) -> np.ndarray:
    L = _lower(c6) @ _u(y)
    return L @ np.transpose(L, (0, 2, 1))


def loss_and_dy(A, samples, y, c6):
    """Mean loss over samples and its gradient with respect to y [n, 8].
    A: scipy sparse (n_dof x n_dof); samples [S, n_dof]."""
    M = blocks(y, c6)
    n = M.shape[0]
    S = samples.shape[0]
    G = np.zeros((n, 3, 3))
    loss = 0.0
    for r in samples:
        r3 = r.reshape(n, 3)
        z = np.einsum("nij,nj->ni", M, r3).ravel()
        e = r - A @ z
        loss += float(e @ e)
        q = (A @ e).reshape(n, 3)
        G += -2.0 * np.einsum("ni,nj->nij", q, r3)
    G = 0.5 * (G + np.transpose(G, (0, 2, 1))) / S
    C, U = _lower(c6), _u(y)
    Ct = np.transpose(C, (0, 2, 1))
    D = 2.0 * Ct @ G @ C @ U
    dy = np.zeros((n, NO))
    dy[:, 0] = D[:, 0, 0] * U[:, 0, 0]
    dy[:, 1] = D[:, 1, 1] * U[:, 1, 1]
    dy[:, 2] = D[:, 2, 2] * U[:, 2, 2]
    dy[:, 3], dy[:, 4], dy[:, 5] = D[:, 1, 0], D[:, 2, 0], D[:, 2, 1]
    return loss / S, dy
