"""CPU checks of the learned-block oracle (numpy): its analytic backward and
loss gradient against central finite differences in float64, its BF16
rounding, and the zero-output identity M = D^-1 (block Jacobi)."""
import numpy as np
import scipy.sparse as sp

from oracle import learned_oracle as lo


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 1e-3, 0.0], dtype=np.float32)
    r = lo.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # tie -> even
    assert r[2] == np.float32(1.0 + 4 * 2.0 ** -8)  # tie -> even (upwards)
    assert r[3] == -2.5
    assert abs(r[4] - 1e-3) <= 1e-3 * 2.0 ** -8
    assert r[5] == 0.0
    # every result is representable in 16 bits
    assert np.all((r.view(np.uint32) & 0xFFFF) == 0)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(5)
    p = lo.init_like_gpu_shapes(rng, last_scale=0.3)
    p[lo.N_PARAMS - 8:] = rng.standard_normal(8) * 0.1
    feat = rng.standard_normal((7, lo.NF))
    dy = rng.standard_normal((7, lo.NO))
    y, cache = lo.forward(p, feat, emulate_bf16=False)
    g = lo.backward(cache, dy)
    idx = rng.choice(lo.N_PARAMS, 60, replace=False)
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fp = np.sum(lo.forward(pp, feat, emulate_bf16=False)[0] * dy)
        fm = np.sum(lo.forward(pm, feat, emulate_bf16=False)[0] * dy)
        fd = (fp - fm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def _spd_block_matrix(n_nodes, rng):
    B = rng.standard_normal((3 * n_nodes, 3 * n_nodes)) * 0.3
    A = B @ B.T + 3 * n_nodes * np.eye(3 * n_nodes)
    A[np.abs(A) < 0.5] = 0.0  # some sparsity
    A = 0.5 * (A + A.T) + 2 * np.eye(3 * n_nodes)
    return sp.csr_matrix(A)


def test_loss_gradient_matches_finite_differences():
    rng = np.random.default_rng(9)
    n = 5
    A = _spd_block_matrix(n, rng)
    D = lo.diag_blocks(A.indptr, A.indices, A.data, n)
    c6 = lo.chol_of_inverse(D)
    y = rng.standard_normal((n, lo.NO)) * 0.2
    samples = rng.standard_normal((3, 3 * n))
    loss, dy = lo.loss_and_dy(A, samples, y, c6)
    h = 1e-6
    for node in range(n):
        for k in range(6):
            yp, ym = y.copy(), y.copy()
            yp[node, k] += h
            ym[node, k] -= h
            fd = (lo.loss_and_dy(A, samples, yp, c6)[0] - lo.loss_and_dy(A, samples, ym, c6)[0]) / (2 * h)
            assert abs(fd - dy[node, k]) <= 1e-6 * max(1.0, abs(fd)), (node, k, fd, dy[node, k])
    assert np.all(dy[:, 6:] == 0.0)


def test_zero_output_is_block_jacobi():
    rng = np.random.default_rng(2)
    n = 4
    A = _spd_block_matrix(n, rng)
    D = lo.diag_blocks(A.indptr, A.indices, A.data, n)
    M = lo.blocks(np.zeros((n, lo.NO)), lo.chol_of_inverse(D))
    np.testing.assert_allclose(M, np.linalg.inv(D), rtol=1e-12, atol=1e-14)
    # any output gives SPD blocks
    M2 = lo.blocks(rng.standard_normal((n, lo.NO)), lo.chol_of_inverse(D))
    assert np.all(np.linalg.eigvalsh(M2) > 0)
