"""The FP64 oracle of the surrogate network, pinned without a GPU.

There is no reference implementation of the learned surrogate, so the
oracle's backward pass is pinned by central finite differences of its own
forward pass (FP64, relative error < 1e-6 on parameters drawn from every
block); the BF16-quantised variant (the points where the kernels hold BF16
operands) stays within BF16 rounding of the exact one.
"""
import numpy as np
import pytest

from oracle import mpnn_oracle as O


def _case(seed=0, n=60, n_recv=40, radius=0.12):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, 0.35, size=(n, 3)).astype(np.float32)
    pos4 = np.concatenate([pos, np.zeros((n, 1), np.float32)], 1)
    vel4 = np.concatenate([rng.normal(0, 0.5, size=(n, 3)), np.zeros((n, 1))], 1).astype(np.float32)
    x = np.zeros((n, 16))
    x[:, :10] = rng.normal(0, 1, size=(n, 10))
    send, recv = O.radius_graph(pos, n_recv, radius)
    theta = O.init_theta(seed).astype(np.float64)
    theta[O.N3_W:O.N3_W + 6 * 128] *= 30.0  # larger output layer: every block gets a sizeable gradient
    target = np.zeros((n_recv, 16))
    target[:, :6] = rng.normal(0, 1, size=(n_recv, 6))
    return dict(theta=theta, x=x, pos4=pos4, vel4=vel4, send=send, recv=recv, n_recv=n_recv, radius=radius,
                target=target)


def _loss(c, theta, quantize=False):
    out, cache = O.forward(theta, c["x"], c["pos4"], c["vel4"], c["send"], c["recv"], c["n_recv"],
                           1.0 / c["radius"], 1.0, 1.0 / 8.0, quantize=quantize)
    L, d_out = O.loss(out, c["target"])
    return L, d_out, cache


def test_radius_graph_is_symmetric_and_exact():
    c = _case()
    pos = c["pos4"][:, :3]
    pairs = set(zip(c["recv"].tolist(), c["send"].tolist()))
    assert len(pairs) == len(c["send"]) > 0
    for i, j in pairs:
        d = pos[j] - pos[i]
        assert (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2] < np.float32(c["radius"]) ** 2
        if j < c["n_recv"]:
            assert (j, i) in pairs
    assert all(i != j for i, j in pairs)


def test_backward_matches_central_differences():
    c = _case()
    L, d_out, cache = _loss(c, c["theta"])
    g = O.backward(cache, d_out)
    rng = np.random.default_rng(1)
    blocks = [(O.E1_W, O.E1_W + 7 * 16), (O.E1_B, O.E2_W), (O.E2_W, O.E2_B), (O.E2_B, O.N1_W),
              (O.N1_W, O.N1_B), (O.N1_B, O.N2_W), (O.N2_W, O.N2_B), (O.N2_B, O.N3_W),
              (O.N3_W, O.N3_W + 6 * 128), (O.N3_B, O.N3_B + 6)]
    idx = []
    for a, b in blocks:
        cand = np.arange(a, b)
        if a == O.E1_W:  # only the 7 used input columns of each row
            cand = np.array([r * 16 + k for r in range(128) for k in range(7)])
        if a == O.N1_W:
            cand = np.array([r * 16 + k for r in range(128) for k in range(10)]) + O.N1_W
        idx += list(rng.choice(cand, 6, replace=False))
    eps = 1e-6
    for i in idx:
        tp, tm = c["theta"].copy(), c["theta"].copy()
        tp[i] += eps
        tm[i] -= eps
        fd = (_loss(c, tp)[0] - _loss(c, tm)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-5 * np.abs(g).max(), (i, fd, g[i])


def test_quantized_oracle_is_within_bf16_of_exact():
    c = _case(seed=3)
    out_q, cache_q = O.forward(c["theta"], c["x"], c["pos4"], c["vel4"], c["send"], c["recv"], c["n_recv"],
                               1.0 / c["radius"], 1.0, 1.0 / 8.0, quantize=True)
    out, cache = O.forward(c["theta"], c["x"], c["pos4"], c["vel4"], c["send"], c["recv"], c["n_recv"],
                           1.0 / c["radius"], 1.0, 1.0 / 8.0)
    assert np.abs(out_q - out).max() <= 3e-2 * np.abs(out).max()
    _, d_out = O.loss(out, c["target"])
    g, gq = O.backward(cache, d_out), O.backward(cache_q, d_out)
    assert np.linalg.norm(gq - g) <= 5e-2 * np.linalg.norm(g)


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 0.0], dtype=np.float32)
    r = O.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 * 2.0 ** -7 and r[3] == -2.5 and r[4] == 0.0
