"""FP64 oracle of the learned surrogate's network (test infrastructure only).

A NumPy restatement of the message-passing network declared in
include/sphdem_mpnn.h -- forward pass, mean-squared-error loss and the full
backward pass -- used by the tests to check the tensor-core kernels'
outputs and gradients.  There is no reference implementation of this network
(hojin9908/Warp_SPH_GPT has no learned component); the oracle is pinned by
central finite differences of its own forward pass (tests/test_mpnn_oracle.py).

``quantize=True`` rounds to BF16 at exactly the points where the GPU kernels
hold BF16 operands (node and edge inputs, weights, hidden activations and the
gradient operands of the tensor-core products); everything else is FP64.
"""
from __future__ import annotations

import numpy as np

H = 128
E1_W, E1_B, E2_W, E2_B = 0, 2048, 2176, 18560
N1_W, N1_B, N2_W, N2_B = 18688, 20736, 20864, 37248
N3_W, N3_B, NPARAM = 37376, 39424, 39440


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _ident(a):
    return np.asarray(a, dtype=np.float64)


def unpack(theta):
    t = np.asarray(theta, dtype=np.float64)
    return dict(E1=t[E1_W:E1_B].reshape(128, 16), b_E1=t[E1_B:E2_W], E2=t[E2_W:E2_B].reshape(128, 128),
                b_E2=t[E2_B:N1_W], N1=t[N1_W:N1_B].reshape(128, 16), b_N1=t[N1_B:N2_W],
                N2=t[N2_W:N2_B].reshape(128, 128), b_N2=t[N2_B:N3_W], N3=t[N3_W:N3_B].reshape(16, 128),
                b_N3=t[N3_B:NPARAM])


def init_theta(seed: int = 0) -> np.ndarray:
    """He-style initialisation; the unused output rows 6..15 are zero."""
    rng = np.random.default_rng(seed)
    th = np.zeros(NPARAM, dtype=np.float32)

    def w(off, rows, cols, fan_in):
        th[off:off + rows * cols] = rng.normal(0.0, np.sqrt(2.0 / fan_in), rows * cols)

    w(E1_W, 128, 16, 7)
    w(E2_W, 128, 128, 128)
    w(N1_W, 128, 16, 13)
    w(N2_W, 128, 128, 128)
    th[N3_W:N3_W + 6 * 128] = rng.normal(0.0, 0.1 * np.sqrt(1.0 / 128), 6 * 128)
    return th


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def edge_features(pos4, vel4, send, recv, inv_r, inv_vs):
    d = pos4[send, :3].astype(np.float64) - pos4[recv, :3]
    dist = np.sqrt((d * d).sum(1, keepdims=True))
    dv = vel4[send, :3].astype(np.float64) - vel4[recv, :3]
    e = np.zeros((len(send), 16))
    e[:, 0:3] = d * inv_r
    e[:, 3:4] = dist * inv_r
    e[:, 4:7] = dv * inv_vs
    return e


def forward(theta, x, pos4, vel4, send, recv, n_recv, inv_r, inv_vs, inv_norm, quantize=False):
    """Network output [n_recv,16] and the activations the backward pass needs."""
    q = bf16 if quantize else _ident
    # the layer-1 edge bias rides in the tensor-core product (as a BF16 weight)
    W = {k: (q(v) if k in ("E1", "E2", "N1", "N2", "N3", "b_E1") else v) for k, v in unpack(theta).items()}
    x = q(x)
    n = len(x)
    e = q(edge_features(pos4, vel4, send, recv, inv_r, inv_vs))
    p = e @ W["E1"].T + W["b_E1"]
    z = q(np.maximum(p, 0.0))
    f = z @ W["E2"].T + W["b_E2"]
    z0 = x @ W["N1"].T + W["b_N1"]
    h0 = q(silu(z0))
    agg1 = np.zeros((n_recv, H))
    np.add.at(agg1, recv, f * h0[send])
    h1 = h0.copy()
    h1[:n_recv] = q(h0[:n_recv] + inv_norm * agg1)
    z2 = h1 @ W["N2"].T + W["b_N2"]
    h2 = q(silu(z2))
    agg2 = np.zeros((n_recv, H))
    np.add.at(agg2, recv, f * h2[send])
    h3 = q(h2[:n_recv] + inv_norm * agg2)
    out = h3 @ W["N3"].T + W["b_N3"]
    cache = dict(W=W, x=x, e=e, p=p, z=z, f=f, z0=z0, h0=h0, h1=h1, z2=z2, h2=h2, h3=h3, send=send, recv=recv,
                 n_recv=n_recv, inv_norm=inv_norm, n=n, quantize=quantize)
    return out, cache


def loss(out, target):
    d = (out[:, :6] - target[:, :6])
    L = (d * d).mean()
    d_out = np.zeros_like(out)
    d_out[:, :6] = 2.0 * d / d.size
    return L, d_out


def backward(cache, d_out):
    """dL/dtheta [NPARAM] given dL/d out."""
    q = bf16 if cache["quantize"] else _ident
    W, s, r, nr, s_n = cache["W"], cache["send"], cache["recv"], cache["n_recv"], cache["inv_norm"]
    g = np.zeros(NPARAM)
    dq = q(d_out)
    g[N3_W:N3_B] = (dq.T @ cache["h3"]).ravel()
    g[N3_B:NPARAM] = d_out.sum(0)
    g2 = dq @ W["N3"]                       # dL/dh3 [nr,128]
    d_h2 = np.zeros((cache["n"], H))
    d_h2[:nr] = g2
    np.add.at(d_h2, s, s_n * cache["f"] * g2[r])
    d_z2 = d_h2 * silu_grad(cache["z2"])
    g[N2_B:N3_W] = d_z2.sum(0)
    d_z2q = q(d_z2)
    g[N2_W:N2_B] = (d_z2q.T @ cache["h1"]).ravel()
    d_h1 = d_z2q @ W["N2"]
    g1 = d_h1[:nr]
    d_h0 = d_h1.copy()
    np.add.at(d_h0, s, s_n * cache["f"] * g1[r])
    df = s_n * (g1[r] * cache["h0"][s] + g2[r] * cache["h2"][s])
    g[E2_B:N1_W] = df.sum(0)
    dfq = q(df)
    g[E2_W:E2_B] = (dfq.T @ cache["z"]).ravel()
    dz = dfq @ W["E2"]
    dp = dz * (cache["z"] > 0)
    g[E1_B:E2_W] = dp.sum(0)
    g[E1_W:E1_B] = (q(dp).T @ cache["e"]).ravel()
    d_z0 = d_h0 * silu_grad(cache["z0"])
    g[N1_B:N2_W] = d_z0.sum(0)
    g[N1_W:N1_B] = (q(d_z0).T @ cache["x"]).ravel()
    return g


def radius_graph(pos, n_recv, radius, inst=None):
    """Edges j -> i (i < n_recv, j != i, |x_j - x_i|^2 < radius^2), sorted by
    receiver; senders in ascending index order (the GPU lists them in cell
    order, so tests compare per-receiver sets)."""
    pos = np.asarray(pos, dtype=np.float32)
    r2 = np.float32(radius) * np.float32(radius)
    send, recv = [], []
    for i in range(n_recv):
        d = pos - pos[i]
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        m = d2 < r2
        m[i] = False
        if inst is not None:
            m &= inst == inst[i]
        js = np.nonzero(m)[0]
        send.append(js)
        recv.append(np.full(len(js), i))
    if not send:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    return np.concatenate(send), np.concatenate(recv)
