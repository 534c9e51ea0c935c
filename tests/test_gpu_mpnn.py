"""Tensor-core kernels of the learned surrogate against the FP64 oracle.

* The tcgen05 GEMM core (BF16 operands, FP32 accumulation in tensor memory)
  equals an FP32 product of the same BF16 values, for every operand shape the
  network uses, full and ragged tiles.
* The weight-gradient reduction over rows (transposed operand staging,
  accumulation across tiles in tensor memory, per-CTA partials) likewise.
* The radius graph lists exactly the oracle's edges (per receiver, as sets).
* Forward output and every parameter block of the gradient match the oracle:
  within 2e-2 (output, relative to its largest magnitude) and 3e-2 (gradient,
  relative L2 per block) of the BF16-quantised FP64 oracle, and within 6e-2
  of the exact FP64 oracle -- the BF16 operands are the only approximation.
* Adam steps of the library's kernels drive the loss of a fixed sample down.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import mpnn_oracle as O

pytestmark = pytest.mark.gpu


def _lib():
    from warp_sph_gpt_gb300 import _lib as L

    return L, L.load()


def _p(t):
    return C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("k,n", [(16, 16), (16, 128), (128, 16), (128, 128)])
@pytest.mark.parametrize("m", [1, 130, 1000])
def test_gemm_core_matches_fp32_product(k, n, m):
    L, lib = _lib()
    g = torch.Generator(device="cuda").manual_seed(k * 7 + n + m)
    a = torch.randn(m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16)
    c = torch.full((m, n), float("nan"), device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    L.check(lib.sphdem_mpnn_gemm(_p(a), _p(b), _p(c), m, n, k, _p(status), _stream()), "gemm")
    ref = a.float() @ b.float().T
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    err = (c - ref).abs().max().item()
    assert err <= 1e-5 * max(1.0, ref.abs().max().item()), err


@pytest.mark.parametrize("n", [16, 128])
@pytest.mark.parametrize("rows", [5, 1000, 40000])
def test_wgrad_matches_fp32_product(n, rows):
    L, lib = _lib()
    g = torch.Generator(device="cuda").manual_seed(rows + n)
    p = torch.randn(rows, 128, device="cuda", generator=g).to(torch.bfloat16)
    q = torch.randn(rows, n, device="cuda", generator=g).to(torch.bfloat16)
    c = torch.full((128, n), float("nan"), device="cuda")
    part = torch.zeros(int(lib.sphdem_mpnn_partial_floats()), device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    L.check(lib.sphdem_mpnn_wgrad(_p(p), _p(q), _p(c), rows, n, _p(part), _p(status), _stream()), "wgrad")
    ref = p.float().T @ q.float()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    err = (c - ref).abs().max().item()
    assert err <= 2e-5 * max(1.0, ref.abs().max().item()), err


def _synthetic(seed, n=900, n_recv=600, radius=0.1):
    from warp_sph_gpt_gb300.surrogate import Graph, SurrogateConfig

    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, 0.5, size=(n, 3)).astype(np.float32)
    vel = rng.normal(0, 0.5, size=(n, 3)).astype(np.float32)
    x = np.zeros((n, 16), np.float32)
    x[:, :10] = rng.normal(0, 1, size=(n, 10))
    x = O.bf16(x).astype(np.float32)
    cfg = SurrogateConfig(radius=radius, dt=1e-4, rho0=1000.0, norm=8.0)
    g = Graph(cfg, "cuda")
    g._ensure(n, n_recv)
    g.n_nodes, g.n_recv = n, n_recv
    b = g.buf
    b["node_pos3"][:n] = torch.tensor(pos, device="cuda")
    b["node_pos4"][:n, :3] = torch.tensor(pos, device="cuda")
    b["node_vel4"][:n, :3] = torch.tensor(vel, device="cuda")
    b["x"][:n] = torch.tensor(x, device="cuda").to(torch.bfloat16).view(torch.int16)
    g.build()
    pos4 = np.concatenate([pos, np.zeros((n, 1), np.float32)], 1)
    vel4 = np.concatenate([vel, np.zeros((n, 1), np.float32)], 1)
    return g, cfg, dict(pos=pos, pos4=pos4, vel4=vel4, x=x.astype(np.float64), n=n, n_recv=n_recv,
                        radius=radius)


def test_graph_lists_the_oracle_edges():
    g, cfg, d = _synthetic(0)
    off = g.buf["offset"][: d["n_recv"] + 1].cpu().numpy()
    snd = g.buf["sender"][: off[-1]].cpu().numpy()
    rcv = g.buf["receiver"][: off[-1]].cpu().numpy()
    s_ref, r_ref = O.radius_graph(d["pos"], d["n_recv"], d["radius"])
    assert off[-1] == len(s_ref) > 10 * d["n_recv"]
    for i in range(d["n_recv"]):
        assert (rcv[off[i]:off[i + 1]] == i).all()
        assert set(snd[off[i]:off[i + 1]].tolist()) == set(s_ref[r_ref == i].tolist())


def _oracle_edges(g, d):
    off = g.buf["offset"][: d["n_recv"] + 1].cpu().numpy()
    snd = g.buf["sender"][: off[-1]].cpu().numpy().astype(np.int64)
    rcv = g.buf["receiver"][: off[-1]].cpu().numpy().astype(np.int64)
    return snd, rcv


def _rel_err(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def test_forward_and_gradients_match_the_oracle():
    from warp_sph_gpt_gb300.surrogate import Network

    g, cfg, d = _synthetic(1)
    net = Network(cfg, "cuda", seed=5)
    th = net.theta.cpu().numpy().astype(np.float64)
    th[O.N3_W:O.N3_W + 6 * 128] *= 30.0
    net.theta.copy_(torch.tensor(th, dtype=torch.float32))
    net.pack()
    out = g.forward(net, store_pre=True).cpu().numpy().astype(np.float64)
    snd, rcv = _oracle_edges(g, d)
    args = (th, d["x"], d["pos4"], d["vel4"], snd, rcv, d["n_recv"], 1.0 / d["radius"], 1.0 / cfg.v_scale,
            1.0 / cfg.norm)
    ref_q, cache_q = O.forward(*args, quantize=True)
    ref, cache = O.forward(*args, quantize=False)
    assert _rel_err(out, ref_q) <= 2e-2
    assert _rel_err(out, ref) <= 6e-2
    target = np.zeros((d["n_recv"], 16))
    target[:, :6] = np.random.default_rng(2).normal(0, 1, size=(d["n_recv"], 6))
    tt = torch.tensor(target, dtype=torch.float32, device="cuda")
    loss = g.loss(tt).item()
    L_ref, d_out = O.loss(out, target)
    assert abs(loss - L_ref) <= 1e-5 * L_ref
    grad = g.backward(net).cpu().numpy().astype(np.float64)
    assert int(g.status()) == 0
    gq, g64 = O.backward(cache_q, d_out), O.backward(cache, d_out)
    blocks = dict(E1_W=(O.E1_W, O.E1_B), E1_B=(O.E1_B, O.E2_W), E2_W=(O.E2_W, O.E2_B), E2_B=(O.E2_B, O.N1_W),
                  N1_W=(O.N1_W, O.N1_B), N1_B=(O.N1_B, O.N2_W), N2_W=(O.N2_W, O.N2_B), N2_B=(O.N2_B, O.N3_W),
                  N3_W=(O.N3_W, O.N3_B), N3_B=(O.N3_B, O.NPARAM))
    for name, (a, b) in blocks.items():
        e_q = np.linalg.norm(grad[a:b] - gq[a:b]) / max(np.linalg.norm(gq[a:b]), 1e-30)
        e_64 = np.linalg.norm(grad[a:b] - g64[a:b]) / max(np.linalg.norm(g64[a:b]), 1e-30)
        assert e_q <= 3e-2, (name, e_q)
        assert e_64 <= 6e-2, (name, e_64)


def test_adam_steps_reduce_the_loss_of_a_fixed_sample():
    from warp_sph_gpt_gb300.surrogate import Network

    g, cfg, d = _synthetic(4)
    net = Network(cfg, "cuda", seed=0)
    rng = np.random.default_rng(0)
    target = torch.tensor(np.concatenate([rng.normal(0, 1, (d["n_recv"], 6)), np.zeros((d["n_recv"], 10))], 1),
                          dtype=torch.float32, device="cuda")
    losses = []
    for it in range(60):
        g.forward(net, store_pre=True)
        losses.append(g.loss(target).item())
        g.backward(net)
        net.adam(3e-3)
    assert losses[-1] < 0.5 * losses[0], losses[::10]
    assert int(g.status()) == 0


def test_inference_forward_matches_training_forward():
    """The inference pass forms the residuals while staging the next layer's
    operand tile; the training pass stores them.  Same network, same output
    (up to the order of the FP32 atomics at run boundaries)."""
    from warp_sph_gpt_gb300.surrogate import Network

    g, cfg, d = _synthetic(3)
    net = Network(cfg, "cuda", seed=7)
    th = net.theta.clone()
    th[O.N3_W:O.N3_W + 6 * 128] *= 30.0
    net.theta.copy_(th)
    net.pack()
    a = g.forward(net, store_pre=True).clone()
    b = g.forward(net, store_pre=False).clone()
    torch.cuda.synchronize()
    assert int(g.status()) == 0
    err = (a - b).abs().max().item() / max(a.abs().max().item(), 1e-30)
    assert err <= 1e-3, err


def test_edge_loss_matches_its_formula():
    """lambda / E * sum over edges (i <- j) of |dx_i - dx_j|^2, dx_j = 0 for
    senders that are not receivers; gradient added to d_out."""
    g, cfg, d = _synthetic(5)
    nr = d["n_recv"]
    rng = np.random.default_rng(1)
    out = rng.normal(0, 1, (nr, 16)).astype(np.float32)
    tgt = rng.normal(0, 1, (nr, 16)).astype(np.float32)
    g.buf["out"][:nr] = torch.tensor(out, device="cuda")
    t = torch.tensor(tgt, device="cuda")
    g.loss(t)
    base_loss = g.buf["loss"].item()
    base_grad = g.buf["d_out"][:nr].cpu().numpy().copy()
    lam = 0.7
    total = g.edge_loss(lam, t).item()
    grad = g.buf["d_out"][:nr].cpu().numpy()
    snd, rcv = _oracle_edges(g, d)
    dx = out[:, :3].astype(np.float64) - tgt[:, :3]
    dj = np.where((snd < nr)[:, None], dx[np.minimum(snd, nr - 1)], 0.0)
    diff = dx[rcv] - dj
    E = len(snd)
    ref = lam / E * (diff * diff).sum()
    assert abs((total - base_loss) - ref) <= 1e-4 * ref
    gref = np.zeros((nr, 16))
    np.add.at(gref[:, :3], rcv, 2 * lam / E * diff)
    m = snd < nr
    np.add.at(gref[:, :3], snd[m], -2 * lam / E * diff[m])
    np.testing.assert_allclose(grad - base_grad, gref, rtol=1e-4, atol=1e-7)


def test_inference_node_layers_run_on_receivers_and_senders():
    """The inference pass lists the non-receiver nodes that send an edge
    (each once) and runs the node layers on the receivers and those only; the
    output equals the pass over every node (up to the order of the FP32
    atomics at run boundaries)."""
    import ctypes as C

    from warp_sph_gpt_gb300.surrogate import Network

    g, cfg, d = _synthetic(5, n=1400, n_recv=500, radius=0.04)
    net = Network(cfg, "cuda", seed=3)
    th = net.theta.clone()
    th[O.N3_W:O.N3_W + 6 * 128] *= 30.0
    net.theta.copy_(th)
    net.pack()
    a = g.forward(net, store_pre=False).clone()
    torch.cuda.synchronize()
    nr = d["n_recv"]
    off = g.buf["offset"][: nr + 1].cpu().numpy()
    snd = g.buf["sender"][: off[-1]].cpu().numpy()
    static = np.unique(snd[snd >= nr])
    lst = g.buf["active_list"].cpu().numpy()
    assert 0 < lst[0] == len(static) < d["n"] - nr  # some non-receivers send, not all
    assert np.array_equal(np.sort(lst[1:1 + lst[0]]), static)
    full = g._net(net)
    full.active = None
    full.active_list = None
    g.lib.sphdem_mpnn_forward(C.byref(full), 0, g.stream())
    b = g.buf["out"][:nr].clone()
    torch.cuda.synchronize()
    err = (a - b).abs().max().item() / max(a.abs().max().item(), 1e-30)
    assert err <= 1e-3, err
