"""Learned K-step surrogate of the coupled WCSPH-DEM step.

A small message-passing network over the radius graph of all particles
(network, graph and kernels: include/sphdem_mpnn.h, csrc/mpnn.cu) predicts
where every fluid particle and DEM sphere will be ``m`` plain steps after the
current one.  One *jump* of K = m + 1 steps is

  1. one plain step (graph replay of the coupled step): fresh density,
     pressure and acceleration a_s;
  2. the network's correction on top of the constant-acceleration prior
       x += m dt v + dt^2 a_s m(m+1)/2,  v += m dt a_s
     (the prior is what m symplectic-Euler substeps give if a_s stays fixed);
  3. the judge: the plain density kernel evaluated at the new positions.  If
     any fluid density moved by more than ``tol * rho0`` over the jump (or,
     with judge = 1, if the density deviation max_i |rho_i - rho0| / rho0
     exceeds tol), the jump is undone and m plain steps run instead.

The plain step is therefore both the fallback and the judge of the density
error.  The network is trained on trajectories of the batched plain solver
(``batch.Ensemble``) by the library's own forward and backward kernels and an
Adam update (``train``).  DEM spin and contact history are advanced only by
the plain steps (a jump keeps omega and the tangential springs).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .grid import HashGrid

NPARAM = 39440
PACKED = 73728
HIDDEN = 128
E1_W, E1_B, E2_W, E2_B = 0, 2048, 2176, 18560
N1_W, N1_B, N2_W, N2_B = 18688, 20736, 20864, 37248
N3_W, N3_B = 37376, 39424


@dataclass
class SurrogateConfig:
    """Geometry of the graph and the scales of inputs and outputs."""
    radius: float                  # edge radius (the SPH support 2h)
    dt: float
    rho0: float
    substeps: int = 9              # m learned substeps after the plain step (K = m + 1)
    v_scale: float = 1.0           # velocity scale of node and edge inputs [m/s]
    a_scale: float = 10.0          # acceleration scale of node inputs [m/s^2]
    norm: float = 32.0             # aggregation normaliser (sum / norm)
    scale: tuple = (1e-4, 1e-1, 1e-4, 1e-1)  # output scales: x fluid, v fluid, x DEM, v DEM
    tol: float = 0.01              # judge tolerance (fraction of rho0)
    pos_tol: float = 0.0           # > 0: largest correction displacement a jump may apply [m]
    judge: int = 0                 # 0: max change of rho over the jump; 1: max |rho - rho0| / rho0
    edges_per_receiver: int = 160  # initial edge capacity per receiver


def init_theta(seed: int = 0) -> np.ndarray:
    """He-style initialisation; output rows 6..15 stay zero."""
    rng = np.random.default_rng(seed)
    th = np.zeros(NPARAM, dtype=np.float32)
    for off, rows, cols, fan in ((E1_W, 128, 16, 7), (E2_W, 128, 128, 128), (N1_W, 128, 16, 13),
                                 (N2_W, 128, 128, 128)):
        th[off:off + rows * cols] = rng.normal(0.0, math.sqrt(2.0 / fan), rows * cols)
    th[N3_W:N3_W + 6 * 128] = rng.normal(0.0, 0.1 / math.sqrt(128), 6 * 128)
    return th


class Network:
    """FP32 master parameters, their BF16 operand images and Adam moments."""

    def __init__(self, cfg: SurrogateConfig, device="cuda", seed: int = 0, theta=None):
        self.cfg = cfg
        self.device = torch.device(device)
        th = init_theta(seed) if theta is None else np.asarray(theta, dtype=np.float32)
        self.theta = torch.tensor(th, device=self.device)
        self.packed = torch.zeros(PACKED, dtype=torch.int16, device=self.device)
        self.m = torch.zeros_like(self.theta)
        self.v = torch.zeros_like(self.theta)
        self.grad = torch.zeros_like(self.theta)
        self.ema = None  # exponential moving average of theta (train(..., ema=decay))
        self.step = 0
        self.lib = _lib.load()
        self.pack()

    def stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def pack(self) -> None:
        _lib.check(self.lib.sphdem_mpnn_pack(_p(self.theta), _p(self.packed), self.stream()), "mpnn_pack")

    def adam(self, lr: float, beta1=0.9, beta2=0.999, eps=1e-8) -> None:
        self.step += 1
        _lib.check(self.lib.sphdem_mpnn_adam(_p(self.theta), _p(self.grad), _p(self.m), _p(self.v), NPARAM,
                                             lr, beta1, beta2, eps, self.step, self.stream()), "mpnn_adam")
        self.pack()

    def ema_update(self, decay: float) -> None:
        if self.ema is None:
            self.ema = self.theta.clone()
        else:
            self.ema.lerp_(self.theta, 1.0 - decay)

    def use_ema(self) -> None:
        """Take the averaged parameters as the network's (and repack)."""
        if self.ema is not None:
            self.theta.copy_(self.ema)
            self.pack()

    def state(self) -> dict:
        c = self.cfg
        return {"theta": self.theta.cpu().numpy(), "radius": c.radius, "dt": c.dt, "rho0": c.rho0,
                "substeps": c.substeps, "v_scale": c.v_scale, "a_scale": c.a_scale, "norm": c.norm,
                "scale": np.array(c.scale), "tol": c.tol, "judge": c.judge, "pos_tol": c.pos_tol}

    def save(self, path) -> None:
        np.savez(path, **self.state())

    @staticmethod
    def load(path, device="cuda") -> "Network":
        z = np.load(path)
        cfg = SurrogateConfig(radius=float(z["radius"]), dt=float(z["dt"]), rho0=float(z["rho0"]),
                              substeps=int(z["substeps"]), v_scale=float(z["v_scale"]),
                              a_scale=float(z["a_scale"]), norm=float(z["norm"]),
                              scale=tuple(float(v) for v in z["scale"]), tol=float(z["tol"]),
                              judge=int(z["judge"]) if "judge" in z else 0,
                              pos_tol=float(z["pos_tol"]) if "pos_tol" in z else 0.0)
        return Network(cfg, device, theta=z["theta"])


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p()


@dataclass
class Sets:
    """Contiguous ranges of the four particle sets forming one graph."""
    P: object
    B: object
    D: object
    W: object
    f: tuple = None   # (start, stop) fluid rows, None = all
    d: tuple = None
    b: tuple = None
    w: tuple = None

    def rng(self, which):
        part = {"f": self.P, "d": self.D, "b": self.B, "w": self.W}[which]
        r = getattr(self, which)
        return (0, part.n) if r is None else r

    def view(self, which, name, src=None):
        part = {"f": self.P, "d": self.D, "b": self.B, "w": self.W}[which]
        a, b = self.rng(which)
        t = getattr(part, name) if src is None else src
        return t[a:b]


class Graph:
    """Device workspace of one radius graph and the network's activations."""

    def __init__(self, cfg: SurrogateConfig, device="cuda"):
        self.cfg = cfg
        self.device = torch.device(device)
        self.lib = _lib.load()
        self.grid = HashGrid()
        self.grid.radius = float(np.float32(cfg.radius))
        self.ctl = torch.zeros(16, dtype=torch.int32, device=self.device)
        self.n_nodes = self.n_recv = 0
        self.capacity = 0
        self.buf = {}
        self.gbuf = {}
        self.scan = None

    def stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    # -- buffers -------------------------------------------------------------------
    def _ensure(self, n_nodes: int, n_recv: int) -> None:
        dev = self.device
        if n_nodes > self.buf.get("_nodes", 0):
            n = int(n_nodes * 1.1) + 16
            f32 = dict(dtype=torch.float32, device=dev)
            i16 = dict(dtype=torch.int16, device=dev)
            self.buf.update(_nodes=n, node_pos3=torch.zeros(n, 3, **f32), node_pos4=torch.zeros(n, 4, **f32),
                            node_vel4=torch.zeros(n, 4, **f32), x=torch.zeros(n, 16, **i16),
                            z0=torch.zeros(n, HIDDEN, **f32), h0=torch.zeros(n, HIDDEN, **i16),
                            h1=torch.zeros(n, HIDDEN, **i16), z2=torch.zeros(n, HIDDEN, **f32),
                            h2=torch.zeros(n, HIDDEN, **i16), active=torch.zeros(n, dtype=torch.int32, device=dev),
                            active_list=torch.zeros(n + 1, dtype=torch.int32, device=dev))
            self.gbuf = {}
        if n_recv > self.buf.get("_recv", 0) or "offset" not in self.buf:
            n = int(max(n_recv, 1) * 1.1) + 16
            f32 = dict(dtype=torch.float32, device=dev)
            self.buf.update(_recv=n, offset=torch.zeros(n + 1, dtype=torch.int32, device=dev),
                            agg=torch.zeros(n, HIDDEN, **f32), h3=torch.zeros(n, HIDDEN, dtype=torch.int16, device=dev),
                            out=torch.zeros(n, 16, **f32), target=torch.zeros(n, 16, **f32),
                            d_out=torch.zeros(n, 16, **f32), loss=torch.zeros(1, **f32),
                            x_t=torch.zeros(n, 3, **f32), v_t=torch.zeros(n, 3, **f32))
            self.scan = torch.zeros(int(self.lib.sphdem_scan_scratch(n)), dtype=torch.int32, device=dev)
            self.gbuf = {}
        need = max(n_recv, 1) * self.cfg.edges_per_receiver
        if need > self.capacity:
            self._alloc_edges(need)

    def _alloc_edges(self, cap: int) -> None:
        self.capacity = int(cap)
        i32 = dict(dtype=torch.int32, device=self.device)
        self.buf["sender"] = torch.zeros(self.capacity, **i32)
        self.buf["receiver"] = torch.zeros(self.capacity, **i32)

    # -- nodes and edges -------------------------------------------------------------
    def set_nodes(self, sets: Sets, acc=None) -> None:
        """Node inputs of the particle ranges in ``sets`` (fluid, DEM, wall, DEM wall)."""
        cfg = self.cfg
        nf = sets.rng("f")[1] - sets.rng("f")[0]
        nd = sets.rng("d")[1] - sets.rng("d")[0]
        nb = sets.rng("b")[1] - sets.rng("b")[0]
        nw = sets.rng("w")[1] - sets.rng("w")[0]
        self._ensure(nf + nd + nb + nw, nf + nd)
        self.n_nodes, self.n_recv = nf + nd + nb + nw, nf + nd
        self.n_fluid, self.n_dem = nf, nd
        a = _lib.MpnnNodesT()
        P, D = sets.P, sets.D
        a.f_pos = _lib.fptr(sets.view("f", "pos"))
        a.f_vel = _lib.fptr(sets.view("f", "vel"))
        a.f_acc = _lib.fptr(sets.view("f", "acc", acc[0] if acc else None))
        a.f_rho = _lib.fptr(sets.view("f", "rho"))
        a.f_por = _lib.fptr(sets.view("f", "porosity"))
        a.n_fluid = nf
        a.d_pos = _lib.fptr(sets.view("d", "pos")) if nd else _lib.c_float_p()
        a.d_vel = _lib.fptr(sets.view("d", "vel")) if nd else _lib.c_float_p()
        a.d_acc = _lib.fptr(sets.view("d", "acc", acc[1] if acc else None)) if nd else _lib.c_float_p()
        a.d_rad = _lib.fptr(sets.view("d", "radius")) if nd else _lib.c_float_p()
        a.n_dem = nd
        a.b_pos = _lib.fptr(sets.view("b", "pos"))
        a.b_rho = _lib.fptr(sets.view("b", "rho"))
        a.n_wall = nb
        a.w_pos = _lib.fptr(sets.view("w", "pos")) if nw else _lib.c_float_p()
        a.w_rad = _lib.fptr(sets.view("w", "radius")) if nw else _lib.c_float_p()
        a.n_dem_wall = nw
        a.rho0, a.inv_vscale, a.inv_ascale = cfg.rho0, 1.0 / cfg.v_scale, 1.0 / cfg.a_scale
        a.inv_radius = 1.0 / cfg.radius
        b = self.buf
        a.node_pos3, a.node_pos4, a.node_vel4 = _lib.fptr(b["node_pos3"]), _lib.fptr(b["node_pos4"]), _lib.fptr(
            b["node_vel4"])
        a.x = C.cast(b["x"].data_ptr(), _lib.c_u16_p)
        self.nodes = a
        _lib.check(self.lib.sphdem_mpnn_nodes(C.byref(a), self.stream()), "mpnn_nodes")

    def build(self, check: bool = True) -> None:
        """Radius graph of the current nodes; with check, grow and rebuild on overflow."""
        g = self.grid
        if g.geometry is None:
            pts = self.buf["node_pos3"][: self.n_nodes]
            lo = pts.min(0).values.cpu().numpy() - 4 * self.cfg.radius
            hi = pts.max(0).values.cpu().numpy() + 4 * self.cfg.radius
            hi[2] += 0.5 * (hi[2] - lo[2])
            g.ensure_geometry(lo.tolist(), hi.tolist(), self.n_nodes, self.device)
        while True:
            gt = _lib.GridT()
            g.fill(gt, self.n_nodes)
            b = self.buf
            _lib.check(self.lib.sphdem_mpnn_graph(
                C.byref(gt), _p(b["node_pos3"]), _p(b["node_pos4"]), self.n_recv, float(self.cfg.radius),
                _p(b["offset"]), _p(b["sender"]), _p(b["receiver"]), self.capacity, _p(self.scan),
                _p(self.ctl), self.stream()), "mpnn_graph")
            if not check:
                return
            flags = int(self.ctl[3].item())
            if flags & 0x8:  # edge capacity
                e = int(b["offset"][self.n_recv].item())
                self.ctl[3] = 0
                self._alloc_edges(int(e * 1.25) + 1024)
                continue
            if flags:
                self.ctl[3] = 0
                raise RuntimeError(f"mpnn graph build raised device status 0x{flags:x}")
            return

    def n_edges(self) -> int:
        return int(self.buf["offset"][self.n_recv].item())

    # -- network -----------------------------------------------------------------
    def _net(self, net: Network) -> "_lib.MpnnNetT":
        b = self.buf
        n = _lib.MpnnNetT()
        n.n_nodes, n.n_recv, n.edge_capacity = self.n_nodes, self.n_recv, self.capacity
        n.inv_radius, n.inv_vscale, n.inv_norm = 1.0 / self.cfg.radius, 1.0 / self.cfg.v_scale, 1.0 / self.cfg.norm
        u16 = lambda t: C.cast(t.data_ptr(), _lib.c_u16_p)
        n.node_pos4, n.node_vel4, n.x = _lib.fptr(b["node_pos4"]), _lib.fptr(b["node_vel4"]), u16(b["x"])
        n.offset, n.sender, n.receiver = _lib.iptr(b["offset"]), _lib.iptr(b["sender"]), _lib.iptr(b["receiver"])
        n.theta, n.packed = _lib.fptr(net.theta), u16(net.packed)
        n.z0, n.h0, n.agg, n.h1 = _lib.fptr(b["z0"]), u16(b["h0"]), _lib.fptr(b["agg"]), u16(b["h1"])
        n.z2, n.h2, n.h3, n.out = _lib.fptr(b["z2"]), u16(b["h2"]), u16(b["h3"]), _lib.fptr(b["out"])
        n.status = C.cast(self.ctl.data_ptr() + 12, _lib.c_int_p)
        n.active, n.active_list = _lib.iptr(b["active"]), _lib.iptr(b["active_list"])
        return n

    def forward(self, net: Network, store_pre: bool = False) -> torch.Tensor:
        self._netst = self._net(net)
        _lib.check(self.lib.sphdem_mpnn_forward(C.byref(self._netst), int(store_pre), self.stream()),
                   "mpnn_forward")
        return self.buf["out"][: self.n_recv]

    def backward(self, net: Network, d_out: torch.Tensor = None) -> torch.Tensor:
        """net.grad = dL/dtheta after forward(store_pre=True); d_out defaults to the loss's."""
        if not self.gbuf:
            n = self.buf["_nodes"]
            r = self.buf["_recv"]
            f32 = dict(dtype=torch.float32, device=self.device)
            self.gbuf = dict(g2=torch.zeros(r, HIDDEN, **f32), d_h2=torch.zeros(n, HIDDEN, **f32),
                             d_h1=torch.zeros(n, HIDDEN, **f32), d_h0=torch.zeros(n, HIDDEN, **f32),
                             bf_a=torch.zeros(n, HIDDEN, dtype=torch.int16, device=self.device),
                             bf_b=torch.zeros(r, 16, dtype=torch.int16, device=self.device),
                             partial=torch.zeros(int(self.lib.sphdem_mpnn_partial_floats()), **f32))
        gb = self.gbuf
        u16 = lambda t: C.cast(t.data_ptr(), _lib.c_u16_p)
        g = _lib.MpnnGradT()
        g.d_out = _lib.fptr(d_out if d_out is not None else self.buf["d_out"])
        g.g2, g.d_h2, g.d_h1, g.d_h0 = (_lib.fptr(gb[k]) for k in ("g2", "d_h2", "d_h1", "d_h0"))
        g.bf_a, g.bf_b = u16(gb["bf_a"]), u16(gb["bf_b"])
        g.partial, g.grad = _lib.fptr(gb["partial"]), _lib.fptr(net.grad)
        netst = self._net(net)
        _lib.check(self.lib.sphdem_mpnn_backward(C.byref(netst), C.byref(g), self.stream()), "mpnn_backward")
        return net.grad

    def loss(self, target: torch.Tensor = None) -> torch.Tensor:
        """MSE of the last forward against target (default: the target buffer); sets d_out."""
        b = self.buf
        t = target if target is not None else b["target"]
        _lib.check(self.lib.sphdem_mpnn_loss(_p(b["out"]), _p(t), self.n_recv, _p(b["loss"]), _p(b["d_out"]),
                                             self.stream()), "mpnn_loss")
        return b["loss"]

    def edge_loss(self, lam: float, target: torch.Tensor = None) -> torch.Tensor:
        """Adds the edge term (relative displacement errors of neighbours) to the
        loss and d_out of the last loss() call."""
        b = self.buf
        t = target if target is not None else b["target"]
        _lib.check(self.lib.sphdem_mpnn_edge_loss(_p(b["offset"]), _p(b["sender"]), _p(b["receiver"]), self.n_recv,
                                                  self.capacity, _p(b["out"]), _p(t), float(lam), _p(b["loss"]),
                                                  _p(b["d_out"]), self.stream()), "mpnn_edge_loss")
        return b["loss"]

    def status(self) -> int:
        return int(self.ctl[3].item())


def _apply(lib, graph: Graph, sets: Sets, net_out, cfg: SurrogateConfig, target_state=None, acc=None):
    """Prior + correction into the particle arrays, or (target_state given) the
    normalised residual target rows of the graph's receivers."""
    nf, nd = graph.n_fluid, graph.n_dem
    f_pos, f_vel = sets.view("f", "pos"), sets.view("f", "vel")
    f_acc = sets.view("f", "acc", acc[0] if acc else None)
    d_pos = sets.view("d", "pos") if nd else None
    d_vel = sets.view("d", "vel") if nd else None
    d_acc = sets.view("d", "acc", acc[1] if acc else None) if nd else None
    # host array read by the call itself (not by the kernel): a named local, so
    # it outlives the call whatever ctypes does with temporaries
    scale_host = (C.c_float * 4)(*(float(v) for v in cfg.scale))
    scale = C.c_void_p(C.addressof(scale_host))
    if target_state is None:
        rc = lib.sphdem_mpnn_apply(_p(f_pos), _p(f_vel), _p(f_acc), nf, _p(d_pos), _p(d_vel), _p(d_acc), nd,
                                   _p(net_out), cfg.substeps, cfg.dt, scale, None, None, None, graph.stream())
    else:
        x_t, v_t = target_state
        rc = lib.sphdem_mpnn_apply(_p(f_pos), _p(f_vel), _p(f_acc), nf, _p(d_pos), _p(d_vel), _p(d_acc), nd, None,
                                   cfg.substeps, cfg.dt, scale, _p(x_t), _p(v_t), _p(graph.buf["target"]),
                                   graph.stream())
    _lib.check(rc, "mpnn_apply")


# ---------------------------------------------------------------------------
# training data from the batched plain solver
# ---------------------------------------------------------------------------
@dataclass
class Snapshot:
    f_pos: torch.Tensor
    f_vel: torch.Tensor
    f_acc: torch.Tensor
    f_rho: torch.Tensor
    f_por: torch.Tensor
    b_rho: torch.Tensor
    d_pos: torch.Tensor
    d_vel: torch.Tensor
    d_acc: torch.Tensor
    x_t: torch.Tensor      # [n_fluid + n_dem, 3] per member block: fluid rows then DEM rows
    v_t: torch.Tensor
    step: int


@dataclass
class TrainingSet:
    ensemble: object
    snapshots: list = field(default_factory=list)


def generate(ensemble, n_steps: int, cfg: SurrogateConfig, log=None) -> TrainingSet:
    """Advance the ensemble n_steps plain steps; every K = m + 1 steps record the
    state after a plain step and, m plain steps later, the positions and
    velocities the surrogate must predict."""
    ts = TrainingSet(ensemble)
    E = ensemble
    m = cfg.substeps
    K = m + 1
    step = 0
    t0 = time.perf_counter()
    while step + K <= n_steps:
        E.run(step, 1)
        P, B, D = E.P, E.B, E.D
        snap = dict(f_pos=P.pos.clone(), f_vel=P.vel.clone(), f_acc=P.acc.clone(), f_rho=P.rho.clone(),
                    f_por=P.porosity.clone(), b_rho=B.rho.clone(), d_pos=D.pos.clone(), d_vel=D.vel.clone(),
                    d_acc=D.acc.clone())
        E.run(step + 1, m)
        xs, vs = [], []
        for k in range(E.ninst):
            xs += [E.member(k, "sph", "pos"), E.member(k, "dem", "pos")]
            vs += [E.member(k, "sph", "vel"), E.member(k, "dem", "vel")]
        ts.snapshots.append(Snapshot(**snap, x_t=torch.cat(xs).clone(), v_t=torch.cat(vs).clone(), step=step))
        step += K
    torch.cuda.synchronize()
    if log:
        log(f"generated {len(ts.snapshots)} snapshots x {E.ninst} members in {time.perf_counter() - t0:.1f} s")
    return ts


class _Proxy:
    """A particle struct whose named fields are replaced by snapshot tensors."""

    def __init__(self, base, **fields):
        self._base = base
        self.__dict__.update(fields)
        self.n = base.n

    def __getattr__(self, name):
        return getattr(self._base, name)


def sample_sets(ts: TrainingSet, snap: Snapshot, k: int):
    """Sets of member k at snapshot `snap` and its target rows."""
    E = ts.ensemble
    o = E.offsets
    P = _Proxy(E.P, pos=snap.f_pos, vel=snap.f_vel, acc=snap.f_acc, rho=snap.f_rho, porosity=snap.f_por)
    B = _Proxy(E.B, rho=snap.b_rho)
    D = _Proxy(E.D, pos=snap.d_pos, vel=snap.d_vel, acc=snap.d_acc)
    sets = Sets(P, B, D, E.W, f=(int(o["sph"][k]), int(o["sph"][k + 1])), d=(int(o["dem"][k]), int(o["dem"][k + 1])),
                b=(int(o["bnd"][k]), int(o["bnd"][k + 1])), w=(int(o["dembnd"][k]), int(o["dembnd"][k + 1])))
    r0 = int(o["sph"][k] + o["dem"][k])
    r1 = int(o["sph"][k + 1] + o["dem"][k + 1])
    return sets, snap.x_t[r0:r1], snap.v_t[r0:r1]


def collect_on_policy(net: Network, cases, n_steps: int, log=None) -> list:
    """Samples from the states a judged learned rollout visits (dataset
    aggregation): along each case's rollout, the state after every plain step
    is paired with the plain method's own continuation m steps later; the
    rollout then moves on with the learned jump if the density judge accepts
    it, else with that plain continuation.  Returns [(sets, x_t, v_t), ...]."""
    from .kernels import Kernel_density_sph

    cfg, lib = net.cfg, net.lib
    m, K = cfg.substeps, cfg.substeps + 1
    g = Graph(cfg, net.device)
    out_samples = []
    accepted = total = 0
    t0 = time.perf_counter()
    for case in cases:
        P, B, D, W = case.P, case.B, case.D, case.W
        step = 0
        while step + K <= n_steps:
            case.run(step, 1)
            st = case.snapshot()
            case.run(step + 1, m)
            x_t = torch.cat([P.pos, D.pos]).clone()
            v_t = torch.cat([P.vel, D.vel]).clone()
            plain_next = case.snapshot()
            sets = Sets(_Proxy(P, pos=st[("P", "pos")], vel=st[("P", "vel")], acc=st[("P", "acc")],
                               rho=st[("P", "rho")], porosity=st[("P", "porosity")]),
                        _Proxy(B, rho=st[("B", "rho")]),
                        _Proxy(D, pos=st[("D", "pos")], vel=st[("D", "vel")], acc=st[("D", "acc")]), W)
            out_samples.append((sets, x_t, v_t))
            # the learned jump from the same state, judged like a rollout
            case.restore(st)
            live = Sets(P, B, D, W)
            g.set_nodes(live)
            g.build()
            _apply(lib, g, live, g.forward(net), cfg)
            Kernel_density_sph(P, B, case.grids[0], case.grids[1], case.solv.support, case.solv.h)
            dev = ((P.rho - st[("P", "rho")]).abs().max() / cfg.rho0).item()
            total += 1
            if dev <= cfg.tol:
                accepted += 1
            else:
                case.restore(plain_next)
            step += K
    if log:
        log(f"on-policy: {len(out_samples)} samples from {len(cases)} cases, {accepted}/{total} jumps accepted, "
            f"{time.perf_counter() - t0:.1f} s")
    return out_samples


def prepare_target(lib, g: Graph, sets: Sets, x_t, v_t, cfg: SurrogateConfig) -> None:
    _apply(lib, g, sets, None, cfg, target_state=(x_t, v_t))


def fit_scales(ts: TrainingSet, cfg: SurrogateConfig, members, device) -> None:
    """Output scales = RMS of the prior's residual per type (fluid, DEM)."""
    lib = _lib.load()
    unit = SurrogateConfig(**{**cfg.__dict__, "scale": (1.0, 1.0, 1.0, 1.0)})
    g = Graph(unit, device)
    acc = {"fx": [], "fv": [], "dx": [], "dv": []}
    for snap in ts.snapshots[:: max(1, len(ts.snapshots) // 10)]:
        for k in members:
            sets, x_t, v_t = sample_sets(ts, snap, k)
            nf = sets.rng("f")[1] - sets.rng("f")[0]
            nd = sets.rng("d")[1] - sets.rng("d")[0]
            g._ensure(nf + nd + 1, nf + nd)
            g.n_fluid, g.n_dem, g.n_recv = nf, nd, nf + nd
            prepare_target(lib, g, sets, x_t, v_t, unit)
            t = g.buf["target"][: nf + nd]
            acc["fx"].append(t[:nf, :3].pow(2).mean().item())
            acc["fv"].append(t[:nf, 3:6].pow(2).mean().item())
            if nd:
                acc["dx"].append(t[nf:, :3].pow(2).mean().item())
                acc["dv"].append(t[nf:, 3:6].pow(2).mean().item())
    rms = {k: math.sqrt(sum(v) / len(v)) if v else 0.0 for k, v in acc.items()}
    fx = max(rms["fx"], 1e-9)
    fv = max(rms["fv"], 1e-9)
    cfg.scale = (fx, fv, max(rms["dx"], 1e-9) if rms["dx"] else fx, max(rms["dv"], 1e-9) if rms["dv"] else fv)


def evaluate(net: Network, ts: TrainingSet, members, graph: Graph = None, zero: bool = False) -> float:
    """Mean loss over all snapshots of the given members (zero=True: the prior alone)."""
    lib = net.lib
    g = graph or Graph(net.cfg, net.device)
    tot, cnt = 0.0, 0
    for snap in ts.snapshots:
        for k in members:
            sets, x_t, v_t = sample_sets(ts, snap, k)
            g.set_nodes(sets)
            prepare_target(lib, g, sets, x_t, v_t, net.cfg)
            if zero:
                g.buf["out"].zero_()
            else:
                g.build()
                g.forward(net)
            tot += g.loss().item()
            cnt += 1
    return tot / max(cnt, 1)


def _noisy(sets: Sets, sigma_x: float, sigma_v: float, gen) -> Sets:
    """The sample with Gaussian noise on fluid and DEM positions and
    velocities (the target stays the true future state, so the network learns
    to correct perturbed inputs -- as a rollout feeds it its own errors)."""
    def jitter(t, s):
        return t + s * torch.randn(t.shape, device=t.device, generator=gen) if s > 0 else t
    a, b = sets.rng("f")
    P = _Proxy(sets.P, pos=_pad_slice(jitter(sets.view("f", "pos"), sigma_x), a, sets.P.n),
               vel=_pad_slice(jitter(sets.view("f", "vel"), sigma_v), a, sets.P.n))
    c, d = sets.rng("d")
    D = sets.D
    if d > c:
        D = _Proxy(sets.D, pos=_pad_slice(jitter(sets.view("d", "pos"), sigma_x), c, sets.D.n),
                   vel=_pad_slice(jitter(sets.view("d", "vel"), sigma_v), c, sets.D.n))
    return Sets(P, sets.B, D, sets.W, f=sets.f, d=sets.d, b=sets.b, w=sets.w)


def _pad_slice(t, start, n):
    """A [n, ...] view-compatible tensor whose rows [start, start + len(t)) are t
    (the other rows are never read)."""
    out = torch.empty((n,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
    out[start:start + t.shape[0]] = t
    return out


def train(net: Network, ts: TrainingSet, members, iters: int, lr: float = 1e-3, seed: int = 0, log=None,
          log_every: int = 200, edge_weight: float = 0.0, noise: tuple = (0.0, 0.0), extra=None,
          extra_fraction: float = 0.5, ema: float = 0.0) -> list:
    """Adam on single-member samples drawn uniformly from the training set.
    edge_weight > 0 adds the edge term (relative displacement errors of
    neighbours, which is what the density judge sees) to the loss; noise =
    (sigma_x [m], sigma_v [m/s]) perturbs the inputs (targets unchanged);
    extra = [(sets, x_t, v_t), ...] samples (collect_on_policy) drawn with
    probability extra_fraction.  ema > 0 keeps an exponential moving average
    of the parameters with that decay (Network.use_ema takes it): each
    iteration's gradient comes from one member's graph, so the averaged
    weights are less noisy than the last iterate."""
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=net.device).manual_seed(seed)
    lib = net.lib
    g = Graph(net.cfg, net.device)
    hist = []
    t0 = time.perf_counter()
    for it in range(iters):
        if extra and rng.random() < extra_fraction:
            sets, x_t, v_t = extra[int(rng.integers(len(extra)))]
        else:
            snap = ts.snapshots[int(rng.integers(len(ts.snapshots)))]
            k = int(members[int(rng.integers(len(members)))])
            sets, x_t, v_t = sample_sets(ts, snap, k)
        if noise[0] > 0.0 or noise[1] > 0.0:
            sets = _noisy(sets, noise[0], noise[1], gen)
        g.set_nodes(sets)
        g.build(check=(it % 50 == 0))
        prepare_target(lib, g, sets, x_t, v_t, net.cfg)
        g.forward(net, store_pre=True)
        L = g.loss()
        if edge_weight > 0.0:
            L = g.edge_loss(edge_weight)
        g.backward(net)
        cos = 0.5 * (1.0 + math.cos(math.pi * it / max(iters, 1)))
        net.adam(lr * (0.05 + 0.95 * cos))
        if ema > 0.0:
            net.ema_update(ema)
        if log_every and (it % log_every == 0 or it == iters - 1):
            hist.append((it, L.item()))
            if log:
                log(f"train it {it}: loss {hist[-1][1]:.4f} ({time.perf_counter() - t0:.1f} s)")
    if g.status():
        raise RuntimeError(f"mpnn kernels raised device status 0x{g.status():x}")
    return hist


# ---------------------------------------------------------------------------
# rollout: plain step + learned jump + density judge
# ---------------------------------------------------------------------------
def rollout_accounting(stats: dict, counts, m: int, k_jump: int, k_body: int) -> bool:
    """Add one device-judged chunk to ``stats``.  counts = sphdem_rollout's
    device counters [jumps, fallbacks, largest accepted judge value (float
    bits), last fell back, largest accepted position term (float bits)];
    every jump ran 1 plain step and every fallback m
    more; k_jump / k_body = kernel nodes of the chunk's jump graphs and of
    their fallback bodies (-1: not captured).  Returns whether the number of
    plain steps is odd (each swaps the DEM contact CSR sides once)."""
    jumps, fb, maxbits = int(counts[0]), int(counts[1]), int(counts[2])
    plain = jumps + m * fb
    stats["jumps"] += jumps
    stats["fallbacks"] += fb
    stats["plain_steps"] += plain
    stats["learned_steps"] += m * (jumps - fb)
    stats["max_dev_accepted"] = max(stats["max_dev_accepted"], float(np.array(maxbits, np.int32).view(np.float32)))
    if len(counts) > 4:
        stats["max_pos_accepted"] = max(stats.get("max_pos_accepted", 0.0),
                                        float(np.array(int(counts[4]), np.int32).view(np.float32)))
    stats["jump_kernels"] += max(k_jump, 0) + (max(k_body, 0) * fb) // max(jumps, 1)
    return plain % 2 == 1


class LearnedRollout:
    """Advance a case with jumps of K = m + 1 steps (one plain, m learned).

    Each jump is a CUDA graph: plain step, network, prior + correction,
    density judge.  By default (``native``) the judge decides on the device:
    a conditional node in the same graph undoes the jump and runs the m steps
    with the plain method when the judge value is above ``tol`` (or a graph
    capacity overflowed), so jumps are launched back to back and the host
    reads the outcome once per chunk (sphdem_rollout).  The host-judged path
    (sphdem_jump, the value read back after every jump) runs the first jump
    and is kept as ``native = False``."""

    CHUNK = 50  # jumps per device-judged launch sequence (one host read each)

    def __init__(self, case, net: Network, reuse_grid: bool = True):
        from .engine import context_for

        self.case = case
        self.reuse_grid = reuse_grid  # after an accepted jump, its judge's fluid grid serves the next
        self.net = net
        self.cfg = net.cfg
        self.lib = net.lib
        self.g = Graph(net.cfg, net.device)
        c = case
        self.ctx = context_for(c.P, c.B, c.D, c.W, tuple(c.grids))
        self.keep = torch.zeros(6 * c.P.n + 6 * c.D.n + c.P.n, dtype=torch.float32, device=net.device)
        self.dev = torch.zeros(2, dtype=torch.float32, device=net.device)  # density term, position term
        self.host = torch.zeros(4, dtype=torch.float32).pin_memory()
        self.jump = None
        self._kernels = {}
        self.last_accepted = False  # the last jump of the last run() was accepted
        self.native = True          # device-judged jumps (sphdem_rollout); False: host-judged
        self._warm = False          # one host-judged jump has run (kernel attributes set)
        self.dstats = torch.zeros(6, dtype=torch.int32, device=net.device)
        self.hstats = torch.zeros(6, dtype=torch.int32).pin_memory()
        self.stats = dict(jumps=0, fallbacks=0, plain_steps=0, learned_steps=0, max_dev_accepted=0.0,
                          max_pos_accepted=0.0, jump_kernels=0)

    def _setup(self) -> None:
        c, g = self.case, self.g
        self.ctx.set_params(c.solv, c.scales)
        self.ctx.prepare(rebuild_moving=False,
                         wall_key=(float(np.float32(c.solv.support)), float(np.float32(c.solv.h))))
        g.set_nodes(Sets(c.P, c.B, c.D, c.W))
        g.build(check=True)  # node grid geometry and edge capacity
        j = _lib.JumpT()
        j.nodes = g.nodes
        j.net = g._net(self.net)
        g.grid.fill(j.node_grid, g.n_nodes)
        j.scan_scratch = _lib.iptr(g.scan)
        j.graph_ctl = C.c_void_p(g.ctl.data_ptr())
        j.radius = float(self.cfg.radius)
        j.substeps = int(self.cfg.substeps)
        for i in range(4):
            j.scale[i] = float(self.cfg.scale[i])
        j.keep = _lib.fptr(self.keep)
        j.dev = _lib.fptr(self.dev)
        j.judge = int(self.cfg.judge)
        j.pos_tol = float(self.cfg.pos_tol)
        self.jump = j

    def run(self, first_step: int, n_steps: int) -> dict:
        """Advance n_steps from first_step: jumps judged on the device
        (sphdem_rollout: launched back to back, the fallback inside the graph),
        in chunks of CHUNK jumps with one host read each; the first jump of a
        rollout goes through the host-judged path (it sets kernel attributes
        eagerly), steps short of a jump run plain."""
        c, cfg, lib = self.case, self.cfg, self.lib
        m, K = cfg.substeps, cfg.substeps + 1
        if self.jump is None:
            self._setup()
        ctx, D = self.ctx, c.D
        step, end = first_step, first_step + n_steps
        ctx.set_params(c.solv, c.scales)  # constant over the rollout (the plain fallback sets its own)
        fresh = 0  # the caller may have moved or restored the state: re-bin in the first jump
        if not self._warm and end - step >= K:
            fresh = self._run_hosted(step, K, fresh)
            self._warm = True
            step += K
        st = self.g.stream()
        while self.native and end - step >= K:
            n = min((end - step) // K, self.CHUNK)
            self.dstats.zero_()
            _lib.check(lib.sphdem_rollout(C.byref(ctx.ctx), C.byref(ctx.params), C.byref(self.jump), step, n,
                                          float(cfg.tol), fresh, C.c_void_p(self.dstats.data_ptr()), st),
                       "sphdem_rollout")
            k_jump = int(lib.sphdem_rollout_kernels(C.byref(ctx.ctx), step, n, fresh, 0))
            k_body = int(lib.sphdem_rollout_kernels(C.byref(ctx.ctx), step, n, fresh, 1))
            self.hstats.copy_(self.dstats, non_blocking=True)
            self.host[1:2].copy_(self.g.ctl[3:4], non_blocking=True)
            self.host[2:3].copy_(ctx.ctl[3:4], non_blocking=True)
            torch.cuda.current_stream(self.net.device).synchronize()
            counts = [int(v) for v in self.hstats.tolist()]
            if rollout_accounting(self.stats, counts, m, k_jump, k_body):  # odd plain steps: CSR sides swapped
                D._flip("dem")
                D._flip("bnd")
            last = counts[3]
            gflags, cflags = int(self.host[1]), int(self.host[2])
            if cflags:
                ctx._raise_for(cflags)
            if gflags & 0x8:  # edge capacity: those jumps fell back; grow and re-capture
                self.g.ctl[3] = 0
                self.g._alloc_edges(self._grown_capacity())
                self._setup()
            elif gflags:
                raise RuntimeError(f"learned jump raised device status 0x{gflags:x}")
            self.last_accepted = not last
            fresh = 1 if self.reuse_grid else 0  # the judge or the fallback body re-binned the fluid
            step += n * K
        if not self.native and end - step >= K:
            fresh = self._run_hosted(step, (end - step) // K * K, fresh)
            step = end - (end - step) % K
        if step < end:
            c.run(step, end - step)
            self.stats["plain_steps"] += end - step
            self.last_accepted = False
        return dict(self.stats)

    def _run_hosted(self, first_step: int, n_steps: int, fresh: int) -> int:
        """Jumps judged on the host: one sphdem_jump per jump, the judge value read
        back, undo + plain steps above tolerance.  Returns the grid-fresh flag."""
        c, cfg, lib = self.case, self.cfg, self.lib
        m, K = cfg.substeps, cfg.substeps + 1
        if self.jump is None:
            self._setup()
        ctx, D = self.ctx, c.D
        step, end = first_step, first_step + n_steps
        st = self.g.stream()
        while step < end:
            if end - step < K:
                c.run(step, end - step)
                self.stats["plain_steps"] += end - step
                self.last_accepted = False
                fresh = 0
                break
            _lib.check(lib.sphdem_jump(C.byref(ctx.ctx), C.byref(ctx.params), C.byref(self.jump), step, fresh, st),
                       "sphdem_jump")
            shep = step == 0 or (c.solv.shepard_step > 0 and step % c.solv.shepard_step == 0)
            variant = int(shep) + 2 * fresh
            nk = self._kernels.get(variant, 0)  # kernel nodes of this variant's jump graph
            if nk <= 0:  # (0 until the graph is captured: the first jumps run eagerly)
                nk = max(0, int(lib.sphdem_jump_kernels(C.byref(ctx.ctx), variant)))
                self._kernels[variant] = nk
            self.stats["jump_kernels"] += nk
            D._flip("dem")  # the plain step of the jump swapped both contact CSRs
            D._flip("bnd")
            self.host[0:1].copy_(self.dev[0:1], non_blocking=True)
            self.host[1:2].copy_(self.g.ctl[3:4], non_blocking=True)
            self.host[2:3].copy_(ctx.ctl[3:4], non_blocking=True)
            self.host[3:4].copy_(self.dev[1:2], non_blocking=True)
            torch.cuda.current_stream(self.net.device).synchronize()
            self.stats["jumps"] += 1
            self.stats["plain_steps"] += 1
            dev, dpos = float(self.host[0]), float(self.host[3])
            gflags, cflags = int(self.host[1]), int(self.host[2])
            if cflags:
                ctx._raise_for(cflags)
            if gflags & 0x8:  # edge capacity: grow, re-capture, run this jump's substeps plain
                self.g.ctl[3] = 0
                self.g._alloc_edges(self._grown_capacity())
                self.jump = None
                self._kernels = {}
            elif gflags:
                raise RuntimeError(f"learned jump raised device status 0x{gflags:x}")
            if self.jump is not None and dev <= cfg.tol and (cfg.pos_tol <= 0.0 or dpos <= cfg.pos_tol):
                self.stats["learned_steps"] += m
                self.stats["max_dev_accepted"] = max(self.stats["max_dev_accepted"], dev)
                self.stats["max_pos_accepted"] = max(self.stats.get("max_pos_accepted", 0.0), dpos)
                fresh = 1 if self.reuse_grid else 0
                self.last_accepted = True
            else:
                fresh = 0
                self.last_accepted = False
                _lib.check(lib.sphdem_jump_undo(C.byref(ctx.ctx), C.byref(self.jump or self._rebuild_jump()), st),
                           "sphdem_jump_undo")
                self.stats["fallbacks"] += 1
                c.run(step + 1, m)
                self.stats["plain_steps"] += m
            step += K
        return fresh

    def _grown_capacity(self) -> int:
        """Edge capacity after an overflow: the last graph's full edge count
        (its counting pass completes even when the fill overflows) + 25%, and
        at least 1.5x the old capacity."""
        need = int(self.g.buf["offset"][self.g.n_recv].item())
        return max(int(need * 1.25) + 1024, int(self.g.capacity * 1.5))

    def _rebuild_jump(self):
        self._setup()
        return self.jump
