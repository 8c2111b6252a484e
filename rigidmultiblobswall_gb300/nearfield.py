"""Near-field augmented preconditioner (GPU): the first Neumann term of the
near inter-body blocks of M on top of the block-diagonal preconditioner, with
exact blob-level couplings for close pairs and network-predicted couplings of
the bodies' 11 low-order modes (translations, rotations, strains) further out.
The network is trained on the GPU on the pair couplings of few-body
clusters that the plain method's own machinery computes.

Use::

    sys_.build_pc()
    attach_exact(sys_, cutoff=6 * R)                   # exact near field only
    model = NearfieldModel(body_radius=R, cutoff=9 * R)      # messages between bodies < 3R apart
    graphs = cluster_training_data(shell, a, eta, 1024, d_range=(2 * R + 2 * a, 9 * R),
                                   z_range=(1.1 * R, 3 * R))
    model.train(graphs, steps=2000)
    model.attach(sys_, exact_cutoff=6 * R)             # exact < 6R <= learned < 9R
    result = solve_with_fallback(sys_, model, rhs, exact_cutoff=6 * R)

The network is a message-passing network over the bodies: embeddings from
each body's height and neighbour count, three rounds of messages between
bodies closer than 3R, and a readout per pair that predicts, from both
embeddings and the pair's horizontal distance d and heights z_i, z_j (units of
the body radius), the 11x11 response G_ij of body i's modes to body j's mode
moments (force, torque, stresslet) in the frame whose x axis is the
horizontal separation; the kernels rotate it into the lab frame.  It trains
on clusters of two to eight bodies.  Changing only the rigid-body (6x6) part of the preconditioner - even
with the exact many-body mobility - was found to cost GMRES iterations: the
blob rows of the correction must stay consistent, which the Neumann form
guarantees.
"""
import ctypes

import numpy as np

from . import _native
from . import suspensions as S
from .rigid import RigidSystem

N_NODE_FEAT, N_EDGE_FEAT, N_MODES = 2, 3, 11
N_TARGET = N_MODES * N_MODES
# rotation by pi about the wall normal in the mode basis (translations,
# rotations, strains (xx-yy), (2zz-xx-yy), xy, xz, yz)
Q_PI = np.diag([-1.0, -1.0, 1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 1.0, -1.0, -1.0])
_S2, _S6 = 1.0 / np.sqrt(2.0), 1.0 / np.sqrt(6.0)
_STRAINS = np.array([np.diag([_S2, -_S2, 0.0]), np.diag([-_S6, -_S6, 2.0 * _S6]),
                     [[0, _S2, 0], [_S2, 0, 0], [0, 0, 0]], [[0, 0, _S2], [0, 0, 0], [_S2, 0, 0]],
                     [[0, 0, 0], [0, 0, _S2], [0, _S2, 0]]], dtype=np.float64)


def mode_rotations(c, s):
    """Q = diag(Rz, Rz, R5) (n, 11, 11) for rotations about the wall normal with cos c, sin s (arrays)."""
    c = np.asarray(c, dtype=np.float64).reshape(-1)
    s = np.asarray(s, dtype=np.float64).reshape(-1)
    n = c.size
    Rz = np.zeros((n, 3, 3))
    Rz[:, 0, 0], Rz[:, 0, 1], Rz[:, 1, 0], Rz[:, 1, 1], Rz[:, 2, 2] = c, -s, s, c, 1.0
    Q = np.zeros((n, N_MODES, N_MODES))
    Q[:, :3, :3] = Rz
    Q[:, 3:6, 3:6] = Rz
    T = np.einsum("nap,lpq,nbq->nlab", Rz, _STRAINS, Rz)
    Q[:, 6:, 6:] = np.einsum("kab,nlab->nkl", _STRAINS, T)
    return Q


def _sizes():
    vals = [ctypes.c_int(0) for _ in range(6)]
    _native.call("rmw_nearfield_sizes", *[ctypes.byref(v) for v in vals])
    return [v.value for v in vals]


class _Graph(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int32), ("n_mp", ctypes.c_int32), ("n_band", ctypes.c_int32),
                ("node_feat", ctypes.c_void_p), ("mp_src", ctypes.c_void_p), ("mp_dst", ctypes.c_void_p),
                ("mp_off", ctypes.c_void_p), ("mp_rev", ctypes.c_void_p), ("mp_feat", ctypes.c_void_p),
                ("band_i", ctypes.c_void_p), ("band_j", ctypes.c_void_p), ("band_off", ctypes.c_void_p),
                ("band_rev", ctypes.c_void_p), ("band_feat", ctypes.c_void_p), ("target", ctypes.c_void_p)]


def graph_arrays(centres, cluster, R, r_mp, band_lo, band_hi):
    """numpy arrays of the message-passing graph of bodies at centres (n, 3) grouped by cluster id (edges
    only within a cluster): message edges below r_mp, band edges in [band_lo, band_hi) (centre distance),
    each sorted by destination with CSR offsets and reverse-edge indices."""
    c = np.asarray(centres, dtype=np.float64).reshape(-1, 3)
    n = c.shape[0]
    cl = np.asarray(cluster)
    d = np.linalg.norm(c[:, None] - c[None], axis=-1)
    same = cl[:, None] == cl[None]
    np.fill_diagonal(same, False)

    def edges(mask):
        dst, src = np.nonzero(mask)
        order = {(int(i), int(j)): e for e, (i, j) in enumerate(zip(dst, src))}
        rev = np.array([order[(int(j), int(i))] for i, j in zip(dst, src)], dtype=np.int32)
        off = np.zeros(n + 1, dtype=np.int32)
        np.add.at(off, dst + 1, 1)
        off = np.cumsum(off).astype(np.int32)
        dh = np.hypot(c[dst, 0] - c[src, 0], c[dst, 1] - c[src, 1])
        feat = (np.stack([dh, c[dst, 2], c[src, 2]], axis=1) / R).astype(np.float32)
        return dst.astype(np.int32), src.astype(np.int32), off, rev, feat

    mdst, msrc, moff, mrev, mfeat = edges(same & (d < r_mp))
    bi, bj, boff, brev, bfeat = edges(same & (d >= band_lo) & (d < band_hi))
    deg = np.diff(moff)
    node = np.stack([c[:, 2] / R, deg / 8.0], axis=1).astype(np.float32)
    return {"n_nodes": n, "node_feat": node, "mp_src": msrc, "mp_dst": mdst, "mp_off": moff, "mp_rev": mrev,
            "mp_feat": mfeat, "band_i": bi, "band_j": bj, "band_off": boff, "band_rev": brev, "band_feat": bfeat}


class DeviceGraph:
    """A graph's arrays on the GPU (torch tensors kept alive) and the C struct pointing at them."""

    def __init__(self, arrays, target=None, device="cuda"):
        import torch
        self.arrays = arrays
        self._t = {}
        for k, v in arrays.items():
            if isinstance(v, np.ndarray):
                self._t[k] = torch.as_tensor(np.ascontiguousarray(v), device=device)
        if target is not None:
            self._t["target"] = torch.as_tensor(target, dtype=torch.float32, device=device).contiguous()
        g = _Graph()
        g.n_nodes = int(arrays["n_nodes"])
        g.n_mp = int(len(arrays["mp_src"]))
        g.n_band = int(len(arrays["band_i"]))
        for name, _ in _Graph._fields_[3:]:
            t = self._t.get(name)
            setattr(g, name, t.data_ptr() if t is not None and t.numel() > 0 else None)
        self.c = g

    @property
    def n_band(self):
        return self.c.n_band


class NearfieldModel:
    """Owner of an rmw message-passing near-field network on the current CUDA device."""

    def __init__(self, body_radius, cutoff, seed=0, mp_cutoff=None):
        h = ctypes.c_void_p()
        _native.call("rmw_nearfield_create", ctypes.byref(h), float(body_radius), float(cutoff), int(seed))
        self._h = h
        self.body_radius = float(body_radius)
        self.cutoff = float(cutoff)
        self.mp_cutoff = float(mp_cutoff) if mp_cutoff is not None else 3.0 * float(body_radius)
        _native.call("rmw_nearfield_set_cutoffs", self._h, self.mp_cutoff, self.cutoff)
        self.n_weights, self.n_biases, self.n_norm, self.width, self.n_out, self.n_target = _sizes()

    def __del__(self):
        try:
            if self._h is not None and self._h.value:
                _native.load().rmw_nearfield_destroy(self._h)
        except Exception:
            pass

    # -- parameters --------------------------------------------------------------
    def get_params(self):
        w = np.zeros(self.n_weights, dtype=np.float32)
        b = np.zeros(self.n_biases, dtype=np.float32)
        nrm = np.zeros(self.n_norm, dtype=np.float32)
        _native.call("rmw_nearfield_get", self._h, w.ctypes.data, b.ctypes.data, nrm.ctypes.data)
        return w, b, nrm

    def set_params(self, w=None, b=None, norm=None):
        keep = [np.ascontiguousarray(x, dtype=np.float32) if x is not None else None for x in (w, b, norm)]
        _native.call("rmw_nearfield_set", self._h, *[None if k is None else k.ctypes.data for k in keep])

    def save(self, path):
        w, b, nrm = self.get_params()
        np.savez(path, w=w, b=b, norm=nrm, radius=self.body_radius, cutoff=self.cutoff, mp_cutoff=self.mp_cutoff)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        m = cls(float(d["radius"]), float(d["cutoff"]), mp_cutoff=float(d["mp_cutoff"]))
        m.set_params(d["w"], d["b"], d["norm"])
        return m

    # -- network -------------------------------------------------------------------
    def forward(self, graph: DeviceGraph):
        """Normalised outputs (n_band, 121) of a graph (numpy)."""
        import torch
        out = torch.empty((graph.n_band, N_TARGET), dtype=torch.float32, device="cuda")
        _native.call("rmw_nearfield_forward", self._h, ctypes.byref(graph.c), out.data_ptr(),
                     torch.cuda.current_stream().cuda_stream)
        return out.cpu().numpy()

    def grad(self, graph: DeviceGraph):
        """Gradients (weights, biases) and loss of the mean squared error on the graph's targets."""
        gW = np.zeros(self.n_weights, dtype=np.float32)
        gb = np.zeros(self.n_biases, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _native.call("rmw_nearfield_grad", self._h, ctypes.byref(graph.c), gW.ctypes.data, gb.ctypes.data,
                     loss.ctypes.data)
        return gW, gb, float(loss[0])

    def train(self, graphs, steps=2000, lr=2e-3):
        """Adam over training graphs (one per step, cycling).  Returns the loss history."""
        import torch
        arr = (_Graph * len(graphs))(*[g.c for g in graphs])
        hist = np.zeros(steps, dtype=np.float32)
        _native.call("rmw_nearfield_train", self._h, arr, len(graphs), int(steps), float(lr), hist.ctypes.data,
                     torch.cuda.current_stream().cuda_stream)
        return hist

    def attach(self, sys_: RigidSystem, exact_cutoff=0.0, learned_from=0.0):
        """Augment sys_'s preconditioner (already built): exact couplings below
        exact_cutoff, learned ones from max(exact_cutoff, learned_from) up to the
        network's cutoff.  Returns the (exact, learned) ordered pair counts."""
        return _set(sys_, self._h, exact_cutoff, learned_from)


def _set(sys_, net, exact_cutoff, learned_from=0.0):
    n = (ctypes.c_int64 * 2)()
    _native.call("rmw_rigid_set_nearfield_bands", sys_._h, net, float(exact_cutoff), float(learned_from), n)
    return int(n[0]), int(n[1])


def attach_exact(sys_: RigidSystem, cutoff):
    """Exact near-field couplings only (no network)."""
    return _set(sys_, None, cutoff)


def detach(sys_: RigidSystem):
    """Back to the plain block-diagonal preconditioner."""
    _set(sys_, None, 0.0)


def _place_cluster(rng, n, R, a, d_range, z_range):
    """Centres of one cluster: each new body within d_range of a random earlier one, heights in z_range,
    no two closer than 2R + 2a."""
    c = [np.array([0.0, 0.0, rng.uniform(*z_range)])]
    while len(c) < n:
        base = c[rng.integers(len(c))]
        z = rng.uniform(*z_range)
        dist = rng.uniform(*d_range)
        dz = z - base[2]
        if dz * dz >= dist * dist:
            continue
        h = np.sqrt(dist * dist - dz * dz)
        t = rng.uniform(0.0, 2 * np.pi)
        p = np.array([base[0] + h * np.cos(t), base[1] + h * np.sin(t), z])
        if all(np.linalg.norm(p - q) >= 2 * R + 2 * a for q in c):
            c.append(p)
    return np.array(c)


def cluster_training_data(shell, a, eta, n_clusters, d_range, z_range, sizes=(2, 8), clusters_per_graph=64,
                          r_mp=None, seed=0, device="cuda"):
    """Training graphs from clusters of 2..8 bodies (the plain method's couplings as targets).

    Every cluster grows body by body, each new shell at a centre distance in d_range from a random earlier
    one, heights in z_range, random orientations.  One handle holds all clusters' shells (clusters far
    apart); the block-diagonal preconditioner forms each body's M^-1 and rmw_rigid_pair_coupling_list the
    11 x 11 coupling G_ij of every ordered pair of a cluster within d_range, turned into the pair's frame
    (x axis along the horizontal separation).  Returns a list of DeviceGraph (clusters_per_graph clusters
    each, message edges below r_mp = 3R by default)."""
    import torch
    rng = np.random.default_rng(seed)
    R = float(np.linalg.norm(shell[0]))
    r_mp = 3.0 * R if r_mp is None else float(r_mp)
    cents, cid = [], []
    for k in range(n_clusters):
        n = int(rng.integers(sizes[0], sizes[1] + 1))
        c = _place_cluster(rng, n, R, a, d_range, z_range)
        c[:, 0] += 1000.0 * R * (k % 64)
        c[:, 1] += 1000.0 * R * (k // 64)
        cents.append(c)
        cid.extend([k] * n)
    cen = np.concatenate(cents)
    cid = np.asarray(cid)
    q = S.random_quaternions(rng, cen.shape[0])
    r = S.blob_positions(cen, q, shell)
    nb = shell.shape[0]
    graphs = []
    sys_ = RigidSystem([nb] * cen.shape[0], eta, a, device=device)
    try:
        sys_.set_configuration(r, cen)
        sys_.build_pc()
        for g0 in range(0, n_clusters, clusters_per_graph):
            sel = (cid >= g0) & (cid < g0 + clusters_per_graph)
            idx = np.nonzero(sel)[0]
            arrays = graph_arrays(cen[idx], cid[idx], R, r_mp, d_range[0], d_range[1])
            nbnd = len(arrays["band_i"])
            if nbnd == 0:
                continue
            pairs = np.stack([idx[arrays["band_i"]], idx[arrays["band_j"]]], axis=1).astype(np.int32)
            pt = torch.as_tensor(pairs.reshape(-1), device=sys_.device)
            G = torch.empty(nbnd * N_TARGET, dtype=torch.float64, device=sys_.device)
            _native.call("rmw_rigid_pair_coupling_list", sys_._h, pt.data_ptr(), nbnd, G.data_ptr())
            G = G.reshape(nbnd, N_MODES, N_MODES).cpu().numpy()
            sep = cen[idx[arrays["band_j"]]] - cen[idx[arrays["band_i"]]]
            rho = np.hypot(sep[:, 0], sep[:, 1])
            Q = mode_rotations(sep[:, 0] / rho, sep[:, 1] / rho)
            Gp = np.einsum("nka,nkl,nlb->nab", Q, G, Q)  # Q^T G Q
            graphs.append(DeviceGraph(arrays, Gp.reshape(nbnd, N_TARGET).astype(np.float32), device=device))
    finally:
        sys_.close()
    return graphs


def solve_with_fallback(sys_, model, rhs, tol=1e-8, restart=60, maxiter=1000, mode="mixed", reference=None,
                        exact_cutoff=0.0, learned_from=0.0):
    """Solve with the augmented preconditioner and keep it only when it helps.

    model may be None (exact near field only).  reference: (iterations,
    relative residual) of the plain block-diagonal solve on the same system, if
    known; otherwise it is measured here.  Returns a dict with both solves and
    the one kept ("plain" or "augmented"); the handle is left with that
    preconditioner.
    """
    import time
    import torch
    if reference is None:
        detach(sys_)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xp, infop, itp, rrp = sys_.solve(rhs, tol=tol, restart=restart, maxiter=maxiter, mode=mode)
        torch.cuda.synchronize()
        plain = {"iterations": itp, "relres": rrp, "info": infop, "s": time.perf_counter() - t0, "x": xp}
    else:
        plain = {"iterations": reference[0], "relres": reference[1], "info": 0, "s": None, "x": None}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pairs = (model.attach(sys_, exact_cutoff, learned_from) if model is not None
             else attach_exact(sys_, exact_cutoff))
    xl, infol, itl, rrl = sys_.solve(rhs, tol=tol, restart=restart, maxiter=maxiter, mode=mode)
    torch.cuda.synchronize()
    aug = {"iterations": itl, "relres": rrl, "info": infol, "s": time.perf_counter() - t0, "x": xl,
           "pairs": pairs}
    worse = infol != 0 or itl > plain["iterations"] or rrl > max(plain["relres"], tol)
    if worse:
        detach(sys_)
    return {"plain": plain, "augmented": aug, "kept": "plain" if worse else "augmented"}
