"""Oracle (test infrastructure only) for the message-passing near-field network.

numpy restatement of the network the GPU trains and runs (csrc/nearfield.cu), with the same BF16
rounding (round to nearest even) of weights, GEMM inputs and stored activations, FP64 accumulation
(the GPU accumulates in FP32), SiLU activations, straight-through gradients through every rounding,
and BF16-rounded output gradients in the backward GEMMs (the GPU runs them on the tensor cores too).
Used to check the GPU forward pass and training gradients; checked itself against finite differences
with the rounding switched off.

Graph (one or many clusters of bodies above the wall):
  nodes       bodies; raw features (z / R, degree / 8)
  mp edges    (dst <- src) for centre distances below the message cutoff, sorted by dst, with the
              index of the reverse edge; raw features (horizontal distance, z_dst, z_src) / R
  band edges  (i <- j) whose 11 x 11 mode coupling G_ij is predicted (the learned band), sorted by i,
              with the reverse edge; raw features as for mp edges
Network (widths 64, inputs zero-padded to 16):
  h0 = silu(W0 x + b0)
  3 x:  m_e = silu(Wm [h_src; e] + bm);  M_i = mean_{e -> i} m_e;  h <- h + silu(Wu [h_i; M_i] + bu)
  readout per band edge: 144 -> 64 -> 64 -> 128 (121 outputs = G_ij in the pair frame, normalised)
"""
import numpy as np

from .nearfield import bf16, silu, silu_grad

IN, W, OUT, TARGET = 16, 64, 128, 121
N_NODE_FEAT, N_EDGE_FEAT = 2, 3
MP_LAYERS = 3
# (name, n_in, n_out, activation)
LAYERS = ([("embed", IN, W, True)] +
          [x for t in range(MP_LAYERS) for x in ((("msg%d" % t), W + IN, W, True), (("upd%d" % t), 2 * W, W, True))] +
          [("ro0", 2 * W + IN, W, True), ("ro1", W, W, True), ("ro2", W, OUT, False)])
# normalisation: node feature mean/scale, edge feature mean/scale, target scale
N_NORM = 2 * N_NODE_FEAT + 2 * N_EDGE_FEAT + TARGET


def sizes():
    nw = sum(ni * no for _, ni, no, _ in LAYERS)
    nb = sum(no for _, _, no, _ in LAYERS)
    return nw, nb


def split(w, b):
    out, ow, ob = {}, 0, 0
    for name, ni, no, act in LAYERS:
        out[name] = (np.asarray(w[ow:ow + ni * no], dtype=np.float64).reshape(no, ni),
                     np.asarray(b[ob:ob + no], dtype=np.float64), act)
        ow += ni * no
        ob += no
    return out


def _r(x, rounding):
    return bf16(x).astype(np.float64) if rounding else np.asarray(x, dtype=np.float64)


def normalise(g, norm):
    """Padded, normalised GEMM inputs: node X0 (n x 16), mp E (e x 16), band E (b x 16)."""
    nm, ns = norm[0:2], norm[2:4]
    em, es = norm[4:7], norm[7:10]
    X0 = np.zeros((g["n_nodes"], IN))
    X0[:, :N_NODE_FEAT] = (g["node_feat"] - nm) / ns
    Em = np.zeros((len(g["mp_src"]), IN))
    Em[:, :N_EDGE_FEAT] = (g["mp_feat"] - em) / es
    Eb = np.zeros((len(g["band_i"]), IN))
    Eb[:, :N_EDGE_FEAT] = (g["band_feat"] - em) / es
    return X0, Em, Eb


def _dense(L, name, X, rounding):
    Wt, b, act = L[name]
    Z = _r(X, rounding) @ _r(Wt, rounding).T + b
    return Z, (silu(Z) if act else Z)


def forward(w, b, norm, g, rounding=True):
    """Outputs (band edges x 121, normalised) and the saved intermediates."""
    L = split(w, b)
    X0, Em, Eb = normalise(g, norm)
    src, dst = g["mp_src"], g["mp_dst"]
    deg = np.bincount(dst, minlength=g["n_nodes"]).astype(np.float64)
    inv = 1.0 / np.maximum(deg, 1.0)
    cache = {"X0": X0}
    Z, Y = _dense(L, "embed", X0, rounding)
    cache["Z_embed"] = Z
    h = _r(Y, rounding)
    hs = [h]
    for t in range(MP_LAYERS):
        Xm = np.concatenate([h[src], Em], axis=1)
        Zm, m = _dense(L, "msg%d" % t, Xm, rounding)
        m = _r(m, rounding)
        M = np.zeros((g["n_nodes"], W))
        np.add.at(M, dst, m)
        M = _r(M * inv[:, None], rounding)
        Xu = np.concatenate([h, M], axis=1)
        Zu, u = _dense(L, "upd%d" % t, Xu, rounding)
        h = _r(h + u, rounding)
        cache.update({"Xm%d" % t: Xm, "Zm%d" % t: Zm, "Xu%d" % t: Xu, "Zu%d" % t: Zu})
        hs.append(h)
    bi, bj = g["band_i"], g["band_j"]
    Xr = np.concatenate([h[bi], h[bj], Eb], axis=1)
    Z0, A0 = _dense(L, "ro0", Xr, rounding)
    A0 = _r(A0, rounding)
    Z1, A1 = _dense(L, "ro1", A0, rounding)
    A1 = _r(A1, rounding)
    Z2, Y2 = _dense(L, "ro2", A1, rounding)
    cache.update({"Xr": Xr, "Zr0": Z0, "Ar0": A0, "Zr1": Z1, "Ar1": A1, "hs": hs, "inv": inv})
    return Y2[:, :TARGET], cache


def grad(w, b, norm, g, T, rounding=True):
    """(gW, gb, loss): gradients of the mean squared error over the band edges' 121 outputs (targets T,
    normalised), by the backward pass the GPU runs."""
    L = split(w, b)
    Y, c = forward(w, b, norm, g, rounding)
    P = Y.shape[0]
    d = Y - T
    loss = float((d * d).sum() / (P * TARGET))
    gW, gB = {}, {}

    def back(name, dZ, X):
        Wt, _, _ = L[name]
        dZr = _r(dZ, rounding)
        gW[name] = dZr.T @ _r(X, rounding)
        gB[name] = dZ.sum(axis=0)
        return dZr @ _r(Wt, rounding)

    dY = np.zeros((P, OUT))
    dY[:, :TARGET] = 2.0 * d / (P * TARGET)
    dA1 = back("ro2", dY, c["Ar1"])
    dA0 = back("ro1", dA1 * silu_grad(c["Zr1"]), c["Ar0"])
    dXr = back("ro0", dA0 * silu_grad(c["Zr0"]), c["Xr"])
    n = g["n_nodes"]
    dh = np.zeros((n, W))
    np.add.at(dh, g["band_i"], dXr[:, :W])
    np.add.at(dh, g["band_j"], dXr[:, W:2 * W])
    src, dst, inv = g["mp_src"], g["mp_dst"], c["inv"]
    for t in range(MP_LAYERS - 1, -1, -1):
        # h_t = h_{t-1} + silu(Zu): straight through the rounding
        dZu = dh * silu_grad(c["Zu%d" % t])
        dXu = back("upd%d" % t, dZu, c["Xu%d" % t])
        dprev = dh + dXu[:, :W]
        dM = dXu[:, W:] * inv[:, None]
        dm = dM[dst]
        dZm = dm * silu_grad(c["Zm%d" % t])
        dXm = back("msg%d" % t, dZm, c["Xm%d" % t])
        np.add.at(dprev, src, dXm[:, :W])
        dh = dprev
    back("embed", dh * silu_grad(c["Z_embed"]), c["X0"])
    gw = np.concatenate([gW[name].reshape(-1) for name, _, _, _ in LAYERS])
    gb = np.concatenate([gB[name] for name, _, _, _ in LAYERS])
    return gw, gb, loss


def graph_from_positions(centres, cluster, R, r_mp, band_lo, band_hi):
    """Graph arrays of bodies at centres (n, 3), grouped by cluster id (edges only inside a cluster), as
    the GPU builds them: mp edges below r_mp, band edges in [band_lo, band_hi) (3-D centre distance)."""
    c = np.asarray(centres, dtype=np.float64)
    n = c.shape[0]
    d = np.linalg.norm(c[:, None] - c[None], axis=-1)
    same = np.asarray(cluster)[:, None] == np.asarray(cluster)[None]
    np.fill_diagonal(same, False)
    mp = same & (d < r_mp)
    band = same & (d >= band_lo) & (d < band_hi)

    def edges(mask):
        dst, src = np.nonzero(mask)  # sorted by dst, then src
        idx = {(int(i), int(j)): e for e, (i, j) in enumerate(zip(dst, src))}
        rev = np.array([idx[(int(j), int(i))] for i, j in zip(dst, src)], dtype=np.int64)
        dh = np.hypot(c[dst, 0] - c[src, 0], c[dst, 1] - c[src, 1])
        feat = np.stack([dh, c[dst, 2], c[src, 2]], axis=1) / R
        return dst.astype(np.int64), src.astype(np.int64), rev, feat

    mdst, msrc, mrev, mfeat = edges(mp)
    bi, bj, brev, bfeat = edges(band)
    deg = np.bincount(mdst, minlength=n)
    node_feat = np.stack([c[:, 2] / R, deg / 8.0], axis=1)
    return {"n_nodes": n, "node_feat": node_feat, "mp_src": msrc, "mp_dst": mdst, "mp_rev": mrev,
            "mp_feat": mfeat, "band_i": bi, "band_j": bj, "band_rev": brev, "band_feat": bfeat}
