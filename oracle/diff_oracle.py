"""FP64 host oracle for the differentiable leaf shading.

TEST INFRASTRUCTURE ONLY.  Restates, in float64 numpy, the shading model of
svo_diff_forward (the viewer's shade(), Main.cpp:81-90, with per-leaf rgb and
normal parameters) and its gradients, given a per-ray hit-leaf buffer from
the CPU raymarch (oracle raymarch = VoxelOctree::raymarch, VoxelOctree.cpp:
207-346, which returns the leaf index):

    n = p/|p|, a = |l.n|, r = d - 2 (n.d) n, s = max(l.r, 0)
    rgb_k = c_k 0.9 a + 0.2 s^2
    L = sum over rays and channels of w (rgb - target)^2
"""
import numpy as np


def _terms(p, d, l):
    length = np.sqrt((p * p).sum(-1))
    inv = np.where(length > 0, 1.0 / np.where(length > 0, length, 1.0), 0.0)
    n = p * inv[:, None]
    ln = (l * n).sum(-1)
    nd = (n * d).sum(-1)
    r = d - 2.0 * nd[:, None] * n
    s = np.maximum((l * r).sum(-1), 0.0)
    return n, inv, ln, nd, s


def shade(leaf, dirs, lights, p_rgb, p_n):
    """rgb per ray (float64); rays with leaf == 0xFFFFFFFF give 0."""
    hit = leaf != 0xFFFFFFFF
    out = np.zeros((leaf.size, 3))
    li = leaf[hit].astype(np.int64)
    d = dirs[hit].astype(np.float64)
    l = lights[hit].astype(np.float64)
    n, inv, ln, nd, s = _terms(p_n[li].astype(np.float64), d, l)
    out[hit] = p_rgb[li].astype(np.float64) * 0.9 * np.abs(ln)[:, None] + (0.2 * s * s)[:, None]
    return out


def loss(leaf, dirs, lights, p_rgb, p_n, target, w):
    c = shade(leaf, dirs, lights, p_rgb, p_n)
    return float((w * (c - target) ** 2).sum())


def gradient(leaf, dirs, lights, p_rgb, p_n, target, w, n_words, leaves=None):
    """Analytic dL/dp_rgb, dL/dp_n (float64, n_words x 3 each); with
    `leaves`, only those leaves' rows (len(leaves) x 3 each, in that order)."""
    if leaves is not None:
        leaves = np.asarray(leaves, np.int64)
        pos = {int(v): i for i, v in enumerate(leaves)}
        sel = np.isin(leaf.astype(np.int64), leaves)
        remap = np.full(leaf.shape, 0xFFFFFFFF, np.uint32)
        remap[sel] = [pos[int(v)] for v in leaf[sel]]
        sub_rgb = np.zeros((len(leaves), 3), np.float32)
        sub_n = np.zeros((len(leaves), 3), np.float32)
        sub_rgb[:] = p_rgb[leaves]
        sub_n[:] = p_n[leaves]
        return gradient(remap[sel], dirs[sel], lights[sel], sub_rgb, sub_n, target[sel], w, len(leaves))
    c = shade(leaf, dirs, lights, p_rgb, p_n)
    g = 2.0 * w * (c - target)
    hit = leaf != 0xFFFFFFFF
    li = leaf[hit].astype(np.int64)
    d = dirs[hit].astype(np.float64)
    l = lights[hit].astype(np.float64)
    gh = g[hit]
    n, inv, ln, nd, s = _terms(p_n[li].astype(np.float64), d, l)
    g_rgb = np.zeros((n_words, 3))
    np.add.at(g_rgb, li, gh * 0.9 * np.abs(ln)[:, None])
    wl = 0.9 * np.sign(ln) * (gh * p_rgb[li].astype(np.float64)).sum(-1)
    ws = np.where(s > 0, -0.8 * gh.sum(-1) * s, 0.0)
    gn = wl[:, None] * l + ws[:, None] * (nd[:, None] * l + ln[:, None] * d)
    gp = (gn - n * (n * gn).sum(-1)[:, None]) * inv[:, None]
    g_n = np.zeros((n_words, 3))
    np.add.at(g_n, li, gp)
    return g_rgb, g_n


def finite_differences(leaf, dirs, lights, p_rgb, p_n, target, w, leaves, h=1e-3, richardson=False):
    """Central differences of L for every component of the given leaves'
    parameters; only rays hitting the leaf change, so only those are
    re-shaded.  Returns (fd_rgb, fd_n, kink) with shape (len(leaves), 3);
    kink marks components whose +-h step crosses |l.n| = 0 or l.r = 0 for
    some contributing ray (where the loss is not differentiable).
    richardson=True returns (4 D(h/2) - D(h)) / 3, which cancels the h^2
    truncation term of the central difference D (the normalisation p/|p|
    makes that term ~ h^2/|p|^2, large for short parameter vectors)."""
    if richardson:
        a_rgb, a_n, kink = finite_differences(leaf, dirs, lights, p_rgb, p_n, target, w, leaves, h)
        b_rgb, b_n, _ = finite_differences(leaf, dirs, lights, p_rgb, p_n, target, w, leaves, h / 2)
        return (4 * b_rgb - a_rgb) / 3, (4 * b_n - a_n) / 3, kink
    fd_rgb = np.zeros((len(leaves), 3))
    fd_n = np.zeros((len(leaves), 3))
    kink = np.zeros((len(leaves), 3), bool)
    order = np.argsort(leaf, kind="stable")
    sorted_leaf = leaf[order]
    for j, lf in enumerate(leaves):
        lo, hi = np.searchsorted(sorted_leaf, lf), np.searchsorted(sorted_leaf, lf, side="right")
        rows = order[lo:hi]
        d = dirs[rows].astype(np.float64)
        l = lights[rows].astype(np.float64)
        t = target[rows]
        ww = w if np.isscalar(w) else w[rows]
        base_rgb = p_rgb[lf].astype(np.float64)
        base_n = p_n[lf].astype(np.float64)

        def part(c_vec, p_vec):
            n, inv, ln, nd, s = _terms(np.broadcast_to(p_vec, d.shape), d, l)
            col = c_vec[None, :] * 0.9 * np.abs(ln)[:, None] + (0.2 * s * s)[:, None]
            return float((ww * (col - t) ** 2).sum()), ln, (l * (d - 2.0 * nd[:, None] * n)).sum(-1)

        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            fd_rgb[j, k] = (part(base_rgb + e, base_n)[0] - part(base_rgb - e, base_n)[0]) / (2 * h)
            lp, ln_p, lr_p = part(base_rgb, base_n + e)
            lm, ln_m, lr_m = part(base_rgb, base_n - e)
            fd_n[j, k] = (lp - lm) / (2 * h)
            kink[j, k] = bool(np.any(np.sign(ln_p) != np.sign(ln_m)) or np.any((lr_p > 0) != (lr_m > 0)))
    return fd_rgb, fd_n, kink
