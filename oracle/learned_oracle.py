"""CPU oracle of the learned opening criterion (test infrastructure only).

Only the tests may import this module; the product never does. It restates
in FP64 numpy what the CUDA kernels of galactic-tides_gb300/csrc/learned.cu
and learned_walk.cu compute, so that the tests can check them:

  * the training label of a (group, cell) pair: the largest
    |a_multipole - a_exact| over the group's targets, a_exact the FP64 direct
    sum over the cell's bodies with Plummer softening (the sum of
    src/gravity.cpp:28-45 restricted to the cell), a_multipole the cell's
    monopole + quadrupole field in the form of the list evaluator
    (include/galactic_tides/kernels/gravity_kernels.h:109-135), in log2 of
    units of G M_total / L^2;
  * the six features of a pair and the physical prior;
  * the network (6 -> 64 -> 64 -> 1, ReLU), its mean-squared-error loss on
    the normalised correction and the loss's gradient by backpropagation,
    for checking the training kernels' gradients;
  * the same network with BF16-rounded weights and activations, for checking
    the walk's tensor-core inference.

The reference has no learned criterion; what is pinned here is the
project's own definition, and the label arithmetic is pinned against the
reference's direct sum and cell formula above.
"""

import numpy as np

FEAT, HID = 6, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + FEAT * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID
PARAMS = OFF_B3 + 1
OFF_MEAN = PARAMS
OFF_STD = OFF_MEAN + FEAT
OFF_YMEAN = OFF_STD + FEAT
OFF_YSTD = OFF_YMEAN + 1
OFF_BAND = OFF_YSTD + 1
MODEL_FLOATS = OFF_BAND + 1
PRIOR_BASE = 3.3773  # log2(2 * 3^1.5)
FEW_BODIES = 2


def unpack(model):
    m = np.asarray(model, dtype=np.float64)
    return dict(
        W1=m[OFF_W1:OFF_B1].reshape(FEAT, HID), b1=m[OFF_B1:OFF_W2],
        W2=m[OFF_W2:OFF_B2].reshape(HID, HID), b2=m[OFF_B2:OFF_W3], W3=m[OFF_W3:OFF_B3],
        b3=m[OFF_B3], mean=m[OFF_MEAN:OFF_STD], std=m[OFF_STD:OFF_YMEAN], ymean=m[OFF_YMEAN],
        ystd=m[OFF_YSTD], band=m[OFF_BAND])


def prior(feat):
    f = np.asarray(feat, dtype=np.float64)
    return PRIOR_BASE + f[:, 3] + 3.0 * f[:, 1] - 5.0 * f[:, 2]


def net_forward(p, x):
    """x: normalised features (n, 6) -> (z1, z2, out)."""
    z1 = x @ p["W1"] + p["b1"]
    z2 = np.maximum(z1, 0.0) @ p["W2"] + p["b2"]
    out = np.maximum(z2, 0.0) @ p["W3"] + p["b3"]
    return z1, z2, out


def predict(model, feat):
    """Predicted log2 error of each pair (FP64)."""
    p = unpack(model)
    x = (np.asarray(feat, np.float64) - p["mean"]) / p["std"]
    return prior(feat) + p["ymean"] + p["ystd"] * net_forward(p, x)[2]


def loss_and_grad(model, feat, label):
    """Mean squared error of the normalised correction and its gradient with
    respect to the PARAMS network parameters (the normalisation is fixed)."""
    p = unpack(model)
    feat = np.asarray(feat, np.float64)
    x = (feat - p["mean"]) / p["std"]
    y = (np.asarray(label, np.float64) - prior(feat) - p["ymean"]) / p["ystd"]
    z1, z2, out = net_forward(p, x)
    n = feat.shape[0]
    err = out - y
    loss = float(np.mean(err * err))
    gout = 2.0 * err / n
    h2 = np.maximum(z2, 0.0)
    h1 = np.maximum(z1, 0.0)
    d2 = (gout[:, None] * p["W3"][None, :]) * (z2 > 0)
    d1 = (d2 @ p["W2"].T) * (z1 > 0)
    g = np.zeros(PARAMS)
    g[OFF_W1:OFF_B1] = (x.T @ d1).ravel()
    g[OFF_B1:OFF_W2] = d1.sum(0)
    g[OFF_W2:OFF_B2] = (h1.T @ d2).ravel()
    g[OFF_B2:OFF_W3] = d2.sum(0)
    g[OFF_W3:OFF_B3] = h2.T @ gout
    g[OFF_B3] = gout.sum()
    return loss, g


def bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a32 = np.asarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def predict_bf16(model, feat):
    """The walk's inference: normalised features, weights, biases of layer 1
    and hidden activations rounded to BF16, sums in high precision."""
    p = unpack(model)
    feat = np.asarray(feat, np.float64)
    x = bf16((feat - p["mean"]) / p["std"])
    z1 = x @ bf16(p["W1"]) + bf16(p["b1"])
    h1 = bf16(np.maximum(z1, 0.0))
    z2 = h1 @ bf16(p["W2"]) + p["b2"]
    out = np.maximum(z2, 0.0) @ p["W3"] + p["b3"]
    return prior(feat) + p["ymean"] + p["ystd"] * out


# ---- labels and features of (group, cell) pairs ----------------------------

def cell_field(targets, com, mass, quad, G, eps2):
    """Monopole + quadrupole field of a cell at the targets (FP64), in the
    list evaluator's form. quad = (xx, yy, zz, xy, xz, yz)."""
    d = targets - com
    r2 = np.einsum("ij,ij->i", d, d) + eps2
    inv = 1.0 / np.sqrt(r2)
    inv3, inv5, inv7 = inv ** 3, inv ** 5, inv ** 7
    xx, yy, zz, xy, xz, yz = quad
    qd = np.stack([xx * d[:, 0] + xy * d[:, 1] + xz * d[:, 2],
                   xy * d[:, 0] + yy * d[:, 1] + yz * d[:, 2],
                   xz * d[:, 0] + yz * d[:, 1] + zz * d[:, 2]], axis=1)
    rqr = np.einsum("ij,ij->i", d, qd)
    return (-G * mass * inv3)[:, None] * d + G * (qd * inv5[:, None]
                                                 - 2.5 * (rqr * inv7)[:, None] * d)


def direct_field(targets, src_pos, src_mass, G, eps2):
    d = targets[:, None, :] - src_pos[None, :, :]
    r2 = np.einsum("ijk,ijk->ij", d, d) + eps2
    inv3 = r2 ** -1.5
    return -G * np.einsum("ij,ijk->ik", src_mass[None, :] * inv3, d)


def pair_label(targets, src_pos, src_mass, com, mass, quad, G, eps2, L, mtot):
    """log2 of the largest error over the targets, in units of G mtot / L^2."""
    err = np.linalg.norm(cell_field(targets, com, mass, quad, G, eps2)
                         - direct_field(targets, src_pos, src_mass, G, eps2), axis=1).max()
    return np.log2(max(err * L * L / (G * mtot), 1e-30))


def pair_features(gbox_half, box_dist, half, mass, qnorm, delta, L, mtot):
    """The six features (FP64 restatement of the device's FP32 arithmetic)."""
    lg = lambda v: np.log2(max(v, 1e-30))
    return np.array([
        lg(max(max(gbox_half) / L, 1e-9)),
        lg(half / L),
        lg(max(box_dist / L, 1e-9)),
        lg(mass / mtot),
        lg(qnorm / max(mass, 1e-30) / (L * L) + 1e-12),
        delta / max(half, 1e-30),
    ])


def quad_norm(q):
    """Frobenius norm of the symmetric tensor (xx, yy, zz, xy, xz, yz)."""
    xx, yy, zz, xy, xz, yz = q
    return np.sqrt(xx * xx + yy * yy + zz * zz + 2.0 * (xy * xy + xz * xz + yz * yz))


# ---- the learned walk's decisions -------------------------------------------
#
# A restatement of galactic-tides_gb300/csrc/learned_walk.cu's walk on a given
# tree: the node and group records in FP32 as the device packs them, the
# verdict of every (group, node) test the walk makes -- the reference's
# overlap test (group_lists.cpp:147) and the guard open; cells of at most two
# bodies accepted; the centred prior decides when it clears the tolerance by
# more than the band; the network (BF16 emulation) decides the rest -- and
# the cells and bodies each group ends with. The walk visits a node when its
# parent was visited and opened (the root is always opened when it has
# children). Rounds, parts and hand-offs to warps only order the device's
# lists, so multisets are compared. Each test's distance from its threshold
# is returned too: device and oracle may differ where the two FP32 pipelines
# (FMA contraction, the fast log2 and exp2) or the BF16 emulation round a
# test to the other side.

KIND_GEOM, KIND_PRIOR, KIND_NET = 0, 1, 2


def _f32(v):
    return np.asarray(v, dtype=np.float32)


def _log2f(v):
    return _f32(np.log2(np.asarray(v, np.float64)))


def _fmaf(a, b, c):
    return _f32(np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64))


def children_of(nodes):
    """Each node's children in octant order (every child after its parent)."""
    parent = np.asarray(nodes["parent"], np.int64)
    kids = [[] for _ in range(len(nodes))]
    for i in range(1, len(nodes)):
        kids[parent[i]].append(i)
    # the device numbers siblings last octant first, the reference first
    # octant first: order them by their first body, which follows the octants
    begin = np.asarray(nodes["begin"], np.int64)
    return [sorted(k, key=lambda c: begin[c]) for k in kids]


def moments32(nodes, bodies):
    """The FP32 moment estimates the learned walk decides from
    (tree_build.cu: leaf_moments32 / node_moments32): the reference's sums
    (octree.cpp:46-102) in FP32, each product and sum rounded on its own, on
    the FP32 bodies relative to the root centre. -> cells (m, 12) in GTCell
    layout and delta (m,)."""
    f = np.float32
    origin = nodes["center"][0]
    cen = (nodes["center"] - origin).astype(np.float32)
    m_nodes = len(nodes)
    cells = np.zeros((m_nodes, 12), np.float32)
    delta = np.zeros(m_nodes, np.float32)
    kids = children_of(nodes)
    b = np.asarray(bodies, np.float32)
    three = f(3.0)

    def finish(p, m, cx, cy, cz, q):
        cells[p, :4] = (cx, cy, cz, m)
        cells[p, 4:8] = q[:4]
        cells[p, 8:10] = q[4:]
        ex, ey, ez = f(cx - cen[p, 0]), f(cy - cen[p, 1]), f(cz - cen[p, 2])
        delta[p] = f(np.sqrt(f(f(f(ex * ex) + f(ey * ey)) + f(ez * ez))))

    def com(p, m, cx, cy, cz):
        if m > 0:
            return f(cx / m), f(cy / m), f(cz / m)
        return cen[p, 0], cen[p, 1], cen[p, 2]

    def quad(terms):
        q = [f(0.0)] * 6
        for w, dx, dy, dz, qa in terms:
            r2 = f(f(f(dx * dx) + f(dy * dy)) + f(dz * dz))
            adds = (f(w * f(f(f(three * dx) * dx) - r2)), f(w * f(f(f(three * dy) * dy) - r2)),
                    f(w * f(f(f(three * dz) * dz) - r2)), f(f(f(w * three) * dx) * dy),
                    f(f(f(w * three) * dx) * dz), f(f(f(w * three) * dy) * dz))
            for k in range(6):
                q[k] = f(q[k] + (f(qa[k] + adds[k]) if qa is not None else adds[k]))
        return q

    depth = np.zeros(m_nodes, np.int64)
    for i in range(1, m_nodes):
        depth[i] = depth[int(nodes["parent"][i])] + 1
    for p in sorted(range(m_nodes), key=lambda i: -depth[i]):  # children before parents
        if not kids[p]:
            rows = b[int(nodes["begin"][p]):int(nodes["end"][p])]
            m, cx, cy, cz = f(0.0), f(0.0), f(0.0), f(0.0)
            for x, y, z, w in rows:
                m, cx, cy, cz = f(m + w), f(cx + f(w * x)), f(cy + f(w * y)), f(cz + f(w * z))
            cx, cy, cz = com(p, m, cx, cy, cz)
            q = quad([(w, f(x - cx), f(y - cy), f(z - cz), None) for x, y, z, w in rows])
        else:
            m, cx, cy, cz = f(0.0), f(0.0), f(0.0), f(0.0)
            for c in kids[p]:
                w = cells[c, 3]
                m = f(m + w)
                cx, cy, cz = (f(cx + f(w * cells[c, 0])), f(cy + f(w * cells[c, 1])),
                              f(cz + f(w * cells[c, 2])))
            cx, cy, cz = com(p, m, cx, cy, cz)
            q = quad([(cells[c, 3], f(cells[c, 0] - cx), f(cells[c, 1] - cy),
                       f(cells[c, 2] - cz), (cells[c, 4], cells[c, 5], cells[c, 6], cells[c, 7],
                                             cells[c, 8], cells[c, 9])) for c in kids[p]])
        finish(p, m, cx, cy, cz, q)
    return cells, delta


def node_records(nodes, bodies, theta_guard, y_mean):
    """Per node, the FP32 record the learned walk reads -- centre and slack
    relative to the root centre from the FP64 geometry, the centre of mass,
    guard^2 and the prior's node part from the FP32 moment estimates -- and
    the cell-only features."""
    origin = nodes["center"][0]
    L = float(nodes["half"][0])
    cells, delta = moments32(nodes, bodies)
    mt = float(cells[0, 3])  # the root's mass, as the walk takes it
    inv_l, inv_mt = _f32(1.0 / L), _f32(1.0 / mt)
    rec = {
        "c": _f32(nodes["center"] - origin), "slack": _f32(nodes["half"] * 1.0001),
        "m": cells[:, :3].copy(),
        "nbody": (nodes["end"].astype(np.int64) - nodes["begin"]),
        "leaf": nodes["n_children"] == 0,
    }
    half = _f32(nodes["half"])
    mass = cells[:, 3]
    qa, qb = cells[:, 4:8], cells[:, 8:12]
    qn = _f32(np.sqrt(qa[:, 0] ** 2 + qa[:, 1] ** 2 + qa[:, 2] ** 2
                      + 2.0 * (qa[:, 3] ** 2 + qb[:, 0] ** 2 + qb[:, 1] ** 2)))
    f1 = _log2f(np.maximum(half * inv_l, 1e-30))
    f3 = _log2f(np.maximum(mass * inv_mt, 1e-30))
    f4 = _log2f(np.maximum(qn / np.maximum(mass, _f32(1e-30)) * inv_l * inv_l + _f32(1e-12),
                           1e-30))
    f5 = _f32(delta / np.maximum(half, _f32(1e-30)))
    prior = _f32(_f32(PRIOR_BASE) + f3 + _f32(3.0) * f1)
    crit = _fmaf(_f32(2.0) * half, _f32(1.0 / theta_guard), delta)
    rec.update(guard2=_f32(crit * crit), f1=f1, f3=f3, f4=f4, f5=f5, prior=prior,
               pscale=_f32(np.exp2(np.float64(0.4) * (prior.astype(np.float64) + y_mean))),
               inv_l=inv_l, inv_mt=inv_mt, L=L, mt=mt, origin=origin)
    return rec


def group_records(tpos, ranges, amag, rec, alpha, G):
    """Per group: the FP32 box (centre relative to the root centre,
    half-extent), the group feature f0 and the tolerance tau."""
    ng = len(ranges)
    gc = np.zeros((ng, 3), np.float32)
    gh = np.zeros((ng, 3), np.float32)
    tau = np.zeros(ng, np.float32)
    for g, (b, e) in enumerate(ranges):
        p = tpos[b:e]
        lo_, hi_ = p.min(0), p.max(0)
        gc[g] = _f32((lo_ + hi_) * 0.5 - rec["origin"])
        gh[g] = _f32((hi_ - lo_) * 0.5)
        a = _f32(amag[b:e])
        asum = np.float32(0.0)
        for v in a:  # in target order, FP32
            asum = np.float32(asum + v)
        ag = max(a.min(), np.float32(np.float32(0.5) * asum / np.float32(max(e - b, 1))))
        v = alpha * float(ag) * rec["L"] * rec["L"] / (G * rec["mt"])
        tau[g] = np.float32(np.log2(v)) if v > 0 else np.float32(-1e30)
    f0 = _log2f(np.maximum(gh.max(1) * rec["inv_l"], _f32(1e-9)))
    return gc, gh, f0, tau


def walk_lists(nodes, bodies, tpos, ranges, amag, model, alpha, G=1.0, theta_guard=1.5,
               band=None):
    """The learned walk on a tree whose every node comes after its parent
    (nodes['parent']; the device's walk order and the reference's layout
    both qualify), bodies the FP32 bodies relative to the root centre (tree
    order), amag the previous |a| of each body in tree order. Returns, per group, the accepted cells
    (node indices) and the bodies (tree positions, with repeats), and per
    group the margins of its tests: a list of (node, kind, margin), margin
    relative to the threshold for FP32 tests (KIND_GEOM, KIND_PRIOR) and in
    log2 units for the network (KIND_NET)."""
    p = unpack(model)
    band = float(p["band"]) if band is None or band < 0 else float(band)
    rec = node_records(nodes, bodies, theta_guard, float(p["ymean"]))
    gc, gh, f0, tau = group_records(tpos, ranges, amag, rec, alpha, G)
    ng, m = len(ranges), len(nodes)
    l2 = _f32(_f32(1.0) / (rec["inv_l"] * rec["inv_l"]))
    acc_d2 = _f32(_f32(np.exp2(np.float64(0.4) * (band - tau.astype(np.float64)))) * l2)
    open_d2 = _f32(_f32(np.exp2(np.float64(0.4) * (-band - tau.astype(np.float64)))) * l2)
    parent = nodes["parent"].astype(np.int64)
    visited = np.zeros((ng, m), bool)
    final = np.zeros((ng, m), np.int8)  # 0 open, 1 accept
    margins = [[] for _ in range(ng)]
    root_opened = not rec["leaf"][0]
    for i in range(m):
        if i == 0:
            vis = np.full(ng, not root_opened)
            if root_opened:
                visited[:, 0] = False
                final[:, 0] = 0
                continue
        else:
            q = parent[i]
            vis = (visited[:, q] | ((q == 0) & root_opened)) & (final[:, q] == 0) & \
                ~rec["leaf"][q]
        visited[:, i] = vis
        if not vis.any():
            continue
        gsel = np.nonzero(vis)[0]
        c, s, mm = rec["c"][i], rec["slack"][i], rec["m"][i]
        # overlap: every axis |c - gc| <= slack + gh
        lhs = np.abs(c - gc[gsel])
        rhs = _f32(s + gh[gsel])
        overlap = np.all(lhs <= rhs, axis=1)
        axis_margin = np.abs(lhs - rhs) / np.maximum(np.abs(rhs), _f32(1e-30))
        d = np.maximum(np.abs(mm - gc[gsel]) - gh[gsel], _f32(0.0))
        d2 = _fmaf(d[:, 0], d[:, 0], _fmaf(d[:, 1], d[:, 1], _f32(d[:, 2] * d[:, 2])))
        guard = rec["guard2"][i]
        verdict = np.full(len(gsel), 2, np.int8)
        opened = overlap | ~(d2 > guard)
        verdict[opened] = 0
        few = ~opened & (rec["nbody"][i] <= FEW_BODIES)
        verdict[few] = 1
        rest = ~opened & ~few
        acc_t = _f32(rec["pscale"][i] * acc_d2[gsel])
        open_t = _f32(rec["pscale"][i] * open_d2[gsel])
        verdict[rest & (d2 > acc_t)] = 1
        verdict[rest & ~(d2 > acc_t) & (d2 < open_t)] = 0
        gm = np.minimum(axis_margin.min(1),
                        np.abs(d2 - guard) / np.maximum(guard, _f32(1e-30)))
        pm = np.minimum(np.abs(d2 - acc_t) / np.maximum(acc_t, _f32(1e-30)),
                        np.abs(d2 - open_t) / np.maximum(open_t, _f32(1e-30)))
        for k, g in enumerate(gsel):
            margins[g].append((i, KIND_GEOM, float(gm[k])))
            if rest[k]:
                margins[g].append((i, KIND_PRIOR, float(pm[k])))
        final[gsel, i] = np.where(verdict == 1, 1, 0)
        # the network decides the deferred pairs of this node (before any of
        # its children is visited)
        dsel = verdict == 2
        if dsel.any():
            gs_, d2s = gsel[dsel], d2[dsel]
            f2 = _log2f(np.maximum(np.sqrt(d2s.astype(np.float64)).astype(np.float32)
                                   * rec["inv_l"], _f32(1e-9)))
            feat = np.stack([f0[gs_], np.full(len(gs_), rec["f1"][i]), f2,
                             np.full(len(gs_), rec["f3"][i]), np.full(len(gs_), rec["f4"][i]),
                             np.full(len(gs_), rec["f5"][i])], axis=1)
            pred = predict_bf16(model, feat)
            acc = pred < tau[gs_]
            final[gs_, i] = np.where(acc, 1, 0)
            for g, mg in zip(gs_, np.abs(pred - tau[gs_])):
                margins[g].append((i, KIND_NET, float(mg)))
    cells_out, bodies_out = [], []
    nb, leaf = rec["nbody"], rec["leaf"]
    begin = nodes["begin"].astype(np.int64)
    for g in range(ng):
        vis = np.nonzero(visited[g])[0]
        fin = final[g, vis]
        acc = vis[(fin == 1) & (nb[vis] > FEW_BODIES)]
        src = vis[((fin == 1) & (nb[vis] <= FEW_BODIES)) | ((fin == 0) & leaf[vis])]
        cells_out.append(np.sort(acc))
        bodies_out.append(np.sort(np.concatenate(
            [np.arange(begin[j], begin[j] + nb[j]) for j in src]) if len(src) else
            np.zeros(0, np.int64)))
    return cells_out, bodies_out, margins
