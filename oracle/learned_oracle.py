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
