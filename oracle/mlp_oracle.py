"""CPU restatement of the learned-guess network (test infrastructure only).

The device kernels (mdoodz6.0_gb300/csrc/mlp.cu) run an 8 -> 64 -> 64 -> 2
ReLU network with BF16 operands and FP32 accumulation.  This module computes
the same forward pass and the gradient of the mean squared error in FP64,
optionally rounding exactly the operands the device rounds to BF16 (inputs,
weights, hidden activations, output and hidden deltas), so the device
gradients can be checked against it; with bf16=False it is the plain FP64
network, whose gradient is checked against finite differences.

Parameter layout (flat): W1[64][8], b1[64], W2[64][64], b2[64], W3[2][64], b3[2].
The network has no counterpart in the reference (which starts every local
Newton solve from the smallest creep viscosity, SOURCE/RheologyDensity.c:44-707).
"""
import numpy as np

NPARAM = 4866
SLICES = {"W1": (0, (64, 8)), "b1": (512, (64,)), "W2": (576, (64, 64)), "b2": (4672, (64,)),
          "W3": (4736, (2, 64)), "b3": (4864, (2,))}


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in SLICES.items()}


def pack(d):
    p = np.zeros(NPARAM)
    for k, (o, s) in SLICES.items():
        p[o:o + int(np.prod(s))] = np.asarray(d[k]).ravel()
    return p


def _r(x, on):
    return bf16(x) if on else np.asarray(x, np.float64)


def forward(p, x, bf=True):
    w = unpack(p)
    X = _r(x, bf)
    h1 = _r(np.maximum(X @ _r(w["W1"], bf).T + w["b1"], 0.0), bf)
    h2 = _r(np.maximum(h1 @ _r(w["W2"], bf).T + w["b2"], 0.0), bf)
    y = h2 @ _r(w["W3"], bf).T + w["b3"]
    return X, h1, h2, y


def loss_and_gradients(p, x, lab, bf=True):
    """Mean over rows of sum_o (y_o - label_o)^2 and its gradient (flat)."""
    w = unpack(p)
    n = len(x)
    X, h1, h2, y = forward(p, x, bf)
    e = y - lab
    loss = float(np.sum(e * e) / n)
    dy = 2.0 * e / n
    dyb = _r(dy, bf)
    dh2 = (dyb @ _r(w["W3"], bf)) * (h2 > 0)
    dh2b = _r(dh2, bf)
    dh1 = (dh2b @ _r(w["W2"], bf)) * (h1 > 0)
    dh1b = _r(dh1, bf)
    g = {"W3": dyb.T @ h2, "b3": dy.sum(0), "W2": dh2b.T @ h1, "b2": dh2.sum(0),
         "W1": dh1b.T @ X, "b1": dh1.sum(0)}
    return loss, pack(g)
