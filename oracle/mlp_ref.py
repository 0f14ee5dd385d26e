"""FP64 CPU reference of the surrogate network -- TEST INFRASTRUCTURE ONLY.

Forward and backward of the 48 -> 128 -> 128 -> 48 SiLU MLP in numpy FP64,
with optional rounding to BF16 at the points where the device kernels round
(inputs, weights, hidden activations, output and hidden gradients), so the
device gradients can be checked element by element.  `finite_difference`
verifies this reference itself.
"""
import numpy as np

IN, HID, OUT = 48, 128, 48


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    o = 0
    out = []
    for shape in [(HID, IN), (HID,), (HID, HID), (HID,), (OUT, HID), (OUT,)]:
        n = int(np.prod(shape))
        out.append(np.asarray(p[o:o + n], np.float64).reshape(shape))
        o += n
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s + z * s * (1.0 - s)


def forward(p, x, round_bf16=True):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, np.float64))
    x = r(x)
    z1 = x @ r(w1).T + b1
    h1 = r(silu(z1))
    z2 = h1 @ r(w2).T + b2
    h2 = r(silu(z2))
    y = h2 @ r(w3).T + b3
    return dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, y=y)


def loss_and_grads(p, x, t, nvalid=38, round_bf16=True):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, np.float64))
    f = forward(p, x, round_bf16)
    B = x.shape[0]
    mask = np.zeros(OUT)
    mask[:nvalid] = 1
    d = (f["y"] - t) * mask
    loss = float((d * d).sum() / (B * nvalid))
    dy = r(2.0 * d / (B * nvalid))
    dz2 = r((dy @ r(w3)) * dsilu(f["z2"]))
    dz1 = r((dz2 @ r(w2)) * dsilu(f["z1"]))
    g = [dz1.T @ f["x"], dz1.sum(0), dz2.T @ f["h1"], dz2.sum(0), dy.T @ f["h2"], dy.sum(0)]
    return loss, np.concatenate([a.reshape(-1) for a in g])


def finite_difference(p, x, t, idx, eps=1e-6, nvalid=38):
    g = []
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        g.append((loss_and_grads(pp, x, t, nvalid, False)[0] - loss_and_grads(pm, x, t, nvalid, False)[0]) / (2 * eps))
    return np.array(g)
