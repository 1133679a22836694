"""TEST INFRASTRUCTURE: NumPy oracle of the surrogate MLP (7 -> 4 x 128 SiLU -> 1).

Restates, on the CPU, the forward pass and the gradient of the weighted MSE that
the tensor-core kernels compute (thoth_gb300/csrc/surrogate.cu), rounding to
bf16 at the same places: the bf16 weight copies W1..W4, the bf16 activations fed
to the next layer, the bf16 loss gradients dz. Each input feature enters as a
bf16 pair (hi, lo) in columns f and f + 7 of the first layer, whose two columns
hold one tied weight. Accumulation is FP64 here, FP32 on
the device, so agreement is to bf16/FP32 rounding, not bit-exact.
"""
import numpy as np

H, KIN, NF = 128, 16, 7
OFF_W1 = 0
OFF_B1 = H * KIN
OFF_W2 = OFF_B1 + H
LAYER = H * H + H
OFF_W5 = OFF_W2 + 3 * LAYER
OFF_B5 = OFF_W5 + H
N_PARAMS = OFF_B5 + 1


def bf16(x):
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def unpack(p):
    W = {1: p[OFF_W1:OFF_B1].reshape(H, KIN)}
    b = {1: p[OFF_B1:OFF_W2]}
    for l in range(2, 5):
        o = OFF_W2 + (l - 2) * LAYER
        W[l] = p[o:o + H * H].reshape(H, H)
        b[l] = p[o + H * H:o + LAYER]
    return W, b, p[OFF_W5:OFF_B5], p[OFF_B5]


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x):
    W, b, w5, b5 = unpack(np.asarray(p, dtype=np.float64))
    a = np.zeros((len(x), KIN))
    hi = bf16(x)
    a[:, :NF] = hi
    a[:, NF:2 * NF] = bf16(np.asarray(x, dtype=np.float32) - hi.astype(np.float32))
    a = bf16(a)
    zs, acts = {}, {0: a}
    for l in range(1, 5):
        z = acts[l - 1] @ bf16(W[l]).T + b[l]
        zs[l] = z
        acts[l] = bf16(silu(z))
    yhat = silu(zs[4]) @ w5 + b5
    return yhat, zs, acts


def gradient(p, x, y, scale):
    p = np.asarray(p, dtype=np.float64)
    W, b, w5, b5 = unpack(p)
    n = len(x)
    yhat, zs, acts = forward(p, x)
    w = 1.0 / np.asarray(scale, dtype=np.float64) ** 2
    e = yhat - y
    loss = np.sum(w * e * e) / n
    dy = 2.0 * e * w / n
    g = np.zeros(N_PARAMS)
    g[OFF_W5:OFF_B5] = dy @ silu(zs[4])
    g[OFF_B5] = dy.sum()
    dz = bf16(dy[:, None] * w5[None, :] * dsilu(zs[4]))
    for l in range(4, 0, -1):
        gw = dz.T @ acts[l - 1]
        if l == 1:
            g[OFF_W1:OFF_B1] = gw.ravel()
            g[OFF_B1:OFF_W2] = dz.sum(0)
        else:
            o = OFF_W2 + (l - 2) * LAYER
            g[o:o + H * H] = gw.ravel()
            g[o + H * H:o + LAYER] = dz.sum(0)
            dz = bf16((dz @ bf16(W[l])) * dsilu(zs[l - 1]))
    g[OFF_W1:OFF_B1].reshape(H, KIN)[:, 2 * NF:] = 0.0
    return g, loss
