"""FP64 restatement of the warm-start MLP of the engine (k_mlp.cu), the
checker for its forward pass, gradients, minibatch draws and Adam steps.

Layout of the flat parameter array: per layer the [out][in] matrix, then the
bias: 4 -> 128 -> 128 -> 128 -> 1, SiLU after the three hidden layers; loss
= mean squared error."""
import numpy as np

SIZES = [(128, 4), (128, 128), (128, 128), (1, 128)]


def unpack(p):
    p = np.asarray(p, np.float64)
    out, off = [], 0
    for o, i in SIZES:
        W = p[off:off + o * i].reshape(o, i)
        off += o * i
        b = p[off:off + o]
        off += o
        out.append((W, b))
    assert off == p.size
    return out


def pack(layers):
    return np.concatenate([np.concatenate([W.reshape(-1), b]) for W, b in layers])


def sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sig(z)


def dsilu(z):
    s = sig(z)
    return s * (1.0 + z * (1.0 - s))


def forward(p, x):
    layers = unpack(p)
    h = np.asarray(x, np.float64)
    zs, hs = [], [h]
    for l, (W, b) in enumerate(layers):
        z = h @ W.T + b
        if l < 3:
            zs.append(z)
            h = silu(z)
            hs.append(h)
        else:
            return z[:, 0], zs, hs


def loss_and_grad(p, x, t):
    """Mean squared error over the points and its gradient (flat)."""
    y, zs, hs = forward(p, x)
    t = np.asarray(t, np.float64)
    B = y.size
    e = y - t
    loss = float(np.mean(e * e))
    layers = unpack(p)
    d = (2.0 * e / B)[:, None]                      # dL/dy
    grads = [None] * 4
    grads[3] = (d.T @ hs[3], d.sum(0))
    dh = d @ layers[3][0]                           # dL/dh3
    for l in (2, 1, 0):
        dz = dh * dsilu(zs[l])
        grads[l] = (dz.T @ hs[l], dz.sum(0))
        dh = dz @ layers[l][0]
    return loss, pack(grads)


def adam_step(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """Adam (Kingma & Ba 2015, Algorithm 1), step number t >= 1."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def minibatch(orc, n, B, step, seed):
    """Indices of the engine's minibatch of step `step`: Philox4x32-10 with key
    {seed, 0x4d4c5000} at counter {k, step, 0x57A27, 0}, index = (r0 * n) >> 32."""
    idx = np.zeros(B, np.int64)
    for k in range(B):
        r = orc.philox([k, step, 0x57A27, 0], [seed, 0x4D4C5000], 10)
        idx[k] = (int(r[0]) * n) >> 32
    return idx
