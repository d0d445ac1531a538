"""CPU oracle of the warm-start MLP — TEST INFRASTRUCTURE ONLY.

float64 numpy restatement of the network the library trains
(12 -> 128 -> 128 -> 64, exact-erf GELU, mean-squared loss over all
outputs): forward pass and an independent hand-written backward pass.  The
weights are rounded to BF16 first, as the device GEMMs read BF16 weights
(the gradient is taken with respect to those rounded values).
"""
import math

import numpy as np

SIZES = [("W1", (128, 12)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)),
         ("W3", (64, 128)), ("b3", (64,))]
COUNT = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(params):
    out, off = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(params[off:off + n], np.float64).reshape(shape)
        off += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SIZES])


def bf16_round(x):
    """Round float32 values to the nearest BF16 (ties to even), as float64."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    cdf = 0.5 * (1.0 + _erf(z / math.sqrt(2.0)))
    pdf = np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)
    return cdf + z * pdf


def effective(params):
    """Parameters as the device uses them: BF16 weights, FP32 biases."""
    p = unpack(params)
    for w in ("W1", "W2", "W3"):
        p[w] = bf16_round(p[w])
    return p


def forward(params, x):
    p = effective(params)
    x = np.asarray(x, np.float64)
    z1 = x @ p["W1"].T + p["b1"]
    a1 = gelu(z1)
    z2 = a1 @ p["W2"].T + p["b2"]
    a2 = gelu(z2)
    y = a2 @ p["W3"].T + p["b3"]
    return y, (x, z1, a1, z2, a2)


def loss_and_grad(params, x, t):
    p = effective(params)
    y, (x, z1, a1, z2, a2) = forward(params, x)
    t = np.asarray(t, np.float64)
    cnt = y.size
    d = y - t
    loss = float((d * d).sum() / cnt)
    dy = 2.0 * d / cnt
    g = {"W3": dy.T @ a2, "b3": dy.sum(0)}
    dz2 = (dy @ p["W3"]) * gelu_grad(z2)
    g["W2"] = dz2.T @ a1
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ p["W2"]) * gelu_grad(z1)
    g["W1"] = dz1.T @ x
    g["b1"] = dz1.sum(0)
    return loss, pack(g)


def loss_only(eff, x, t):
    """Loss for already-effective (float64) parameters, for finite differences."""
    z1 = x @ eff["W1"].T + eff["b1"]
    a1 = gelu(z1)
    z2 = a1 @ eff["W2"].T + eff["b2"]
    a2 = gelu(z2)
    y = a2 @ eff["W3"].T + eff["b3"]
    return float(((y - t) ** 2).sum() / y.size)


def forward_bf16_activations(params, x):
    """The forward pass as the tensor-core inference rounds it: inputs and
    hidden activations (after GELU) rounded to BF16, everything else
    float64.  Returns the (n, 64) outputs."""
    p = unpack(params)
    w = {k: bf16_round(p[k]) if k.startswith("W") else p[k] for k in p}
    a = bf16_round(np.asarray(x, np.float32))
    a = bf16_round(gelu(a @ w["W1"].T + w["b1"]).astype(np.float32))
    a = bf16_round(gelu(a @ w["W2"].T + w["b2"]).astype(np.float32))
    return a @ w["W3"].T + w["b3"]
