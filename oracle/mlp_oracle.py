"""CPU oracle of the emulator MLP ensemble (forward, mean-squared-error backward, AdamW).

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` use it, as the checker of the tensor-core kernels in
``holodeck_gb300/csrc/hgb_mlp.cu``; the ``holodeck_gb300`` product never imports it.

The network has no reference counterpart (the reference's emulators are Gaussian processes,
holodeck/gps/gp_utils.py), so the oracle restates the mathematics of the network directly, in numpy,
with the same rounding points as the kernels: weights and the activations between layers are rounded
to bfloat16 (round to nearest even), every product and sum is fp32, pre-activations and outputs stay
fp32, SiLU(z) = z / (1 + exp(-z)).  The loss is the mean of (out - target)^2 over the batch and
outputs; its gradient with respect to the outputs is rounded to bfloat16 before it is propagated, as
are the gradients with respect to each hidden layer's pre-activations.  Parameters are per-member
lists of (W [N][K], b [N]) in fp32.

The kernels sum in a different order (tensor-core fp32 accumulation), so agreement is to fp32
rounding, plus the occasional flip of a bfloat16 rounding that it causes; with small-integer inputs
and weights every sum is exact and the agreement is bit for bit.
"""

import numpy as np


def bf16(x):
    """Round fp32 values to the nearest bfloat16 (ties to even), returned as fp32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def bf16_bits(x):
    """bfloat16 bit patterns (uint16) of fp32 values, rounded to nearest even."""
    return (bf16(x).view(np.uint32) >> 16).astype(np.uint16)


def from_bf16_bits(b):
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def _sigmoid(z):
    with np.errstate(over="ignore"):   # exp(-z) overflows to inf for very negative z: sigmoid is 0 there
        return (1.0 / (1.0 + np.exp(-z.astype(np.float32)))).astype(np.float32)


def silu(z):
    return (z * _sigmoid(z)).astype(np.float32)


def silu_grad(z):
    s = _sigmoid(z)
    return (s * (1.0 + z * (1.0 - s))).astype(np.float32)


def forward(layers, x):
    """One member: x [B][K0] (bf16-valued) -> (acts, pres, out); acts[l] is the bf16 input of layer
    l + 1, pres[l] the fp32 pre-activation of hidden layer l."""
    acts, pres = [], []
    h = np.asarray(x, dtype=np.float32)
    for ll, (w, b) in enumerate(layers):
        z = (h @ bf16(w).T).astype(np.float32) + np.asarray(b, dtype=np.float32)
        if ll == len(layers) - 1:
            return acts, pres, z.astype(np.float32)
        pres.append(z.astype(np.float32))
        h = bf16(silu(z))
        acts.append(h)


def backward(layers, x, target):
    """Loss and fp32 gradients [(dW, db)] of one member for the batch (x, target)."""
    acts, pres, out = forward(layers, x)
    nb, nout = out.shape
    d = (out - np.asarray(target, dtype=np.float32)).astype(np.float32)
    loss = float(np.mean(d.astype(np.float64) ** 2))
    dz = bf16(np.float32(2.0 / (nb * nout)) * d)
    grads = [None] * len(layers)
    for ll in range(len(layers) - 1, -1, -1):
        inp = np.asarray(x, dtype=np.float32) if ll == 0 else acts[ll - 1]
        grads[ll] = ((dz.T @ inp).astype(np.float32), dz.sum(axis=0, dtype=np.float32))
        if ll == 0:
            break
        g = (dz @ bf16(layers[ll][0])).astype(np.float32)
        dz = bf16(g * silu_grad(pres[ll - 1]))
    return loss, grads


def adamw(p, g, m1, m2, step, lr, beta1, beta2, eps, wd, decay):
    """One decoupled AdamW step (in place on p, m1, m2); ``decay`` selects the decayed entries."""
    m1[...] = beta1 * m1 + (1.0 - beta1) * g
    m2[...] = beta2 * m2 + (1.0 - beta2) * g * g
    bc1 = 1.0 - beta1 ** step
    bc2 = 1.0 - beta2 ** step
    p[...] = np.where(decay, p - lr * wd * p, p)
    p[...] = p - lr * (m1 / bc1) / (np.sqrt(m2 / bc2) + eps)
    return p
