"""CPU oracle of the learned-mixing network (test infrastructure only).

Checks the GPU's multilayer perceptron (libqtgpu ``qt_mlp_*``), which has no
counterpart in the reference: the reference's SCBA loop only mixes linearly
(src/gw_mod.f90:747-749).  Parity is pinned two ways:

* ``emulate=False``: plain float64 forward/backward; its analytic gradient is
  checked against central finite differences of the loss (tests).
* ``emulate=True``: the GPU's arithmetic -- every tensor-core operand rounded
  to BF16 (round to nearest even), FP32 pre-activations and biases -- so the
  GPU result is expected to agree up to FP32 accumulation order.

Network: n_in -> width (GELU) x depth -> n_out, loss = mean of (y - t)^2 over
all outputs.  Flat parameters: for each layer W_l (dout x din, row-major) then
b_l (dout), the layout of ``qt_mlp_get_params``.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

ADAM_B1, ADAM_B2, ADAM_EPS = 0.9, 0.999, 1e-8


def layout(n_in, width, depth, n_out):
    """[(din, dout, woff, boff)] per linear layer and the parameter count."""
    out, off = [], 0
    for layer in range(depth + 1):
        din = n_in if layer == 0 else width
        dout = n_out if layer == depth else width
        out.append((din, dout, off, off + din * dout))
        off += din * dout + dout
    return out, off


def glorot(n_in, width, depth, n_out, seed):
    rng = np.random.default_rng(seed)
    lay, n = layout(n_in, width, depth, n_out)
    p = np.zeros(n, dtype=np.float32)
    for din, dout, wo, _ in lay:
        a = np.sqrt(6.0 / (din + dout))
        p[wo:wo + din * dout] = rng.uniform(-a, a, din * dout)
    return p


def bf16(x):
    """Round float32 values to BF16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    r = np.where(nan, (u | 0x400000) & 0xFFFF0000, r)
    return r.astype(np.uint32).view(np.float32).reshape(np.shape(x))


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def _params(p, lay):
    return [(p[wo:wo + din * dout].reshape(dout, din), p[bo:bo + dout])
            for din, dout, wo, bo in lay]


def forward(p, X, dims, emulate=True):
    """Network output and the cache for ``backward``."""
    lay, _ = layout(*dims)
    f = (lambda a: bf16(a).astype(np.float64)) if emulate else (lambda a: np.asarray(a, np.float64))
    cast = (lambda a: a.astype(np.float32).astype(np.float64)) if emulate else (lambda a: a)
    h = f(X)
    ins, pres = [], []
    for layer, (W, b) in enumerate(_params(np.asarray(p), lay)):
        ins.append(h)
        z = cast(h @ f(W).T + np.asarray(b, np.float64))
        if layer < len(lay) - 1:
            pres.append(z)
            h = f(gelu(z))
        else:
            y = z
    return y, (ins, pres)


def loss_and_grad(p, X, T, dims, emulate=True):
    """Mean squared error and its gradient (flat, the parameter layout)."""
    lay, n = layout(*dims)
    y, (ins, pres) = forward(p, X, dims, emulate)
    f = (lambda a: bf16(a).astype(np.float64)) if emulate else (lambda a: np.asarray(a, np.float64))
    d = y - np.asarray(T, np.float64)
    loss = float(np.mean(d * d))
    dP = 2.0 * d / d.size
    if emulate:
        dP = dP.astype(np.float32).astype(np.float64)
    g = np.zeros(n)
    params = _params(np.asarray(p), lay)
    for layer in range(len(lay) - 1, -1, -1):
        din, dout, wo, bo = lay[layer]
        g[wo:wo + din * dout] = (f(dP).T @ ins[layer]).ravel()
        g[bo:bo + dout] = dP.sum(axis=0)
        if layer > 0:
            dact = f(dP) @ f(params[layer][0])
            dP = dact * gelu_grad(pres[layer - 1])
            if emulate:
                dP = dP.astype(np.float32).astype(np.float64)
    return loss, g


def adamw(p, g, m, v, step, lr, wd):
    """One AdamW step (decoupled weight decay on every parameter); returns (p, m, v)."""
    p, g, m, v = (np.asarray(a, np.float64) for a in (p, g, m, v))
    m = ADAM_B1 * m + (1 - ADAM_B1) * g
    v = ADAM_B2 * v + (1 - ADAM_B2) * g * g
    mh = m / (1 - ADAM_B1 ** step)
    vh = v / (1 - ADAM_B2 ** step)
    p = p * (1 - lr * wd) - lr * mh / (np.sqrt(vh) + ADAM_EPS)
    return p, m, v
