"""CPU oracle of the warm-start MLP (test infrastructure only).

FP64 numpy restatement of the network the engine trains
(pyqcm_gb300/csrc/qcmg_mlp.cu): hidden layers tanh(a W^T + b), a linear last
layer, mean squared error, the weights rounded to BF16 (round to nearest
even) in every product and the FP32 master parameters laid out W_0, b_0,
W_1, b_1, ...  Used by the tests as the checker of the device's forward
pass and gradients; never by the engine.  No counterpart in the reference.
"""
import numpy as np


def bf16(a):
    """Rounds float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(widths, p):
    """[(W_l, b_l)] views of the flat parameter vector."""
    out, off = [], 0
    for a, b in zip(widths[:-1], widths[1:]):
        W = p[off:off + a * b].reshape(b, a)
        off += a * b
        bb = p[off:off + b]
        off += b
        out.append((W, bb))
    assert off == len(p)
    return out


def _w(W, rounding):
    return (bf16(W) if rounding else np.asarray(W)).astype(np.float64)


def forward(widths, p, x, rounding=True):
    """(activations a_0..a_L) in FP64; rounding=True uses BF16-rounded weights
    as the engine does (False: the parameters as given, FP64)."""
    acts = [np.asarray(x, np.float64)]
    layers = unpack(widths, np.asarray(p, np.float32 if rounding else np.float64))
    for l, (W, b) in enumerate(layers):
        z = acts[-1] @ _w(W, rounding).T + b.astype(np.float64)
        acts.append(np.tanh(z) if l + 1 < len(layers) else z)
    return acts


def loss_grad(widths, p, x, t, rounding=True):
    """Mean squared error and its gradient with respect to the flat
    parameters (through the BF16-rounded weights when rounding)."""
    layers = unpack(widths, np.asarray(p, np.float32 if rounding else np.float64))
    acts = forward(widths, p, x, rounding)
    y = acts[-1]
    t = np.asarray(t, np.float64)
    n = y.size
    loss = float(np.sum((y - t) ** 2) / n)
    d = 2.0 * (y - t) / n
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        if l + 1 < len(layers):
            d = d * (1.0 - acts[l + 1] ** 2)
        gW = d.T @ acts[l]
        gb = d.sum(axis=0)
        grads.append((gW, gb))
        if l > 0:
            d = d @ _w(layers[l][0], rounding)
    g = []
    for gW, gb in reversed(grads):
        g.append(gW.ravel())
        g.append(gb)
    return loss, np.concatenate(g)
