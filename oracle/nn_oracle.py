"""CPU oracle for the warm-start MLP (TEST INFRASTRUCTURE ONLY).

Float64 forward/backward of the network the library trains (hidden tanh
layers, linear output, mean-squared-error loss), with the same BF16 rounding
of every GEMM operand that the GPU kernels apply, so that the GPU gradients
(FP32 accumulation) can be checked against it.  There is no reference
counterpart: the learned warm start is new in this project.
"""
import numpy as np


def bf16(a):
    """Round to bfloat16 (round-to-nearest-even) and return float64."""
    a32 = np.asarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, widths):
    Ws, bs, off = [], [], 0
    for l in range(len(widths) - 1):
        n_in, n_out = widths[l], widths[l + 1]
        Ws.append(np.asarray(params[off:off + n_in * n_out], dtype=np.float64).reshape(n_out, n_in))
        off += n_in * n_out
        bs.append(np.asarray(params[off:off + n_out], dtype=np.float64))
        off += n_out
    return Ws, bs


def forward(params, widths, x):
    Ws, bs = unpack(params, widths)
    acts = [np.asarray(x, dtype=np.float64)]
    L = len(Ws)
    for l in range(L):
        z = bf16(acts[-1]) @ bf16(Ws[l]).T + bs[l]
        acts.append(np.tanh(z) if l < L - 1 else z)
    return acts


def loss_and_grad(params, widths, x, t):
    Ws, bs = unpack(params, widths)
    acts = forward(params, widths, x)
    y = acts[-1]
    n = y.size
    loss = float(np.mean((y - t) ** 2))
    dz = 2.0 * (y - t) / n
    L = len(Ws)
    grads = []
    for l in range(L - 1, -1, -1):
        if l < L - 1:
            dz = dz * (1.0 - acts[l + 1] ** 2)
        dW = bf16(dz).T @ bf16(acts[l])
        db = dz.sum(0)
        grads.append((dW, db))
        if l > 0:
            dz = bf16(dz) @ bf16(Ws[l])
    flat = []
    for (dW, db) in reversed(grads):
        flat.append(dW.ravel())
        flat.append(db)
    return loss, np.concatenate(flat)
