"""FP64 numpy restatement of the learned-guess MLP (forward, MSE loss,
backward) used to check the GPU kernels' gradients.  TEST INFRASTRUCTURE:
only the tests import it.

It rounds to BF16 at the same places as the GPU kernels (GEMM inputs:
network input, hidden activations, weights, loss gradient and back-propagated
pre-activation gradients) and keeps pre-activations in FP32, so the remaining
difference is the accumulation order (FP32 tensor-core sums vs FP64 here)."""
import numpy as np


def bf16(x):
    """Round-to-nearest-even FP32 -> BF16, returned as FP32 values."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(params, nin, width, depth, nout):
    dims = [nin] + [width] * depth + [nout]
    out, off = [], 0
    for l in range(depth + 1):
        di, do = dims[l], dims[l + 1]
        W = params[off:off + di * do].reshape(do, di); off += di * do
        b = params[off:off + do]; off += do
        out.append((W, b))
    return out


def silu(z):
    return z / (1 + np.exp(-z))


def loss_and_grads(params, x, t, nin, width, depth, nout):
    layers = unpack(np.asarray(params, np.float32), nin, width, depth, nout)
    a = [bf16(x).astype(np.float64)]
    zs = []
    for l, (W, b) in enumerate(layers):
        z = a[-1] @ bf16(W).astype(np.float64).T + b.astype(np.float64)
        if l < depth:
            z32 = z.astype(np.float32)
            zs.append(z32)
            a.append(bf16(silu(z32.astype(np.float64)).astype(np.float32)).astype(np.float64))
        else:
            y = z.astype(np.float32)
    ny = y.size
    d = y.astype(np.float64) - t
    loss = float((d * d).sum() / ny)
    dz = bf16((2 * d / ny).astype(np.float32)).astype(np.float64)
    grads = [None] * (depth + 1)
    for l in range(depth, -1, -1):
        W, _ = layers[l]
        dW = dz.T @ a[l]
        db = dz.sum(axis=0)
        grads[l] = (dW, db)
        if l == 0:
            break
        da = dz @ bf16(W).astype(np.float64)
        z = zs[l - 1].astype(np.float64)
        s = 1 / (1 + np.exp(-z))
        dz = bf16((da * s * (1 + z * (1 - s))).astype(np.float32)).astype(np.float64)
    flat = np.concatenate([np.concatenate([g[0].ravel(), g[1].ravel()]) for g in grads])
    return loss, flat
