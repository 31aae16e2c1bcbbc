"""CPU restatement of the warm-start network (TEST INFRASTRUCTURE ONLY).

The network of pffrgsolver.jl_gb300/csrc/pffrg_mlp.cu in numpy, FP64: dense
layers y = tanh(x W + b) with a linear last layer, parameters stored layer by
layer as W[n_in][n_out] then b[n_out], loss = mean((y - t)^2) over all
outputs of the batch.  Only tests use it, as the checker of the GPU kernels.
"""
import numpy as np


def unpack(params, sizes):
    out, o = [], 0
    for nin, nout in zip(sizes[:-1], sizes[1:]):
        W = params[o:o + nin * nout].reshape(nin, nout)
        o += nin * nout
        b = params[o:o + nout]
        o += nout
        out.append((W, b))
    return out


def forward(params, sizes, X):
    layers = unpack(np.asarray(params, dtype=np.float64), sizes)
    acts = [np.asarray(X, dtype=np.float64)]
    for l, (W, b) in enumerate(layers):
        z = acts[-1] @ W + b
        acts.append(np.tanh(z) if l + 1 < len(layers) else z)
    return acts


def loss_and_grad(params, sizes, X, T):
    layers = unpack(np.asarray(params, dtype=np.float64), sizes)
    acts = forward(params, sizes, X)
    Y = acts[-1]
    n = Y.size
    loss = float(np.mean((Y - T) ** 2))
    d = 2.0 * (Y - T) / n
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        W, b = layers[l]
        if l + 1 < len(layers):
            d = d * (1.0 - acts[l + 1] ** 2)
        grads.append((acts[l].T @ d, d.sum(axis=0)))
        d = d @ W.T
    flat = []
    for gW, gb in reversed(grads):
        flat.append(gW.ravel())
        flat.append(gb)
    return loss, np.concatenate(flat)
