"""CPU oracle of the learned proposal's network and loss (numpy, FP64).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the library's
tensor-core training kernels.  The product library never imports it.

The network is the one the library trains and runs: 8 inputs, two hidden
layers of 32 with ReLU, 2 outputs; weights FP32, row-major [in][out], packed
W1 b1 W2 b2 W3 b3 (1410 floats).  Per record (12 floats: 8 features, target
t0, label y1, mask m0, spare) the loss is

    reg * m0 * (out0 - t0)^2 + softplus(out1) - y1 * out1

and the batch loss is the mean.  With emulate_bf16=True the forward and
backward passes round what the kernels feed to the BF16 MMA (inputs,
weights, hidden activations and back-propagated gradients) to BF16, round to
nearest even, and accumulate in FP64; bias gradients use the unrounded
values, as the kernels do.  With emulate_bf16=False everything is FP64.
The proposal has no counterpart in the reference (its search is not
learned), so this oracle is pinned by finite differences instead.
"""
import numpy as np

N_IN, N_HID, N_OUT = 8, 32, 2
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_IN * N_HID
OFF_W2 = OFF_B1 + N_HID
OFF_B2 = OFF_W2 + N_HID * N_HID
OFF_W3 = OFF_B2 + N_HID
OFF_B3 = OFF_W3 + N_HID * N_OUT
N_WEIGHTS = OFF_B3 + N_OUT
REC = 12


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), as float64."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w):
    w = np.asarray(w, np.float64)
    return (w[OFF_W1:OFF_B1].reshape(N_IN, N_HID), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(N_HID, N_HID),
            w[OFF_B2:OFF_W3], w[OFF_W3:OFF_B3].reshape(N_HID, N_OUT), w[OFF_B3:N_WEIGHTS])


def forward_backward(w, rec, reg=1.0, emulate_bf16=True):
    """-> (mean loss, gradient of the mean loss wrt the 1410 weights, outputs)."""
    rec = np.asarray(rec, np.float32)
    n = len(rec)
    r = (lambda a: bf16(np.float32(a))) if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(w)
    W1b, W2b, W3b = r(W1), r(W2), r(W3)
    X = r(rec[:, :N_IN])
    t0 = rec[:, 8].astype(np.float64)
    y1 = rec[:, 9].astype(np.float64)
    m0 = (rec[:, 10] > 0).astype(np.float64)
    Z1 = X @ W1b + b1
    H1 = r(np.maximum(Z1, 0.0))
    Z2 = H1 @ W2b + b2
    H2 = r(np.maximum(Z2, 0.0))
    O = H2 @ W3b + b3
    o0, o1 = O[:, 0], O[:, 1]
    e = o0 - t0
    sp = np.maximum(o1, 0.0) + np.log1p(np.exp(-np.abs(o1)))
    loss = np.mean(reg * m0 * e * e + sp - y1 * o1)
    dO = np.stack([2.0 * reg * m0 * e / n, (1.0 / (1.0 + np.exp(-o1)) - y1) / n], axis=1)
    dOb = r(dO)
    gW3 = H2.T @ dOb
    gb3 = dO.sum(0)
    dZ2 = (dOb @ W3b.T) * (H2 > 0)
    gb2 = dZ2.sum(0)
    dZ2b = r(dZ2)
    gW2 = H1.T @ dZ2b
    dZ1 = (dZ2b @ W2b.T) * (H1 > 0)
    gb1 = dZ1.sum(0)
    dZ1b = r(dZ1)
    gW1 = X.T @ dZ1b
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g, O


def predict(w, feats):
    """FP64 outputs (n, 2) for features (n, 8)."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    H1 = np.maximum(np.asarray(feats, np.float64) @ W1 + b1, 0.0)
    H2 = np.maximum(H1 @ W2 + b2, 0.0)
    return H2 @ W3 + b3
