"""CPU restatement of the learned BP warm-start network (test infrastructure).

Checks the library's training kernels (ug_mlp_*, driven by
upside2-md_gb300/warm_start.py): the same network, 64 -> 128 -> 128 -> 8 with
ReLU, with every bf16 rounding point of the GPU path reproduced (inputs,
weights, hidden activations and back-propagated gradients rounded to bf16;
products accumulated in FP32), and the soft-target softmax cross-entropy over
each row's first n_rot logits.  Only the tests import this module.
"""
import numpy as np


def bf16(x):
    """Round FP32 to the nearest bf16 (ties to even), returned as FP32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def forward(X, w):
    Xb = bf16(X)
    H1 = bf16(np.maximum(Xb @ bf16(w["W1"]) + w["b1"], 0))
    H2 = bf16(np.maximum(H1 @ bf16(w["W2"]) + w["b2"], 0))
    Z = H2 @ bf16(w["W3"]) + w["b3"]
    return Xb, H1, H2, Z


def loss_and_grads(X, T, nrot, w):
    Xb, H1, H2, Z = forward(X, w)
    M = X.shape[0]
    valid = nrot > 1
    scale = 1.0 / max(1, int(valid.sum()))
    dZ = np.zeros_like(Z)
    loss = 0.0
    for i in np.nonzero(valid)[0]:
        n = nrot[i]
        z = Z[i, :n].astype(np.float64)
        p = np.exp(z - z.max())
        p /= p.sum()
        dZ[i, :n] = (p - T[i, :n]) * scale
        logp = z - z.max() - np.log(np.exp(z - z.max()).sum())
        loss -= scale * float((T[i, :n] * logp)[T[i, :n] > 0].sum())
    g = {}
    dZb = bf16(dZ)
    g["W3"] = H2.T @ dZb
    g["b3"] = dZ.sum(0)
    dH = dZb @ bf16(w["W3"]).T
    dH[H2 <= 0] = 0
    dHb = bf16(dH)
    g["W2"] = H1.T @ dHb
    g["b2"] = dH.sum(0)
    dH1 = dHb @ bf16(w["W2"]).T
    dH1[H1 <= 0] = 0
    dH1b = bf16(dH1)
    g["W1"] = Xb.T @ dH1b
    g["b1"] = dH1.sum(0)
    del M
    return loss, g
