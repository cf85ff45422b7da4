"""FP64 numpy restatement of the schedule selector's MLP (forward, masked MSE loss, backward).

TEST INFRASTRUCTURE ONLY: the checker for the GPU forward / backward / Adam kernels of
sptrsv_gb300/csrc/mlp.cu.  The product package never imports this module.

The network and its flat parameter layout follow the library's definition: W1 (h1 x in,
row-major), b1, W2 (h2 x h1), b2, W3 (out x h2), b3; hidden layers ReLU; inputs standardised as
(x - mean) * scale; loss = sum mask (P - Y)^2 / sum mask.  There is no reference counterpart (the
reference has no learned part), so parity here is against the mathematics, in FP64.
"""
import numpy as np


def sizes(dims):
    i, h1, h2, o = dims
    return [("W1", (h1, i)), ("b1", (h1,)), ("W2", (h2, h1)), ("b2", (h2,)), ("W3", (o, h2)), ("b3", (o,))]


def unpack(p, dims):
    out, k = {}, 0
    for name, shp in sizes(dims):
        cnt = int(np.prod(shp))
        out[name] = np.asarray(p[k:k + cnt], dtype=np.float64).reshape(shp)
        k += cnt
    return out


def pack(d, dims):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in sizes(dims)])


def forward(p, dims, X, mean=None, scale=None):
    W = unpack(p, dims)
    Xn = np.asarray(X, dtype=np.float64)
    if mean is not None:
        Xn = (Xn - mean) * scale
    H1 = np.maximum(Xn @ W["W1"].T + W["b1"], 0.0)
    H2 = np.maximum(H1 @ W["W2"].T + W["b2"], 0.0)
    P = H2 @ W["W3"].T + W["b3"]
    return Xn, H1, H2, P


def loss_grad(p, dims, X, Y, M, mean=None, scale=None):
    """Masked MSE loss and its gradient with respect to the flat parameters."""
    W = unpack(p, dims)
    Xn, H1, H2, P = forward(p, dims, X, mean, scale)
    M = np.asarray(M, dtype=np.float64)
    cnt = max(float(np.count_nonzero(M)), 1.0)
    D = np.where(M != 0, P - np.asarray(Y, dtype=np.float64), 0.0)
    loss = float(np.sum(D * D) / cnt)
    dP = 2.0 * D / cnt
    g = {"W3": dP.T @ H2, "b3": dP.sum(0)}
    dH2 = (dP @ W["W3"]) * (H2 > 0)
    g["W2"] = dH2.T @ H1
    g["b2"] = dH2.sum(0)
    dH1 = (dH2 @ W["W2"]) * (H1 > 0)
    g["W1"] = dH1.T @ Xn
    g["b1"] = dH1.sum(0)
    return loss, pack(g, dims)


def adam_step(p, g, m1, m2, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One bias-corrected Adam update (t = 1-based step); returns (p, m1, m2)."""
    m1 = beta1 * m1 + (1 - beta1) * g
    m2 = beta2 * m2 + (1 - beta2) * g * g
    c1, c2 = 1 - beta1 ** t, 1 - beta2 ** t
    return p - lr * (m1 / c1) / (np.sqrt(m2 / c2) + eps), m1, m2
