"""CPU restatement of the guiding network (numpy) — test infrastructure only.

Mirrors kazen_proto_gb300's guiding kernels: 51 input features (8-band
sin/cos encoding of the position in the scene box + normal, padded to 64),
three 64-wide ReLU layers, 40 outputs = 8 von Mises-Fisher lobes (anchor
point, concentration = 0.05 + softplus, weight = softmax). A lobe's mean
direction points from the shading point p01 to its anchor, both in scene-box
coordinates, measured in world units: normalize((anchor - p01) * ext), ext =
the box extent. `bf16=True` rounds to
bfloat16 (round to nearest even) exactly where the kernels store BF16:
inputs, weights, activations after ReLU, and the back-propagated
gradients; products accumulate in higher precision. The guiding network has
no counterpart in the reference (kazen_proto), so this restatement is
checked by finite differences (float64) in tests/.
"""
from __future__ import annotations

import numpy as np

N_PARAMS = 15080
OFF = {"W1": 0, "b1": 4096, "W2": 4160, "b2": 8256, "W3": 8320, "b3": 12416, "W4": 12480, "b4": 15040}
KAPPA_MIN, KAPPA_MAX = 0.05, 2000.0


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(x.shape)


def unpack(p):
    p = np.asarray(p)
    return {
        "W1": p[OFF["W1"]:OFF["b1"]].reshape(64, 64), "b1": p[OFF["b1"]:OFF["W2"]],
        "W2": p[OFF["W2"]:OFF["b2"]].reshape(64, 64), "b2": p[OFF["b2"]:OFF["W3"]],
        "W3": p[OFF["W3"]:OFF["b3"]].reshape(64, 64), "b3": p[OFF["b3"]:OFF["W4"]],
        "W4": p[OFF["W4"]:OFF["b4"]].reshape(40, 64), "b4": p[OFF["b4"]:N_PARAMS],
    }


def features(p01, n, dtype=np.float32):
    p01 = np.asarray(p01, dtype).reshape(-1, 3)
    n = np.asarray(n, dtype).reshape(-1, 3)
    X = np.zeros((len(p01), 64), dtype)
    for j in range(48):
        a, b = j >> 4, (j & 15) >> 1
        x = p01[:, a] * dtype(1 << b) * dtype(np.pi)
        X[:, j] = np.cos(x) if (j & 1) else np.sin(x)
    X[:, 48:51] = n
    return X


def softplus(x):
    return np.where(x > 20, x, np.log1p(np.exp(np.minimum(x, 20))))


def lobe_axes(raw, p01, ext=(1.0, 1.0, 1.0)):
    """(anchor - p01) * ext per lobe, (n, 8, 3)."""
    raw = np.asarray(raw, np.float64).reshape(-1, 8, 5)
    p01 = np.asarray(p01, np.float64).reshape(-1, 1, 3)
    return (raw[:, :, 0:3] - p01) * np.asarray(ext, np.float64).reshape(1, 1, 3)


def mixture(raw, p01, ext=(1.0, 1.0, 1.0)):
    raw = np.asarray(raw, np.float64).reshape(-1, 8, 5)
    m = lobe_axes(raw, p01, ext)
    ln = np.linalg.norm(m, axis=2, keepdims=True)
    mu = np.where(ln > 1e-12, m / np.maximum(ln, 1e-30), np.array([0, 0, 1.0]))
    kap = np.minimum(KAPPA_MIN + softplus(raw[:, :, 3]), KAPPA_MAX)
    z = raw[:, :, 4] - raw[:, :, 4].max(axis=1, keepdims=True)
    w = np.exp(z)
    w /= w.sum(axis=1, keepdims=True)
    return mu, kap, w


def vmf(mu, kap, d):
    lognorm = np.log(kap) - np.log(2 * np.pi) - np.log1p(-np.exp(-2 * kap))
    return np.exp(lognorm + kap * ((mu * d[:, None, :]).sum(2) - 1))


def pdf(raw, d, p01, ext=(1.0, 1.0, 1.0)):
    mu, kap, w = mixture(raw, p01, ext)
    return (w * vmf(mu, kap, np.asarray(d, np.float64))).sum(1)


def nll_and_grad(raw, d, scale, p01, ext=(1.0, 1.0, 1.0)):
    """-log q(d) per row and d(scale * -log q)/d(raw) (n, 40), float64."""
    raw = np.asarray(raw, np.float64).reshape(-1, 8, 5)
    d = np.asarray(d, np.float64)
    mu, kap, w = mixture(raw, p01, ext)
    v = vmf(mu, kap, d)
    q = np.maximum((w * v).sum(1), 1e-30)
    resp = w * v / q[:, None]
    cosd = (mu * d[:, None, :]).sum(2)
    e = np.exp(-2 * kap)
    dlogv = 1 / kap - 2 * e / (1 - e) + (cosd - 1)
    kraw = KAPPA_MIN + softplus(raw[:, :, 3])
    dk = np.where(kraw < KAPPA_MAX, 1 / (1 + np.exp(-raw[:, :, 3])), 0.0)
    s = np.asarray(scale, np.float64)[:, None]
    g = np.zeros_like(raw)
    g[:, :, 4] = s * (w - resp)
    g[:, :, 3] = s * (-resp * dlogv * dk)
    ln = np.linalg.norm(lobe_axes(raw, p01, ext), axis=2)
    proj = (d[:, None, :] - mu * cosd[:, :, None]) / np.maximum(ln, 1e-30)[:, :, None]
    proj = proj * np.asarray(ext, np.float64).reshape(1, 1, 3)  # d axis / d anchor = diag(ext)
    g[:, :, 0:3] = np.where((ln > 1e-12)[:, :, None], (-resp * kap * s)[:, :, None] * proj, 0.0)
    return -np.log(q), g.reshape(-1, 40)


def forward(params, p01, n, use_bf16=True):
    P = unpack(np.asarray(params, np.float32 if use_bf16 else np.float64))
    r = bf16 if use_bf16 else (lambda a: np.asarray(a, np.float64))
    X = r(features(p01, n, np.float32 if use_bf16 else np.float64))
    W = {k: r(P[k]) for k in ("W1", "W2", "W3", "W4")}
    c = {"X": X}
    A = X
    for l in (1, 2, 3):
        Z = (A.astype(np.float64) @ W[f"W{l}"].T.astype(np.float64)) + P[f"b{l}"]
        c[f"Z{l}"] = Z
        A = r(np.maximum(Z, 0).astype(np.float32 if use_bf16 else np.float64))
        c[f"H{l}"] = A
    c["O"] = (A.astype(np.float64) @ W["W4"].T.astype(np.float64)) + P["b4"]
    c["W"] = W
    return c


def loss_and_grad(params, p01, n, d, weights, wscale, use_bf16=True, ext=(1.0, 1.0, 1.0)):
    """Loss sum(w * wscale * -log q) and its gradient in the parameter layout."""
    r = bf16 if use_bf16 else (lambda a: np.asarray(a, np.float64))
    c = forward(params, p01, n, use_bf16)
    s = np.asarray(weights, np.float64) * wscale
    nll, dO = nll_and_grad(c["O"], d, s, p01, ext)
    loss = float((s * nll).sum())
    W = c["W"]
    ft = np.float32 if use_bf16 else np.float64
    dOb = r(dO.astype(ft)).astype(np.float64)
    dZ3 = r((dOb @ W["W4"].astype(np.float64) * (c["Z3"] > 0)).astype(ft)).astype(np.float64)
    dZ2 = r((dZ3 @ W["W3"].astype(np.float64) * (c["Z2"] > 0)).astype(ft)).astype(np.float64)
    dZ1 = r((dZ2 @ W["W2"].astype(np.float64) * (c["Z1"] > 0)).astype(ft)).astype(np.float64)
    g = np.zeros(N_PARAMS, np.float64)
    H = {0: c["X"], 1: c["H1"], 2: c["H2"], 3: c["H3"]}
    for l, dZ in ((1, dZ1), (2, dZ2), (3, dZ3), (4, dOb)):
        dW = dZ.T @ H[l - 1].astype(np.float64)
        g[OFF[f"W{l}"]:OFF[f"W{l}"] + dW.size] = dW.reshape(-1)
        g[OFF[f"b{l}"]:OFF[f"b{l}"] + dZ.shape[1]] = dZ.sum(0)
    g[OFF["W1"]:OFF["b1"]].reshape(64, 64)[:, 51:] = 0.0
    return loss, g


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, np.float32)
    for l, (rows, fan) in enumerate(((64, 51), (64, 64), (64, 64), (40, 64)), 1):
        bound = np.sqrt(6.0 / fan) if l < 4 else 0.5 * np.sqrt(3.0 / fan)
        W = np.zeros((rows, 64), np.float32)
        W[:, :fan] = rng.uniform(-bound, bound, (rows, fan))
        p[OFF[f"W{l}"]:OFF[f"W{l}"] + W.size] = W.reshape(-1)
        p[OFF[f"b{l}"]:OFF[f"b{l}"] + rows] = rng.uniform(-0.1, 0.1, rows)
    return p
