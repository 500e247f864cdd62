"""Float64 CPU restatement of the subtree-surrogate GRU (forward and backward).

TEST INFRASTRUCTURE ONLY: the checker for the GPU training kernels and for the
port phase of the step kernel; never imported by the product.

The GRU has no counterpart in the reference: it is the learned part this build
adds in front of the reference's staggered step.  Its equations are the usual
GRU cell (hidden H = 64, inputs X = 4)::

    r  = sigmoid(Wx_r x + bx_r + Wh_r h~ + bh_r)
    z  = sigmoid(Wx_z x + bx_z + Wh_z h~ + bh_z)
    hn = Wh_n h~ + bh_n
    n  = tanh(Wx_n x + bx_n + r * hn)
    h' = (1 - z) n + z h
    y  = wo . h' + bo

With ``quantize=True`` the oracle rounds at the same points as the kernels:
``Wh`` and ``h~ = h`` are BF16 operands of the recurrent product; the inputs
and biases enter the same tensor-core product as an extra K block, so ``Wx`` is
BF16, ``x`` counts as ``bf16(x) + bf16(x - bf16(x))`` and every bias (the r
and z blocks use ``bx + bh`` summed in float32) as the sum of its two BF16
halves; the backward products use the BF16-rounded gate gradients ``dG`` and
``h~`` (the input and bias gradients are taken at full precision, as the
kernels do).  With
``quantize=False`` everything is float64 and the gradient is exact, which the
CPU tests check against finite differences.  Loss: mean over (sequence, step)
of ``(y - y_target)^2``; truncated BPTT within one window.
"""

from __future__ import annotations

import numpy as np

__all__ = ["H", "X", "NPARAM", "bf16", "unpack", "init_params", "step", "forward", "backward", "loss_and_grad"]

H = 64
X = 4
G3 = 3 * H
OFF_WH = 0
OFF_WX = OFF_WH + G3 * H
OFF_BX = OFF_WX + G3 * X
OFF_BH = OFF_BX + G3
OFF_WO = OFF_BH + G3
OFF_BO = OFF_WO + H
NPARAM = OFF_BO + 1


def bf16(a) -> np.ndarray:
    """Round to BF16 (round to nearest even, through float32), returned as float64."""
    f = np.ascontiguousarray(np.asarray(a, dtype=np.float64).astype(np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def unpack(theta: np.ndarray) -> dict:
    t = np.asarray(theta, dtype=np.float64)
    return {
        "Wh": t[OFF_WH:OFF_WX].reshape(G3, H),
        "Wx": t[OFF_WX:OFF_BX].reshape(G3, X),
        "bx": t[OFF_BX:OFF_BH],
        "bh": t[OFF_BH:OFF_WO],
        "wo": t[OFF_WO:OFF_BO],
        "bo": float(t[OFF_BO]),
    }


def init_params(seed: int = 0, scale: float = 1.0) -> np.ndarray:
    """Uniform(-1/sqrt(H), 1/sqrt(H)) initialisation (the common GRU default)."""
    rng = np.random.default_rng(seed)
    k = scale / np.sqrt(H)
    theta = rng.uniform(-k, k, size=NPARAM)
    theta[OFF_BO] = 0.0
    return theta.astype(np.float32).astype(np.float64)


def _sig(x):
    return 1.0 / (1.0 + np.exp(-x))


def _split(a) -> np.ndarray:
    """A float32 value as the sum of two BF16 halves (as the kernels feed it)."""
    f = np.asarray(a, dtype=np.float64).astype(np.float32).astype(np.float64)
    hi = bf16(f)
    return hi + bf16(f - hi)


def _preact(p: dict, h, x, quantize: bool):
    """Pre-activations (r, z, hn, nx) of a batch: h [B, H], x [B, X]."""
    if quantize:
        Wh, Wx, xe = bf16(p["Wh"]), bf16(p["Wx"]), _split(x)
        b_rz = _split(p["bx"][:2 * H].astype(np.float32) + p["bh"][:2 * H].astype(np.float32))
        b_hn, b_nx = _split(p["bh"][2 * H:]), _split(p["bx"][2 * H:])
        hq = bf16(h)
    else:
        Wh, Wx, xe, hq = p["Wh"], p["Wx"], x, h
        b_rz = p["bx"][:2 * H] + p["bh"][:2 * H]
        b_hn, b_nx = p["bh"][2 * H:], p["bx"][2 * H:]
    a = hq @ Wh.T
    xi = xe @ Wx.T
    rz = a[:, :2 * H] + xi[:, :2 * H] + b_rz
    return rz[:, :H], rz[:, H:], a[:, 2 * H:] + b_hn, xi[:, 2 * H:] + b_nx


def step(theta, x, h, quantize: bool = True):
    """One GRU step for a batch: x [B, X], h [B, H] -> (h' [B, H], y [B])."""
    p = unpack(theta)
    pr, pz, hn, nx = _preact(p, h, x, quantize)
    r, z = _sig(pr), _sig(pz)
    n = np.tanh(nx + r * hn)
    h_new = (1.0 - z) * n + z * h
    return h_new, h_new @ p["wo"] + p["bo"]


def forward(theta, x, h0, quantize: bool = True):
    """x: [B, T, X], h0: [B, H] -> (y [B, T], h_T [B, H], cache)."""
    p = unpack(theta)
    B, T, _ = x.shape
    h = np.array(h0, dtype=np.float64)
    ys = np.zeros((B, T))
    cache = {"h": np.zeros((B, T, H)), "r": np.zeros((B, T, H)), "z": np.zeros((B, T, H)),
             "n": np.zeros((B, T, H)), "hn": np.zeros((B, T, H))}
    for t in range(T):
        pr, pz, hn, nx = _preact(p, h, x[:, t, :], quantize)
        r, z = _sig(pr), _sig(pz)
        n = np.tanh(nx + r * hn)
        cache["h"][:, t] = h
        cache["r"][:, t], cache["z"][:, t], cache["n"][:, t], cache["hn"][:, t] = r, z, n, hn
        h = (1.0 - z) * n + z * h
        ys[:, t] = h @ p["wo"] + p["bo"]
    return ys, h, cache


def backward(theta, x, y_target, ys, cache, quantize: bool = True) -> np.ndarray:
    """Gradient of mean((y - y_target)^2) over one window (flat, the layout of theta)."""
    p = unpack(theta)
    WhT = (bf16(p["Wh"]) if quantize else p["Wh"]).T   # [H, 3H]
    B, T, _ = x.shape
    g = np.zeros(NPARAM)
    gWh = g[OFF_WH:OFF_WX].reshape(G3, H)
    gWx = g[OFF_WX:OFF_BX].reshape(G3, X)
    dys = 2.0 * (ys - y_target) / (B * T)
    carry = np.zeros((B, H))
    for t in range(T - 1, -1, -1):
        h_old, r, z, n, hn = (cache[k][:, t] for k in ("h", "r", "z", "n", "hn"))
        dy = dys[:, t][:, None]
        h_new = (1.0 - z) * n + z * h_old
        dh = carry + dy * p["wo"][None, :]
        dn = dh * (1.0 - z)
        dz = dh * (h_old - n)
        dh_dir = dh * z
        dan = dn * (1.0 - n * n)
        dar = dan * hn * r * (1.0 - r)
        daz = dz * z * (1.0 - z)
        dhn = dan * r
        dGx = np.concatenate([dar, daz, dan], axis=1)
        dGh = np.concatenate([dar, daz, dhn], axis=1)
        gWx += dGx.T @ x[:, t, :]
        g[OFF_BX:OFF_BH] += dGx.sum(0)
        g[OFF_BH:OFF_WO] += dGh.sum(0)
        g[OFF_WO:OFF_BO] += (dy * h_new).sum(0)
        g[OFF_BO] += dy.sum()
        dGq = bf16(dGh) if quantize else dGh
        hq = bf16(h_old) if quantize else h_old
        gWh += dGq.T @ hq
        carry = dh_dir + dGq @ WhT.T
    return g


def loss_and_grad(theta, x, y_target, h0, quantize: bool = False):
    ys, _, cache = forward(theta, x, h0, quantize)
    loss = float(np.mean((ys - y_target) ** 2))
    return loss, backward(theta, x, y_target, ys, cache, quantize)
