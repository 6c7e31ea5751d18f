"""CPU restatement of the learned radiance cache's network: encoding, forward pass, relative L2
loss and its gradient, Adam.

ORACLE — test infrastructure, used only by tests/ to check the CUDA kernels
(trenchanttracer_gb300/csrc/tt_nrc.cu). The reference has no learned component, so this is
the project's own statement of the math, in FP64, with the same BF16 rounding points as the
device code (weights, the encoding, every stored activation and pre-activation gradient):

  H_0 = bf16(encode(record));  Z_l = W_l H_l;  H_{l+1} = bf16(relu(Z_l)), l < 5;  Y = W_5 H_5
  p = exp(min(Y, 20));  loss = mean_rows sum_c (p - t)^2 / (p^2 + 0.01)   (denominator not
  differentiated);  dY = bf16(2 (p - t) / (p^2 + 0.01) p / rows);  dZ_4 = bf16(dY W_5 * [H_5 > 0]);
  dZ_{l-1} = bf16(dZ_l W_l * [H_l > 0]);  dW_l = dZ_l^T H_l.
"""
from __future__ import annotations

import numpy as np

IN, HIDDEN, LAYERS, OUT, OUT_PAD = 160, 64, 6, 3, 8
POS_FREQ, DIR_FREQ = 12, 6


def layer_in(l: int) -> int:
    return IN if l == 0 else HIDDEN


def layer_out(l: int) -> int:
    return OUT_PAD if l == LAYERS - 1 else HIDDEN


def offsets() -> list[int]:
    off = [0]
    for l in range(LAYERS):
        off.append(off[-1] + layer_in(l) * layer_out(l))
    return off


NUM_PARAMS = offsets()[-1]


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    return np.where(np.isnan(f), np.nan, out)


def unpack(w: np.ndarray) -> list[np.ndarray]:
    """Compact weight vector -> [W_l (out, in)]."""
    off = offsets()
    return [np.asarray(w[off[l]:off[l + 1]], np.float64).reshape(layer_out(l), layer_in(l)) for l in range(LAYERS)]


def pack(ws: list[np.ndarray]) -> np.ndarray:
    return np.concatenate([np.asarray(x, np.float64).ravel() for x in ws])


def encode(rec: np.ndarray, lo, hi) -> np.ndarray:
    """(n, 16) records -> (n, 160) encoding (layout in tt_nrc.cuh). The arguments of the sines are
    formed in FP32 as the device forms them (p_hat = (p - lo) * float(1 / (hi - lo)), x = (d + 1) /
    2, then exact doublings); sin(pi x) and cos(pi x) are evaluated in FP64."""
    rec32 = np.asarray(rec, np.float32)
    rec = rec32.astype(np.float64)
    n = rec.shape[0]
    lo32, hi32 = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    ext = hi32 - lo32
    inv = np.where(ext > 0, np.float32(1.0) / np.where(ext > 0, ext, np.float32(1.0)), np.float32(1.0))
    ph32 = ((rec32[:, 0:3] - lo32) * inv).astype(np.float32)
    ph = ph32.astype(np.float64)
    xd = ((rec32[:, 3:6] + np.float32(1.0)) * np.float32(0.5)).astype(np.float64)
    xn = ((rec32[:, 6:9] + np.float32(1.0)) * np.float32(0.5)).astype(np.float64)
    e = np.zeros((n, IN))
    for i in range(3):
        for k in range(POS_FREQ):
            a = np.pi * (ph[:, i] * 2.0 ** k)
            e[:, 24 * i + 2 * k], e[:, 24 * i + 2 * k + 1] = np.sin(a), np.cos(a)
        for k in range(DIR_FREQ):
            ad = np.pi * (xd[:, i] * 2.0 ** k)
            an = np.pi * (xn[:, i] * 2.0 ** k)
            e[:, 72 + 12 * i + 2 * k], e[:, 72 + 12 * i + 2 * k + 1] = np.sin(ad), np.cos(ad)
            e[:, 108 + 12 * i + 2 * k], e[:, 108 + 12 * i + 2 * k + 1] = np.sin(an), np.cos(an)
    e[:, 144] = rec[:, 9]
    e[:, 145:148] = rec[:, 10:13]
    e[:, 148] = 1.0
    e[:, 149:152] = rec[:, 3:6]
    e[:, 152:155] = rec[:, 6:9]
    e[:, 155:158] = ph
    e[:, 158] = rec[:, 13]
    return e


def forward(h0: np.ndarray, w: np.ndarray, rounding: bool = True) -> tuple[np.ndarray, list[np.ndarray]]:
    """h0 (n, 160) encoded inputs (already BF16 values when rounding) -> raw outputs Y (n, 3) and
    the activations H_0..H_5."""
    W = unpack(w)
    if rounding:
        W = [bf16(x) for x in W]
    hs = [np.asarray(h0, np.float64)]
    for l in range(LAYERS - 1):
        z = hs[-1] @ W[l].T
        h = np.maximum(z, 0.0)
        hs.append(bf16(h) if rounding else h)
    y = hs[-1] @ W[-1].T
    return y[:, :OUT], hs


def radiance(h0: np.ndarray, w: np.ndarray, rounding: bool = True) -> np.ndarray:
    y, _ = forward(h0, w, rounding)
    return np.exp(np.minimum(y, 20.0))


def loss_and_gradient(h0: np.ndarray, w: np.ndarray, target: np.ndarray, rounding: bool = True,
                      den: np.ndarray | None = None) -> tuple[float, np.ndarray]:
    """Mean relative L2 loss and its gradient w.r.t. the compact weights. `den` (n, 3) fixes the
    loss denominators (default p^2 + 0.01 at these weights), as the device treats them."""
    W = unpack(w)
    if rounding:
        W = [bf16(x) for x in W]
    y, hs = forward(h0, w, rounding)
    n = y.shape[0]
    p = np.exp(np.minimum(y, 20.0))
    t = np.asarray(target, np.float64)
    if den is None:
        den = p * p + 0.01
    diff = p - t
    loss = float(np.sum(diff * diff / den) / n)
    dy = np.where(y < 20.0, 2.0 * diff / den * p / n, 0.0)
    dyp = np.zeros((n, OUT_PAD))
    dyp[:, :OUT] = bf16(dy) if rounding else dy
    grads = [None] * LAYERS
    grads[LAYERS - 1] = dyp.T @ hs[LAYERS - 1]
    dz = dyp
    for l in range(LAYERS - 1, 0, -1):
        dh = dz @ W[l]
        dz = dh * (hs[l] > 0)
        if rounding:
            dz = bf16(dz)
        grads[l - 1] = dz.T @ hs[l - 1]
    return loss, pack(grads)


def adam(w, m, v, g, t: int, lr: float, b1: float = 0.9, b2: float = 0.99, eps: float = 1e-10):
    """One Adam step (t = 1 for the first); returns new (w, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v


def init_weights(seed: int) -> np.ndarray:
    """Random weights for tests (He-uniform, output rows 3..7 zero)."""
    rng = np.random.default_rng(seed)
    ws = []
    for l in range(LAYERS):
        s = np.sqrt(6.0 / layer_in(l)) * (0.1 if l == LAYERS - 1 else 1.0)
        x = rng.uniform(-s, s, (layer_out(l), layer_in(l)))
        if l == LAYERS - 1:
            x[OUT:] = 0.0
        ws.append(x)
    return pack(ws).astype(np.float32)
