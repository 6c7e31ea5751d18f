"""The radiance cache's CPU oracle (oracle/nrc_oracle.py) checked on its own: BF16 rounding
against torch, the analytic gradient against finite differences in FP64, Adam against
torch.optim.Adam."""
import numpy as np
import pytest

from oracle import nrc_oracle as nrc

torch = pytest.importorskip("torch")


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(0, 1, 5000), rng.normal(0, 1e-30, 100), [0.0, -0.0, 1.0, 65504.0, 3.0e38]])
    x = x.astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(nrc.bf16(x), ref)


def test_parameter_layout():
    assert nrc.NUM_PARAMS == 160 * 64 + 4 * 64 * 64 + 8 * 64 == 27136
    w = nrc.init_weights(3)
    ws = nrc.unpack(w)
    assert [x.shape for x in ws] == [(64, 160), (64, 64), (64, 64), (64, 64), (64, 64), (8, 64)]
    assert not ws[-1][3:].any()
    assert np.array_equal(nrc.pack(ws).astype(np.float32), w)


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    rec = np.zeros((n, 16))
    rec[:, 0:3] = rng.uniform(-2, 2, (n, 3))
    d = rng.normal(size=(n, 3))
    rec[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.normal(size=(n, 3))
    rec[:, 6:9] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    rec[:, 9] = rng.uniform(0, 1, n)
    rec[:, 10:13] = rng.uniform(0, 1, (n, 3))
    rec[:, 13] = rng.integers(0, 7, n) / 8.0
    return rec


def test_encoding_layout():
    rec = _inputs(5, 1)
    e = nrc.encode(rec, [-2, -2, -2], [2, 2, 2])
    ph = (rec[:, 0:3] + 2.0) / 4.0
    assert np.allclose(e[:, 24 * 1 + 2 * 3], np.sin(np.pi * ph[:, 1] * 8))
    assert np.allclose(e[:, 72 + 12 * 2 + 2 * 5 + 1], np.cos(np.pi * (rec[:, 5] + 1) * 0.5 * 32))
    assert np.allclose(e[:, 148], 1.0) and np.allclose(e[:, 145:148], rec[:, 10:13])
    assert np.all(e[:, 159] == 0.0)


def test_gradient_against_finite_differences():
    """The analytic gradient (denominators held fixed, as the loss defines them) against
    central differences of the same loss in FP64 without rounding."""
    n = 6
    rec = _inputs(n, 2)
    h0 = nrc.encode(rec, [-2] * 3, [2] * 3)
    w = nrc.init_weights(5).astype(np.float64)
    rng = np.random.default_rng(7)
    target = rng.uniform(0.2, 3.0, (n, 3))
    y, _ = nrc.forward(h0, w, rounding=False)
    p = np.exp(y)
    den = p * p + 0.01
    _, g = nrc.loss_and_gradient(h0, w, target, rounding=False, den=den)
    off = nrc.offsets()
    idx = np.concatenate([rng.integers(off[l], off[l + 1], 12) for l in range(nrc.LAYERS)])
    idx = idx[(idx < off[5]) | ((idx - off[5]) // 64 < 3)]  # skip the zero padding rows
    h = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        lp, _ = nrc.loss_and_gradient(h0, wp, target, rounding=False, den=den)
        lm, _ = nrc.loss_and_gradient(h0, wm, target, rounding=False, den=den)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_adam_matches_torch():
    rng = np.random.default_rng(3)
    w0 = rng.normal(size=50)
    grads = rng.normal(size=(4, 50))
    p = torch.nn.Parameter(torch.from_numpy(w0.copy()))
    opt = torch.optim.Adam([p], lr=1e-2, betas=(0.9, 0.99), eps=1e-10)
    w, m, v = w0.copy(), np.zeros(50), np.zeros(50)
    for t in range(4):
        p.grad = torch.from_numpy(grads[t].copy())
        opt.step()
        w, m, v = nrc.adam(w, m, v, grads[t], t + 1, 1e-2)
    assert np.allclose(p.detach().numpy(), w, rtol=1e-12, atol=1e-14)
