"""GPU tests of the MLP surrogate: gradients of the hand-written forward /
backward kernels against the FP64 oracle (oracle/mlp_oracle.py), training on
the GPU, and the surrogate with its BEM fallback.

Gradient tolerances (relative to the largest gradient entry): split-BF16
products 2e-4, plain BF16 products 5e-2 (8-bit mantissas of the operands).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _net(agb):
    from andromeda_gb300.surrogate import MLP
    return MLP(device=0, seed=3)


def test_mlp_gradient_matches_oracle(agb):
    import mlp_oracle as mo
    net = _net(agb)
    rng = np.random.default_rng(1)
    n = 96
    X = rng.uniform(0.2, 1.8, (n, 5)).astype(np.float32)
    T = rng.normal(size=(n, 21)).astype(np.float32)
    xm, xs = X.mean(0), X.std(0) + 1e-3
    ym, ys = T.mean(0), T.std(0) + 1e-3
    net.set_normalization(xm, xs, ym, ys)
    p = net.params()
    loss_ref, g_ref = mo.loss_and_grad(p.astype(np.float64), X, T, xm.astype(np.float64), xs.astype(np.float64),
                                       ym.astype(np.float64), ys.astype(np.float64))
    scale = np.max(np.abs(g_ref))
    g_split, loss_split = net.gradient(X, T, split=True)
    g_plain, loss_plain = net.gradient(X, T, split=False)
    assert abs(loss_split - loss_ref) < 1e-4 * loss_ref
    assert np.max(np.abs(g_split - g_ref)) < 2e-4 * scale
    assert np.max(np.abs(g_plain - g_ref)) < 5e-2 * scale
    net.close()


def test_fused_inference_matches_layer_gemms_and_oracle(agb):
    """The fused one-kernel split-BF16 inference against the layer-by-layer
    split-BF16 GEMMs (same accumulation order and FP32 epilogues: equal up to
    1 ulp of the outputs) and against the FP64 oracle forward (split-BF16
    products carry ~16 mantissa bits: 1e-4 of the largest output), on a
    query count that is not a multiple of the 128-query CTA tile."""
    import mlp_oracle as mo
    net = _net(agb)
    rng = np.random.default_rng(5)
    n = 1000
    X = rng.uniform(0.2, 1.8, (n, 5)).astype(np.float32)
    xm, xs = X.mean(0), X.std(0) + 1e-3
    ym = rng.normal(size=21).astype(np.float32)
    ys = rng.uniform(0.5, 2.0, 21).astype(np.float32)
    net.set_normalization(xm, xs, ym, ys)
    p = net.params()
    p = p + rng.normal(scale=0.05, size=p.shape).astype(np.float32)  # non-zero biases
    net.set_params(p)
    Yf, _ = net.predict(X, split=True, fused=True)
    Yg, _ = net.predict(X, split=True, fused=False)
    assert np.all(np.isfinite(Yf))
    assert np.max(np.abs(Yf - Yg)) <= 2.0 * np.max(np.spacing(np.abs(Yg)))
    Xn = (X.astype(np.float64) - xm) / xs
    Yo, _ = mo.forward(p.astype(np.float64), Xn)
    Yo = Yo * ys + ym
    assert np.max(np.abs(Yf - Yo)) < 1e-4 * np.max(np.abs(Yo))
    net.close()


def test_mlp_trains_on_the_gpu(agb):
    """A smooth 5 -> 21 map is learned: the loss falls by two orders of magnitude."""
    net = _net(agb)
    rng = np.random.default_rng(2)
    X = rng.uniform(0.0, 1.0, (4096, 5)).astype(np.float32)
    W = rng.normal(size=(5, 21))
    Y = (np.sin(X @ W) + 0.1 * (X ** 2) @ W).astype(np.float32)
    net.set_normalization(X.mean(0), X.std(0), Y.mean(0), Y.std(0))
    hist, st = net.train(X, Y, epochs=120, batch=256, lr=2e-3)
    assert hist[-1] < 1e-2 * hist[0]
    assert st["adam_steps"] == 120 * 16 and st["launches"] > 0
    Yp, _ = net.predict(X[:512])
    assert np.sqrt(np.mean((Yp - Y[:512]) ** 2)) < 0.1 * np.std(Y)
    net.close()


def test_surrogate_with_bem_fallback(agb):
    """Trained on BEM tensors of coarse superellipsoids: an ensemble of four
    networks, its agreement threshold calibrated on held-out BEM tensors, and
    on a second held-out set every accepted answer within 1e-3 (max-entry,
    relative) of the BEM; the rest -- outside the hull or above the threshold --
    answered by the BEM itself; the networks answer orders of magnitude faster
    than the BEM."""
    from andromeda_gb300 import surrogate as S
    bem = dict(n_elem=120, outer_level=1, outer_radius=20.0, eps=1e-8)
    # a narrower shape family than the many-body workload's, so that a few
    # thousand coarse bodies and a few seconds of training suffice
    rng = np.random.default_rng(5)
    P = np.column_stack([rng.uniform(0.5, 1.0, (3600, 2)), rng.uniform(0.6, 1.4, (3600, 2))])
    R, st = S.bem_tensors(P, **bem)
    sur = S.Surrogate(device=0, seed=4, bem_kwargs=bem, members=4)
    hist, _ = sur.fit(P[:3000], R[:3000], epochs=800, batch=128, lr=2e-3, lr_final=2e-5)
    assert hist[-1] < 0.01 * hist[0]
    cal = sur.calibrate(P[3000:3300], R[3000:3300], target=1e-3, margin=0.7)
    Rp, acc, info = sur.predict(P[3300:], bem=False)
    err = S.rel_err(Rp[acc], R[3300:][acc])
    print("calibration", cal, "held-out accepted", int(acc.sum()), "of", len(acc),
          "max err", float(err.max()) if len(err) else None, "fallback", info["n_bem"])
    assert acc.sum() >= 0.2 * len(acc), (int(acc.sum()), cal)
    assert np.all(err <= 1e-3), float(err.max())
    assert info["n_bem"] == len(acc) - int(acc.sum())
    # out of the hull (b = 0.1 < every training b): the BEM answers
    q = np.array([[0.1, 0.5, 1.0, 1.0], [0.6, 0.6, 1.0, 1.0]])
    Rq, accq, _ = sur.predict(q)
    assert not accq[0]
    Rd, _ = S.bem_tensors(q[:1], **bem)
    assert np.max(np.abs(Rq[0] - Rd[0])) <= 1e-12 * np.max(np.abs(Rd[0]))
    # throughput: ensemble inferences per second vs BEM solves per second
    many = np.repeat(P[:400], 50, axis=0)
    _, _, ms = sur.ensemble(S.features(many))
    mlp_rate = len(many) / (ms / 1000.0)
    bem_rate = len(P) / (st["device_ms"] / 1000.0)
    assert mlp_rate > 100 * bem_rate
    sur.close()
