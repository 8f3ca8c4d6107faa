"""Learned fixed-rate selection: features, network, training, and what the
network gains over plain bisection.

The oracle (oracle/lfx.py) restates the feature sums and the network's
forward and backward passes on the CPU; the GPU's feature sums must equal it
exactly (integers), its features and gradients must agree to float
precision.  The end-to-end test trains a network on the GPU from real
compress passes and checks it against bisection on held-out fields.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import fields as GF  # noqa: E402
from oracle import lfx as OL  # noqa: E402


def _params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    p = (rng.normal(size=OL.P_TOTAL) * 0.2 * scale).astype(np.float32)
    p[OL.P_MU:OL.P_MU + 32] = rng.normal(size=32).astype(np.float32)
    p[OL.P_SD:OL.P_SD + 32] = rng.uniform(0.5, 2.0, 32).astype(np.float32)
    return p


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = _params(2).astype(np.float64)
    X = rng.normal(size=(7, 32))
    y = rng.normal(size=7)
    loss, g = OL.mlp_loss_grad(p, X, y)
    for k in rng.choice(OL.P_NTRAIN, 40, replace=False):
        e = 1e-6
        q = p.copy()
        q[OL.P_W1 + k] += e
        lp, _ = OL.mlp_loss_grad(q, X, y)
        q[OL.P_W1 + k] -= 2 * e
        lm, _ = OL.mlp_loss_grad(q, X, y)
        assert abs((lp - lm) / (2 * e) - g[k]) <= 1e-6 + 1e-5 * abs(g[k]), k


def test_oracle_features_of_simple_fields():
    x = np.zeros(128 * 100, np.float32)
    rng, a = OL.sums(x)
    assert rng == 0 and a[0] == 3 and a[17] == 3 and all(a[1:17] == 12)   # coarse: sampled blocks 0, 4, 8
    for t in (4.0, 8.0, 16.0, 32.0):
        f = OL.features(GF.make("smooth", 1 << 16, np.float32), t)
        assert f[0] == np.log2(t)
        assert np.all(np.diff(f[5:13]) >= -1e-12)    # the ratio grows with the bound
        assert np.all(np.diff(f[13:29]) >= -1e-12)
        assert f[4] <= f[1] <= f[4] + 0.25           # the aim lies in the 1/64-step window
        yq = (OL.center(OL.sums(GF.make("smooth", 1 << 16, np.float32))[1], t) + 128) / 64.0
        assert yq - 2.0 <= f[4] <= yq + 1.75          # inside the quarter-step window
        assert abs(f[3]) < 0.5                        # the second sample agrees closely on a smooth field
        if f[13] < 0 <= f[28]:
            assert abs(f[1] - f[4] - 0.125) <= 0.125


# ------------------------------------------------------------------ GPU

@pytest.fixture(scope="module")
def L():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required")
    from szx_gb300 import build
    build.build()
    from szx_gb300 import learned
    return learned


def _dev_fields(torch):
    xs = [GF.make(n, 1 << 16, np.float32) for n in GF.FIELDS]
    rng = np.random.default_rng(3)
    xs += [rng.normal(size=70001).astype(np.float32), (np.cumsum(rng.normal(size=300000)) * 1e-3).astype(np.float32),
           np.zeros(5000, np.float32), rng.normal(size=1000).astype(np.float32)]
    return xs, [torch.tensor(x, device="cuda") for x in xs]


@pytest.mark.gpu
def test_features_match_oracle(L):
    import torch
    xs, ts = _dev_fields(torch)
    # an unaligned field too: a view one value into a buffer
    base = torch.tensor(np.concatenate([[0], xs[1]]).astype(np.float32), device="cuda")
    ts.append(base[1:])
    xs.append(xs[1])
    b = L.Batch(ts)
    rows = np.repeat(np.arange(len(ts)), 2)
    tg = np.tile([8.0, 20.0], len(ts)).astype(np.float32)
    X, rg = b.features(rows, tg)
    X = X.cpu().numpy().astype(np.float64)
    for r, (f, t) in enumerate(zip(rows, tg)):
        want_rng, acc = OL.sums(xs[f])
        assert rg[f] == want_rng, f
        mq = OL.center(acc, t)
        mu = int(round(X[r, 4] * 64))
        assert mu == OL.center2(float(OL.sampled_blocks(xs[f])), OL.probe_sums(xs[f], mq, 16), t, mq), (f, t)
        want = OL.features(xs[f], t, mq, mu)
        np.testing.assert_allclose(X[r], want, rtol=1e-5, atol=2e-6, err_msg=f"field {f}")
    b.close()


@pytest.mark.gpu
def test_network_forward_and_gradient_match_oracle(L):
    import torch
    rng = np.random.default_rng(4)
    p = _params(5)
    m = L.Mlp(0, params=p)
    for n in (1, 33, 200):
        X = rng.normal(size=(n, 32)).astype(np.float32)
        y = rng.normal(size=n).astype(np.float32)
        Xt, yt = torch.tensor(X, device="cuda"), torch.tensor(y, device="cuda")
        out = m.forward(Xt).cpu().numpy()
        want, _ = OL.mlp_forward(p.astype(np.float64), X)
        np.testing.assert_allclose(out, want, rtol=1e-4, atol=1e-5)
        loss, g = m.gradient(Xt, yt)
        wl, wg = OL.mlp_loss_grad(p.astype(np.float64), X, y)
        assert abs(loss - wl) <= 1e-4 * abs(wl) + 1e-6
        g = g.cpu().numpy()
        np.testing.assert_allclose(g, wg, rtol=2e-3, atol=1e-5 * np.abs(wg).max())
    m.close()


@pytest.mark.gpu
def test_training_is_reproducible_and_fits(L):
    import torch
    rng = np.random.default_rng(6)
    X = rng.normal(size=(3000, 32)).astype(np.float32)
    w = rng.normal(size=32)
    y = (np.tanh(X @ w / 6.0) * 4.0 - 10.0).astype(np.float32)
    Xt, yt = torch.tensor(X, device="cuda"), torch.tensor(y, device="cuda")
    m1, l1 = L.train(Xt, yt, seed=3, epochs=40, batch=256)
    m2, l2 = L.train(Xt, yt, seed=3, epochs=40, batch=256)
    assert l1 == l2 and np.array_equal(m1.params(), m2.params())
    base = float(((y - y.mean()) ** 2).mean())
    assert l1 < 0.05 * base, (l1, base)
    pred = m1.forward(Xt).cpu().numpy()
    assert float(((pred - y) ** 2).mean()) < 0.05 * base


@pytest.mark.gpu
def test_learned_selection_beats_bisection_and_the_zero_network(L):
    """Trained on the GPU from real compress passes, the learned selection
    reaches the target ratio within 5% on fields it was not trained on with
    at least 3x fewer real compress passes than plain bisection on these
    small fields (at least 4x on the larger fields of the fixed-rate
    benchmark), reaches every
    field bisection reaches, and leaves the codec's own streams at its bounds.
    And the network earns its place: against the same search with a zero
    network (the first sample's crossing alone), networks trained from three
    seeds each need fewer real passes on the held-out fields, and the gain is
    larger than the spread between the three trained networks.  (The network
    sees a second, disjoint block sample that the crossing does not use.)"""
    from szx_gb300 import api
    train_f, _ = L.synthetic_fields(600, 15, 19, seed=11)
    tb = L.Batch(train_f)
    X, y, _ = L.training_set(tb, passes=16, seed=12)
    tb.close()
    del train_f
    models = []
    for seed in (13, 14, 15):
        m, loss = L.train(X, y, seed=seed, epochs=200, batch=512)
        assert loss < float(y.var()), (loss, float(y.var()))
        models.append(m)
    zero = L.Mlp(0, params=np.concatenate([np.zeros(32), np.ones(32), np.zeros(OL.P_NTRAIN)]).astype(np.float32))
    test_f, _ = L.synthetic_fields(160, 16, 19, seed=21)
    b = L.Batch(test_f)
    zero_passes, bisect_passes, reached, learned_passes = [], [], [], [[] for _ in models]
    for target in (8.0, 16.0):
        eb_b, cr_b, ps_b = b.fixed_rate(target, None, 0.05, 20)
        _, cr_z, ps_z = b.fixed_rate(target, zero, 0.05, 20)
        ok_b = np.abs(cr_b / target - 1) <= 0.05
        zero_passes.append(ps_z)
        bisect_passes.append(ps_b)
        for j, m in enumerate(models):
            eb_l, cr_l, ps_l = b.fixed_rate(target, m, 0.05, 20)
            ok_l = np.abs(cr_l / target - 1) <= 0.05
            reached.append(bool(ok_l[ok_b].all()))
            learned_passes[j].append(ps_l)
    pz = float(np.concatenate(zero_passes).mean())
    pb = float(np.concatenate(bisect_passes).mean())
    pl = np.array([np.concatenate(p).mean() for p in learned_passes])
    gain = pz - pl
    res = dict(bisection=pb, zero=pz, learned=pl.tolist(), gain=gain.tolist(), spread=float(pl.max() - pl.min()))
    print(res)
    assert all(reached), res
    # small fields (2^16..2^19 values) are the hard case for a sampled model
    assert pl.max() * 3 <= pb, res
    assert (gain > 0).all(), res
    assert gain.mean() > pl.max() - pl.min(), res
    # the last learned run (target 16) left its streams in the plan
    for k in range(0, 96, 17):
        s = b.stream(k)
        x = test_f[k].cpu().numpy()
        assert len(s) == pytest.approx(x.size * 4 / cr_l[k], rel=1e-6)
        assert s == api.compress_host(2, x, 128, 0, float(eb_l[k]), 0.0)
    b.close()
