"""The learned radiance cache on the tensor cores against its numpy restatement
(oracle/mlp.py): feature encoding, forward pass, gradients and training.

Tolerances: features 5e-4 absolute (the band-0 sin/cos of the two sides differ by an ulp or two, which angle doubling amplifies up to 2^11 times); network
outputs and gradients compare BF16 products accumulated in FP32 in different orders, so
1e-2 of the output scale and 3e-2 relative norm per gradient tensor; against the FP64
network, the BF16 restatement's own error (factor 1.5, plus 2^-10) bounds the GPU's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAYERS = [(64, 96), (64, 64), (64, 64), (64, 64), (16, 64)]


def flatten(p):
    return np.concatenate([np.concatenate([w.ravel(), b]) for w, b in zip(p["W"], p["b"])]).astype(np.float32)


def unflatten(v):
    W, b, off = [], [], 0
    for o, k in LAYERS:
        W.append(v[off:off + o * k].reshape(o, k).copy())
        off += o * k
        b.append(v[off:off + o].copy())
        off += o
    return {"W": W, "b": b}


def queries(n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-0.5, 0.5, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return pos, d.astype(np.float32)


def target_fn(pos, d):
    """A smooth synthetic radiance field to learn."""
    r = 0.8 + 0.4 * np.sin(3 * pos[:, 0]) * np.cos(2 * pos[:, 1]) + 0.2 * d[:, 1]
    return np.stack([r, 0.8 * r + 0.1 * pos[:, 2], 0.5 * r], 1).astype(np.float32)


@pytest.fixture(scope="module")
def cache(built):
    import narvalengine_gb300 as ne
    ctx = ne.Context(0)
    c = ne.RadianceCache(ctx, seed=1)
    yield c
    c.close()
    ctx.close()


def test_layout_constants():
    from oracle import mlp
    assert sum(o * k + o for o, k in LAYERS) == 19728 == flatten(mlp.init_params(0)).size


def test_encoding(cache):
    from oracle import mlp
    pos, d = queries(4096, 1)
    g = cache.encode(pos, d)
    c = mlp.encode(pos, d)
    assert np.abs(g - c).max() < 5e-4
    assert np.all(g[:, 88:] == 0)


@pytest.mark.parametrize("n", [5, 128, 1000, 20000])
def test_forward_matches_oracle(cache, n):
    from oracle import mlp
    p = mlp.init_params(7)
    cache.set_params(flatten(p))
    assert np.array_equal(cache.params(), flatten(p))
    pos, d = queries(n, n)
    feats = cache.encode(pos, d)
    got = cache.infer(feats=feats)
    want = mlp.forward(p, feats)[0][:, :3]
    scale = np.abs(want).max() + 1e-3
    assert np.abs(got - want).max() <= 1e-2 * scale, (np.abs(got - want).max(), scale)
    # the fused encoding gives the same outputs as precomputed features
    assert np.allclose(cache.infer(pos=pos, dirs=d), got, rtol=0, atol=1e-6 * scale + 1e-7)


@pytest.mark.parametrize("n", [300, 65536])
def test_gradients_match_oracle(cache, n):
    from oracle import mlp
    p = mlp.init_params(11)
    cache.set_params(flatten(p))
    pos, d = queries(n, 5)
    feats = cache.encode(pos, d)
    t = target_fn(pos, d)
    loss, g = cache.train(t, feats=feats, apply=False, want_grads=True)
    out, xs, zs = mlp.forward(p, feats)
    want_loss, gout = mlp.loss_and_grad_out(out, t)
    gW, gb = mlp.backward(p, xs, zs, gout)
    assert abs(loss - want_loss) <= 1e-3 * want_loss
    G = unflatten(g)
    for i in range(5):
        for name, a, b in (("W", G["W"][i], gW[i]), ("b", G["b"][i], gb[i])):
            rel = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-12)
            assert rel < 3e-2, f"layer {i} {name}: relative error {rel:.3e}"
    # apply=False leaves the parameters alone
    assert np.array_equal(cache.params(), flatten(p))


@pytest.mark.parametrize("n", [1000, 65536])
def test_gradients_against_fp64(cache, n):
    """Gradients against the FP64 network (no BF16 rounding anywhere, oracle/mlp.py with
    quant=False). Tolerance from BF16 rounding: operands carry 8 significand bits (relative
    rounding up to 2^-9), so each tensor's error against FP64 may be what the BF16-quantised
    restatement's own error is, within a factor 1.5 plus 2^-10 of the tensor's norm (the
    GPU sums its FP32 partial products in another order). That error is itself large where a
    gradient is a sum of many products of both signs (layer 0's weights over 1000 samples: about
    6% of a norm that cancellation makes small), so the bound is relative to it, not fixed."""
    from oracle import mlp
    p = mlp.init_params(13)
    cache.set_params(flatten(p))
    pos, d = queries(n, 8)
    feats = cache.encode(pos, d)
    t = target_fn(pos, d)
    _, g = cache.train(t, feats=feats, apply=False, want_grads=True)
    G = unflatten(g)
    out64, xs64, zs64 = mlp.forward(p, feats, quant=False)
    _, gout64 = mlp.loss_and_grad_out(out64, t)
    gW64, gb64 = mlp.backward(p, xs64, zs64, gout64, quant=False)
    outq, xsq, zsq = mlp.forward(p, feats)
    _, goutq = mlp.loss_and_grad_out(outq, t)
    gWq, gbq = mlp.backward(p, xsq, zsq, goutq)
    for i in range(5):
        for name, a, q, ref in (("W", G["W"][i], gWq[i], gW64[i]), ("b", G["b"][i], gbq[i], gb64[i])):
            nref = np.linalg.norm(ref) + 1e-30
            e_gpu = np.linalg.norm(a - ref) / nref
            e_bf16 = np.linalg.norm(q - ref) / nref
            assert e_gpu <= 1.5 * e_bf16 + 2.0 ** -10, \
                f"layer {i} {name}: GPU {e_gpu:.3e} vs BF16 restatement {e_bf16:.3e} against FP64"


def test_training_follows_oracle_and_converges(cache):
    from oracle import mlp
    p = mlp.init_params(3)
    cache.set_params(flatten(p))
    adam = mlp.Adam(p)
    n = 8192
    losses_gpu, losses_cpu = [], []
    for step in range(5):
        pos, d = queries(n, 100 + step)
        feats = cache.encode(pos, d)
        t = target_fn(pos, d)
        lg, _ = cache.train(t, feats=feats)
        losses_gpu.append(lg)
        losses_cpu.append(mlp.train_step(p, adam, feats, t))
    assert np.allclose(losses_gpu, losses_cpu, rtol=5e-2), (losses_gpu, losses_cpu)
    rel = np.linalg.norm(cache.params() - flatten(p)) / np.linalg.norm(flatten(p))
    assert rel < 2e-2, rel
    for step in range(300):
        pos, d = queries(n, 1000 + step)
        lg, _ = cache.train(target_fn(pos, d), pos=pos, dirs=d)
    pos, d = queries(20000, 99)
    pred = np.maximum(cache.infer(pos=pos, dirs=d), 0)
    t = target_fn(pos, d)
    rel_l2 = np.mean((pred - t) ** 2 / (t * t + 0.01))
    assert lg < losses_gpu[0] / 10 and rel_l2 < 0.05, (losses_gpu[0], lg, rel_l2)
