"""The surrogate MLP's tensor-core kernels (kura_mlp_*) against the CPU oracle.

Forward outputs and gradients are compared with the oracle that rounds to BF16 where the
GPU stores BF16 (then only FP32 accumulation order differs), and with the exact FP64
network (the BF16 storage error itself, a few 1e-3 relative).  A training step is checked
against the oracle's Adam update, and training is checked to fit a smooth target.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu

IN, OUT = 14, 2


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, IN)).astype(np.float32)
    t = np.stack([np.tanh(x[:, 0] + 0.5 * x[:, 1] * x[:, 2]), 0.3 * np.sin(x[:, 3]) + 0.1 * x[:, 4] ** 2], 1)
    return x, t.astype(np.float32)


@pytest.mark.parametrize("hidden,batch", [(256, 512), (128, 256), (64, 128)])
def test_init_forward_matches_oracle(native, hidden, batch):
    with native.MLP(IN, OUT, hidden=hidden, batch=batch, seed=11) as m:
        p = m.params()
        dims = mo.dims_of(IN, hidden, OUT)
        assert np.array_equal(p.astype(np.float64), mo.init_params(dims, 11))
        x, _ = data(batch + 77, 1)  # two chunks, the second partial
        y = m.forward(x)
        ref, _ = mo.forward(p, x, dims, bf16=True)
        exact, _ = mo.forward(p, x, dims, bf16=False)
        assert np.max(np.abs(y - ref)) <= 2e-3 * np.max(np.abs(ref)) + 1e-6
        assert rel(y, exact) < 2e-2


@pytest.mark.parametrize("n", [512, 300])
def test_gradients_match_oracle(native, n):
    with native.MLP(IN, OUT, hidden=256, batch=512, seed=3) as m:
        rng = np.random.default_rng(5)
        p = m.params() + rng.normal(0, 0.02, m.param_count).astype(np.float32)  # biases nonzero too
        m.set_params(p)
        assert np.array_equal(m.params(), p)
        x, t = data(n, 2)
        loss, g = m.gradients(x, t)
        dims = mo.dims_of(IN, 256, OUT)
        lref, gref = mo.loss_and_grads(p, x, t, dims, bf16=True)
        lex, gex = mo.loss_and_grads(p, x, t, dims, bf16=False)
        assert abs(loss - lref) <= 1e-3 * lref
        # per layer and part (W, b): BF16-emulating oracle tight, exact FP64 loose
        k = 0
        for i, o in zip(dims[:-1], dims[1:]):
            for size in (o * i, o):
                sl = slice(k, k + size)
                assert rel(g[sl], gref[sl]) < 1e-2, (k, size, rel(g[sl], gref[sl]))
                assert rel(g[sl], gex[sl]) < 6e-2, (k, size, rel(g[sl], gex[sl]))
                k += size
        assert k == g.size


def test_one_training_step_is_oracle_adam(native):
    with native.MLP(IN, OUT, hidden=256, batch=256, seed=9) as m:
        p0 = m.params().astype(np.float64)
        x, t = data(256, 4)
        losses, ms = m.train(x, t, epochs=1, lr=1e-3, seed=1)  # one batch: the permutation is the identity set
        p1 = m.params().astype(np.float64)
        dims = mo.dims_of(IN, 256, OUT)
        _, g = mo.loss_and_grads(p0, x, t, dims, bf16=True)
        want, _, _ = mo.adam_step(p0, g, np.zeros_like(g), np.zeros_like(g), 0, 1e-3)
        d = p1 - p0
        big = np.abs(g) > 1e-5 * np.max(np.abs(g))
        # a first Adam step moves every parameter by lr * sign(g) (up to eps)
        assert np.mean(np.abs(d[big] - (want - p0)[big]) <= 2e-5) > 0.99
        assert ms > 0 and losses.size == 1 and np.isfinite(losses[0])


def test_training_fits_smooth_target(native):
    x, t = data(8192, 6)
    xv, tv = data(2048, 7)
    with native.MLP(IN, OUT, hidden=256, batch=512, seed=2) as m:
        base = float(np.mean((m.forward(xv) - tv) ** 2))
        losses, ms = m.train(x, t, epochs=60, lr=2e-3, lr_final=2e-4, seed=3)
        val = float(np.mean((m.forward(xv) - tv) ** 2))
    assert losses[-1] < 0.1 * losses[0]
    assert val < 0.05 * base and val < 5e-3, (base, val)
    assert np.all(np.isfinite(losses))


def test_rejects_unsupported(native):
    for kw in (dict(in_dim=65, out_dim=2), dict(in_dim=4, out_dim=2, hidden=100), dict(in_dim=4, out_dim=2, batch=100)):
        with pytest.raises(native.KuraError) as e:
            native.MLP(**kw)
        assert e.value.code == -7
