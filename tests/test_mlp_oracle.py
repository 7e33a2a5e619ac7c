"""The surrogate MLP's CPU oracle, pinned by central finite differences in FP64 (the
reference has no learned component, so there are no reference outputs to pin it to), and
its BF16 rounding checked against exact values."""
import numpy as np

from oracle import mlp_oracle as mo


def test_bf16_round_known_values():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 0.0, 3.0e-39],
                 np.float32)
    # ties to even at 2^-8 spacing above 1; 1 + 2^-9 is a tie that rounds down to 1
    want = np.array([1.0, 1.0, 1.0 + 4 * 2 ** -8, 1.0, 1.0 + 2 * 2 ** -8, -2.5, 0.0, 0.0])
    got = mo.bf16_round(x)
    assert np.array_equal(got[:7], want[:7])
    assert abs(got[7]) < 1e-38


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    dims = mo.dims_of(5, 8, 3)
    p = rng.normal(0, 0.5, sum(o * i + o for i, o in zip(dims[:-1], dims[1:])))
    x = rng.normal(size=(7, 5))
    t = rng.normal(size=(7, 3))
    loss, g = mo.loss_and_grads(p, x, t, dims, bf16=False)
    eps = 1e-6
    for k in rng.choice(p.size, 40, replace=False):
        q = p.copy()
        q[k] += eps
        lp, _ = mo.loss_and_grads(q, x, t, dims, bf16=False)
        q[k] -= 2 * eps
        lm, _ = mo.loss_and_grads(q, x, t, dims, bf16=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def test_adam_first_step_is_signed_learning_rate():
    g = np.array([0.3, -2.0, 1e-3])
    p, m, v = mo.adam_step(np.zeros(3), g, np.zeros(3), np.zeros(3), 0, 0.01)
    assert np.allclose(p, -0.01 * np.sign(g), rtol=1e-4)


def test_init_params_layout():
    dims = mo.dims_of(14, 256, 2)
    p = mo.init_params(dims, 7)
    assert p.size == 14 * 256 + 256 + 2 * (256 * 256 + 256) + 256 * 2 + 2
    layers = mo.split(p, dims)
    for (W, b), (i, o) in zip(layers, zip(dims[:-1], dims[1:])):
        assert W.shape == (o, i) and np.all(b == 0)
        assert np.max(np.abs(W)) <= np.sqrt(6.0 / (i + o))
