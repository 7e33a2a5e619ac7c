"""The learned sweep placement end to end, at a size that runs in seconds.

Training data come from the batched multi-network solver. The MLP is trained by the
library's kernels. A sweep over c for one network places 64 points where the predicted
steady statistics of r change fastest, and the DP45 solver integrates every point and checks
each prediction.  A dense DP45 sweep of the same network locates the true transition, and
the test measures what the network gains over the method without it (64 evenly spaced
points): how many points land in the transition window, and what an even sweep would cost to
reach the same spacing there.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, T1 = 2000, 40.0


@pytest.fixture(scope="module")
def trained(native):
    from kuramoto_gb300 import surrogate as S
    rng = np.random.default_rng(11)
    X, Y, st = S.generate(3072, N, T1, rng, cauchy_frac=0.0)
    assert X.shape == (3072, 14) and Y.shape == (3072, 2)
    assert np.all(np.isfinite(X)) and np.all(np.isfinite(Y))
    sur = S.Surrogate(hidden=256, batch=512, seed=4)
    losses, ms = sur.fit(X[:2560], Y[:2560], epochs=150, lr=2e-3, lr_final=1e-4)
    yield S, sur, X[2560:], Y[2560:], losses
    sur.close()


def test_surrogate_learns_steady_statistics(trained):
    S, sur, Xv, Yv, losses = trained
    assert losses[-1] < 0.5 * losses[0]
    pred = sur.predict(Xv)
    # held-out networks: the predicted spread of r explains most of its variance
    resid = np.mean((pred[:, 1] - Yv[:, 1]) ** 2)
    assert resid < 0.3 * np.var(Yv[:, 1]), (resid, np.var(Yv[:, 1]))
    assert np.mean(np.abs(pred[:, 0] - Yv[:, 0]) <= 0.02) >= 0.99


def test_sweep_placement_beats_even_spacing(trained):
    S, sur, _, _, _ = trained
    k, f, seed = 5, 1.0, 77
    res = S.sweep(sur, N, k, f, 0, seed, np.random.default_rng(3), npoints=64, candidates=64, t1=T1)
    # every prediction checked by DP45; the tolerance of the sweep is 0.02 in r
    assert res["within_tol"].mean() >= 0.95
    assert np.all(np.isfinite(res["value"]))
    # the true transition from a dense DP45 sweep of the same network
    c = np.linspace(0, 6, 121).astype(np.float32)
    ones = np.ones(c.size)
    orders, _ = S.simulate(N, c, (k * ones).astype(int), (seed * ones).astype(int), [res["theta0"]] * c.size,
                           [res["omega"]] * c.size, T1)
    truth = S.targets(orders, T1)
    lo, hi = S.transition_window(c, truth[:, 1])
    assert 0.5 < lo < hi < 4.0, (lo, hi)
    width = max(hi - lo, 0.05)
    inside = int(np.sum((res["points"] >= lo) & (res["points"] <= hi)))
    even = 64 * width / 6.0
    assert inside >= 2.0 * even, (inside, even, lo, hi)
    # cost of an even sweep with the surrogate's spacing inside the window, in full runs,
    # against the surrogate's 64 full runs plus its short runs
    even_runs = 6.0 / (width / max(inside, 1))
    spent = res["osc_steps_full"] + res["osc_steps_short"]
    per_full = res["osc_steps_full"] / 64
    assert even_runs * per_full > 1.3 * spent, (even_runs, per_full, spent)
