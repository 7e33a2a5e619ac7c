"""Host-side arithmetic of the learned sweep placement (kuramoto_gb300/surrogate.py) on the
CPU: targets and features of a record set, the placement density and its inverse-CDF
points, and the transition window of a sweep."""
import numpy as np

from kuramoto_gb300 import surrogate as S


def test_targets_are_mean_and_std_over_the_second_half():
    t1, dt = 10.0, 1.0
    rec = np.arange(11, dtype=np.float32)[None, :] * np.float32([[1.0], [0.5]])
    tg = S.targets(rec, t1, dt)
    w = rec[:, 5:].astype(np.float64)
    assert tg.shape == (2, 2)
    assert np.allclose(tg[:, 0], w.mean(1)) and np.allclose(tg[:, 1], w.std(1))


def test_features_hold_parameters_then_early_records():
    rec = np.random.default_rng(0).random((3, 20)).astype(np.float32)
    c, k, f, ca = np.float32([1, 2, 3]), np.array([2, 5, 8]), np.float32([0.5, 1, 2]), np.array([0, 1, 0])
    x = S.features(c, k, f, ca, rec)
    assert x.shape == (3, 4 + S.N_EARLY)
    assert np.array_equal(x[:, :4], np.stack([c, k, f, ca], 1).astype(np.float32))
    assert np.array_equal(x[:, 4:], rec[:, :S.N_EARLY])


def test_uniform_density_places_points_at_equal_quantiles():
    cg = np.linspace(0.0, 6.0, 64)
    pts = S.place_points(cg, np.full(64, 1.0 / 6.0), 12)
    assert np.allclose(pts, (np.arange(12) + 0.5) / 12 * 6.0, atol=1e-5)


def test_density_concentrates_points_where_the_prediction_moves():
    cg = np.linspace(0.0, 6.0, 64)
    step = 1.0 / (1.0 + np.exp(-(cg - 2.0) / 0.1))  # a sharp transition at c = 2
    pred = np.stack([step, 0.3 * (1 - step)], 1)
    dens = S.placement_density(cg, pred)
    assert abs(S._trapezoid(dens, cg) - 1.0) < 1e-6
    assert np.all(dens >= 0.15 / 6.0 - 1e-12)
    pts = S.place_points(cg, dens, 64)
    assert np.all(np.diff(pts) >= 0)
    near = np.mean(np.abs(pts - 2.0) < 0.5)  # a sixth of the range holds most of the points
    assert near > 0.5


def test_transition_window_brackets_the_drop():
    c = np.linspace(0.0, 6.0, 121)
    std_r = 0.05 + 0.25 / (1.0 + np.exp((c - 3.0) / 0.2))  # falls from 0.30 to 0.05 around c = 3
    lo, hi = S.transition_window(c, std_r)
    assert lo < 3.0 < hi
    # 80 % and 20 % of the drop are at c = 3 -/+ 0.2 ln 4
    assert abs(lo - (3.0 - 0.2 * np.log(4.0))) < 0.1 and abs(hi - (3.0 + 0.2 * np.log(4.0))) < 0.1
