"""Learned placement of coupling-sweep points near the volcano transition.

The pipeline:

1. The batched multi-network solver (``MultiNetworks``) integrates networks with random
   coupling c, volcano rank K, frequency scale f and frequency family (Cauchy or normal).
   Each run gives r(t) at t = 0, dt, ..., t1.
2. A 4-layer MLP (``MLP``, trained by libkura's tensor-core kernels) learns the map
       (c, K, f, family, r(0..9)) -> (mean r, std r over the steady window t >= t1/2).
   Below the transition r fluctuates at the 1/sqrt(N) level; above it the phases lock into
   the volcano pattern, the fluctuations collapse and the mean shifts.
3. For a sweep over c, short runs of the candidate couplings (t <= 9) give the features. The
   network predicts the steady statistics, and the sweep points go where the predicted
   statistics change fastest.
4. Every placed point is then integrated to t1 by the DP45 solver. The solver checks each
   prediction (tolerance 0.02 in r), and its values replace the predictions that miss.

The reference has no counterpart; it integrates one network per process and leaves
the choice of c to the user.
"""
import numpy as np

from .native import MLP, MultiNetworks

FEATURES = ["c", "K", "freq_scale", "cauchy"] + ["r%d" % i for i in range(10)]
TARGETS = ["mean_r", "std_r"]
N_EARLY = 10  # records r(0..9) used as features (dt = 1)


def sample_params(count, rng, c_range=(0.0, 6.0), k_range=(2, 8), f_range=(0.5, 2.0), cauchy_frac=0.5):
    """Random (c, K, f, family) per network."""
    c = rng.uniform(*c_range, count).astype(np.float32)
    k = rng.integers(k_range[0], k_range[1] + 1, count)
    f = np.exp(rng.uniform(np.log(f_range[0]), np.log(f_range[1]), count)).astype(np.float32)
    cauchy = (rng.random(count) < cauchy_frac).astype(np.int32)
    return c, k, f, cauchy


def network_inputs(n, f, cauchy, rng):
    """theta0 uniform in [0, 2pi); omega = f * (Cauchy or standard normal)."""
    th = (rng.random(n) * 2 * np.pi).astype(np.float32)
    if cauchy:
        om = f * np.tan(np.pi * (rng.random(n) - 0.5))
    else:
        om = f * rng.standard_normal(n)
    return th, om.astype(np.float32)


def simulate(n, c, k, seeds, thetas, omegas, t1, dt=1.0, device=0, cluster_size=0, block_threads=0):
    """r(t) records of every network to t1 in one multi-network launch; returns
    (orders [count, records], stats)."""
    count = len(c)
    with MultiNetworks([n] * count, k, seeds, c, t1, dt, device=device, cluster_size=cluster_size,
                       block_threads=block_threads) as m:
        order, _, acc = m.integrate(omegas, thetas, want_theta=False)
        st = m.stats()
    st["accepted_per_network"] = acc
    return order, st


def features(c, k, f, cauchy, orders):
    early = np.asarray(orders, np.float32)[:, :N_EARLY]
    return np.concatenate([np.stack([c, k, f, cauchy], 1).astype(np.float32), early], 1)


def targets(orders, t1, dt=1.0):
    o = np.asarray(orders, np.float64)
    i0 = int(round(0.5 * t1 / dt))
    w = o[:, i0:]
    return np.stack([w.mean(1), w.std(1)], 1).astype(np.float32)


def generate(count, n, t1, rng, device=0, **ranges):
    """Training data from the batched solver: (X [count, 14], Y [count, 2], stats)."""
    c, k, f, cauchy = sample_params(count, rng, **ranges)
    seeds = rng.integers(1, 1 << 30, count)
    thetas, omegas = [], []
    for i in range(count):
        th, om = network_inputs(n, f[i], cauchy[i], rng)
        thetas.append(th)
        omegas.append(om)
    orders, st = simulate(n, c, k, seeds, thetas, omegas, t1, device=device)
    return features(c, k, f, cauchy, orders), targets(orders, t1), st


class Surrogate:
    """Standardised features and targets around an ``MLP``."""

    def __init__(self, hidden=256, batch=512, seed=1, device=0):
        self.net = MLP(len(FEATURES), len(TARGETS), hidden=hidden, batch=batch, seed=seed, device=device)
        self.xm = self.xs = self.ym = self.ys = None

    def fit(self, X, Y, epochs=200, lr=2e-3, lr_final=1e-4, seed=1):
        X = np.asarray(X, np.float64)
        Y = np.asarray(Y, np.float64)
        self.xm, self.xs = X.mean(0), X.std(0) + 1e-12
        self.ym, self.ys = Y.mean(0), Y.std(0) + 1e-12
        losses, ms = self.net.train((X - self.xm) / self.xs, (Y - self.ym) / self.ys, epochs, lr=lr,
                                    lr_final=lr_final, seed=seed)
        return losses, ms

    def predict(self, X):
        y = self.net.forward((np.asarray(X, np.float64) - self.xm) / self.xs)
        return y * self.ys + self.ym

    def close(self):
        self.net.close()


def _trapezoid(y, x):
    return float(np.sum(0.5 * (y[1:] + y[:-1]) * np.diff(x)))


def placement_density(cgrid, pred, floor=0.15):
    """Density over the candidate grid: the smoothed speed of change of the predicted
    (mean, std), each scaled by its range, plus a uniform floor."""
    p = np.asarray(pred, np.float64)
    speed = np.zeros(len(cgrid))
    for j in range(p.shape[1]):
        y = np.convolve(p[:, j], np.ones(5) / 5, mode="same")
        g = np.abs(np.gradient(y, cgrid))
        speed += g / (np.ptp(y) + 1e-12)
    speed = np.convolve(speed, np.ones(5) / 5, mode="same")
    speed /= _trapezoid(speed, cgrid) + 1e-30
    return (1 - floor) * speed + floor / (cgrid[-1] - cgrid[0])


def place_points(cgrid, density, npoints):
    """npoints couplings at equal quantiles of the density (inverse CDF)."""
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (density[1:] + density[:-1]) * np.diff(cgrid))])
    cdf /= cdf[-1]
    q = (np.arange(npoints) + 0.5) / npoints
    return np.interp(q, cdf, cgrid).astype(np.float32)


def sweep(sur, n, k, f, cauchy, seed, rng, npoints=64, candidates=64, c_range=(0.0, 6.0), t1=60.0, tol=0.02,
          device=0):
    """Surrogate-guided sweep of c for one network (fixed seed, omega and theta0).

    Returns a dict with the candidate grid and its predictions, the placed points, the
    DP45 statistics at every point, the prediction errors and the accepted values
    (prediction where it is within `tol` of the DP45 value, the DP45 value otherwise), and the
    oscillator-steps spent on the short and the full runs."""
    th, om = network_inputs(n, f, cauchy, rng)
    cgrid = np.linspace(c_range[0], c_range[1], candidates).astype(np.float32)
    ones = np.ones(candidates)
    early, st_short = simulate(n, cgrid, (k * ones).astype(int), (seed * ones).astype(int), [th] * candidates,
                               [om] * candidates, float(N_EARLY - 1), device=device)
    pred_grid = sur.predict(features(cgrid, k * ones, f * ones, cauchy * ones, early))
    pts = place_points(cgrid, placement_density(cgrid, pred_grid), npoints)
    ones = np.ones(npoints)
    full, st_full = simulate(n, pts, (k * ones).astype(int), (seed * ones).astype(int), [th] * npoints,
                             [om] * npoints, t1, device=device)
    truth = targets(full, t1)
    pred = sur.predict(features(pts, k * ones, f * ones, cauchy * ones, full))
    err = np.abs(pred - truth)
    ok = err[:, 0] <= tol
    value = np.where(ok[:, None], pred, truth)
    return dict(cgrid=cgrid, pred_grid=pred_grid, points=pts, truth=truth, pred=pred, err=err, within_tol=ok,
                value=value, osc_steps_short=st_short["osc_steps"], osc_steps_full=st_full["osc_steps"],
                theta0=th, omega=om)


def transition_window(c, std_r, lo=0.2, hi=0.8):
    """The c interval over which the steady std r falls from `hi` to `lo` of its drop
    (incoherent plateau -> locked plateau), from a sweep sorted by c."""
    c = np.asarray(c, np.float64)
    s = np.convolve(np.asarray(std_r, np.float64), np.ones(3) / 3, mode="same")
    s[0], s[-1] = std_r[0], std_r[-1]
    q = max(3, len(s) // 4)
    top, bot = np.max(s[:q]), np.min(s[-q:])
    frac = (s - bot) / max(top - bot, 1e-30)
    i_hi = int(np.argmax(frac < hi))
    i_lo = int(np.argmax(frac < lo))
    return float(c[max(i_hi - 1, 0)]), float(c[max(i_lo, i_hi)])
