"""Many independent volcano networks of uneven size in one launch (kura_multi_*).

Every network of a batch is checked on its own against the FP64 oracle run of the same
network (the reference program run once per network with -A), with the tolerance of the
single-network runs: r within 1e-4, widened where the network itself amplifies rounding
(by the float32 oracle's deviation and the FP64 oracle's spread under a 1e-9 change of the
first step).  The launch shape (cluster size, block size) changes summation order only,
and the same shape twice gives bitwise the same records.
"""
import numpy as np
import pytest

from helpers import cauchy_inputs, normal_inputs

pytestmark = pytest.mark.gpu


def networks(count, seed, nmin, nmax, kind="cauchy"):
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(nmin), np.log(nmax), count)).astype(np.int64)
    ks = rng.integers(2, 9, count)
    cs = rng.uniform(0.0, 6.0, count).astype(np.float32)
    seeds = rng.integers(1, 100000, count)
    ths, oms = [], []
    for i in range(count):
        if kind == "cauchy":
            th, om = cauchy_inputs(int(ns[i]), seed * 1000 + i)
        else:
            th, om = normal_inputs(int(ns[i]), seed * 1000 + i, init=2 * np.pi)
        ths.append(th)
        oms.append(om)
    return ns, ks, seeds, cs, ths, oms


def oracle_envelope(oracle_lib, th, om, k, c, seed, t1, dt):
    kw = dict(k=int(k), c1=float(c), onthefly=True, seed=int(seed), t1=t1, dt=dt)
    ref = oracle_lib.run(th, om, fp64=True, **kw)
    alts = [oracle_lib.run(th, om, fp64=True, h0=dt / 100 * (1 + e), **kw) for e in (1e-9, -1e-9)]
    r32 = oracle_lib.run(th, om, fp64=False, **kw)
    scale = np.max([np.abs(a.order - ref.order) for a in alts + [r32]], axis=0)
    return ref, 1e-4 + 4 * scale


def test_uneven_networks_match_fp64_oracle(native, oracle_lib):
    ns, ks, seeds, cs, ths, oms = networks(8, 3, 40, 1500)
    ns[0], ns[1] = 1, 2  # the smallest networks the reference accepts
    ths[0], oms[0] = ths[0][:1], oms[0][:1]
    ths[1], oms[1] = ths[1][:2], oms[1][:2]
    t1, dt = 10.0, 1.0
    with native.MultiNetworks(ns, ks, seeds, cs, t1, dt, cluster_size=2, block_threads=256) as m:
        order, thetas, acc = m.integrate(oms, ths)
        st = m.stats()
    assert order.shape == (8, 11)
    assert st["cluster_size"] == 2 and st["block_threads"] == 256 and st["grid"] >= 2
    assert st["accepted"] == acc.sum() and st["osc_steps"] == pytest.approx(float((acc * ns).sum()))
    for i in range(8):
        ref, tol = oracle_envelope(oracle_lib, ths[i], oms[i], ks[i], cs[i], seeds[i], t1, dt)
        assert ref.order.size == 11
        assert np.all(np.abs(order[i] - ref.order) <= tol), (i, ns[i], np.max(np.abs(order[i] - ref.order) - tol))
        assert abs(acc[i] - ref.steps) <= max(2, ref.steps // 50), (i, acc[i], ref.steps)
        assert thetas[i].size == ns[i]


def test_matches_single_network_engine(native):
    """One network through the multi-network launch and through the persistent
    single-network kernel: the same arithmetic up to the order of the sums."""
    n = 6000
    th, om = normal_inputs(n, 17, init=2 * np.pi)
    with native.MultiNetworks([n], [5], [9], [3.0], 10.0, 1.0, cluster_size=4, block_threads=512) as m:
        order, thetas, acc = m.integrate(om, th)
    net = native.Network(n, k=5, coupling=1, seed=9, dense_level=0)
    net.set_frequencies(om)
    net.set_coupling(0, 3.0)
    net.set_state(0, th, 0.0, 0.01)
    net.set_horizon(10.0, 1.0, True)
    net.run()
    r = net.order(0)
    st = net.stats()
    net.close()
    assert np.max(np.abs(order[0] - r)) < 2e-5
    assert abs(int(acc[0]) - st["accepted"]) <= 2


@pytest.mark.parametrize("shape", [(1, 256), (2, 512), (4, 1024), (8, 512)])
def test_launch_shapes_agree(native, shape):
    """Config-3 sizes (N log-uniform in [1000, 20000], K in 2..8, c in [0, 6], Cauchy omega)
    on a short horizon: every shape gives the same records to rounding, and a second
    integration on the same handle is bitwise identical (graph replay)."""
    ns, ks, seeds, cs, ths, oms = networks(24, 5, 1000, 20000)
    t1, dt = 0.02, 0.005
    with native.MultiNetworks(ns, ks, seeds, cs, t1, dt, cluster_size=1, block_threads=512) as m:
        base, _, _ = m.integrate(oms, ths, want_theta=False)
    with native.MultiNetworks(ns, ks, seeds, cs, t1, dt, cluster_size=shape[0], block_threads=shape[1]) as m:
        o1, th1, a1 = m.integrate(oms, ths)
        o2, th2, a2 = m.integrate(oms, ths)
    assert np.array_equal(o1.view(np.uint32), o2.view(np.uint32))
    assert all(np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(th1, th2))
    assert np.array_equal(a1, a2)
    assert np.max(np.abs(o1 - base)) < 2e-5


def test_autotuned_graph(native, oracle_lib):
    ns, ks, seeds, cs, ths, oms = networks(40, 7, 200, 6000, kind="normal")
    t1, dt = 2.0, 0.5
    with native.MultiNetworks(ns, ks, seeds, cs, t1, dt) as m:
        order, _, acc = m.integrate(oms, ths, want_theta=False)
        st = m.stats()
        order2, _, _ = m.integrate(oms, ths, want_theta=False)
    assert st["cluster_size"] in (1, 2, 4, 8, 16) and st["block_threads"] in (256, 512, 1024)
    assert st["tune_ms"] > 0 and st["kernel_ms"] > 0
    assert np.array_equal(order.view(np.uint32), order2.view(np.uint32))
    for i in (0, 13, 39):
        ref, tol = oracle_envelope(oracle_lib, ths[i], oms[i], ks[i], cs[i], seeds[i], t1, dt)
        assert np.all(np.abs(order[i] - ref.order) <= tol)


def test_uncoupled_known_answer(native):
    """K = 0 (and c = 0): the slopes vanish, every accepted step grows h tenfold, and the
    phases are theta0 + omega t exactly; r(t) follows in closed form."""
    ns = [300, 77]
    ths, oms = [], []
    for i, n in enumerate(ns):
        th, om = normal_inputs(n, 40 + i, init=2 * np.pi)
        ths.append(th)
        oms.append(om)
    t1, dt, h0 = 5.0, 0.5, 0.001
    with native.MultiNetworks(ns, [0, 3], [1, 1], [2.0, 0.0], t1, dt, h0=h0, cluster_size=1,
                              block_threads=256) as m:
        order, thetas, acc = m.integrate(oms, ths)
    t, h, steps = 0.0, h0, 0
    while t < t1:
        t += h
        h *= 10.0
        steps += 1
    te = np.float32(dt) * np.arange(int(np.float32(t1) / np.float32(dt)) + 1, dtype=np.float32)
    for i in range(2):
        assert acc[i] == steps
        exact = ths[i].astype(np.float64) + oms[i].astype(np.float64) * t
        assert np.all(np.abs(thetas[i] - exact) <= 4 * np.spacing(np.abs(exact).astype(np.float32)) + 1e-6)
        ph = ths[i][None, :].astype(np.float64) + oms[i][None, :].astype(np.float64) * te[:, None].astype(np.float64)
        r = np.abs(np.exp(1j * ph).mean(axis=1))
        assert np.max(np.abs(order[i] - r)) < 2e-6


def test_errors(native):
    with pytest.raises(native.KuraError) as e:
        native.MultiNetworks([100], [9], [1], [1.0], 1.0, 1.0)
    assert e.value.code == -7
    with pytest.raises(native.KuraError) as e:
        native.MultiNetworks([100], [5], [1], [1.0], 1.0, 1.0, cluster_size=3)
    assert e.value.code == -1
    th, om = normal_inputs(64, 2)
    with native.MultiNetworks([64], [5], [1], [3.0], 1.0, 1.0, atol=1e-30, cluster_size=1, block_threads=256) as m:
        with pytest.raises(native.KuraError) as e:
            m.integrate(om, th)
    assert e.value.code == -5


def test_heavy_network_runs_beside_the_main_launch(native, oracle_lib):
    """One network whose predicted work dwarfs the others' (a Cauchy outlier of |omega| ~ 1e3
    among small normal-frequency networks) is moved to a launch of its own in large clusters
    on a second stream.  Its records match the FP64 oracle, match the same network run alone
    to rounding, and a second integration is bitwise identical."""
    ns, ks, seeds, cs, ths, oms = networks(24, 31, 200, 600, kind="normal")
    th_h, om_h = normal_inputs(3000, 4242, init=2 * np.pi)
    om_h[17] = np.float32(1.2e3)  # one fast oscillator sets the step of the whole network
    ns = np.concatenate([ns, [3000]])
    ks = np.concatenate([ks, [5]])
    seeds = np.concatenate([seeds, [77]])
    cs = np.concatenate([cs, np.float32([4.0])]).astype(np.float32)
    ths, oms = ths + [th_h], oms + [om_h]
    t1, dt = 2.0, 0.25  # about 310 steps for the outlier network, at most 28 for the others
    with native.MultiNetworks(ns, ks, seeds, cs, t1, dt, cluster_size=1, block_threads=256) as m:
        order, _, acc = m.integrate(oms, ths, want_theta=False)
        st = m.stats()
        order2, _, _ = m.integrate(oms, ths, want_theta=False)
    assert st["heavy"] >= 1
    assert np.array_equal(order.view(np.uint32), order2.view(np.uint32))
    h = len(ns) - 1
    assert acc[h] > 10 * np.median(acc[:h])
    with native.MultiNetworks([3000], [5], [77], [4.0], t1, dt, cluster_size=1, block_threads=256) as m:
        alone, _, acc1 = m.integrate([om_h], [th_h], want_theta=False)
        assert m.stats()["heavy"] == 0
    assert np.max(np.abs(order[h] - alone[0])) < 2e-5
    assert abs(int(acc[h]) - int(acc1[0])) <= 2
    ref, tol = oracle_envelope(oracle_lib, th_h, om_h, 5, 4.0, 77, t1, dt)
    assert np.all(np.abs(order[h] - ref.order) <= tol)


@pytest.mark.parametrize("shape", [(1, 256), (16, 256)])
def test_tiny_networks_and_empty_ctas(native, oracle_lib, shape):
    """Networks smaller than the cluster leave CTAs without rows (n = 1 in a 16-CTA cluster);
    ragged sizes around a warp (31, 33) and K = 0 (uncoupled) ride along.  Every network
    matches its FP64 oracle run."""
    ns = np.array([1, 2, 31, 33, 64, 5], np.int64)
    ks = np.array([1, 2, 5, 8, 3, 0])
    seeds = np.array([3, 5, 7, 11, 13, 17])
    cs = np.float32([2.0, 5.0, 3.0, 4.5, 1.0, 3.0])
    ths, oms = [], []
    for i, n in enumerate(ns):
        th, om = normal_inputs(int(n), 900 + i, init=2 * np.pi)
        ths.append(th)
        oms.append(om)
    t1, dt = 4.0, 0.5
    with native.MultiNetworks(ns, ks, seeds, cs, t1, dt, cluster_size=shape[0], block_threads=shape[1]) as m:
        order, thetas, acc = m.integrate(oms, ths)
    for i in range(len(ns)):
        ref, tol = oracle_envelope(oracle_lib, ths[i], oms[i], ks[i], cs[i], seeds[i], t1, dt)
        assert order[i].size == ref.order.size
        assert np.all(np.abs(order[i] - ref.order) <= tol), i
        assert abs(int(acc[i]) - ref.steps) <= max(2, ref.steps // 50), (i, acc[i], ref.steps)
        assert thetas[i].size == ns[i]
