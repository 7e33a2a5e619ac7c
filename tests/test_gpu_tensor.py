"""The shared-adjacency ensemble on tcgen05 tensor cores against the FP64 oracle.

The adjacency enters the GEMM as N*A in BF16 (exact integers for the volcano rule; a
general adjacency as BF16 hi + lo), the phases as BF16 hi + lo of (cos, sin), with FP32
accumulation.  Couplings therefore agree with the oracle to about 2^-16 of their
magnitude, and whole runs to the tolerances of the other parity tests.
"""
import numpy as np
import pytest

from helpers import cauchy_inputs, normal_inputs

pytestmark = pytest.mark.gpu
DENSE = 0
TENSOR = 2


def make(native, n, k, thetas, omega, cs, seed=1, t1=10.0, dt=1.0, adj=None, atol=1e-6, h0=None):
    B = len(thetas)
    net = native.Network(n, k=k, coupling=DENSE, batch=B, seed=seed, atol=atol, dense_level=0, engine=TENSOR)
    net.set_frequencies(omega)
    if adj is None:
        net.generate_adjacency()
    else:
        net.set_adjacency(adj)
    for b in range(B):
        net.set_coupling(b, cs[b])
        net.set_state(b, thetas[b], 0.0, dt / 100 if h0 is None else h0)
    net.set_horizon(t1, dt, True)
    return net


@pytest.mark.parametrize("n,k", [(100, 5), (300, 300), (1000, 6)])
def test_tensor_adjacency_bit_exact(native, oracle_lib, n, k):
    _, om = normal_inputs(n, 1)
    net = make(native, n, k, [om * 0] * 16, om, [1.0] * 16, seed=9)
    a = net.adjacency()
    ref = oracle_lib.volcano_adjacency(9, n, k, fp64=False)
    assert np.array_equal(a.view(np.uint32), ref.view(np.uint32))
    net.close()


# (25600, 128): 200 two-tile units on 152 SMs, so the GEMM runs its last rows as one-tile units
@pytest.mark.parametrize("n,batch,k", [(130, 16, 5), (700, 40, 5), (384, 128, 300), (25600, 128, 5)])
def test_tensor_rhs_matches_oracle(native, oracle_lib, n, batch, k):
    th, om = cauchy_inputs(n, 3)
    thetas = [(th + 0.1 * b).astype(np.float32) for b in range(batch)]
    net = make(native, n, k, thetas, om, [2.5] * batch, seed=3)
    for b in (0, batch // 2, batch - 1):
        f, cp = net.rhs(b, thetas[b])
        # the rank-K form builds the same matrix as the stored volcano adjacency
        fr, cpr = oracle_lib.rhs(thetas[b], om, k=k, c1=2.5, seed=3, fp64=True, onthefly=n > 4096)
        scale = np.max(np.abs(cpr)) + 1e-3
        assert np.max(np.abs(cp - cpr)) <= 3e-5 * scale + 1e-7, np.max(np.abs(cp - cpr))
        assert np.all(np.abs(f - fr) <= 1e-4 * scale + 1e-6 * np.abs(fr))
    net.close()


def test_tensor_general_adjacency_split(native, oracle_lib):
    n, batch = 200, 16
    rng = np.random.default_rng(5)
    adj = (rng.standard_normal((n, n)) / n).astype(np.float32)
    th, om = normal_inputs(n, 4)
    thetas = [(th + 0.2 * b).astype(np.float32) for b in range(batch)]
    net = make(native, n, 5, thetas, om, [1.5] * batch, adj=adj)
    back = net.adjacency()
    # N*A stored as BF16 hi + lo: 16 significant bits, about 2^-16 relative per entry
    assert np.all(np.abs(back - adj) <= 2.0 ** -15 * np.abs(adj) + 1e-12)
    f, cp = net.rhs(3, thetas[3])
    fr, cpr = oracle_lib.rhs(thetas[3], om, k=5, c1=1.5, adj=adj.astype(np.float64), fp64=True)
    assert np.max(np.abs(cp - cpr)) <= 3e-5 * np.max(np.abs(cpr))
    net.close()


@pytest.mark.parametrize("n,batch", [(256, 16), (1000, 24)])
def test_tensor_runs_match_fp64(native, oracle_lib, n, batch):
    _, om = normal_inputs(n, 11)
    thetas = [normal_inputs(n, 100 + b, init=2 * np.pi)[0] for b in range(batch)]
    cs = [1.0 + 0.25 * (b % 9) for b in range(batch)]
    net = make(native, n, 5, thetas, om, cs, seed=2, t1=10.0, dt=1.0)
    net.run()
    st = net.stats()
    assert st["accepted"] > 0
    for b in (0, batch // 3, batch - 1):
        r = net.order(b)
        ref = oracle_lib.run(thetas[b], om, k=5, c1=cs[b], seed=2, fp64=True, t1=10.0, dt=1.0)
        r32 = oracle_lib.run(thetas[b], om, k=5, c1=cs[b], seed=2, fp64=False, t1=10.0, dt=1.0)
        assert r.size == ref.order.size == 11
        env = np.abs(r32.order - ref.order)
        assert np.all(np.abs(r - ref.order) <= 1e-4 + 4 * env), (b, np.max(np.abs(r - ref.order)))
    th_end, t_end, _ = net.state(0)
    assert t_end >= 10.0
    net.close()


def test_tensor_batch_128_long_horizon(native, oracle_lib):
    n, batch = 512, 128
    _, om = normal_inputs(n, 21)
    thetas = [normal_inputs(n, 200 + b, init=2 * np.pi)[0] for b in range(batch)]
    cs = [3.0] * batch
    net = make(native, n, 5, thetas, om, cs, seed=4, t1=40.0, dt=1.0)
    net.run()
    for b in (0, 63, 127):
        r = net.order(b)
        ref = oracle_lib.run(thetas[b], om, k=5, c1=3.0, seed=4, fp64=True, t1=40.0, dt=1.0)
        assert abs(r.mean() - ref.order.mean()) < 1e-3
    net.close()


def test_tensor_rejects_unsupported(native):
    with pytest.raises(native.KuraError):
        native.Network(100, k=5, coupling=1, batch=16, engine=TENSOR)  # volcano coupling
    with pytest.raises(native.KuraError):
        native.Network(100, k=5, coupling=DENSE, batch=16, engine=TENSOR, dense_level=1)


def test_auto_engine_choice(native):
    """KURA_ENGINE_AUTO: the tensor engine (it reports grid 0) for a dense batch of two or more
    that keeps only r, and for any dense batch above 8; the persistent kernel for one trajectory,
    for per-step records (dense level >= 1), for the int8 adjacency and for the -A coupling."""
    def grid(**kw):
        net = native.Network(300, k=5, **kw)
        g = net.stats()["grid"]
        net.close()
        return g
    assert grid(coupling=DENSE, batch=2, dense_level=0) == 0
    assert grid(coupling=DENSE, batch=16, dense_level=0) == 0
    assert grid(coupling=DENSE, batch=1, dense_level=0) > 0
    assert grid(coupling=DENSE, batch=4, dense_level=1) > 0
    assert grid(coupling=DENSE, batch=4, dense_level=0, adj_storage=native.ADJ_I8) > 0
    assert grid(coupling=1, batch=4, dense_level=0) > 0
