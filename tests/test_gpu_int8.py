"""Dense adjacency stored as the integers N*A in int8 (KURA_ADJ_I8).

The reference's volcano rule makes N*A_ij an integer in [-K, K], so int8 storage is exact:
the adjacency read back is bit-identical to the float32 one, the RHS differs from the
float32 path only by where 1/N is applied (one rounding), and whole runs meet the same
FP64-oracle tolerance as the float32 path.
"""
import numpy as np
import pytest

from helpers import cauchy_inputs, normal_inputs

pytestmark = pytest.mark.gpu

DENSE = 0


def network(native, n, k, om, storage, seed=2, c=3.0, batch=1):
    net = native.Network(n, k=k, coupling=DENSE, seed=seed, batch=batch, dense_level=0, adj_storage=storage)
    net.set_frequencies(om)
    net.generate_adjacency()
    for b in range(batch):
        net.set_coupling(b, c)
    return net


@pytest.mark.parametrize("n,k", [(1, 1), (100, 5), (1000, 6), (4099, 8), (513, 127)])
def test_int8_adjacency_bit_exact(native, oracle_lib, n, k):
    _, om = normal_inputs(n, 1)
    net = network(native, n, k, om, native.ADJ_I8, seed=4)
    a = net.adjacency()
    ref = oracle_lib.volcano_adjacency(4, n, k, fp64=False)
    assert np.array_equal(a.view(np.uint32), ref.view(np.uint32))
    net.close()


@pytest.mark.parametrize("n,batch", [(33, 1), (700, 1), (3000, 1), (5000, 1), (21000, 1), (2000, 8)])
def test_int8_rhs_matches_float32_storage(native, n, batch):
    th, om = cauchy_inputs(n, 9)
    out = []
    for storage in (native.ADJ_F32, native.ADJ_I8):
        net = network(native, n, 5, om, storage, batch=batch)
        for b in range(batch):
            net.set_state(b, th + b, 0.0, 0.01)
        out.append([net.rhs(b, th + np.float32(0.3 * b)) for b in range(batch)])
        net.close()
    for (f32, c32), (f8, c8) in zip(*out):
        scale = np.max(np.abs(c32)) + 1e-30
        assert np.max(np.abs(c8 - c32)) <= 4e-6 * scale + 1e-7
        assert np.all(np.abs(f8 - f32) <= 4e-6 * (scale * 3 + np.abs(f32)) + 1e-6)


@pytest.mark.parametrize("kind,n", [("cauchy", 64), ("normal", 1000), ("normal", 5000)])
def test_int8_run_matches_fp64_oracle(native, oracle_lib, kind, n):
    th, om = cauchy_inputs(n, 31 + n) if kind == "cauchy" else normal_inputs(n, 31 + n, init=2 * np.pi)
    net = network(native, n, 5, om, native.ADJ_I8, seed=2)
    net.set_state(0, th, 0.0, 0.01)
    net.set_horizon(10.0, 1.0, True)
    net.run()
    r = net.order(0)
    net.close()
    kw = dict(k=5, c1=3.0, seed=2, t1=10.0, dt=1.0)
    ref = oracle_lib.run(th, om, fp64=True, **kw)
    alts = [oracle_lib.run(th, om, fp64=True, h0=0.01 * (1 + e), **kw) for e in (1e-9, -1e-9)]
    r32 = oracle_lib.run(th, om, fp64=False, **kw)
    scale = np.max([np.abs(a.order - ref.order) for a in alts + [r32]], axis=0)
    assert r.size == ref.order.size == 11
    assert np.all(np.abs(r - ref.order) <= 1e-4 + 4 * scale), np.max(np.abs(r - ref.order))


def test_int8_set_adjacency_accepts_integer_multiples_only(native, oracle_lib):
    n = 300
    _, om = normal_inputs(n, 5)
    net = native.Network(n, k=4, coupling=DENSE, seed=1, adj_storage=native.ADJ_I8)
    ref = oracle_lib.volcano_adjacency(7, n, 4, fp64=False)  # as the reference's adj.dat holds it
    net.set_adjacency(ref)
    assert np.array_equal(net.adjacency().view(np.uint32), ref.view(np.uint32))
    bad = ref.copy()
    bad[3, 5] += np.float32(1e-3)
    with pytest.raises(native.KuraError) as e:
        net.set_adjacency(bad)
    assert e.value.code == -7
    net.close()
    with pytest.raises(native.KuraError) as e:
        native.Network(n, k=200, coupling=DENSE, adj_storage=native.ADJ_I8)
    assert e.value.code == -7
