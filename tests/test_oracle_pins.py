"""Pins of the CPU oracle against the reference's own data and published vectors.

The reference repository has no tests; its data/ directory is the only ground
truth.  These tests check the oracle (oracle/kora_core.hpp) against it:
  * frequencies.dat of seed 1 (normal and Cauchy) byte for byte,
  * the uncoupled (K=0) end state theta = omega * t in fs.dat,
  * avgorder.npy of the uncoupled runs = the seed average of |mean exp(i omega t)|,
  * the published Philox4x32-10 known-answer vectors (Random123 kat_vectors),
and the oracle's own consistency (volcano rule, FP32 vs FP64, -A vs dense).
"""
import hashlib
import json

import numpy as np
import pytest

from helpers import golden


def test_golden_manifest_digests():
    man = json.load(open(golden("manifest.json")))
    assert len(man) >= 13
    for name, info in man.items():
        assert hashlib.sha256(open(golden(name), "rb").read()).hexdigest() == info["sha256"], name


@pytest.mark.parametrize("ctr,key,expect", [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
])
def test_philox_known_answers(oracle_lib, ctr, key, expect):
    assert list(oracle_lib.philox4x32_10(ctr, key)) == expect


def test_philox_stream_layout(oracle_lib):
    # element q of the stream is word q%4 of block q/4 (the curand_init(seed,0,0) stream)
    kora = oracle_lib
    for seed in (1, 7, -3):
        s = seed & 0xFFFFFFFFFFFFFFFF
        key = [s & 0xFFFFFFFF, s >> 32]
        for q in (0, 1, 2, 3, 4, 9, 12345, 2**33 + 5):
            blk = kora.philox4x32_10([q // 4 & 0xFFFFFFFF, q // 4 >> 32, 0, 0], key)
            assert kora.lib().kora_philox_stream_word(seed, q) == blk[q % 4]


@pytest.mark.parametrize("K", [0, 2, 5000])
@pytest.mark.parametrize("normal", [True, False])
def test_frequencies_byte_exact(oracle_lib, K, normal):
    name = "%s_K%d_seed1_frequencies.dat" % ("normal" if normal else "cauchy", K)
    ref = np.fromfile(golden(name), np.float32)
    _, om = oracle_lib.host_random_inputs(1, ref.size, 0.0, 1.0, normal)
    assert np.array_equal(om.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("normal", [True, False])
def test_uncoupled_fs_known_answer(oracle_lib, normal):
    fs = np.fromfile(golden("%s_K0_seed1_fs.dat" % ("normal" if normal else "cauchy")), np.float32)
    om = np.fromfile(golden("%s_K0_seed1_frequencies.dat" % ("normal" if normal else "cauchy")), np.float32)
    n = om.size
    assert fs.size == n + 2
    t = np.float64(fs[n])
    theta = fs[:n].astype(np.float64)
    exact = om.astype(np.float64) * t
    # float32 storage: error bounded by a few ulps of |omega t|
    tol = 4 * np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64) + 1e-4
    assert np.all(np.abs(theta - exact) <= tol)


@pytest.mark.parametrize("normal", [True, False])
def test_uncoupled_avgorder_is_seed_average(oracle_lib, normal):
    """avgorder(N=5000, K=0) equals the mean over seeds 1..750 of |<exp(i omega t)>|."""
    avg = np.load(golden("%s_N5000_K0_avgorder.npy" % ("normal" if normal else "cauchy")))
    idx = np.array([1, 10, 37, 100, 250, 500, 2000, 10000])
    t = (np.float32(0.01) * idx.astype(np.float32)).astype(np.float64)
    acc = np.zeros(idx.size)
    for seed in range(1, 751):
        _, om = oracle_lib.host_random_inputs(seed, 5000, 0.0, 1.0, normal)
        ph = np.outer(t, om.astype(np.float64))
        acc += np.abs(np.exp(1j * ph).mean(1))
    mean = acc / 750
    assert avg[0] == pytest.approx(1.0, abs=1e-6)
    assert np.max(np.abs(mean - avg[idx])) < 5e-5


def test_volcano_rule_integer_symmetric(oracle_lib):
    kora = oracle_lib
    n, k = 60, 5
    a = kora.volcano_adjacency(3, n, k, fp64=True)
    u = kora.volcano_factor(3, n, k).astype(np.float64)
    s = np.array([(-1) ** m for m in range(k)], np.float64)
    expect = (u.T * s) @ u / n
    assert np.array_equal(a, expect)
    assert np.array_equal(a, a.T)
    ki = a * n
    assert np.allclose(ki, np.round(ki)) and np.abs(ki).max() <= k
    a32 = kora.volcano_adjacency(3, n, k, fp64=False)
    assert np.array_equal(a32, (np.round(ki).astype(np.float32) * np.float32(1.0 / n)).astype(np.float32)) or \
        np.array_equal(a32, (np.round(ki).astype(np.float32) * (np.float32(1) / np.float32(n))))


def test_oracle_onthefly_equals_dense(oracle_lib):
    kora = oracle_lib
    n = 300
    rng = np.random.default_rng(0)
    y = rng.random(n) * 6.28
    om = rng.standard_normal(n)
    f1, c1 = kora.rhs(y, om, k=5, c1=3.0, onthefly=True, seed=9, fp64=True)
    f2, c2 = kora.rhs(y, om, k=5, c1=3.0, onthefly=False, seed=9, fp64=True)
    assert np.allclose(f1, f2, atol=1e-12) and np.allclose(c1, c2, atol=1e-12)


def test_oracle_rhs_matches_numpy_restatement(oracle_lib):
    # f_i = omega_i + c sum_j A_ij sin(theta_j - theta_i)... with the reference's sign:
    # f_i = omega_i + c (sin_i (A cos)_i - cos_i (A sin)_i) = omega_i + c sum_j A_ij sin(theta_i - theta_j)
    kora = oracle_lib
    n = 200
    rng = np.random.default_rng(1)
    y = rng.random(n) * 6.28
    om = rng.standard_normal(n)
    A = kora.volcano_adjacency(5, n, 4, fp64=True)
    f, cp = kora.rhs(y, om, k=4, c1=2.5, adj=A, fp64=True)
    expect = om + 2.5 * (A * np.sin(y[:, None] - y[None, :])).sum(1)
    assert np.allclose(f, expect, atol=1e-12)
    assert np.allclose(cp[0::2], A @ np.cos(y)) and np.allclose(cp[1::2], A @ np.sin(y))


def test_oracle_uncoupled_order_analytic(oracle_lib):
    kora = oracle_lib
    th, om = kora.host_random_inputs(4, 500, 0.0, 1.0, True)
    res = kora.run(th, om, k=0, c1=1.75, fp64=True, t1=5.0, dt=0.01, dense=1)
    t = (np.float64(0.01) * np.arange(1, 501))
    analytic = np.abs(np.exp(1j * np.outer(t, om.astype(np.float64))).mean(1))
    assert res.order.size == 501
    assert np.max(np.abs(res.order[1:] - analytic)) < 1e-10
    assert np.allclose(res.thetas[1:], np.outer(t, om.astype(np.float64)), atol=1e-9)


def test_oracle_fp32_tracks_fp64(oracle_lib):
    kora = oracle_lib
    from helpers import cauchy_inputs
    th, om = cauchy_inputs(256, 11)
    r64 = kora.run(th, om, k=5, c1=3.0, seed=2, fp64=True, t1=10, dt=1, dense=1)
    r32 = kora.run(th, om, k=5, c1=3.0, seed=2, fp64=False, t1=10, dt=1, dense=1)
    assert abs(r64.steps - r32.steps) <= max(3, r64.steps // 50)
    assert np.max(np.abs(r64.order - r32.order)) < 1e-4
    # the final record interpolates with k1 replaced by k7, so it differs from the last output row
    assert r64.final_theta.size == 256
    assert np.max(np.abs(r64.final_theta - r64.thetas[-1])) > 0
