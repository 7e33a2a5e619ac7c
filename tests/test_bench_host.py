"""bench.py's host arithmetic on the CPU: the seeded multi-network workload and the roofline
fields of the JSON line (algorithmic bytes or flops per unit over the kernel time)."""
import json
import os
import types

import numpy as np

import bench


def test_multi_inputs_are_seeded_and_in_range():
    w = bench.WORKLOADS["multi512"]
    a = bench.multi_inputs(w, bench.instance_seed(0))
    b = bench.multi_inputs(w, bench.instance_seed(0))
    ns, ks, seeds, cs, ths, oms = a
    assert len(ns) == 512 and int(ns.sum()) == 3135408
    assert ns.min() >= 1000 and ns.max() <= 20000
    assert ks.min() >= 2 and ks.max() <= 8 and cs.min() >= 0.0 and cs.max() <= 6.0
    assert all(t.size == n and o.size == n for t, o, n in zip(ths, oms, ns))
    assert all(np.array_equal(x, y) for x, y in zip(a[4] + a[5], b[4] + b[5]))
    other = bench.multi_inputs(w, bench.instance_seed(1))  # another rank's instance
    assert not np.array_equal(other[0], ns)


def _args(workload, steps):
    return types.SimpleNamespace(workload=workload, steps=steps)


def test_dense_roofline_counts_a_once_per_rhs():
    w = bench.WORKLOADS["dense65536"]
    n = w["n"]
    res = dict(kernel_ms=90.0, launches=1, acc_per_step=6)
    r = bench.roofline(w, res, _args("dense65536", 1))
    expect = 24.0 * n * 6 * n / 0.090 / 1e9  # 6 RHS x 4N^2 bytes per accepted step
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert abs(r["achieved"] - round(expect, 1)) < 0.11
    assert abs(r["frac"] - round(r["achieved"] / r["peak"], 4)) < 1e-4
    prof = json.load(open(os.path.join(bench.ROOT, "profiles", "traffic.json")))["dense65536"]
    assert abs(r["traffic"] - prof["bytes_per_accepted_osc_step"] * 6 * n) < 1.0


def test_int8_roofline_counts_one_byte_per_entry():
    w = bench.WORKLOADS["dense65536i8"]
    n = w["n"]
    r = bench.roofline(w, dict(kernel_ms=39.0, launches=1, acc_per_step=6), _args("dense65536i8", 1))
    assert abs(r["bytes_per_unit"] - 6.0 * n) < 1e-6


def test_tensor_roofline_counts_algorithmic_flops_per_gemm_launch():
    w = bench.WORKLOADS["ensemble65536"]
    n, B = w["n"], len(w["cs"])
    d = dict(accepted=128 * 70, coupling_ms=6 * 2.9, coupling_launches=6)
    r = bench.roofline_tensor(n, B, d, step_ms=1500.0)
    flops = 4.0 * n * n * B  # one RHS of every trajectory: 2 columns x 2 flops x N^2
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert abs(r["achieved"] - round(flops / 2.9e-3 / 1e12, 1)) < 0.051
    assert r["issued_flops_per_launch"] == 2 * r["flops_per_launch"] == 2 * flops
    assert abs(r["whole_step_tflops"] - round(24.0 * n * 128 * 70 * n / 1.5 / 1e12, 1)) < 0.051
    # a batch of 8 (padded to 16 columns) reads the same adjacency for 1/16 of the flops: HBM-bound
    r8 = bench.roofline_tensor(n, 8, d, step_ms=1500.0)
    assert r8["bound"] == "hbm" and r8["unit"] == "GB/s"
    assert abs(r8["achieved"] - round(2.0 * n * n / 2.9e-3 / 1e9, 1)) < 0.051


def test_window_inputs_share_trajectory_zero():
    from oracle import kora
    w = bench.WORKLOADS["ensemble65536"]
    small = dict(w, n=1000, cs=[3.0] * 4)
    th4, om4 = bench.window_inputs(small, 1, kora.host_random_inputs)
    th1, om1 = bench.window_inputs(dict(small, cs=[3.0]), 1, kora.host_random_inputs)
    assert np.array_equal(th4[0], th1[0]) and np.array_equal(om4, om1)
    assert all(t.min() >= 0 and t.max() < 2 * np.pi for t in th4)
    assert not np.array_equal(th4[0], th4[1])


def test_volcano_roofline_reports_issue_with_the_state_bytes_beside():
    w = bench.WORKLOADS["volcano200k"]
    r = bench.roofline(w, dict(kernel_ms=39.9, launches=1, acc_per_step=1023, sms=152,
                               clocks={"sm_mhz": 2070.0}), _args("volcano200k", 1))
    # reported against instruction issue; the nominal state-traffic figure rides along
    assert r["bound"] == "issue"
    h = r["hbm_nominal"]
    assert h["bytes_per_unit"] == bench.STATE_BYTES == 150.0
    assert abs(h["achieved"] - round(150.0 * 1023 * w["n"] / 0.0399 / 1e9, 1)) < 0.11
    rate = 1023 * w["n"] / 0.0399
    assert abs(r["frac"] - r["instructions_per_unit"] * rate / (4 * 152 * 2070e6)) < 1e-4


def test_issue_roofline_counts_instructions_per_unit():
    """An issue-bound kernel: warp instructions per accepted oscillator-step (the ncu count in
    profiles/issue.json) times the rate, over 4 issue slots per SM and cycle."""
    t = json.load(open(os.path.join(bench.ROOT, "profiles", "issue.json")))["volcano200k"]
    r = bench.issue_roofline("volcano200k", 5e9, {"sm_mhz": 2000.0}, sms=152)
    peak = 4 * 152 * 2000e6
    assert r["bound"] == "issue"
    assert abs(r["achieved"] - t["warp_instructions_per_accepted_osc_step"] * 5e9 / 1e9) < 0.01
    assert abs(r["frac"] - t["warp_instructions_per_accepted_osc_step"] * 5e9 / peak) < 1e-4
    assert bench.issue_roofline("no-such-workload", 5e9, None, sms=152) is None
