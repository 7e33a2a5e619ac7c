#!/usr/bin/env python
"""Benchmark: accepted DP45 steps x N x batch per second on one GB300.

Workload (default ``volcano200k``): the large on-the-fly volcano network,
N=200000 oscillators, rank K=5, adjacency regenerated from Philox (-A) and never
stored, coupling constant swept over c in {1,2,3,4,5} as a batch of 5
trajectories sharing the network, normal frequencies (glibc rand, seed 1, -n),
initial phases uniform in [0, pi) (seeded), t=50, output every dt=1,
atol=1e-6, rtol=0.  One bench step = the whole integration of all 5
trajectories from t=0 to t=50.  Synthetic inputs of that shape; nothing is read
from disk.

Arms:
  --impl native (default): libkura through its C ABI.  ``value`` times the
      integration with inputs already resident in HBM; ``e2e`` times the same
      through host buffers (frequencies and phases copied in from pinned memory,
      order parameter and final phases copied out, inside the timed region).
  --impl reference: the reference's CPU path, i.e. the oracle's restatement of the
      reference program (float32, reference arithmetic), on all host threads.

Multi-GPU: each rank integrates its own instance (network seed 1 + rank) of the
same workload; no collective on the data path (weak scaling).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "volcano200k": dict(n=200000, k=5, coupling=1, cs=[1.0, 2.0, 3.0, 4.0, 5.0], normal=True, init=np.pi,
                        t1=50.0, dt=1.0, atol=1e-6, rtol=0.0, shared_theta=True),
    # the reference's default dense case (configs: N=5000, K=5, c=3, Cauchy, theta0=0, t=100, dt=1)
    "dense5000": dict(n=5000, k=5, coupling=0, cs=[3.0], normal=False, init=0.0, t1=100.0, dt=1.0, atol=1e-6,
                      rtol=0.0, shared_theta=True, fresh=True),
    # the same with N*A stored as int8 (exact for the volcano rule): 25 MB, a quarter of the bytes per RHS
    "dense5000i8": dict(n=5000, k=5, coupling=0, cs=[3.0], normal=False, init=0.0, t1=100.0, dt=1.0, atol=1e-6,
                        rtol=0.0, shared_theta=True, fresh=True, adj_storage=1),
    # the plain FP32 path at N=65536 (17.2 GB adjacency read once per RHS; x8: shared by 8
    # trajectories of one pass), Cauchy omega, theta0 uniform in [0, 2pi); the Cauchy
    # outliers of N=65536 force steps of ~1e-4, so the horizon is short
    "dense65536": dict(n=65536, k=5, coupling=0, cs=[3.0], normal=False, init=2 * np.pi, t1=0.004, dt=0.001,
                       atol=1e-6, rtol=0.0, shared_theta=False),
    "dense65536x8": dict(n=65536, k=5, coupling=0, cs=[3.0] * 8, normal=False, init=2 * np.pi, t1=0.004,
                         dt=0.001, atol=1e-6, rtol=0.0, shared_theta=False),
    # the same network with N*A stored as int8 (exact for the volcano rule): 4.3 GB per RHS
    "dense65536i8": dict(n=65536, k=5, coupling=0, cs=[3.0], normal=False, init=2 * np.pi, t1=0.004, dt=0.001,
                         atol=1e-6, rtol=0.0, shared_theta=False, adj_storage=1),
    # the shared-adjacency ensemble on tensor cores: N=65536, K=5 dense volcano adjacency,
    # 128 trajectories with distinct theta0 uniform in [0, 2pi), shared Cauchy omega, c=3,
    # integrated toward t=20 with records every 0.01; one bench step is 64 step attempts of every
    # trajectory that continue the same integration (the warm-up steps start it from t=0).  The
    # plain FP32 path (`dense65536w`) runs trajectory 0 of the same inputs beside it.
    "ensemble65536": dict(kind="windows", n=65536, k=5, cs=[3.0] * 128, init=2 * np.pi, t1=20.0, dt=0.01,
                          attempts=64, atol=1e-6, rtol=0.0, engine="tensor", plain="dense65536w"),
    "dense65536w": dict(kind="windows", n=65536, k=5, cs=[3.0], init=2 * np.pi, t1=20.0, dt=0.01, attempts=64,
                        atol=1e-6, rtol=0.0, engine="persistent"),
    # the same ensemble at N=32768 (a 2.1 GB BF16 adjacency, larger than L2): profiling captures
    "ensemble32768": dict(kind="windows", n=32768, k=5, cs=[3.0] * 128, init=2 * np.pi, t1=20.0, dt=0.01,
                          attempts=192, atol=1e-6, rtol=0.0, engine="tensor"),
    # a batch of 8 on either engine (the choice KURA_ENGINE_AUTO makes for small dense batches)
    "ensemble65536x8": dict(kind="windows", n=65536, k=5, cs=[3.0] * 8, init=2 * np.pi, t1=20.0, dt=0.01,
                            attempts=128, atol=1e-6, rtol=0.0, engine="tensor", plain="dense65536w"),
    "dense65536x8w": dict(kind="windows", n=65536, k=5, cs=[3.0] * 8, init=2 * np.pi, t1=20.0, dt=0.01,
                          attempts=32, atol=1e-6, rtol=0.0, engine="persistent"),
    # the same ensemble at N=16384 (a 512 MiB BF16 adjacency, still larger than L2): profiling captures
    "ensemble16384": dict(n=16384, k=5, coupling=0, cs=[3.0] * 128, normal=False, init=2 * np.pi, t1=0.004,
                          dt=0.001, atol=1e-6, rtol=0.0, shared_theta=False, engine="tensor"),
    # 512 independent regenerated-volcano networks of uneven size in one launch: N log-uniform
    # in [1000, 20000], K uniform in 2..8, c uniform in [0, 6], Cauchy omega (scale 1), theta0
    # uniform in [0, 2pi), each with its own adaptive step, t=100, records every dt=1
    "multi512": dict(kind="multi", count=512, nmin=1000, nmax=20000, kmin=2, kmax=8, cmax=6.0, t1=100.0, dt=1.0,
                     atol=1e-6, rtol=0.0),
    # the learned sweep placement: 20000 training networks at N=10000 from the batched solver
    # (c uniform in [0, 6], K uniform in 2..8, frequency scale log-uniform in [0.5, 2], 10 %
    # Cauchy), a 4 x 256 MLP trained on them, then surrogate-guided sweeps of 64 points,
    # each verified by a DP45 run to t=60
    "surrogate": dict(kind="surrogate", networks=20000, n=10000, t1=60.0, cauchy_frac=0.1, epochs=60,
                      sweeps=[(5, 1.0, 0), (3, 0.7, 0), (8, 1.5, 0), (6, 1.5, 1)]),
    "dense16384": dict(n=16384, k=5, coupling=0, cs=[3.0], normal=False, init=2 * np.pi, t1=0.004, dt=0.001,
                       atol=1e-6, rtol=0.0, shared_theta=False),
    "dense16384i8": dict(n=16384, k=5, coupling=0, cs=[3.0], normal=False, init=2 * np.pi, t1=0.004, dt=0.001,
                         atol=1e-6, rtol=0.0, shared_theta=False, adj_storage=1),
    "dense16384x8": dict(n=16384, k=5, coupling=0, cs=[3.0] * 8, normal=False, init=2 * np.pi, t1=0.004,
                         dt=0.001, atol=1e-6, rtol=0.0, shared_theta=False),
}
# algorithmic bytes per accepted oscillator-step of the dominant kernel
#   volcano: the DP45 state a step moves in the reference design (~150 B)
#   dense:   6 RHS x 4N bytes of A per step, shared by the trajectories of one pass
STATE_BYTES = 150.0


def inputs(w, seed, host_rng=None):
    """Frequencies from glibc rand of `seed` (libkura's generator, or the oracle's byte-identical
    one for the reference arm, which loads no product library) and seeded theta0."""
    if host_rng is None:
        import kuramoto_gb300 as kg
        host_rng = kg.random_inputs
    n = w["n"]
    # a fresh start draws N values for theta0 before the frequencies (kuramoto.cu:498-541); a run
    # whose phases come from a file through -R draws only the frequencies
    _, om = host_rng(seed, n, 0.0, 1.0, w["normal"], gen_theta=bool(w.get("fresh")))
    rng = np.random.default_rng(seed)
    B = len(w["cs"])
    if w["shared_theta"]:
        th = (rng.random(n) * w["init"]).astype(np.float32)
        thetas = [th] * B
    else:
        thetas = [(rng.random(n) * w["init"]).astype(np.float32) for _ in range(B)]
    return thetas, om


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 2 + i and r[2 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def instance_seed(rank):
    """Each rank integrates its own network instance (weak scaling, no data exchange)."""
    return 1 + rank


def combine_ranks(units, ms, device):
    """Whole-job units (sum over ranks) and time (max over ranks)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(units), float(ms)
    t = torch.tensor([float(units), float(ms)], dtype=torch.float64, device=device)
    u = t[:1].clone()
    m = t[1:].clone()
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return float(u.item()), float(m.item())


def run_native(args, w):
    import torch
    import kuramoto_gb300 as kg

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    seed = instance_seed(rank)
    thetas, om = inputs(w, seed)
    n, B = w["n"], len(w["cs"])
    stream = torch.cuda.current_stream()
    eng = kg.ENGINE_TENSOR if w.get("engine") == "tensor" else kg.ENGINE_PERSISTENT
    net = kg.Network(n, k=w["k"], coupling=w["coupling"], batch=B, seed=seed, atol=w["atol"], rtol=w["rtol"],
                     dense_level=0, device=local, stream=stream.cuda_stream, adj_storage=w.get("adj_storage", 0),
                     engine=eng)
    net.set_frequencies(om)
    if w["coupling"] == 0:
        net.generate_adjacency()
    for b, c in enumerate(w["cs"]):
        net.set_coupling(b, c)
    dev_th = [torch.from_numpy(t).cuda() for t in thetas]
    h0 = w["dt"] / 100
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 129 MB L2

    def step_resident():
        for b in range(B):
            net.set_state_device(b, dev_th[b].data_ptr(), 0.0, h0)
        net.set_horizon(w["t1"], w["dt"], True)
        net.run()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step_resident()
    # ---- value: inputs resident in HBM, L2 flushed between steps (outside the events)
    st0 = net.stats()
    barrier()
    evs = []
    with Clocks(local) as clk:
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step_resident()
            e1.record(stream)
            evs.append((e0, e1))
        barrier()
        t_wall = time.perf_counter() - t_wall
    st1 = net.stats()
    ms = sum(a.elapsed_time(b) for a, b in evs)
    acc = st1["accepted"] * args.steps  # accepted steps of the last run, all trajectories
    acc_per_step = st1["accepted"]
    launches = st1["launches"] - st0["launches"]
    kernel_ms = st1["kernel_ms"] - st0["kernel_ms"]
    barriers = st1["barriers"] - st0["barriers"]
    units, ms = combine_ranks(acc_per_step * n * args.steps, ms, "cuda")
    value = units / (ms / 1e3)
    orders = [net.order(b) for b in range(B)]

    # ---- e2e: host buffers through the C ABI, copies inside the timed region.  Inputs and
    # the final phases live in pinned host memory (numpy views of pinned torch tensors)
    e2e_ms = 0.0
    h2d = d2h = 0

    om_pin = pinned(om)
    th_pin = [pinned(t) for t in thetas]
    fin_pin = [pinned(np.zeros(n, np.float32)) for _ in range(B)]
    for it in range(args.steps):
        flush.zero_()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        net.set_frequencies(om_pin)
        for b in range(B):
            net.set_state(b, th_pin[b], 0.0, h0)
        net.set_horizon(w["t1"], w["dt"], True)
        net.run()
        rs = [net.order(b) for b in range(B)]
        finals = [net.state(b, out=fin_pin[b])[0] for b in range(B)]
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms += e0.elapsed_time(e1)
        if it == 0:
            h2d = 4 * n + 4 * n * B
            d2h = sum(4 * r.size for r in rs) + 4 * n * B
    e2e_units, e2e_ms = combine_ranks(acc_per_step * n * args.steps, e2e_ms, "cuda")
    e2e_value = e2e_units / (e2e_ms / 1e3)
    net.close()
    res = dict(value=value, ms=ms, wall=t_wall, kernel_ms=kernel_ms, launches=launches, acc_per_step=acc_per_step,
               barriers=barriers,
               e2e_value=e2e_value, h2d=h2d, d2h=d2h, clocks=clk.summary(), orders=orders, thetas=thetas, om=om,
               rank=rank, ws=ws, B=B)
    return res


def issue_roofline(workload, osc_steps_per_s, clocks, sms=None):
    """Roofline of a kernel bound by instruction issue: warp instructions per accepted
    oscillator-step (one ncu count of the same kernel, profiles/issue.json) times the measured
    rate, against 4 issue slots per SM and cycle at the SM clock sampled during the run."""
    try:
        t = json.load(open(os.path.join(ROOT, "profiles", "issue.json"))).get(workload)
    except Exception:
        t = None
    if not t:
        return None
    if sms is None:
        try:
            import torch
            sms = torch.cuda.get_device_properties(0).multi_processor_count
        except Exception:
            return None
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
    peak = 4.0 * sms * mhz * 1e6
    ach = t["warp_instructions_per_accepted_osc_step"] * osc_steps_per_s
    return {"bound": "issue", "achieved": round(ach / 1e9, 2), "peak": round(peak / 1e9, 2),
            "unit": "G warp-instructions/s", "frac": round(ach / peak, 4),
            "peak_source": "4 issue slots x %d SMs x %.0f MHz (median SM clock of the run)" % (sms, mhz),
            "instructions_per_unit": t["warp_instructions_per_accepted_osc_step"],
            "ncu_issue_active": t["issue_active"], "instructions_source": t["source"]}


def roofline(w, res, args):
    import json as _json
    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    src = "measured" if "hbm_gbs" in peaks else "fallback"
    n = w["n"]
    if w.get("engine") == "tensor":
        # tensor-bound: algorithmic flops 24 N per accepted oscillator-step (2 products, 2 flop
        # per multiply-add, 6 RHS); the split-BF16 product issues 2x that (hi and lo columns).
        # The GEMMs run back to back for the whole step: the sustained bf16 figure applies.
        peak = peaks.get("bf16_tflops_sustained", 1700.0)
        run_s = res["kernel_ms"] / 1e3 / max(args.steps, 1)
        flops = 24.0 * n * res["acc_per_step"] * n / max(run_s, 1e-12)
        return {"bound": "tensor", "achieved": round(flops / 1e12, 2), "peak": peak, "unit": "TFLOP/s",
                "frac": round(flops / 1e12 / peak, 4), "traffic": None,
                "peak_source": "measured" if "bf16_tflops_sustained" in peaks else "fallback",
                "flops_per_unit": 24.0 * n, "issued_flops_per_unit": 48.0 * n,
                "kernel_ms_per_step": round(run_s * 1e3, 3)}
    kernel_s = res["kernel_ms"] / 1e3 / max(res["launches"], 1)
    acc_per_launch = res["acc_per_step"] * args.steps / max(res["launches"], 1)
    if w["coupling"] == 1:
        per_unit = STATE_BYTES
        bytes_per_launch = per_unit * acc_per_launch * n
    else:
        # 6 RHS x N entries of A per accepted step and oscillator: 4 bytes each (float32) or 1 (int8)
        per_unit = (6.0 if w.get("adj_storage") else 24.0) * n / len(w["cs"])
        bytes_per_launch = per_unit * acc_per_launch * n
    achieved = bytes_per_launch / kernel_s / 1e9
    traffic = None
    try:
        prof = _json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        t = prof.get(args.workload)
        if t:
            traffic = t["bytes_per_accepted_osc_step"] * acc_per_launch * n
    except Exception:
        pass
    out = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
           "frac": round(achieved / hbm, 4), "traffic": traffic, "peak_source": src,
           "bytes_per_unit": per_unit, "kernel_ms_per_launch": round(kernel_s * 1e3, 3)}
    if w["coupling"] == 1:
        # the regenerated coupling keeps its state in L2: instruction issue binds it, not DRAM
        iss = issue_roofline(args.workload, acc_per_launch * n / kernel_s, res.get("clocks"), res.get("sms"))
        if iss:
            iss["traffic"] = traffic
            iss["kernel_ms_per_launch"] = out["kernel_ms_per_launch"]
            iss["hbm_nominal"] = {k: out[k] for k in ("achieved", "peak", "unit", "frac", "bytes_per_unit")}
            out = iss
    if w["coupling"] == 1 and res.get("barriers"):
        # the DP45 state of this workload stays in L2, so DRAM does not bind it: every coupling
        # evaluation and every error norm is one grid barrier, and the time between barriers
        # (phase A, the gather, phase C at one CTA per SM) is what the kernel costs
        out["binding"] = {"kind": "latency: one grid barrier per coupling evaluation and per error norm",
                          "us_per_barrier_interval": round(res["kernel_ms"] * 1e3 / res["barriers"], 2),
                          "barriers_per_accepted_step": round(res["barriers"] / max(acc_per_launch *
                                                                                     res["launches"] /
                                                                                     len(w["cs"]), 1), 2)}
    return out


def multi_inputs(w, seed):
    """Seeded networks of the multi-network workload (sizes, ranks, couplings, Philox seeds)
    and their inputs, one array per network."""
    rng = np.random.default_rng(seed)
    count = w["count"]
    ns = np.exp(rng.uniform(np.log(w["nmin"]), np.log(w["nmax"]), count)).astype(np.int64)
    ks = rng.integers(w["kmin"], w["kmax"] + 1, count)
    cs = rng.uniform(0.0, w["cmax"], count).astype(np.float32)
    seeds = rng.integers(1, 1 << 30, count)
    ths = [(rng.random(int(n)) * 2 * np.pi).astype(np.float32) for n in ns]
    oms = [np.tan(np.pi * (rng.random(int(n)) - 0.5)).astype(np.float32) for n in ns]
    return ns, ks, seeds, cs, ths, oms


def pinned(a):
    """A float32 copy of `a` in pinned host memory (a numpy view of a pinned torch tensor)."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).pin_memory().numpy()


def run_multi(args, w):
    import torch
    import kuramoto_gb300 as kg

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    nets = multi_inputs(w, instance_seed(rank))
    ns, ks, seeds, cs, ths, oms = nets
    om = pinned(np.concatenate(oms))  # the e2e leg copies them in from pinned memory
    th = pinned(np.concatenate(ths))
    m = kg.MultiNetworks(ns, ks, seeds, cs, w["t1"], w["dt"], atol=w["atol"], rtol=w["rtol"], device=local)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 129 MB L2

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):  # the first one runs the autotuner and captures the graph
        order, _, acc = m.integrate(om, th, want_theta=False)
    barrier()
    # one timed step = one integration of every network.  `value` counts the device time of
    # the persistent launch (CUDA events on the library's stream around the graph launch,
    # inputs already in HBM); e2e times the whole synchronous call with host buffers (H2D
    # of omega and theta0, the launch, D2H of the records and the final phases)
    kern_ms = e2e_ms = osc = 0.0
    with Clocks(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            barrier()
            t0 = time.perf_counter()
            order, thetas, acc = m.integrate(om, th, want_theta=True)
            e2e_ms += (time.perf_counter() - t0) * 1e3
            st = m.stats()
            kern_ms += st["kernel_ms"]
            osc += st["osc_steps"]
    units, ms = combine_ranks(osc, kern_ms, "cuda")
    e2e_units, e2e_ms = combine_ranks(osc, e2e_ms, "cuda")
    tot = int(ns.sum())
    res = dict(value=units / (ms / 1e3), ms=ms, kernel_ms=kern_ms, launches=args.steps,
               e2e_value=e2e_units / (e2e_ms / 1e3), h2d=8 * tot, d2h=4 * order.size + 4 * tot + 8 * len(ns),
               clocks=clk.summary(), orders=order, nets=nets, osc_per_step=osc / args.steps,
               shape=(st["cluster_size"], st["block_threads"], st["grid"], st["heavy"]), tune_ms=st["tune_ms"],
               acc=acc)
    m.close()
    return res


def _multi_worker(job):
    """One network on one host core (the reference runs one process per network)."""
    from oracle import kora
    th, om, k, c, seed, t1, dt, atol, rtol = job
    r = kora.run(th, om, k=int(k), c1=float(c), onthefly=True, seed=int(seed), fp64=False, t1=t1, dt=dt, atol=atol,
                 rtol=rtol, threads=1)
    return r.steps * th.size


def multi_cpu(w, nets, threads, t1):
    """Every network of the workload to t1 on `threads` host processes, one network per task
    (spawned, so that no child inherits a CUDA context)."""
    import multiprocessing as mp
    ns, ks, seeds, cs, ths, oms = nets
    jobs = [(ths[i], oms[i], ks[i], cs[i], seeds[i], t1, w["dt"], w["atol"], w["rtol"]) for i in np.argsort(-ns)]
    with mp.get_context("spawn").Pool(threads) as pool:
        pool.map(_multi_worker, jobs[:threads], chunksize=1)  # children up and the oracle loaded
        t0 = time.perf_counter()
        osc = sum(pool.map(_multi_worker, jobs, chunksize=1))
        el = time.perf_counter() - t0
    return osc / el, el, osc


MULTI_CPU_T1 = 1.0  # horizon of the CPU sample of the multi-network workload (every network)


def main_multi(args, w):
    ws, rank, local = dist_env()
    config = {"workload": args.workload, "networks": w["count"],
              "n": "log-uniform [%d, %d]" % (w["nmin"], w["nmax"]), "k": "uniform %d..%d" % (w["kmin"], w["kmax"]),
              "coupling": "volcano-regenerated", "c": "uniform [0, %g]" % w["cmax"],
              "frequencies": "cauchy (scale 1)", "theta0": "uniform [0, 2pi)", "t1": w["t1"], "dt": w["dt"],
              "atol": w["atol"], "rtol": w["rtol"],
              "l2": "flushed between steps (512 MiB write); the networks' state (~225 MB) exceeds L2",
              "parallelism": "replicas" if ws > 1 else "single"}
    metric = "accepted DP45 steps x N x batch / s"
    threads = os.cpu_count() or 1
    sample = ("every one of the %d networks to t=%g (%g%% of the horizon), one network per task on %d host "
              "processes (the reference runs one process per network), float32 oracle restating the reference "
              "program" % (w["count"], MULTI_CPU_T1, 100 * MULTI_CPU_T1 / w["t1"], threads))
    if args.impl == "reference":
        if rank != 0:
            return
        nets = multi_inputs(w, 1)
        for _ in range(args.warmup):
            multi_cpu(w, nets, threads, MULTI_CPU_T1 / 4)
        osc = el = 0.0
        for _ in range(args.steps):
            v, e, o = multi_cpu(w, nets, threads, MULTI_CPU_T1)
            osc += o
            el += e
        value = osc / el
        print(json.dumps({"impl": "reference", "metric": metric, "value": value, "unit": "osc-steps/s",
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config,
                          "cpu_baseline": {"value": value, "unit": "osc-steps/s", "cores": threads, "kind": "port",
                                           "sample": sample},
                          "e2e": {"value": value, "unit": "osc-steps/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return
    res = run_multi(args, w)
    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    achieved = STATE_BYTES * res["osc_per_step"] / (res["kernel_ms"] / args.steps / 1e3) / 1e9
    traffic = None
    try:
        t = json.load(open(os.path.join(ROOT, "profiles", "traffic.json"))).get(args.workload)
        if t:
            traffic = t["bytes_per_accepted_osc_step"] * res["osc_per_step"]
    except Exception:
        pass
    line = {"metric": metric, "value": res["value"], "unit": "osc-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config}
    line["e2e"] = {"value": res["e2e_value"], "unit": "osc-steps/s", "h2d_bytes_per_step": res["h2d"],
                   "d2h_bytes_per_step": res["d2h"]}
    line["gpu_launches"] = res["launches"]
    rl = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
          "frac": round(achieved / hbm, 4), "traffic": traffic,
          "peak_source": "measured" if "hbm_gbs" in peaks else "fallback", "bytes_per_unit": STATE_BYTES}
    # the networks' state stays in L2: instruction issue and latency bind the kernel, not DRAM
    iss = issue_roofline(args.workload, res["osc_per_step"] / (res["kernel_ms"] / args.steps / 1e3), res["clocks"])
    if iss:
        iss["traffic"] = traffic
        iss["hbm_nominal"] = {k: rl[k] for k in ("achieved", "peak", "unit", "frac", "bytes_per_unit")}
        rl = iss
    line["roofline"] = dict(rl, **{
                        "kernel_ms_per_launch": round(res["kernel_ms"] / args.steps, 3),
                        "binding": {"kind": "latency: the networks' state stays in L2; the integration ends when "
                                            "its longest networks (the most accepted steps) end",
                                    "accepted_steps_max_network": int(res["acc"].max()),
                                    "us_per_step_of_longest_network": round(res["kernel_ms"] / args.steps * 1e3 /
                                                                            max(int(res["acc"].max()), 1), 3)}})
    line["clocks"] = res["clocks"]
    line["launch_shape"] = {"cluster_size": res["shape"][0], "block_threads": res["shape"][1],
                            "grid": res["shape"][2], "heavy_networks_in_large_clusters": res["shape"][3],
                            "autotune_trial_ms": round(res["tune_ms"], 3)}
    line["accepted_steps_per_network"] = {"mean": float(res["acc"].mean()), "max": int(res["acc"].max())}
    if not args.no_cpu:
        v, el, osc = multi_cpu(w, res["nets"], threads, MULTI_CPU_T1)
        line["cpu_baseline"] = {"value": v, "unit": "osc-steps/s", "cores": threads, "kind": "port",
                                "sample": sample + " (%.1f s)" % el}
        # r error of the two smallest networks against the FP64 oracle over the records t <= 10
        from oracle import kora
        ns, ks, seeds, cs, ths, oms = res["nets"]
        errs = []
        for i in np.argsort(ns)[:2]:
            r = kora.run(ths[i], oms[i], k=int(ks[i]), c1=float(cs[i]), onthefly=True, seed=int(seeds[i]),
                         fp64=True, t1=10.0, dt=w["dt"], atol=w["atol"], rtol=w["rtol"], threads=threads)
            errs.append(float(np.max(np.abs(r.order - res["orders"][i][:r.order.size]))))
        line["r_err_vs_fp64"] = max(errs)
    print(json.dumps(line))


def main_surrogate(args, w):
    """The learned part end to end on one GPU.  ``value`` is the batched solver's throughput
    while it generates the training data (the dominant cost); the other keys report the
    training, the held-out accuracy and, for each swept network, the DP45 verification and
    the gain over an even sweep."""
    ws, rank, local = dist_env()
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned component or batched "
                              "solver; its per-network CPU cost is the multi512 workload's reference arm"}))
        return
    import torch
    from kuramoto_gb300 import surrogate as S
    torch.cuda.set_device(local)
    rng = np.random.default_rng(instance_seed(rank))
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        X, Y, st = S.generate(w["networks"], w["n"], w["t1"], rng, device=local, cauchy_frac=w["cauchy_frac"])
        gen_wall = time.perf_counter() - t0
        nval = len(X) // 10
        sur = S.Surrogate(hidden=256, batch=512, seed=instance_seed(rank), device=local)
        losses, train_ms = sur.fit(X[nval:], Y[nval:], epochs=w["epochs"], lr=2e-3, lr_final=1e-4)
        pred = sur.predict(X[:nval])
        sweeps = []
        for (k, f, cauchy) in w["sweeps"]:
            seed = 1000 + len(sweeps)
            res = S.sweep(sur, w["n"], k, f, cauchy, seed, rng, npoints=64, candidates=64, t1=w["t1"], device=local)
            c = np.linspace(0, 6, 121).astype(np.float32)
            ones = np.ones(c.size)
            orders, st_dense = S.simulate(w["n"], c, (k * ones).astype(int), (seed * ones).astype(int),
                                          [res["theta0"]] * c.size, [res["omega"]] * c.size, w["t1"], device=local)
            lo, hi = S.transition_window(c, S.targets(orders, w["t1"])[:, 1])
            width = max(hi - lo, 0.05)
            inside = int(np.sum((res["points"] >= lo) & (res["points"] <= hi)))
            spent = res["osc_steps_full"] + res["osc_steps_short"]
            even_runs = 6.0 / (width / max(inside, 1))
            sweeps.append({"k": k, "f": f, "family": "cauchy" if cauchy else "normal",
                           "transition_window": [round(lo, 3), round(hi, 3)],
                           "points_in_window": inside, "even_points_in_window": round(64 * width / 6.0, 1),
                           "within_0.02": float(res["within_tol"].mean()),
                           "max_err_mean_r": float(res["err"][:, 0].max()),
                           "cost_vs_even_sweep_same_spacing": round(even_runs * res["osc_steps_full"] / 64 / spent, 2)})
        sur.close()
    steps_total = (len(X) - nval) // 512 * w["epochs"]
    mlp_flops = 6.0 * 512 * (64 * 256 + 2 * 256 * 256 + 256 * 64) * steps_total  # fwd + 2 bwd GEMMs per layer
    line = {"metric": "accepted DP45 steps x N x batch / s", "value": st["osc_steps"] / (st["kernel_ms"] / 1e3),
            "unit": "osc-steps/s", "n_gpus": ws, "steps": 1, "warmup": 0, "ms_per_step": st["kernel_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 solver, bf16 MLP",
            "data": "synthetic",
            "config": {"workload": args.workload, "networks": w["networks"], "n": w["n"], "t1": w["t1"],
                       "c": "uniform [0, 6]", "k": "uniform 2..8", "freq_scale": "log-uniform [0.5, 2]",
                       "cauchy_fraction": w["cauchy_frac"], "mlp": "14 -> 256 -> 256 -> 256 -> 2, SiLU",
                       "epochs": w["epochs"], "batch": 512, "l2": "not flushed (one pass)"},
            "e2e": {"value": st["osc_steps"] / gen_wall, "unit": "osc-steps/s", "h2d_bytes_per_step": 8 * len(X) * w["n"],
                    "d2h_bytes_per_step": 4 * len(X) * (int(w["t1"]) + 1)},
            "gpu_launches": 1 + steps_total * 19,
            "training": {"samples": len(X) - nval, "steps": steps_total, "device_ms": round(train_ms, 1),
                         "first_epoch_loss": float(losses[0]), "last_epoch_loss": float(losses[-1]),
                         "achieved_tflops": round(mlp_flops / (train_ms / 1e3) / 1e12, 3)},
            "holdout": {"networks": nval, "mean_r_within_0.02": float(np.mean(np.abs(pred[:, 0] - Y[:nval, 0]) <= 0.02)),
                        "std_r_r2": float(1 - np.mean((pred[:, 1] - Y[:nval, 1]) ** 2) / np.var(Y[:nval, 1]))},
            "sweeps": sweeps, "clocks": clk.summary(),
            "accepted_steps_per_network": {"mean": float(st["accepted_per_network"].mean()),
                                           "max": int(st["accepted_per_network"].max())}}
    if rank == 0:
        print(json.dumps(line))


# the CPU sample of a dense workload: about this many multiply-adds (12 N^2 per step attempt:
# six RHS, two GEMV passes each), some 10-30 s of host time
CPU_DENSE_MACS = 3e11


def cpu_sample_attempts(w):
    """None (the whole workload) for the regenerated coupling, whose CPU cost is O(N K) per RHS;
    a bounded number of step attempts of the first trajectory for a dense adjacency."""
    if w["coupling"] == 1:
        return None
    return max(1, int(CPU_DENSE_MACS / (12.0 * w["n"] * w["n"])))


def cpu_baseline(w, om, thetas, threads):
    from oracle import kora
    n = w["n"]
    att = cpu_sample_attempts(w)
    cs = w["cs"] if att is None else w["cs"][:1]
    t0 = time.perf_counter()
    steps = 0
    for b, c in enumerate(cs):
        r = kora.run(thetas[b], om, k=w["k"], c1=c, onthefly=w["coupling"] == 1, seed=1, fp64=False, t1=w["t1"],
                     dt=w["dt"], atol=w["atol"], rtol=w["rtol"], threads=threads, max_attempts=att)
        steps += r.steps
    el = time.perf_counter() - t0
    return steps * n / el, el, steps


def volcano_accuracy(w, thetas, om, seed, device, threads, t_phase=10.0):
    """The accuracy contract of the large regenerated network, for every c of the batch: phases
    within 1e-4 rad of the FP64 oracle for t <= t_phase (plus one float32 ulp of the phase), and
    the time-averaged r within 1e-3 over the whole horizon.  One extra GPU integration with the
    phases recorded at every output time; the FP64 oracle runs each trajectory on the host."""
    import kuramoto_gb300 as kg
    from oracle import kora
    n, B = w["n"], len(w["cs"])
    net = kg.Network(n, k=w["k"], coupling=w["coupling"], batch=B, seed=seed, atol=w["atol"], rtol=w["rtol"],
                     dense_level=1, device=device)
    net.set_frequencies(om)
    for b, c in enumerate(w["cs"]):
        net.set_coupling(b, c)
        net.set_state(b, thetas[b], 0.0, w["dt"] / 100)
    net.set_horizon(w["t1"], w["dt"], True)
    rows = int(round(t_phase / w["dt"])) + 1  # records at t = 0, dt, .., t_phase
    th_gpu = {b: [] for b in range(B)}
    net.run(on_output=lambda b, i, te, r, th, cp: (len(th_gpu[b]) < rows and th_gpu[b].append(th)) and False)
    r_gpu = [net.order(b) for b in range(B)]
    net.close()
    per_c = []
    for b, c in enumerate(w["cs"]):
        ref = kora.run(thetas[b], om, k=w["k"], c1=c, onthefly=w["coupling"] == 1, seed=seed, fp64=True, t1=w["t1"],
                       dt=w["dt"], atol=w["atol"], rtol=w["rtol"], dense=1, threads=threads)
        tg = np.stack(th_gpu[b]).astype(np.float64)
        tr = ref.thetas[:rows]
        d = np.abs((tg - tr + np.pi) % (2 * np.pi) - np.pi)
        ulp = np.spacing(np.abs(tr).astype(np.float32)).astype(np.float64)
        m = min(r_gpu[b].size, ref.order.size)
        per_c.append({"c": c, "theta_err_max_t_le_%g" % t_phase: float(d.max()),
                      "theta_err_over_1e-4_plus_ulp": float((d - 1e-4 - ulp).max()),
                      "r_err_max": float(np.max(np.abs(r_gpu[b][:m] - ref.order[:m]))),
                      "mean_r_err": float(abs(np.mean(r_gpu[b][:m], dtype=np.float64) - np.mean(ref.order[:m])))})
    return {"vs": "FP64 oracle (rank-K coupling, the reference's -A arithmetic in double)",
            "theta_window": [0.0, t_phase], "r_window": [0.0, w["t1"]], "per_c": per_c,
            "max_theta_err": max(x["theta_err_max_t_le_%g" % t_phase] for x in per_c),
            "max_mean_r_err": max(x["mean_r_err"] for x in per_c)}


def r_error_vs_fp64(w, om, theta, c, gpu_order, threads, t1=3.0):
    """max |r_gpu - r_fp64| over the first outputs (the FP64 oracle on a bounded horizon)."""
    from oracle import kora
    r = kora.run(theta, om, k=w["k"], c1=c, onthefly=w["coupling"] == 1, seed=1, fp64=True, t1=t1, dt=w["dt"],
                 atol=w["atol"], rtol=w["rtol"], threads=threads)
    m = min(r.order.size, gpu_order.size)
    return float(np.max(np.abs(r.order[:m] - gpu_order[:m])))


# ------------------------------------------------------------------ windowed workloads
def window_inputs(w, seed, host_rng):
    """Shared Cauchy omega of scale 1 as the reference draws it on a fresh start (glibc rand of
    `seed`, N draws for theta0 first: its frequencies.dat) and one theta0 per trajectory, uniform
    in [0, init), from a numpy stream of `seed`.  Trajectory 0 is the same for every batch size,
    so the plain path integrates the ensemble's first member."""
    n, B = w["n"], len(w["cs"])
    _, om = host_rng(seed, n, 0.0, 1.0, False)
    rng = np.random.default_rng(seed)
    return [(rng.random(n) * w["init"]).astype(np.float32) for _ in range(B)], om


class Windowed:
    """One integration toward t1 on one handle, advanced a budget of step attempts at a time
    (kura_advance): every trajectory keeps its phases, FSAL slope and step size on the device, so
    the steps are consecutive pieces of one uninterrupted run, and every trajectory stays active
    (no trajectory waits for the others at a step boundary)."""

    def __init__(self, w, thetas, om, seed, device, stream):
        import kuramoto_gb300 as kg
        self.w = w
        self.n, self.B = w["n"], len(thetas)
        eng = kg.ENGINE_TENSOR if w["engine"] == "tensor" else kg.ENGINE_PERSISTENT
        self.net = kg.Network(self.n, k=w["k"], coupling=kg.COUPLING_DENSE, batch=self.B, seed=seed, atol=w["atol"],
                              rtol=w["rtol"], dense_level=0, device=device, stream=stream, engine=eng)
        self.net.set_frequencies(om)
        self.net.generate_adjacency()
        for b in range(self.B):
            self.net.set_coupling(b, w["cs"][b])
            self.net.set_state(b, thetas[b], 0.0, w["dt"] / 100)
        self.net.set_horizon(w["t1"], w["dt"], True)
        self.running = self.B
        self.rec = [dict() for _ in range(self.B)]  # t_eval -> r

    def step(self):
        rec = self.rec
        self.running = self.net.advance(self.w["attempts"], on_output=lambda b, i, te, r, th, cp:
                                        rec[b].__setitem__(round(te, 9), r) and False)

    def times(self):
        return [self.net.state(b)[1] for b in range(self.B)]

    def close(self):
        self.net.close()


def timed_windows(win, steps, stream):
    """`steps` budgets of step attempts timed with CUDA events on the handle's stream (fewer when
    every trajectory reaches t1 first); returns the accepted oscillator-steps, the event time, the
    stats deltas and the steps taken."""
    import torch
    st0 = win.net.stats()
    ms = 0.0
    done = 0
    for _ in range(steps):
        if win.running == 0:
            break
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        win.step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
        done += 1
    st1 = win.net.stats()
    d = {k: st1[k] - st0[k] for k in ("accepted", "rejected", "launches", "kernel_ms", "coupling_ms",
                                     "coupling_launches")}
    d["steps"] = done
    return d["accepted"] * win.n, ms, d


def fp64_records(w, theta0, om, c, t1, threads, seed=1):
    """r of one trajectory from the FP64 oracle (rank-K form: the same matrix as the stored
    dense volcano adjacency, at O(N K) per RHS) at t = 0, dt, .., keyed like the GPU records."""
    from oracle import kora
    r = kora.run(theta0, om, k=w["k"], c1=c, onthefly=True, seed=seed, fp64=True, t1=t1, dt=w["dt"],
                 atol=w["atol"], rtol=w["rtol"], threads=threads)
    keys = [round(float(np.float32(np.float32(w["dt"]) * np.float32(i))), 9) for i in range(r.order.size)]
    keys[0] = 0.0
    return dict(zip(keys, r.order)), r.steps


def window_cpu_model(w, om, threads):
    """The float32 oracle port of the reference program holding the workload's dense volcano
    adjacency (4 N^2 bytes of host memory, built once), as the reference stores it and streams
    it twice per RHS (two GEMVs, kuramoto.cu:113-114)."""
    from oracle import kora
    t0 = time.perf_counter()
    M = kora.Model(om, k=w["k"], seed=1, fp64=False, threads=threads)
    return M, time.perf_counter() - t0


def window_cpu(w, M, theta0, c, attempts):
    """`attempts` step attempts of one trajectory from t = 0 on the CPU port."""
    t0 = time.perf_counter()
    r = M.run(theta0, c1=c, t1=w["t1"], dt=w["dt"], atol=w["atol"], rtol=w["rtol"], max_attempts=attempts)
    el = time.perf_counter() - t0
    return r.steps * w["n"] / el, el, r.steps


CPU_ATTEMPTS = 2  # the CPU sample: step attempts of one trajectory from t = 0 (dense FP32 port)


def main_windows(args, w):
    ws, rank, local = dist_env()
    n, B = w["n"], len(w["cs"])
    threads = os.cpu_count() or 1
    metric = "accepted DP45 steps x N x batch / s"
    config = {"workload": args.workload, "n": n, "k": w["k"], "coupling": "dense volcano adjacency (seed 1)",
              "engine": "tcgen05 split-BF16 ensemble" if w["engine"] == "tensor" else "plain FP32 persistent",
              "batch": B, "c": w["cs"][0], "theta0": "uniform [0, 2pi), one numpy stream per seed",
              "frequencies": "cauchy scale 1 (glibc rand, seed 1), shared", "t1": w["t1"], "dt": w["dt"],
              "atol": w["atol"], "rtol": w["rtol"],
              "step": "%d step attempts of every trajectory (kura_advance) continuing one integration toward "
                      "t1; the warm-up steps start it from t=0" % w["attempts"],
              "l2": "inputs larger than L2 (the adjacency, %.1f GB, is streamed by every RHS); not flushed"
                    % (n * n * (2 if w["engine"] == "tensor" else 4) / 1e9),
              "parallelism": "replicas" if ws > 1 else "single"}
    sample = ("trajectory b = step mod %d, %d step attempts from t=0, float32 oracle restating the reference "
              "program with the dense adjacency in host memory (two GEMV passes per RHS), OpenMP"
              % (B, CPU_ATTEMPTS))
    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import kora
        thetas, om = window_inputs(w, 1, kora.host_random_inputs)
        M, _ = window_cpu_model(w, om, threads)
        for i in range(args.warmup):
            window_cpu(w, M, thetas[i % B], w["cs"][i % B], 1)
        units = el = 0.0
        for i in range(args.steps):
            v, e, st = window_cpu(w, M, thetas[i % B], w["cs"][i % B], CPU_ATTEMPTS)
            units += st * n
            el += e
        M.close()
        value = units / el
        print(json.dumps({"impl": "reference", "metric": metric, "value": value, "unit": "osc-steps/s",
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config,
                          "cpu_baseline": {"value": value, "unit": "osc-steps/s", "cores": threads, "kind": "port",
                                           "sample": sample},
                          "e2e": {"value": value, "unit": "osc-steps/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return

    if args.until is not None:  # one whole integration to t1 = args.until, timed after the warm-up
        w = dict(w, t1=args.until)
        args.steps = 1 << 30
    import torch
    import kuramoto_gb300 as kg
    os.environ.setdefault("KURA_TIME_COUPLING", "1")
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    seed = instance_seed(rank)
    thetas, om = window_inputs(w, seed, kg.random_inputs)
    stream = torch.cuda.current_stream()
    win = Windowed(w, thetas, om, seed, local, stream.cuda_stream)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        win.step()
    barrier()
    with Clocks(local) as clk:
        units, ms, d = timed_windows(win, args.steps, stream)
        barrier()
    steps = d["steps"]
    units_all, ms_max = combine_ranks(units, ms, "cuda")
    value = units_all / (ms_max / 1e3)
    t_reached = win.times()

    # ---- e2e: further steps through host buffers: the frequencies and every trajectory's phases
    # copied in from pinned memory with their own t and h (as a -R resume through fs.dat), the
    # budget of attempts, then the records and the phases copied out
    om_pin = pinned(om)
    th_pin = [pinned(np.zeros(n, np.float32)) for _ in range(B)]
    th_t = [0.0] * B
    th_h = [0.0] * B
    for b in range(B):
        _, th_t[b], th_h[b] = win.net.state(b, out=th_pin[b])
    e2e_units = e2e_s = 0.0
    h2d = d2h = 0
    for it in range(0 if (args.no_e2e or args.until is not None) else steps):
        if min(th_t) >= w["t1"]:
            break
        barrier()
        t0 = time.perf_counter()
        win.net.set_frequencies(om_pin)
        for b in range(B):
            win.net.set_state(b, th_pin[b], th_t[b], th_h[b])
        win.net.set_horizon(w["t1"], w["dt"], False)
        win.net.advance(w["attempts"])
        rs = [win.net.order(b) for b in range(B)]
        for b in range(B):
            _, th_t[b], th_h[b] = win.net.state(b, out=th_pin[b])
        e2e_s += time.perf_counter() - t0
        e2e_units += win.net.stats()["accepted"] * n  # set_state restarts the per-trajectory counts
        if it == 0:
            h2d = 4 * n + 4 * n * B
            d2h = sum(4 * r.size for r in rs) + 4 * n * B
    e2e_units, e2e_ms = combine_ranks(e2e_units, e2e_s * 1e3, "cuda")
    e2e_value = e2e_units / (e2e_ms / 1e3) if e2e_ms > 0 else None
    rec = win.rec
    win.close()

    # ---- the plain FP32 path on trajectory 0 of the same inputs
    plain = None
    if w.get("plain") and args.until is None:
        pw = dict(WORKLOADS[w["plain"]], t1=w["t1"])
        pwin = Windowed(pw, thetas[:1], om, seed, local, stream.cuda_stream)
        for _ in range(2):
            pwin.step()
        pu, pms, pd = timed_windows(pwin, 2, stream)
        pwin.close()
        pval = pu / (pms / 1e3)
        pk = pd["kernel_ms"] / max(pd["launches"], 1)
        bytes_launch = 24.0 * n * pd["accepted"] * n / max(pd["launches"], 1)
        plain = {"value": pval, "unit": "osc-steps/s", "steps": pd["steps"], "attempts_per_step": pw["attempts"],
                 "accepted_steps": pd["accepted"], "ratio_batched_over_plain": value / pval,
                 "roofline": roofline_hbm(bytes_launch, pk)}
    if rank != 0:
        return
    line = {"metric": metric, "value": value, "unit": "osc-steps/s", "n_gpus": ws, "steps": steps,
            "warmup": args.warmup, "ms_per_step": ms_max / max(steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 state, bf16 split operands, f32 accumulation",
            "data": "synthetic", "config": config}
    line["e2e"] = {"value": e2e_value, "unit": "osc-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    if w["engine"] == "tensor":
        # per attempt: coefficients, 6 x (stage phases, GEMM), error, decision, 2 output kernels;
        # per step: the first-slope kernels (their GEMM is skipped once the slopes are on the device)
        line["gpu_launches"] = 17 * d["launches"] + 6 * steps
        line["roofline"] = roofline_tensor(n, B, d, ms, args.workload)
    else:
        # one persistent launch per step; A is read once per RHS for the whole batch
        line["gpu_launches"] = d["launches"]
        line["roofline"] = roofline_hbm(24.0 * n * n * d["accepted"] / B / max(d["launches"], 1),
                                        d["kernel_ms"] / max(d["launches"], 1))
    line["clocks"] = clk.summary()
    line["accepted_steps"] = {"timed": d["accepted"], "rejected": d["rejected"],
                              "per_trajectory_per_step": d["accepted"] / B / max(steps, 1),
                              "t_reached": {"min": round(min(t_reached), 4), "mean": round(float(np.mean(t_reached)), 4),
                                            "max": round(max(t_reached), 4)}}
    if plain:
        line["plain_fp32"] = plain
    if not args.no_cpu:
        M, build_s = window_cpu_model(w, om, threads)
        v, el, st = window_cpu(w, M, thetas[0], w["cs"][0], CPU_ATTEMPTS)
        M.close()
        line["cpu_baseline"] = {"value": v, "unit": "osc-steps/s", "cores": threads, "kind": "port",
                                "sample": "trajectory 0, %d step attempts from t=0 (%d accepted, %.1f s; the dense "
                                          "adjacency built once beforehand in %.1f s), float32 oracle restating the "
                                          "reference program, two GEMV passes per RHS, OpenMP"
                                          % (CPU_ATTEMPTS, st, el, build_s)}
    if not args.no_cpu or args.until is not None:
        errs, cnt = [], 0
        for b in sorted({0, B // 2, B - 1}):
            ref, _ = fp64_records(w, thetas[b], om, w["cs"][b], t_reached[b], threads, seed)
            common = [t for t in rec[b] if t in ref]
            cnt += len(common)
            if common:
                errs.append(max(abs(float(rec[b][t]) - float(ref[t])) for t in common))
        line["r_err_vs_fp64"] = max(errs) if errs else None
        line["r_err_sample"] = ("trajectories %s, %d records from t=0 to each one's time reached, against the "
                                "FP64 oracle" % (sorted({0, B // 2, B - 1}), cnt))
    print(json.dumps(line))


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def roofline_hbm(bytes_per_launch, kernel_ms_per_launch, traffic=None):
    peaks = _peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    ach = bytes_per_launch / (kernel_ms_per_launch / 1e3) / 1e9 if kernel_ms_per_launch > 0 else 0.0
    return {"bound": "hbm", "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s", "frac": round(ach / hbm, 4),
            "traffic": traffic, "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
            "kernel_ms_per_launch": round(kernel_ms_per_launch, 3)}


def traffic_entry(workload, key):
    try:
        t = json.load(open(os.path.join(ROOT, "profiles", "traffic.json"))).get(workload)
        return t.get(key) if t else None
    except Exception:
        return None


def roofline_tensor(n, B, d, step_ms, workload=None):
    """The coupling GEMM: one launch is every trajectory's RHS, C = (N A) [cos|sin]: 4 N^2 B
    algorithmic flops (2 columns x 2 flops per multiply-add), 8 N^2 B issued (hi and lo columns).
    Its duration is the CUDA-event time of the GEMM launches the engine sampled in the timed
    windows (event nodes around the six GEMMs of one attempt in four).  The GEMMs run back to
    back through the whole window, so the sustained bf16 figure is the peak."""
    peaks = _peaks()
    peak = peaks.get("bf16_tflops_sustained", 1700.0)
    src = "measured" if "bf16_tflops_sustained" in peaks else "fallback"
    per = d["coupling_ms"] / max(d["coupling_launches"], 1)
    flops = 4.0 * n * n * B
    ach = flops / (per / 1e3) / 1e12 if per > 0 else 0.0
    step_tf = 24.0 * n * d["accepted"] * n / (step_ms / 1e3) / 1e12 if step_ms > 0 else 0.0
    # the adjacency (N*A in BF16) is read once per launch: a small batch makes the launch HBM-bound
    hbm = peaks.get("hbm_gbs", 6800.0)
    a_gbs = 2.0 * n * n / (per / 1e3) / 1e9 if per > 0 else 0.0
    out = {"bound": "tensor", "achieved": round(ach, 1), "peak": peak, "unit": "TFLOP/s",
           "frac": round(ach / peak, 4), "traffic": traffic_entry(workload, "bytes_per_launch"), "peak_source": src,
           "flops_per_launch": flops, "issued_flops_per_launch": 2 * flops,
           "kernel_ms_per_launch": round(per, 4), "launches_sampled": d["coupling_launches"],
           "whole_step_tflops": round(step_tf, 1), "whole_step_frac": round(step_tf / peak, 4),
           "adjacency_gbs": round(a_gbs, 1), "adjacency_hbm_frac": round(a_gbs / hbm, 4)}
    bp = 16
    while bp < B:
        bp *= 2
    issued = 8.0 * n * n * bp  # hi and lo columns of the padded batch
    out["issued_flops_per_launch"] = issued
    out["issued_frac"] = round(issued / (per / 1e3) / 1e12 / peak, 4) if per > 0 else 0.0
    if a_gbs / hbm > out["issued_frac"]:
        out.update({"bound": "hbm", "achieved": round(a_gbs, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(a_gbs / hbm, 4), "tensor_frac": round(ach / peak, 4),
                    "bytes_per_launch": 2.0 * n * n})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--workload", default="ensemble65536", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--t1", type=float, default=None, help="shorter horizon (profiling captures only)")
    ap.add_argument("--until", type=float, default=None,
                    help="windowed workloads: time windows until the integration reaches this t (e.g. 20)")
    ap.add_argument("--no-e2e", action="store_true", help="windowed workloads: skip the host-buffer leg")
    args = ap.parse_args()
    w = dict(WORKLOADS[args.workload])
    if args.t1 is not None:
        w["t1"] = args.t1
    if w.get("kind") == "multi":
        return main_multi(args, w)
    if w.get("kind") == "surrogate":
        return main_surrogate(args, w)
    if w.get("kind") == "windows":
        return main_windows(args, w)
    ws, rank, local = dist_env()
    n, B = w["n"], len(w["cs"])
    config = {"workload": args.workload, "n": n, "k": w["k"], "coupling": "volcano-regenerated" if w["coupling"] else
              "dense", "batch": B, "c": w["cs"], "t1": w["t1"], "dt": w["dt"], "atol": w["atol"],
              "rtol": w["rtol"], "frequencies": "normal (glibc rand, seed 1)" if w["normal"] else "cauchy",
              "l2": "flushed between steps (512 MiB write)", "parallelism": "replicas" if ws > 1 else "single"}
    if w.get("adj_storage"):
        config["adjacency_storage"] = "int8 (N*A, exact for the volcano rule)"
    metric = "accepted DP45 steps x N x batch / s"
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import kora
        thetas, om = inputs(w, 1, kora.host_random_inputs)
        for _ in range(args.warmup):
            cpu_baseline(w, om, thetas, threads)
        tot_units = 0.0
        tot_s = 0.0
        for _ in range(args.steps):
            v, el, steps = cpu_baseline(w, om, thetas, threads)
            tot_units += steps * n
            tot_s += el
        value = tot_units / tot_s
        line = {"impl": "reference", "metric": metric, "value": value, "unit": "osc-steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_s / args.steps * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": config,
                "cpu_baseline": {"value": value, "unit": "osc-steps/s", "cores": threads, "kind": "port",
                                 "sample": ("whole workload per step (%d trajectories to t=%g)" % (B, w["t1"])
                                            if cpu_sample_attempts(w) is None else
                                            "trajectory 0, %d step attempts from t=0 per step"
                                            % cpu_sample_attempts(w)) +
                                           ", float32 oracle restating the reference program, OpenMP"},
                "e2e": {"value": value, "unit": "osc-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    res = run_native(args, w)
    if rank != 0:
        return
    line = {"metric": metric, "value": res["value"], "unit": "osc-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config}
    line["e2e"] = {"value": res["e2e_value"], "unit": "osc-steps/s", "h2d_bytes_per_step": res["h2d"],
                   "d2h_bytes_per_step": res["d2h"]}
    # launches of our kernels per step: B state uploads + the integrator's own launches
    line["gpu_launches"] = (B * args.steps + res["launches"] * (1 if w.get("engine") != "tensor" else 17))
    line["roofline"] = roofline(w, res, args)
    line["clocks"] = res["clocks"]
    line["accepted_steps_per_run"] = res["acc_per_step"]
    if not args.no_cpu:
        v, el, steps = cpu_baseline(w, res["om"], res["thetas"], threads)
        att = cpu_sample_attempts(w)
        line["cpu_baseline"] = {"value": v, "unit": "osc-steps/s", "cores": threads, "kind": "port",
                                "sample": ("whole workload (%d trajectories to t=%g, " % (B, w["t1"]) if att is None
                                           else "trajectory 0, %d step attempts from t=0 (" % att) +
                                          "%d accepted steps, %.1f s), float32 oracle restating the reference "
                                          "program" % (steps, el)}
        if w["coupling"] == 1:
            acc = volcano_accuracy(w, res["thetas"], res["om"], instance_seed(res["rank"]), 0, threads)
            line["accuracy"] = acc
            line["r_err_vs_fp64"] = max(x["r_err_max"] for x in acc["per_c"])
        else:
            ci = len(w["cs"]) // 2
            line["r_err_vs_fp64"] = r_error_vs_fp64(w, res["om"], res["thetas"][ci], w["cs"][ci], res["orders"][ci],
                                                    threads)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
