"""Runs FILEBASE programs on the same reload inputs and reads their outputs.

The programs are the reference's own ``kuramoto`` / ``kuramoto_64`` (built into oracle/_ref by
oracle/build_ref.py, the checker) and this project's drop-in ``kuramoto`` CLI.  Inputs enter
through the reference's ``-R`` reload path (kuramoto.cu:466-521, 557-566; kuramoto_64.cu:472,
511, 560): ``fs.dat`` = theta0[N], t, h; ``frequencies.dat`` = omega[N]; ``adj.dat`` = A[N*N]
row-major, all float32 for ``kuramoto`` and float64 for ``kuramoto_64``.  A reload run writes no
t = 0 record (kuramoto.cu:587): order.dat holds r at t_eval = dt, 2dt, ..., thetas.dat (D >= 1)
theta there.
"""
import os
import subprocess
import time
from dataclasses import dataclass

import numpy as np


@dataclass
class Outputs:
    order: np.ndarray   # r at each t_eval
    thetas: np.ndarray  # [n_out][N] (D >= 1) or None
    times: np.ndarray   # t after each accepted step (D >= 1) or None
    fs: np.ndarray      # final fs.dat: theta[N], t, h, couplings[2N]
    steps: int          # accepted steps ("steps:" line of FILEBASE.out)
    wall_s: float       # wall time of the process
    stdout: str


def write_inputs(base, theta0, omega, adj=None, t0=0.0, h0=0.01, fp64=False):
    """The reload files of one run, widened exactly to float64 for ``kuramoto_64``."""
    dt = np.float64 if fp64 else np.float32
    th = np.asarray(theta0, np.float32).astype(dt)
    np.concatenate([th, np.array([t0, h0], dt)]).tofile(base + "fs.dat")
    np.asarray(omega, np.float32).astype(dt).tofile(base + "frequencies.dat")
    if adj is not None:
        np.asarray(adj, np.float32).astype(dt).tofile(base + "adj.dat")


def fmt(x):
    return repr(float(x)) if float(x) != int(x) else str(int(x))


def run(exe, base, n, *, k=5, c=3.0, t1=100.0, dt=1.0, volcano=False, seed=1, dense=1, atol=1e-6, rtol=0.0,
        fp64=False, timeout=1200, env=None):
    """One ``-R`` run of a FILEBASE program; returns its outputs."""
    args = [exe, "-N", str(n), "-K", str(k), "-c", fmt(c), "-t", fmt(t1), "-d", fmt(dt), "-a", repr(atol),
            "-r", repr(rtol), "-D", str(dense), "-s", str(seed), "-R"]
    if volcano:
        args.append("-A")
    t0 = time.perf_counter()
    r = subprocess.run(args + [base], capture_output=True, text=True, timeout=timeout, env=env)
    wall = time.perf_counter() - t0
    if r.returncode != 0:
        raise RuntimeError("%s exited %d\n%s\n%s" % (exe, r.returncode, r.stdout[-2000:], r.stderr[-2000:]))
    return read_outputs(base, n, fp64, r.stdout, wall)


def read_outputs(base, n, fp64=False, stdout="", wall=0.0):
    dt = np.float64 if fp64 else np.float32

    def load(suffix):
        p = base + suffix
        return np.fromfile(p, dt) if os.path.exists(p) else None

    thetas = load("thetas.dat")
    steps = -1
    if os.path.exists(base + ".out"):
        for line in open(base + ".out", errors="replace").read().splitlines():
            if line.startswith("steps:"):
                steps = int(line.split()[1])
    return Outputs(order=load("order.dat"), thetas=None if thetas is None else thetas.reshape(-1, n),
                   times=load("times.dat"), fs=load("fs.dat"), steps=steps, wall_s=wall, stdout=stdout)


def wrapped(a, b):
    """|a - b| modulo 2 pi, in float64."""
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return np.abs((d + np.pi) % (2 * np.pi) - np.pi)


def ulp32(x):
    """One float32 ulp at |x| (the storage step of a float32 phase file)."""
    x = np.abs(np.asarray(x, np.float32))
    return np.spacing(x).astype(np.float64)
