"""Reading FILEBASE outputs for downstream analysis, and writing them in the layout the
reference's DMD post-processing reads.

The reference's program writes, for a run named FILEBASE:

* `FILEBASE.out`: line 1 is "N K t1 dt c seed" (kuramoto.cu:418), line 2 the argv;
* `frequencies.dat`: omega;
* `thetas.dat`: theta0, then theta at every output time;
* `order.dat`: r at the same times;
* `times.dat`: t after every accepted step;
* `couplings.dat`: [A cos, A sin] interleaved;
* `fs.dat`: the end record, theta, t, h, couplings.

Files are float32 from `kuramoto` and from this project's CLI, float64 from `kuramoto_64`.
`dmd.py` (dmd.py:38-48) parses line 1 of `.out` and memory-maps float64 `frequencies.dat`
and `thetas.dat`, the latter as int(t1/dt) rows of N.  `load` reads either precision
(detected from the size of frequencies.dat).  `write_dmd` writes a run in the float64
layout `dmd.py` maps, so output of the float32 program can feed it.
"""
import os
import shutil
from dataclasses import dataclass

import numpy as np


@dataclass
class Header:
    N: int
    K: int
    t1: float
    dt: float
    c: float
    seed: int


@dataclass
class Run:
    header: Header
    dtype: type
    omega: np.ndarray
    thetas: np.ndarray        # [records, N] or None
    order: np.ndarray         # [records] or None
    times: np.ndarray         # [accepted steps] or None
    couplings: np.ndarray     # [records, 2N] or None
    final_theta: np.ndarray   # fs.dat
    final_t: float
    final_h: float


def read_header(filebase):
    """Line 1 of FILEBASE.out: N K t1 dt c seed."""
    with open(filebase + ".out") as f:
        v = f.readline().split()
    return Header(int(float(v[0])), int(float(v[1])), float(v[2]), float(v[3]), float(v[4]), int(float(v[5])))


def detect_dtype(filebase, n):
    size = os.path.getsize(filebase + "frequencies.dat")
    if size == 4 * n:
        return np.float32
    if size == 8 * n:
        return np.float64
    raise ValueError("%sfrequencies.dat holds %d bytes, neither %d float32 nor float64 values" % (filebase, size, n))


def _read(path, dtype, width=None):
    if not os.path.exists(path):
        return None
    a = np.fromfile(path, dtype)
    if width:
        if a.size % width:
            raise ValueError("%s holds %d values, not a multiple of %d" % (path, a.size, width))
        a = a.reshape(-1, width)
    return a


def load(filebase):
    """Every file of one run, in the precision it was written."""
    h = read_header(filebase)
    dt = detect_dtype(filebase, h.N)
    fs = _read(filebase + "fs.dat", dt)
    ft = fh = float("nan")
    fth = None
    if fs is not None and fs.size >= h.N + 2:
        fth, ft, fh = fs[:h.N], float(fs[h.N]), float(fs[h.N + 1])
    return Run(header=h, dtype=dt, omega=_read(filebase + "frequencies.dat", dt),
               thetas=_read(filebase + "thetas.dat", dt, h.N), order=_read(filebase + "order.dat", dt),
               times=_read(filebase + "times.dat", dt), couplings=_read(filebase + "couplings.dat", dt, 2 * h.N),
               final_theta=fth, final_t=ft, final_h=fh)


def write_dmd(filebase, out_filebase):
    """Writes `out_filebase` in the layout dmd.py reads: the .out file (its line 1 is the
    header), float64 frequencies.dat and float64 thetas.dat.  Returns the thetas array as
    dmd.py maps it, int(t1/dt) rows of N."""
    run = load(filebase)
    if run.thetas is None:
        raise ValueError("%s has no thetas.dat (run with -D 1 or higher)" % filebase)
    shutil.copyfile(filebase + ".out", out_filebase + ".out")
    run.omega.astype(np.float64).tofile(out_filebase + "frequencies.dat")
    run.thetas.astype(np.float64).tofile(out_filebase + "thetas.dat")
    length = int(run.header.t1 / run.header.dt)
    return np.memmap(out_filebase + "thetas.dat", dtype=np.float64, mode="r", shape=(length, run.header.N))
