"""The FILEBASE reader and the float64 layout dmd.py maps (runs the oracle's CLI
restatements of `kuramoto` and `kuramoto_64`; no GPU)."""
import subprocess

import numpy as np
import pytest

from kuramoto_gb300 import filebase as fb


def run_cli(exe, base, args):
    r = subprocess.run([exe, *args, base], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("fp64", [False, True])
def test_load_reads_both_precisions(oracle_lib, tmp_path, fp64):
    base = str(tmp_path / "run")
    run_cli(oracle_lib.cli_path(fp64), base, ["-N", "50", "-K", "3", "-c", "2", "-t", "4", "-d", "1", "-D", "2",
                                              "-s", "3", "-I", "2"])
    run = fb.load(base)
    assert run.header == fb.Header(50, 3, 4.0, 1.0, 2.0, 3)
    assert run.dtype == (np.float64 if fp64 else np.float32)
    assert run.omega.shape == (50,)
    assert run.thetas.shape == (5, 50) and run.order.shape == (5,) and run.couplings.shape == (5, 100)
    assert np.all(np.diff(run.times) > 0) and run.times[-1] >= 4.0
    assert run.final_theta.shape == (50,) and run.final_t >= 4.0 and run.final_h > 0
    # r recomputed from the stored phases
    r = np.abs(np.exp(1j * run.thetas.astype(np.float64)).mean(1))
    assert np.max(np.abs(r - run.order)) < (1e-12 if fp64 else 2e-6)


def test_write_dmd_layout(oracle_lib, tmp_path):
    base = str(tmp_path / "run")
    run_cli(oracle_lib.cli_path(False), base, ["-N", "40", "-K", "2", "-t", "6", "-d", "0.5", "-D", "1", "-s", "2"])
    out = str(tmp_path / "dmd0")
    X = fb.write_dmd(base, out)
    run = fb.load(base)
    # what dmd.py maps: .out line 1, float64 frequencies and int(t1/dt) rows of thetas
    N, K, t1, dt, c, seed = np.array(open(out + ".out").readline().split(), dtype=np.float64)
    assert (int(N), int(t1 / dt)) == (40, 12)
    om = np.memmap(out + "frequencies.dat", dtype=np.float64, mode="r", shape=(40,))
    assert np.array_equal(om, run.omega.astype(np.float64))
    assert X.shape == (12, 40) and np.array_equal(np.asarray(X), run.thetas[:12].astype(np.float64))
    assert fb.load(out).dtype == np.float64


def test_detect_dtype_rejects_other_sizes(tmp_path):
    base = str(tmp_path / "x")
    open(base + ".out", "w").write("10 2 1.0 1.0 1.0 1\n")
    np.zeros(7, np.float32).tofile(base + "frequencies.dat")
    with pytest.raises(ValueError):
        fb.load(base)
