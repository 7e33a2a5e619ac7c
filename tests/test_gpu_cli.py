"""The `kuramoto` command line as a drop-in for the reference program.

Runs the product CLI and the oracle's restatement of the reference CLI on the
same arguments and compares the FILEBASE files: names, sizes and layout exactly;
generated inputs (frequencies, phases, adjacency) byte for byte; integrated
outputs within tolerance (the float32 oracle follows the reference's float32
arithmetic, so the comparison tolerance is looser than against FP64).
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FILES = ["fs.dat", "order.dat", "thetas.dat", "times.dat", "couplings.dat", "adj.dat", "frequencies.dat"]


def run_pair(native, oracle_lib, tmp_path, args, reload_files=None):
    out = {}
    for name, exe in (("gpu", native.cli_path()), ("cpu", oracle_lib.cli_path(False))):
        d = tmp_path / name
        d.mkdir(exist_ok=True)
        base = str(d / "run")
        if reload_files:
            for suffix, arr in reload_files.items():
                arr.tofile(base + suffix)
        r = subprocess.run([exe, *args, base], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, (name, r.stdout, r.stderr)
        out[name] = (base, r.stdout)
    return out


def load(base, suffix):
    p = base + suffix
    return np.fromfile(p, np.float32) if os.path.exists(p) else None


@pytest.mark.parametrize("volcano", [False, True])
def test_fresh_run_files(native, oracle_lib, tmp_path, volcano):
    n = 300
    args = ["-N", str(n), "-K", "5", "-c", "3", "-t", "10", "-d", "1", "-D", "3", "-I", "6.28", "-s", "4"]
    if volcano:
        args.append("-A")
    res = run_pair(native, oracle_lib, tmp_path, args)
    g, c = res["gpu"][0], res["cpu"][0]
    for f in FILES:
        eg, ec = os.path.exists(g + f), os.path.exists(c + f)
        assert eg == ec, f
        if eg:
            assert os.path.getsize(g + f) == os.path.getsize(c + f) or f == "times.dat", f
    assert os.path.exists(g + "adj.dat") != volcano
    assert np.array_equal(load(g, "frequencies.dat"), load(c, "frequencies.dat"))
    if not volcano:
        assert np.array_equal(load(g, "adj.dat").view(np.uint32), load(c, "adj.dat").view(np.uint32))
    og, oc = load(g, "order.dat"), load(c, "order.dat")
    assert og.size == oc.size == 11 and og[0] == pytest.approx(oc[0], abs=1e-6)
    assert np.max(np.abs(og - oc)) < 2e-3
    tg, tc = load(g, "thetas.dat").reshape(-1, n), load(c, "thetas.dat").reshape(-1, n)
    assert np.array_equal(tg[0], tc[0])
    # the float32 oracle accumulates rounding of order ulp(theta) per step
    assert np.all(np.abs(tg - tc) <= 5e-3 + 1e-5 * np.abs(tc))
    cg, cc = load(g, "couplings.dat").reshape(-1, 2 * n), load(c, "couplings.dat").reshape(-1, 2 * n)
    assert np.max(np.abs(cg - cc)) < 5e-3
    fg, fc = load(g, "fs.dat"), load(c, "fs.dat")
    assert fg.size == fc.size == 3 * n + 2
    assert fg[n] == pytest.approx(fc[n], rel=1e-2)  # end time (overshoots t1)
    assert fg[n] >= 10.0
    assert np.all(np.abs(fg[:n] - fc[:n]) <= 5e-3 + 1e-5 * np.abs(fc[:n]))
    timg, timc = load(g, "times.dat"), load(c, "times.dat")
    # the float32 reference's error estimate carries rounding noise of omega*h, so its step
    # count differs by a few percent
    assert abs(timg.size - timc.size) <= max(3, timc.size // 20) and timg[-1] >= 10.0
    lg = open(g + ".out").read().splitlines()
    lc = open(c + ".out").read().splitlines()
    assert lg[0] == lc[0]
    assert lg[1].split()[1:-1] == lc[1].split()[1:-1]  # argv without the program and FILEBASE paths
    for msg in ("Using random initial conditions", "Using random frequencies", "Using random adjacency matrix"):
        assert msg in lg and msg in lc
    assert any(l.startswith("steps: ") for l in lg)


def test_dense_level_zero_writes_minimal_files(native, tmp_path):
    base = str(tmp_path / "z")
    r = subprocess.run([native.cli_path(), "-N", "100", "-K", "3", "-t", "3", "-D", "0", "-A", base],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(base + "order.dat") and os.path.exists(base + "fs.dat")
    assert os.path.exists(base + "frequencies.dat")
    for f in ("thetas.dat", "times.dat", "couplings.dat", "adj.dat"):
        assert not os.path.exists(base + f)
    assert os.path.getsize(base + "order.dat") == 4 * 4


def test_reload_appends_and_continues(native, oracle_lib, tmp_path):
    """-R: phases, time and step from fs.dat, frequencies and adjacency from files, outputs appended."""
    n = 200
    args = ["-N", str(n), "-K", "4", "-c", "2", "-t", "5", "-d", "1", "-D", "3", "-I", "3", "-s", "8"]
    res = run_pair(native, oracle_lib, tmp_path, args)
    args2 = ["-N", str(n), "-K", "4", "-c", "2", "-t", "8", "-d", "1", "-D", "2", "-s", "8", "-R"]
    res2 = run_pair(native, oracle_lib, tmp_path, args2)
    g, c = res2["gpu"][0], res2["cpu"][0]
    og, oc = load(g, "order.dat"), load(c, "order.dat")
    assert og.size == oc.size == 6 + 3
    assert np.max(np.abs(og - oc)) < 2e-3
    assert load(g, "thetas.dat").size == load(c, "thetas.dat").size == 9 * n
    out = open(g + ".out").read()
    assert "Using initial conditions from file" in out and "Restarting at t=" in out
    assert "Using frequencies from file" in out and "Using adjacency from file" in out


def test_fixed_step_cli(native, oracle_lib, tmp_path):
    n = 64
    args = ["-N", str(n), "-K", "3", "-c", "1", "-t", "2", "-d", "0.5", "-D", "1", "-F", "-I", "2"]
    res = run_pair(native, oracle_lib, tmp_path, args)
    g, c = res["gpu"][0], res["cpu"][0]
    assert load(g, "times.dat").size == load(c, "times.dat").size == 4
    assert np.max(np.abs(load(g, "order.dat") - load(c, "order.dat"))) < 1e-3


@pytest.mark.parametrize("volcano", [False, True])
def test_fault_injection_resume(native, tmp_path, volcano):
    """Preemption and resume without a GPU fault: KURA_FAIL_AT_STEP makes the host process
    exit(3) right after it rewrites fs.dat; rerunning with -R continues from fs.dat and
    appends.  The result matches an uninterrupted run to the float32 checkpoint precision
    (fs.dat stores theta, t and h as float32, as the reference does)."""
    n = 1500
    args = ["-N", str(n), "-K", "5", "-c", "3", "-t", "30", "-d", "1", "-D", "1", "-n", "-s", "4"]
    if volcano:
        args.append("-A")
    full = str(tmp_path / "full")
    r = subprocess.run([native.cli_path(), *args, full], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cut = str(tmp_path / "cut")
    env = dict(os.environ, KURA_CHECKPOINT_STEPS="40", KURA_FAIL_AT_STEP="100")
    r = subprocess.run([native.cli_path(), *args, cut], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 3, (r.returncode, r.stdout, r.stderr)
    assert "injected fault after" in open(cut + ".out").read()
    fs = np.fromfile(cut + "fs.dat", np.float32)
    t_chk = float(fs[n])
    assert fs.size == 3 * n + 2 and 0 < t_chk < 30
    part = load(cut, "order.dat")
    assert 1 <= part.size < 31
    r = subprocess.run([native.cli_path(), *args, "-R", cut], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    a, b = load(full, "order.dat"), load(cut, "order.dat")
    assert a.size == b.size == 31
    assert np.max(np.abs(a - b)) < 1e-4, np.max(np.abs(a - b))
    ta, tb = load(full, "thetas.dat").reshape(-1, n), load(cut, "thetas.dat").reshape(-1, n)
    assert ta.shape == tb.shape
    assert np.max(np.abs(ta - tb) - 4 * np.spacing(np.abs(ta))) < 1e-4
    # the step times: the interrupted run's up to the checkpoint, then the resumed run's
    sa, sb = load(full, "times.dat"), load(cut, "times.dat")
    assert abs(sa.size - sb.size) <= 3
    assert np.all(np.diff(sb) > 0) and sb[-1] >= 30.0
