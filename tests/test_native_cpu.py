"""CPU-side checks of the native library: it loads, exports every entry point of
include/kura.h, its host random generator is byte-identical to the reference's
frequencies.dat, and compute calls fail cleanly (no crash) without a GPU."""
import os
import re
import subprocess

import numpy as np
import pytest

from helpers import golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "kura.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(kura_\w+)\s*\(", src, re.M)))


def test_exports_every_declared_symbol(native):
    syms = header_symbols()
    assert len(syms) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", native.lib_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (kura_\w+)", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    L = native.lib()
    for s in syms:
        assert hasattr(L, s)


@pytest.mark.parametrize("K", [0, 2, 5000])
@pytest.mark.parametrize("normal", [True, False])
def test_host_rng_byte_exact(native, K, normal):
    ref = np.fromfile(golden("%s_K%d_seed1_frequencies.dat" % ("normal" if normal else "cauchy", K)), np.float32)
    _, om = native.random_inputs(1, ref.size, 0.0, 1.0, normal)
    assert np.array_equal(om.view(np.uint32), ref.view(np.uint32))


def test_host_rng_matches_oracle_theta(native, oracle_lib):
    for seed in (1, 5, 123):
        a, b = native.random_inputs(seed, 777, 3.5, 2.0, seed % 2 == 0)
        c, d = oracle_lib.host_random_inputs(seed, 777, 3.5, 2.0, seed % 2 == 0)
        assert np.array_equal(a.view(np.uint32), c.view(np.uint32))
        assert np.array_equal(b.view(np.uint32), d.view(np.uint32))
    # theta0 only, omega only: the rand() sequence restarts at srand(seed)
    _, om_only = native.random_inputs(9, 100, 1.0, 1.0, False, gen_theta=False)
    _, om_ref = oracle_lib.host_random_inputs(9, 100, 1.0, 1.0, False, gen_theta=False)
    assert np.array_equal(om_only, om_ref)


def test_memory_required(native):
    b_dense = native.Network.memory_required(5000, 5, native.COUPLING_DENSE)
    b_volc = native.Network.memory_required(5000, 5, native.COUPLING_VOLCANO)
    assert b_dense > 5000 * 5000 * 4 > b_volc > 0


def test_invalid_config_rejected_without_gpu(native):
    with pytest.raises(native.KuraError):
        native.Network(0)
    with pytest.raises(native.KuraError):
        native.Network(100, k=40, coupling=native.COUPLING_VOLCANO)
    with pytest.raises(native.KuraError):
        native.Network(100, batch=9)
    # multi-network handles: rank above 8, a cluster size that is not a power of two, a
    # block size outside 256/512/1024 and an empty set fail before any device work
    for kw, code in ((dict(ks=[9]), -7), (dict(cluster_size=3), -1), (dict(block_threads=128), -1),
                     (dict(ns=[0]), -7), (dict(ns=[], ks=[], seeds=[], cs=[]), -1)):
        args = dict(ns=[100], ks=[5], seeds=[1], cs=[1.0])
        args.update(kw)
        with pytest.raises(native.KuraError) as e:
            native.MultiNetworks(args.pop("ns"), args.pop("ks"), args.pop("seeds"), args.pop("cs"), 1.0, 1.0, **args)
        assert e.value.code == code


def test_invalid_mlp_rejected_without_gpu(native):
    """Surrogate shapes outside what the tensor-core kernels support fail before any device
    work: input or output width 0 or above 64, a hidden width other than 64/128/256, a batch
    that is not a multiple of 128 in 128..4096."""
    for kw in (dict(in_dim=0), dict(in_dim=65), dict(out_dim=0), dict(out_dim=65), dict(hidden=100),
               dict(batch=100), dict(batch=8192)):
        args = dict(in_dim=14, out_dim=2, hidden=256, batch=512)
        args.update(kw)
        with pytest.raises(native.KuraError) as e:
            native.MLP(**args)
        assert e.value.code == -7


def test_cli_help_runs_without_gpu(native):
    r = subprocess.run([native.cli_path(), "-h"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "usage:" in r.stdout and "filebase" in r.stdout


def test_oracle_cli_files(oracle_lib, tmp_path):
    base = str(tmp_path / "o")
    r = subprocess.run([oracle_lib.cli_path(False), "-N", "64", "-K", "3", "-c", "2", "-t", "3", "-d", "1", "-D", "3",
                        "-I", "6.28", base], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    sz = lambda s: os.path.getsize(base + s)
    assert sz("frequencies.dat") == 64 * 4
    assert sz("adj.dat") == 64 * 64 * 4
    assert sz("order.dat") == 4 * 4
    assert sz("thetas.dat") == 4 * 64 * 4
    assert sz("couplings.dat") == 4 * 128 * 4
    assert sz("fs.dat") == (64 + 2 + 128) * 4
    first = open(base + ".out").readline()
    assert first.startswith("64 3 3.000000 1.000000 2.000000 1")


def test_advance_and_horizon_validate_arguments_without_gpu(native):
    """kura_advance and kura_set_horizon check their arguments before any device work."""
    import ctypes
    L = native.lib()
    running = ctypes.c_int32(-1)
    assert L.kura_advance(None, None, 10, ctypes.byref(running)) == -1
    assert running.value == -1
    assert L.kura_set_horizon(None, 1.0, 0.1, 1) == -1
