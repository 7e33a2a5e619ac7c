"""Pins the Philox stream mapping of the volcano factor against cuRAND itself.

The reference draws u_mn from cuRAND's Philox4_32_10 device generator
(kuramoto.cu:57-101).  tests/cuda/curand_factor.cu draws the same bits through
the cuRAND device API in the reference's call pattern; libkura's own Philox
(and the oracle's) must reproduce them bit for bit.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def curand_bin(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("curand") / "curand_factor")
    subprocess.run([nvcc, "-O2", "-gencode", "arch=compute_103a,code=sm_103a", os.path.join(HERE, "cuda",
                    "curand_factor.cu"), "-o", out], check=True, capture_output=True, timeout=600)
    return out


@pytest.mark.parametrize("seed,n,k", [(1, 5000, 5), (2, 1001, 7), (-5, 333, 3), (77, 20000, 2)])
def test_factor_bits_match_curand(native, oracle_lib, curand_bin, tmp_path, seed, n, k):
    path = str(tmp_path / "bits")
    subprocess.run([curand_bin, str(seed), str(n), str(k), path], check=True, timeout=120)
    ref = np.fromfile(path, np.int8).reshape(k, n)
    assert np.array_equal(native.volcano_factor(seed, n, k), ref)
    assert np.array_equal(oracle_lib.volcano_factor(seed, n, k), ref)
