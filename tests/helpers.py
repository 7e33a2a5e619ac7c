"""Shared helpers of the test suite: seeded inputs and comparisons."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return os.path.join(GOLDEN, name)


def cauchy_inputs(n, seed, init=2 * np.pi, scale=1.0):
    """Seeded theta0 uniform in [0, init) and Cauchy omega of the given scale."""
    rng = np.random.default_rng(seed)
    th = (rng.random(n) * init).astype(np.float32)
    om = (scale * np.tan(np.pi * (rng.random(n) - 0.5))).astype(np.float32)
    return th, om


def normal_inputs(n, seed, init=np.pi):
    rng = np.random.default_rng(seed)
    th = (rng.random(n) * init).astype(np.float32)
    om = rng.standard_normal(n).astype(np.float32)
    return th, om


def wrapped_diff(a, b):
    """|a - b| taken modulo 2*pi (phases)."""
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return np.abs((d + np.pi) % (2 * np.pi) - np.pi)
