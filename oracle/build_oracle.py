"""Build recipe for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Compiles, with g++ only, into ``oracle/_build/``:
  * ``libkora.so``          -- C ABI used through ctypes by tests and bench.py's CPU legs
  * ``kuramoto_oracle``     -- CLI restatement of the reference ``kuramoto`` (float files)
  * ``kuramoto_oracle_64``  -- the same for ``kuramoto_64`` (double files)

``-ffp-contract=off`` keeps the arithmetic identical on x86_64 and aarch64 (no
fused multiply-add contraction), so the oracle gives the same bits on both.
"""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-result"]


def _jobs():
    src = lambda f: os.path.join(HERE, f)
    out = lambda f: os.path.join(OUT, f)
    return [
        ["g++", *FLAGS, "-shared", "-fPIC", src("kora_capi.cpp"), "-o", out("libkora.so")],
        ["g++", *FLAGS, src("kora_cli.cpp"), "-o", out("kuramoto_oracle")],
        ["g++", *FLAGS, "-DKORA_FP64", src("kora_cli.cpp"), "-o", out("kuramoto_oracle_64")],
    ]


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    jobs = _jobs()

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), r.stderr))
        if verbose and r.stderr:
            print(r.stderr)

    with ThreadPoolExecutor(len(jobs)) as ex:
        list(ex.map(run, jobs))
    return OUT


if __name__ == "__main__":
    print(build(verbose=True))
