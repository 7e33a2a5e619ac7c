"""Build recipe of the native parts of kuramoto_gb300 (sm_103a only).

Produces, in ``kuramoto_gb300/_build/``:
  * ``libkura.so``  -- the C ABI of include/kura.h: persistent DP45 kernels and host logic
  * ``kuramoto``    -- the drop-in command line (same flags and FILEBASE files as the
                       reference ``kuramoto``), a C++ program linked against libkura.so

Translation units compile in parallel; no cmake.  Host C++ is compiled with
``-ffp-contract=off`` so that x86_64 and aarch64 builds give identical host arithmetic.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
SRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    cu_flags = [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INC, "-I", SRC]
    if ptxas_info:
        cu_flags += ["-Xptxas", "-v"]
    objs = {
        "kura_kernels.o": [nv, *cu_flags, "-c", os.path.join(SRC, "kura_kernels.cu")],
        "kura_api.o": [nv, *cu_flags, "-c", os.path.join(SRC, "kura_api.cu")],
        "kura_noalloc.o": [nv, *cu_flags, "-c", os.path.join(SRC, "kura_noalloc.cu")],
        "kura_tensor.o": [nv, *cu_flags, "-c", os.path.join(SRC, "kura_tensor.cu")],
        "kura_multi.o": [nv, *cu_flags, "-c", os.path.join(SRC, "kura_multi.cu")],
        "kura_mlp.o": [nv, *cu_flags, "-c", os.path.join(SRC, "kura_mlp.cu")],
        "kura_host_rng.o": ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INC, "-c",
                            os.path.join(SRC, "kura_host_rng.cpp")],
    }
    jobs = [cmd + ["-o", os.path.join(OUT, name)] for name, cmd in objs.items()]
    with ThreadPoolExecutor(len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    lib = os.path.join(OUT, "libkura.so")
    _run([nv, *ARCH, "-shared", "-o", lib, *[os.path.join(OUT, o) for o in objs], "-cudart", "shared"])
    cli = os.path.join(OUT, "kuramoto")
    _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", INC, "-I", os.path.join(cuda_home(), "include"),
          os.path.join(SRC, "kuramoto_cli.cpp"),
          "-o", cli, "-L", OUT, "-lkura", "-Wl,-rpath,$ORIGIN",
          "-L", os.path.join(cuda_home(), "lib64"), "-lcudart"])
    return OUT


if __name__ == "__main__":
    import sys
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
