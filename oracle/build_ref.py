"""Build recipe for the reference programs ``kuramoto`` and ``kuramoto_64`` (TEST INFRASTRUCTURE ONLY).

The reference (znicolaou/kuramoto) is two CUDA programs: ``kuramoto.cu`` + ``dp45.cu`` (FP32) and
``kuramoto_64.cu`` + ``dp45_64.cu`` (FP64), built by the one-line recipe of its README
(``nvcc -lcuda -lcublas -lcurand -O3 -o kuramoto dp45.cu kuramoto.cu``).  Here they are the
checker of the GPU path: tests run them through their ``-R`` reload path on the same
``fs.dat`` / ``frequencies.dat`` / ``adj.dat`` files as this project's integrator.

The build has two stages, because the sources exist only where the reference is checked out
and the GPU host may have another CPU architecture:

  1. ``prepare(ref_dir)`` runs where the reference sources are.  nvcc compiles each of the four
     ``.cu`` files where they lie: device code to sm_103a, embedded as a fat binary in nvcc's
     host-side intermediate (``--cuda``: preprocessed C++ for the host compiler).  Outputs go
     to ``oracle/_ref/*.cu.ii`` only (git-ignored, never committed).
  2. ``finish()`` compiles those intermediates with the host's g++ and links them against the
     CUDA runtime, cuBLAS and cuRAND into ``oracle/_ref/kuramoto`` and ``kuramoto_64``.

``_FORTIFY_SOURCE`` is undefined during preprocessing so that the intermediates carry no
glibc inline wrappers specific to the preprocessing host.  The host compile uses
``-fsigned-char``: the reference stores getopt's int result in a ``char`` and compares it with
-1 (kuramoto.cu:292, 299), which terminates its option loop only where char is signed (x86_64);
with aarch64's unsigned char the loop never ends.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# where this recipe looks for the reference checkout when no directory is given
DEFAULT_REF = "/root/reference"
PROGRAMS = {"kuramoto": ("kuramoto.cu", "dp45.cu"), "kuramoto_64": ("kuramoto_64.cu", "dp45_64.cu")}


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _intermediate(src):
    return os.path.join(OUT, src + ".ii")


def binary(fp64=False):
    """Path of the built reference program (``kuramoto`` or ``kuramoto_64``)."""
    return os.path.join(OUT, "kuramoto_64" if fp64 else "kuramoto")


def available():
    return all(os.path.exists(binary(f)) for f in (False, True))


def prepared():
    return all(os.path.exists(_intermediate(s)) for srcs in PROGRAMS.values() for s in srcs)


def prepare(ref_dir):
    """Stage 1: nvcc on the reference sources where they lie; writes oracle/_ref/*.cu.ii."""
    os.makedirs(OUT, exist_ok=True)
    nv = _nvcc()
    jobs = []
    for srcs in PROGRAMS.values():
        for s in srcs:
            path = os.path.join(ref_dir, s)
            if not os.path.exists(path):
                raise RuntimeError("reference source missing: %s" % path)
            jobs.append([nv, *ARCH, "-O3", "--cuda", "-Xcompiler", "-U_FORTIFY_SOURCE", "-I", ref_dir, path,
                         "-o", _intermediate(s)])
    with ThreadPoolExecutor(len(jobs)) as ex:
        list(ex.map(_run, jobs))


def finish():
    """Stage 2: host compile of the intermediates and link, on the machine that runs them."""
    if not prepared():
        raise RuntimeError("oracle/_ref holds no prepared reference intermediates")
    nv = _nvcc()
    lib64 = os.path.join(_cuda_home(), "lib64")
    objs = {}
    jobs = []
    for srcs in PROGRAMS.values():
        for s in srcs:
            o = os.path.join(OUT, s + ".o")
            objs[s] = o
            jobs.append(["g++", "-O3", "-w", "-fsigned-char", "-c", "-x", "c++-cpp-output", _intermediate(s), "-o", o])
    with ThreadPoolExecutor(len(jobs)) as ex:
        list(ex.map(_run, jobs))
    for name, srcs in PROGRAMS.items():
        _run([nv, *ARCH, "-o", os.path.join(OUT, name), *[objs[s] for s in srcs], "-L", lib64,
              "-lcublas", "-lcurand", "-lcuda"])
    for o in objs.values():
        os.remove(o)


def build(ref_dir=None):
    """Prepare (where the reference sources exist) and finish (where a host compiler and CUDA exist).

    Returns the output folder, or None when neither the sources nor prepared intermediates exist.
    """
    ref_dir = ref_dir or os.environ.get("KURA_REFERENCE_DIR") or DEFAULT_REF
    if ref_dir and os.path.isdir(ref_dir):
        prepare(ref_dir)
    if not prepared():
        return None
    finish()
    return OUT


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
