"""Regenerate the golden fixtures under tests/golden/ from the reference checkout.

Give the reference checkout as the argument (or in the REFERENCE environment variable):
    python tests/golden/make_golden.py REFERENCE_DIR
The fixtures are data files of the reference repository (znicolaou/kuramoto,
data/), copied byte for byte, plus their SHA-256 digests:
  * {normal,cauchy}_K{0,2,5000}_seed1_frequencies.dat  -- frequencies.dat of seed 1, N=5000
    (job1.sh:24-25: `-N 5000 -K K -s 1 -c 1.75 -t 100 -d 0.01 -D 0 [-n] -vR`)
  * {normal,cauchy}_K0_seed1_fs.dat  -- the final fs.dat of the uncoupled runs
    (theta[N], t, h; written by an older revision of the program, N+2 floats)
  * {normal,cauchy}_N5000_K{0,2}_avgorder.npy, normal_N10000_K2000_avgorder.npy
    -- order.dat averaged over the seeds of the job arrays (float32[10001])
"""
import hashlib
import json
import os
import shutil
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE")
HERE = os.path.dirname(os.path.abspath(__file__))

FILES = {}
for K in (0, 2, 5000):
    FILES["normal_K%d_seed1_frequencies.dat" % K] = "data/5000/%d/1frequencies.dat" % K
    FILES["cauchy_K%d_seed1_frequencies.dat" % K] = "data/5000_lorentz/%d/1frequencies.dat" % K
FILES["normal_K0_seed1_fs.dat"] = "data/5000/0/1fs.dat"
FILES["cauchy_K0_seed1_fs.dat"] = "data/5000_lorentz/0/1fs.dat"
FILES["normal_N5000_K0_avgorder.npy"] = "data/5000/0/avgorder.npy"
FILES["cauchy_N5000_K0_avgorder.npy"] = "data/5000_lorentz/0/avgorder.npy"
FILES["normal_N5000_K2_avgorder.npy"] = "data/5000/2/avgorder.npy"
FILES["cauchy_N5000_K2_avgorder.npy"] = "data/5000_lorentz/2/avgorder.npy"
FILES["normal_N10000_K2000_avgorder.npy"] = "data/10000/2000/avgorder.npy"


def main():
    if not REF:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_DIR")
    if not os.path.isdir(REF):
        sys.exit("reference checkout not found: %s" % REF)
    digests = {}
    for dst, src in FILES.items():
        s = os.path.join(REF, src)
        if not os.path.exists(s):
            print("missing", s)
            continue
        shutil.copyfile(s, os.path.join(HERE, dst))
        digests[dst] = {"source": src, "sha256": hashlib.sha256(open(s, "rb").read()).hexdigest()}
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(digests, f, indent=1, sort_keys=True)
    print("wrote", len(digests), "fixtures")


if __name__ == "__main__":
    main()
