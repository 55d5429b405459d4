"""Build the CUDA library (sm_103a) and, for the test suite, the CPU oracle.

    python -m trans_bl_gb300.build          # library + oracle
Outputs (git-ignored, rebuilt on every machine):
    trans_bl_gb300/libtransbl.so
    oracle/_build/libtb_oracle.so
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtransbl.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def build_library(verbose=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I" + os.path.join(ROOT, "include")]
    # extra flags, e.g. the multigrid's tuning macros: TB_NVCC_EXTRA="-DTB_MG_NU_PRE=3"
    common += os.environ.get("TB_NVCC_EXTRA", "").split()
    jobs = []
    for s in srcs:
        obj = os.path.join(BUILD, s.rsplit(".", 1)[0] + ".o")
        if s.endswith(".cu"):
            cmd = [nvcc] + ARCH + ["-lineinfo"] + common + ["-c", os.path.join(CSRC, s), "-o", obj]
        else:
            cmd = [nvcc] + common + ["-x", "c++", "-c", os.path.join(CSRC, s), "-o", obj]
        jobs.append((cmd, obj))
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        outs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    tmp = LIB + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + [o for _, o in jobs] + ["-lcudart"])
    os.replace(tmp, LIB)
    return LIB


def build_oracle():
    odir = os.path.join(ROOT, "oracle")
    _run(["make", "-s", "-C", odir])
    return os.path.join(odir, "_build", "libtb_oracle.so")


def main():
    print(build_library(verbose="-v" in sys.argv))
    print(build_oracle())


if __name__ == "__main__":
    main()
