"""Build libelastic_rtm.so (CUDA, sm_103a) in tree.

Every translation unit under csrc/ is compiled in parallel with nvcc for
sm_103a only and linked into elastic_gb300/libelastic_rtm.so.  Host code is
compiled with -ffp-contract=off so that host-side tables (Ricker wavelet,
sponge filter) are rounded exactly as the reference computes them on every
host architecture (aarch64 compilers fuse multiply-adds by default).  No torch
extension machinery: the library is a plain C-ABI shared object that
Fortran/C callers link directly.
"""
import concurrent.futures as cf
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
# objects per host architecture: a working tree copied between an x86 and an
# Arm machine never links the other's objects
OBJ = os.path.join(HERE, "_build", platform.machine() or "host")
LIB = os.path.join(HERE, "libelastic_rtm.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-diag-suppress", "177"]


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "elastic_rtm.h"))
    jobs = []
    for s in sources():
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s[:-3] + ".o")
        if force or _newer(obj, [src] + headers):
            jobs.append([NVCC, *ARCH, *FLAGS, "-c", src, "-o", obj])
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        return r
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OBJ, s[:-3] + ".o") for s in sources()]
    # the stamp holds the modification time of the library this
    # architecture's objects last linked: a library linked elsewhere (another
    # architecture sharing the tree) does not match and is relinked
    stamp = os.path.join(OBJ, "lib.stamp")
    linked = open(stamp).read().strip() if os.path.exists(stamp) else ""
    current = repr(os.path.getmtime(LIB)) if os.path.exists(LIB) else "none"
    if force or jobs or _newer(LIB, objs) or linked != current:
        run([NVCC, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs])
        with open(stamp, "w") as f:
            f.write(repr(os.path.getmtime(LIB)))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
