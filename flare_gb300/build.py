"""Build libflaregb.so (CUDA, sm_103a) in-tree with nvcc.

Each .cu translation unit is compiled in parallel to an object file under
flare_gb300/_build/, then linked into flare_gb300/libflaregb.so.  Host code is
compiled with -ffp-contract=off so that the cell algebra shared with the
neighbour kernel keeps its documented operation order.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libflaregb.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith((".h", ".cuh"))] + \
        [os.path.join(ROOT, "include", "flaregb.h")]
    flags = [ARCH, "-O3", "-lineinfo", "-std=c++17",
             "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", CSRC,
             "-I", os.path.join(ROOT, "include")]
    jobs = []
    for src in sources():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src[:-3] + ".o")
        if force or _stale(o, [s, __file__] + headers):
            jobs.append([nvcc, *flags, "-c", s, "-o", o])
    objs = [os.path.join(BUILD, s[:-3] + ".o") for s in sources()]

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" +
                               r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    if jobs or not os.path.exists(LIB) or _stale(LIB, objs):
        run([nvcc, ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-lcublas",
             "-lcusolver"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
