"""Build libampe_gb300.so in-tree with nvcc for sm_103a.

The library is a plain C-ABI shared object (include/ampe_gb300.h): no
PyTorch types cross its boundary, so it is compiled straight with nvcc,
one translation unit per source, in parallel, then linked with
``nvcc -shared``.  Output: ampe_gb300/_build/libampe_gb300.so.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libampe_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "--extended-lambda",
    "-Xcompiler",
    "-fPIC",
    "-I" + os.path.join(ROOT, "include"),
    "-I" + CSRC,
]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu")
    )


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, extra_flags=()):
    os.makedirs(OUT, exist_ok=True)
    headers = [
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))
    ] + [os.path.join(ROOT, "include", "ampe_gb300.h")]
    cc = nvcc()
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            cmd = [cc] + ARCH + NVFLAGS + list(extra_flags) + ["-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg.strip():
                print(msg)
    if force or jobs or _newer(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs
        run(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
