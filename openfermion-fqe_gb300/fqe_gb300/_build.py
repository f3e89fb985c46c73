"""In-tree build of libfqegpu.so (CUDA, sm_103a only).

Each translation unit under ``csrc/`` is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into
``fqe_gb300/libfqegpu.so`` next to this file.  The CUDA runtime is linked
statically, so the library depends only on the CUDA driver library (libcuda).
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
LIB = os.path.join(PKG_DIR, "libfqegpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + CSRC,
    "-I" + INCLUDE, "--expt-relaxed-constexpr"
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required")


def sources():
    return sorted(
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _needs(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    headers = [
        os.path.join(CSRC, f) for f in os.listdir(CSRC)
        if f.endswith((".cuh", ".h"))
    ] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD,
                           os.path.basename(src).replace(".cu", ".o"))
        objs.append(obj)
        if force or _needs(obj, [src] + headers):
            jobs.append([cc] + CFLAGS + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" +
                               r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return cmd[-1]

    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(workers) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _needs(LIB, objs):
        run([cc] + ARCH + ["-shared", "-o", LIB] + objs)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
