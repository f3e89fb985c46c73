"""In-tree build of libfqegpu.so (CUDA, sm_103a only).

Each translation unit under ``csrc/`` is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into
``fqe_gb300/libfqegpu.so`` next to this file.  The CUDA runtime is linked
statically, so the library depends only on the CUDA driver library (libcuda).

Rebuilds are keyed on content, not on file times: every object carries a
stamp with the SHA-256 of its compiler command, its source and every header,
and the library a stamp over the objects' stamps and the host machine type.
An object or library copied from another machine (or left from an older
source) is rebuilt because its stamp does not match.
"""

import concurrent.futures
import hashlib
import os
import platform
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


def _digest(cmd, files) -> str:
    h = hashlib.sha256()
    h.update(" ".join(cmd).encode())
    h.update(platform.machine().encode())
    for f in files:
        h.update(f.encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


def _stamp_ok(target, digest) -> bool:
    try:
        with open(target + ".stamp") as fh:
            return os.path.exists(target) and fh.read().strip() == digest
    except OSError:
        return False


def _write_stamp(target, digest) -> None:
    with open(target + ".stamp", "w") as fh:
        fh.write(digest + "\n")


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    headers = sorted([
        os.path.join(CSRC, f) for f in os.listdir(CSRC)
        if f.endswith((".cuh", ".h"))
    ] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)])
    jobs = []
    objs = []
    digests = []
    for src in sources():
        obj = os.path.join(BUILD,
                           os.path.basename(src).replace(".cu", ".o"))
        objs.append(obj)
        cmd = [cc] + CFLAGS + ["-c", src, "-o", obj]
        dg = _digest(cmd, [src] + headers)
        digests.append(dg)
        if force or not _stamp_ok(obj, dg):
            jobs.append((cmd, obj, dg))

    def run(job):
        cmd, target, dg = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" +
                               r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        if dg is not None:
            _write_stamp(target, dg)
        return target

    # the slowest translation units first, so the parallel build ends sooner
    jobs.sort(key=lambda j: -os.path.getsize(j[0][-3]))
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(workers) as ex:
            list(ex.map(run, jobs))
    link = [cc] + ARCH + ["-shared", "-o", LIB] + objs
    ldg = hashlib.sha256((" ".join(link) + platform.machine() +
                          "".join(digests)).encode()).hexdigest()
    if force or jobs or not _stamp_ok(LIB, ldg):
        run((link, LIB, ldg))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
