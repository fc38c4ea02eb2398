"""Build libsid.so (all CUDA sources, sm_103a) in-tree, under sid_gb300/_build/.

Used by ``__graft_entry__.build()`` and by the package loader.  Compiles each
translation unit in parallel with nvcc, then links one shared library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsid.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsid")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj: str, src: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src, *deps])


def _machine_stamp() -> str:
    import platform
    return f"{platform.machine()} {' '.join(ARCH)} {' '.join(NVCC_FLAGS)}"


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "STAMP")
    if not os.path.exists(stamp) or open(stamp).read() != _machine_stamp():
        force = True  # objects from another host architecture or other flags
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "sid.h"))
    exe = nvcc()
    jobs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if force or _stale(obj, src, deps):
            jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [exe, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(compile_one, jobs):
            if verbose and out:
                print(out)
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in sources()]
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libsid.so failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(_machine_stamp())
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
