"""Build of the CUDA library libbse_gb300.so (sm_103a) from csrc/*.cu with nvcc.

Translation units are compiled in parallel and linked against cuBLAS/cuSOLVER; the
result stays in-tree under _build/ (git-ignored)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libbse_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj, deps):
    return not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(d) for d in deps)


def _host_stamp(cc: str) -> str:
    """Machine and compiler the objects were built for: a tree built elsewhere (another CPU
    architecture, another toolkit) is rebuilt from scratch rather than trusted by mtime."""
    r = subprocess.run([cc, "--version"], capture_output=True, text=True)
    return platform.machine() + "\n" + r.stdout.strip().splitlines()[-1] + "\n"


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    stamp_path = os.path.join(OUT, "host.txt")
    stamp = _host_stamp(nvcc())
    try:
        force = force or open(stamp_path).read() != stamp
    except OSError:
        force = True
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers.append(os.path.join(INCLUDE, "bse_gpu.h"))
    srcs = sources()
    objs = [os.path.join(OUT, os.path.basename(s)[:-3] + ".o") for s in srcs]
    cc = nvcc()
    jobs = []
    for s, o in zip(srcs, objs):
        if force or _stale(o, [s] + headers):
            jobs.append([cc] + ARCH + FLAGS + ["-I", INCLUDE, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or not os.path.exists(LIB) or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        run([cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcublas", "-lcusolver", "-lcudart", "-Xlinker", "--no-undefined"])
        os.replace(tmp, LIB)
    with open(stamp_path, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
