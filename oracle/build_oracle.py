"""Build recipe of the CPU oracle (test infrastructure): g++ -O2 -fopenmp on
oracle/bse_oracle.cpp -> oracle/_build/libbse_oracle.so.  Host code only, portable
(no -march flags), so the same recipe runs on x86_64 and aarch64 hosts."""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bse_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libbse_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "..", "include", "bse_gpu.h")]
    # a library built on another machine (CPU architecture) is rebuilt, not trusted by mtime
    stamp_path = os.path.join(OUT_DIR, "host.txt")
    try:
        force = force or open(stamp_path).read() != platform.machine()
    except OSError:
        force = True
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    with open(stamp_path, "w") as f:
        f.write(platform.machine())
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
