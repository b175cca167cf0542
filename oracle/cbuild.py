"""Build the oracle's C baseline (oracle/newmark_cg.c) with gcc + OpenMP into oracle/_build.

Test infrastructure: used by tests, smoke() and the CPU-baseline legs of bench.py only.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle_newmark.so")
SRC = os.path.join(HERE, "newmark_cg.c")


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle baseline")
    os.makedirs(OUT, exist_ok=True)
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, "-O3", "-fopenmp", "-fPIC", "-shared", SRC, "-o", tmp, "-lm"], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle C build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
