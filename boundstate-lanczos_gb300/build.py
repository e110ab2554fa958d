"""Build recipe for libbsl_gb300.so (in-tree, sm_103a only).

    python boundstate-lanczos_gb300/build.py

Compiles the CUDA kernels with nvcc for sm_103a and the host C++ with g++,
in parallel, into boundstate-lanczos_gb300/_build/, and links the shared
library next to this file.  Nothing is installed.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbsl_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose=False, extra_nvcc=()):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I", os.path.join(REPO, "include"), "-I", CSRC]
    jobs = []
    for f in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        if f.endswith(".cu"):
            jobs.append([nvcc, "-c", src, "-o", obj] + ARCH +
                        ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-fvisibility=hidden",
                         "-Xptxas", "-v"] + list(extra_nvcc) + inc)
        elif f.endswith(".cpp"):
            jobs.append(["g++", "-c", src, "-o", obj, "-O3", "-fPIC", "-fvisibility=hidden", "-std=c++17", "-Wall",
                         "-I", os.path.join(cuda, "include")] + inc)
    with ThreadPoolExecutor(max_workers=max(2, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    objs = [j[j.index("-o") + 1] for j in jobs]
    _run([nvcc, "-shared"] + ARCH + objs + ["-o", LIB])
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
