"""Build libyaksa.so (C host library + sm_103a CUDA kernels) in-tree.

    python -m yaksa_gb300.build          # or: python yaksa_gb300/build.py

C sources compile with gcc, CUDA sources with nvcc for sm_103a only, all in parallel;
the objects link into yaksa_gb300/lib/libyaksa.so with the CUDA runtime linked
statically, so the library needs only the NVIDIA driver at run time.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libyaksa.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: the GB300 engine has no CPU build")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".c", ".cu")))


def build(verbose=False, extra_nvcc=()):
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(cuda, "include")]
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    jobs = []
    objs = []
    for f in sources():
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if f.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xptxas", "-v" if verbose else "-O3", *extra_nvcc, *inc, "-c", src, "-o", obj]
        else:
            cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter",
                   *inc, "-c", src, "-o", obj]
        jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=min(16, len(jobs))) as ex:
        results = list(ex.map(_run, jobs))
    if verbose:
        for r in results:
            sys.stderr.write(r.stderr)
    # export the yaksa_* API only: internal yk_* symbols and the static CUDA runtime stay
    # private, so the library can sit in any application without symbol clashes
    vscript = os.path.join(BUILD, "exports.map")
    with open(vscript, "w") as f:
        f.write("{ global: yaksa_*; local: *; };\n")
    _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-Xlinker", "-Bsymbolic",
          "-Xlinker", "--no-undefined", "-Xlinker", "--version-script=" + vscript,
          "-lpthread", "-lrt", "-ldl"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
