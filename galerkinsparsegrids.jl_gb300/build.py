"""In-tree build of libsgdg.so for sm_103a (nvcc + g++, no cmake).

Translation units compile in parallel; the shared library links the CUDA
runtime statically, so loading it needs no libcudart on the path.
"""
import concurrent.futures as cf
import hashlib
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
# SGDG_DEBUG=1 builds (and the package then loads) the debug library, with
# device index checks, into its own directory
DEBUG = os.environ.get("SGDG_DEBUG") == "1"
OUT = os.path.join(HERE, "_build_debug" if DEBUG else "_build")
LIB = os.path.join(OUT, "libsgdg.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off"]
if DEBUG:
    HOST_FLAGS = HOST_FLAGS + ["-DSGDG_DEBUG"]
    NVCC_FLAGS = NVCC_FLAGS + ["-DSGDG_DEBUG"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _sources():
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    return cpp, cu


def _digest():
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for f in sorted(os.listdir(d)):
            if f.endswith((".cpp", ".cu", ".h", ".cuh")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(f.encode() + fh.read())
    h.update(" ".join(ARCH + HOST_FLAGS + NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compile every translation unit and link libsgdg.so; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "stamp")
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        return LIB
    cpp, cu = _sources()
    nvcc = _nvcc()
    jobs = []
    for f in cpp:
        jobs.append(["g++"] + HOST_FLAGS + ["-I", INCLUDE, "-c", os.path.join(CSRC, f),
                                            "-o", os.path.join(OUT, f + ".o")])
    for f in cu:
        jobs.append([nvcc] + ARCH + NVCC_FLAGS + ["-I", INCLUDE, "-c", os.path.join(CSRC, f),
                                                   "-o", os.path.join(OUT, f + ".o")])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OUT, f + ".o") for f in cpp + cu]
    tmp = LIB + ".%d.tmp" % os.getpid()
    run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC"])
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
