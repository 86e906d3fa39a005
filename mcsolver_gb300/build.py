"""Build libmcsgpu.so (sm_103a) and the CPython drop-in modules in-tree.

Outputs (git-ignored) go to ``mcsolver_gb300/lib/``:
    libmcsgpu.so                  the engine (CUDA kernels + C ABI, include/mcsgpu.h)
    isinglib.so xylib.so heisenberglib.so   drop-ins for mcsolver's compiled libraries

Translation units are compiled in parallel; a content stamp skips the build
when no source changed.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "obj")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-extended-lambda",
              "-Xcompiler", "-Wall"] + ARCH


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.isfile(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(nvcc))


def _sources():
    return sorted(os.path.join(SRC, f) for f in os.listdir(SRC)
                  if f.endswith((".cu", ".cpp", ".c", ".h", ".cuh"))) + [os.path.join(INCLUDE, "mcsgpu.h"),
                                                                          os.path.abspath(__file__)]


def _stamp() -> str:
    h = hashlib.sha256()
    for f in _sources():
        with open(f, "rb") as fh:
            h.update(f.encode())
            h.update(fh.read())
    h.update(sys.version.encode())
    return h.hexdigest()


def built_paths():
    return {"engine": os.path.join(LIB, "libmcsgpu.so"),
            "isinglib": os.path.join(LIB, "isinglib.so"),
            "xylib": os.path.join(LIB, "xylib.so"),
            "heisenberglib": os.path.join(LIB, "heisenberglib.so")}


def build(force: bool = False, verbose: bool = False) -> dict:
    os.makedirs(OBJ, exist_ok=True)
    stamp_file = os.path.join(LIB, ".stamp")
    st = _stamp()
    paths = built_paths()
    if (not force and os.path.isfile(stamp_file) and open(stamp_file).read() == st
            and all(os.path.isfile(p) for p in paths.values())):
        return paths
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    jobs = []
    objs = []
    for f in ("mcs_kernels.cu", "mcs_cluster.cu", "mcs_noalloc.cu", "mcs_pt.cu", "mcs_model.cpp", "mcs_engine.cpp", "mcs_server.cpp"):
        o = os.path.join(OBJ, f + ".o")
        objs.append(o)
        cmd = [nvcc] + NVCC_FLAGS + ["-x", "cu" if f.endswith(".cu") else "c++", "-c", os.path.join(SRC, f), "-o", o]
        if f.endswith(".cpp"):
            cmd = [nvcc, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-c",
                   os.path.join(SRC, f), "-o", o]
        jobs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    errs = []
    for j in jobs:
        out, _ = j.communicate()
        if j.returncode != 0:
            errs.append(out.decode(errors="replace"))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if errs:
        raise RuntimeError("CUDA build failed:\n" + "\n".join(errs))
    subprocess.run([nvcc] + ARCH + ["-shared", "-o", paths["engine"]] + objs + ["-lcudart"],
                   check=True, capture_output=not verbose)
    pyinc = sysconfig.get_paths()["include"]
    cc = os.environ.get("CC", "gcc")
    jobs = []
    for i, name in enumerate(("isinglib", "xylib", "heisenberglib"), start=1):
        cmd = [cc, "-O2", "-fPIC", "-shared", "-Wall", "-DMCS_PYMOD=%d" % i, "-I" + pyinc,
               os.path.join(SRC, "mcs_pymod.c"), "-o", paths[name], "-L" + LIB, "-lmcsgpu",
               "-Wl,-rpath,$ORIGIN", "-L" + os.path.join(cuda, "lib64")]
        jobs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    for j in jobs:
        out, _ = j.communicate()
        if j.returncode != 0:
            raise RuntimeError("python module build failed:\n" + out.decode(errors="replace"))
    with open(stamp_file, "w") as fh:
        fh.write(st)
    return paths


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
