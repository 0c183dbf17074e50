"""Build ``tnqvm_gb300/_lib/libgb300mps.so`` for sm_103a with nvcc.

One translation unit per source, compiled in parallel, then linked into one
shared library that exports the ``gb300mps.h`` C ABI.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libgb300mps.so")
SOURCES = ["k_ops.cu", "k_measure.cu", "engine.cu", "serve.cu", "graph.cu", "k_gemm.cu", "k_coop.cu", "wide.cu", "density.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        exe = "/usr/local/cuda/bin/nvcc"
    if exe is None:
        raise RuntimeError("nvcc not found")
    return exe


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp"))]
    headers.append(os.path.join(HERE, "..", "include", "gb300mps.h"))
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc()] + FLAGS + ARCH + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc(), "-shared"] + ARCH + objs + ["-o", LIB, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


VISITOR_DIR = os.path.join(HERE, "visitor")
VISITOR_DEMO = os.path.join(OUT, "visitor_demo")


def build_visitor_demo():
    """Compile the C++ TNQVM visitor plugin (shim build) and its driver, linked
    against libgb300mps.so."""
    lib = build()
    srcs = [os.path.join(VISITOR_DIR, f) for f in ("GpuMpsVisitor.cpp", "GpuPmpsVisitor.cpp", "visitor_demo.cpp")]
    deps = srcs + [os.path.join(VISITOR_DIR, f) for f in os.listdir(VISITOR_DIR) if f.endswith(".hpp")] + [lib]
    if not _stale(VISITOR_DEMO, deps):
        return VISITOR_DEMO
    cmd = ["g++", "-std=c++17", "-O2", "-I", VISITOR_DIR] + srcs + ["-o", VISITOR_DEMO, "-L", OUT, "-lgb300mps",
                                                                    "-Wl,-rpath," + OUT]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("visitor build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return VISITOR_DEMO


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
