"""Build the in-tree shared library ``exadg_gb300/_lib/libexadg_gb300.so`` with nvcc for sm_103a.

Each translation unit compiles in parallel to an object file; the objects are linked into one
shared library that exports the C ABI declared in ``include/exadg_gb300.h``.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libexadg_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", SRC, "-I", os.path.join(HERE, "..", "include")]

SOURCES = [
    "sipg_cart_f64.cu",
    "sipg_cart_f32.cu",
    "sipg_cart_df64.cu",
    "sipg_cartesian.cu",
    "sipg_general.cu",
    "solver_kernels.cu",
    "cg_device.cu",
    "vec_ops.cu",
    "fe_tables.cpp",
    "host.cpp",
    "capi.cpp",
    "noalloc.cu",
    "cnn.cu",
    "lattice.cu",
    "block_jacobi.cu",
]


def _needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(SRC):
        if os.path.getmtime(os.path.join(SRC, f)) > t:
            return True
    hdr = os.path.join(HERE, "..", "include", "exadg_gb300.h")
    return os.path.getmtime(hdr) > t


def _compile(src, verbose=False):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [NVCC] + ARCH + COMMON + ["-c", os.path.join(SRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC] + COMMON + ["-x", "c++", "-c", os.path.join(SRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-8000:]))
    return obj, r.stderr


def build(force=False, verbose=False, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    if not force and not _needs_build():
        return LIB
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [r[0] for r in results]
    if verbose:
        for r in results:
            sys.stderr.write(r[1])
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr[-8000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
