"""Builds libvgpu.so in-tree: the sm_103a kernels (nvcc) and the C11 host
layer (gcc), linked into one shared library next to this file.

    python -m vectra_gb300.build             # or vectra_gb300.build.build()
    python -m vectra_gb300.build --archive   # also libvgpu.a, for linking the
                                             # nodes into the vectra package

No CMake, no torch extension machinery: a handful of translation units
compiled in parallel, then one link step.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvgpu.so")
ARCHIVE = os.path.join(HERE, "libvgpu.a")

CU_SOURCES = ["k_groupby_fastj.cu", "k_groupby_fast.cu", "k_groupby.cu", "jit_agg.cu", "k_filter.cu",
              "k_sort.cu", "k_hashjoin.cu", "k_prof.cu", "k_static.cu", "k_batch.cu", "k_serve.cu",
              "k_pagg.cu", "k_strings.cu"]
# headers the run-time compiler needs, embedded into jit_agg.cu's object
JIT_HEADERS = [("vg_rtc_types.h", CSRC), ("vectra_abi.h", INCLUDE), ("vgpu_internal.h", CSRC),
               ("k_common.cuh", CSRC), ("k_groupby_dev.cuh", CSRC), ("k_jit_lib.cuh", CSRC),
               ("k_jit_kernel.cuh", CSRC), ("k_jit_pagg.cuh", CSRC)]
C_SOURCES = ["runtime.c", "compile.c", "source.c", "node_filter.c",
             "node_project.c", "node_agg.c", "node_join.c", "noalloc.c", "scan_vtr.c", "node_sort.c",
             "strdict.c"]

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def _cuda_include():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return os.path.join(cuda, "include")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _stale(obj, srcs):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def _write_jit_headers():
    """vg_jit_headers.inc: the device headers as string literals, for NVRTC."""
    names, srcs = [], []
    for name, d in JIT_HEADERS:
        text = open(os.path.join(d, name)).read()
        if ")VGJH\"" in text:
            raise RuntimeError("%s contains the raw-string delimiter" % name)
        names.append('"%s"' % name)
        srcs.append('R"VGJH(%s)VGJH"' % text)
    out = ("// generated by build.py from the device headers; do not edit\n"
           "static const char *const kJitHeaderNames[] = {%s};\n"
           "static const char *const kJitHeaderSources[] = {\n%s};\n"
           "static const int kJitHeaderCount = %d;\n") % (", ".join(names), ",\n".join(srcs), len(names))
    path = os.path.join(BUILD, "vg_jit_headers.inc")
    if not os.path.exists(path) or open(path).read() != out:
        with open(path, "w") as f:
            f.write(out)


def build(verbose=False, archive=False):
    """Compiles what changed and links libvgpu.so (and, with archive=True,
    a static libvgpu.a of the same objects).  Returns the .so path."""
    os.makedirs(BUILD, exist_ok=True)
    _write_jit_headers()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    jobs = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([_nvcc(), GENCODE, "-O3", "-lineinfo", "-std=c++17",
                         "-Xcompiler", "-fPIC", "-I", CSRC, "-I", INCLUDE, "-I", BUILD, "-c", src, "-o", obj])
    for f in C_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["gcc", "-std=gnu11", "-O2", "-g", "-fPIC", "-Wall", "-Wno-unused-function",
                         "-I", CSRC, "-I", INCLUDE, "-I", _cuda_include(), "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                sys.stderr.write(r.stdout + r.stderr)
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cuda_lib = os.path.join(os.path.dirname(_cuda_include()), "lib64")
        _run([_nvcc(), GENCODE, "-shared", "-o", tmp] + objs +
             ["-cudart", "static", "-L", cuda_lib, "-lnvrtc", "-lpthread", "-Xlinker", "-rpath=" + cuda_lib])
        os.replace(tmp, LIB)
    if archive:
        if os.path.exists(ARCHIVE):
            os.remove(ARCHIVE)
        _run(["ar", "rcs", ARCHIVE] + objs)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, archive="--archive" in sys.argv[1:]))
