"""Build recipe for libforkmatch.so and the ForkMatch CLI (sm_103a only).

Compiles each translation unit with nvcc in parallel, links the shared
library in-tree at ``forkmatch_gb300/lib/``, and links the CLI against it.
Usage: ``python -m forkmatch_gb300.build`` or ``forkmatch_gb300.build.build()``.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "lib")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I" + INCLUDE, "-I" + CSRC,
                  "--expt-relaxed-constexpr"]
SOURCES = ["fm_host.cu", "fm_match.cu", "fm_graph.cu", "fm_parse.cpp", "fm_static.cu", "fm_batch.cu",
           "fm_serve.cpp", "fm_table.cpp", "fm_ingest.cu"]
HEADERS = ["fm_internal.h", "fm_device.cuh", "fm_pool.h"]


def _nvcc():
    n = shutil.which("nvcc")
    if n is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        n = "/usr/local/cuda/bin/nvcc"
    if n is None:
        raise RuntimeError("nvcc not found")
    return n


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout[-6000:], r.stderr[-6000:]))
    return r


def _newer(out, deps):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose=False):
    os.makedirs(LIB, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "forkmatch.h")]
    objs = []
    jobs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(LIB, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if not _newer(obj, [sp] + hdrs):
            lang = ["-x", "cu"] if src.endswith(".cu") else []
            jobs.append([nvcc] + NVFLAGS + lang + ["-c", sp, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr)
    so = os.path.join(LIB, "libforkmatch.so")
    if not _newer(so, objs):
        tmp = so + ".tmp%d" % os.getpid()
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, so)
    cli = os.path.join(LIB, "ForkMatch")
    cli_src = os.path.join(CSRC, "fm_cli.cpp")
    if not _newer(cli, [so, cli_src, os.path.join(INCLUDE, "forkmatch.h")]):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", cli, "-L" + LIB, "-lforkmatch",
              "-Wl,-rpath,$ORIGIN"])
    return so


if __name__ == "__main__":
    print(build(verbose=True))
