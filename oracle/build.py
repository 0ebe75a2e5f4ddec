"""Build recipe for the oracle (test infrastructure).

* ``oracle/_ref/liboracle.so`` is not produced here; the oracle library is
  ``oracle/liboracle.so`` compiled with gcc from ``fm_oracle.c``.
* ``oracle/_ref/ref_planner`` is the reference's own host query planner,
  compiled from the ForkMatch sources where they lie (``<ref>/src``) together
  with ``ref_planner_probe.cu``.  It is built only when the reference tree is
  present; nothing at run time depends on it.
* ``oracle/_ref/ref_matcher`` is the reference's own GPU matcher built without
  SYMMETRY behind ``ref_matcher_probe.cu``; it generates the golden fixture
  ``tests/golden/ref_matches.json`` on a GPU (``tests/golden/make_ref_matches.py``)
  and is never run by tests or the benchmark.

Outputs are git-ignored.  Run ``python oracle/build.py`` or call ``build()``.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The ForkMatch checkout these recipes read: $FM_REFERENCE_ROOT, else the
# build container's read-only mount.  It is absent on the GPU machine, where only
# the outputs already staged under oracle/_ref/ are used.
REF_ROOT = os.environ.get("FM_REFERENCE_ROOT", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout[-4000:], r.stderr[-4000:]))


def build_oracle():
    out = os.path.join(HERE, "liboracle.so")
    src = os.path.join(HERE, "fm_oracle.c")
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(src),
                                                            os.path.getmtime(os.path.join(HERE, "fm_oracle.h"))):
        return out
    tmp = out + ".tmp%d" % os.getpid()
    _run(["gcc", "-O2", "-std=c11", "-shared", "-fPIC", "-pthread", "-Wall", "-o", tmp, src])
    os.replace(tmp, out)
    return out


def build_ref_planner():
    """Compile the reference's host planner probe; returns its path or None."""
    if not os.path.isdir(REF_SRC) or shutil.which("nvcc") is None:
        return None
    ref_dir = os.path.join(HERE, "_ref")
    os.makedirs(ref_dir, exist_ok=True)
    out = os.path.join(ref_dir, "ref_planner")
    probe = os.path.join(HERE, "ref_planner_probe.cu")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(probe):
        return out
    _run(["nvcc", "-std=c++20", "-Xcompiler", "-std=c++20 -O1 -fpermissive -w", "-w",
          "-I" + REF_SRC, probe, "-o", out])
    return out


# The reference sources the matcher probe needs, staged into oracle/_ref/src
# (git-ignored, like every output of these recipes) so that the probe can be
# compiled on a machine without the reference checkout (the GPU machine has
# another CPU architecture, so nothing compiled here runs there).
REF_FILES = ("smsm.cu", "smsm.cuh", "trie.cuh", "ccsr.cuh", "hostparser.cuh", "intersect.cuh", "tbs.cuh",
             "environment.cuh")


def stage_reference_sources():
    """Copy the reference's src/ files the matcher probe includes into
    oracle/_ref/src; returns that folder, or None without a reference checkout."""
    if not os.path.isdir(REF_SRC):
        return None
    dst = os.path.join(HERE, "_ref", "src")
    os.makedirs(dst, exist_ok=True)
    for name in REF_FILES:
        shutil.copyfile(os.path.join(REF_SRC, name), os.path.join(dst, name))
    return dst


def build_ref_matcher():
    """Compile the reference's own GPU matcher (SYMMETRY undefined) behind
    ref_matcher_probe.cu into oracle/_ref/ref_matcher, from the reference
    checkout or from the staged copy; returns its path or None."""
    src = REF_SRC if os.path.isdir(REF_SRC) else os.path.join(HERE, "_ref", "src")
    if not os.path.isfile(os.path.join(src, "smsm.cu")) or shutil.which("nvcc") is None:
        return None
    out = os.path.join(HERE, "_ref", "ref_matcher")
    probe = os.path.join(HERE, "ref_matcher_probe.cu")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(probe):
        return out
    # the reference's own build line (build.sh) retargeted to sm_103a, without
    # --keep (compiler intermediates are not kept)
    _run(["nvcc", "-rdc=true", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler",
          "-std=c++20 -O3 -fpermissive -w", "-std", "c++20", "-cudart", "static", "-maxrregcount=64", "-w",
          "-I" + src, probe, "-o", out])
    return out


def build():
    build_oracle()
    build_ref_planner()
    stage_reference_sources()


if __name__ == "__main__":
    build()
    print("oracle built", file=sys.stderr)
