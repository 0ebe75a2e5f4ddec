"""Build recipe for the oracle (test infrastructure).

* ``oracle/_ref/liboracle.so`` is not produced here; the oracle library is
  ``oracle/liboracle.so`` compiled with gcc from ``fm_oracle.c``.
* ``oracle/_ref/ref_planner`` is the reference's own host query planner,
  compiled from the ForkMatch sources where they lie (``<ref>/src``) together
  with ``ref_planner_probe.cu``.  It is built only when the reference tree is
  present; nothing at run time depends on it.

Outputs are git-ignored.  Run ``python oracle/build.py`` or call ``build()``.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = os.environ.get("FM_REFERENCE_SRC", "/root/reference/src")


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


def build():
    build_oracle()
    build_ref_planner()


if __name__ == "__main__":
    build()
    print("oracle built", file=sys.stderr)
