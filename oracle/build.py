"""Build recipe for the oracle (test infrastructure only).

* ``liboracle.so``  — the C restatement (fm.c, tho.c) and the reference's
  per-molecule loops for CPU-baseline timing (refpath.c), built everywhere.
* ``_ref/libref.so`` — hfsolver's own src/cints.c and src/qc.c compiled
  unmodified from the reference checkout, linked with fm.c for the c_Fm
  callback that src/qc.f90:90-95 provides in the reference.  Built only where the
  reference sources exist; written only into oracle/_ref/ (git-ignored).

Both use -ffp-contract=off so that x86 and Arm builds round identically.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: HFSOLVER_REFERENCE_SRC, else a checkout named
# "reference" beside this repository
REF_SRC = os.environ.get("HFSOLVER_REFERENCE_SRC") or os.path.normpath(
    os.path.join(HERE, "..", "..", "reference", "src"))
CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr)


def build_oracle():
    out = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, "fm.c"), os.path.join(HERE, "tho.c"), os.path.join(HERE, "refpath.c")]
    _run(["gcc", *CFLAGS, "-fopenmp", *srcs, "-o", out, "-lm"])
    return out


def build_ref():
    """Returns the path of oracle/_ref/libref.so, or None without the sources."""
    cints = os.path.join(REF_SRC, "cints.c")
    qc = os.path.join(REF_SRC, "qc.c")
    if not (os.path.exists(cints) and os.path.exists(qc)):
        return None
    os.makedirs(os.path.join(HERE, "_ref"), exist_ok=True)
    out = os.path.join(HERE, "_ref", "libref.so")
    _run(["gcc", *CFLAGS, "-I", REF_SRC, cints, qc, os.path.join(HERE, "fm.c"), "-o", out, "-lm"])
    return out


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref())
    sys.exit(0)
