"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles the CPU restatement (oracle/*.c) into
  ``oracle/_build/liborc.so`` with gcc.  It runs on any host (x86 or Arm).
* ``build_ref()`` compiles the one part of the reference that builds from its
  own sources with libm alone -- ``qpms/gaunt.c`` (Xu's Gaunt recurrences) --
  into ``oracle/_ref/libgaunt_ref.so``, when the reference tree is present.
  The rest of the reference's hot path needs GSL, LAPACKE/CBLAS and the AMOS
  Fortran/camos Bessel library, none of which exist here, so it is not built.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# root of the reference checkout (read only); QPMS_REFERENCE_ROOT overrides it
REF_ROOT = os.environ.get("QPMS_REFERENCE_ROOT", "/root/reference")
SOURCES = ["orc_specfunc.c", "orc_trans.c", "orc_ewald.c", "orc_scatsys.c", "orc_interp.c", "orc_axsym.c"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle(force=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "liborc.so")
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "orc.h")]
    if force or _newer(out, deps):
        cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-o", out] + srcs + ["-lm"]
        subprocess.check_call(cmd)
    return out


def build_ref(force=False):
    """Compile reference gaunt.c where the reference tree exists; else None."""
    src = os.path.join(REF_ROOT, "qpms", "gaunt.c")
    if not os.path.exists(src):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libgaunt_ref.so")
    if force or _newer(out, [src]):
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-I", os.path.join(REF_ROOT, "qpms"),
               "-o", out, src, "-lm"]
        subprocess.check_call(cmd)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
