"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles the CPU restatement (oracle/*.c) into
  ``oracle/_build/liborc.so`` with gcc.  It runs on any host (x86 or Arm).
* ``build_ref()``, when the reference tree is present, compiles the
  reference's own sources where they lie (read only) into oracle/_ref:
  - ``libgaunt_ref.so``: qpms/gaunt.c (Xu's Gaunt recurrences), libm only;
  - ``libqpms_ref.so``: qpms/translations.c, ewald.c, ewaldsf.c, gaunt.c,
    latticegens.c, lattices2d.c, lll.c, error.c with LATTICESUMS32 (as the
    reference's build defines it), against oracle/refshim: stand-in headers
    for the GSL / CBLAS / Faddeeva declarations those files include and
    refshim.c, which implements the few functions they call over the oracle's
    restatements (Legendre arrays, 3j, spherical Bessel functions for the
    AMOS-backed bessel.c, incomplete gamma, QUADPACK-style qagiu), plus
    refpin.c, plain-argument entry points for ctypes.  GSL, LAPACKE/CBLAS,
    AMOS (camos) and the Faddeeva package are absent here; everything else in
    those files is the reference's code, unchanged.
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




REF_SOURCES = ["translations.c", "ewald.c", "ewaldsf.c", "gaunt.c", "latticegens.c", "lattices2d.c", "lll.c",
               "error.c"]


def build_ref_lib(force=False):
    """The reference's translation / lattice-sum sources over the GSL stand-in
    (oracle/refshim) into oracle/_ref/libqpms_ref.so; None without the tree."""
    qdir = os.path.join(REF_ROOT, "qpms")
    srcs = [os.path.join(qdir, f) for f in REF_SOURCES]
    if not all(os.path.exists(x) for x in srcs):
        return None
    shim = os.path.join(HERE, "refshim")
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libqpms_ref.so")
    ours = [os.path.join(shim, "refshim.c"), os.path.join(shim, "refpin.c"), os.path.join(HERE, "orc_specfunc.c"),
            os.path.join(HERE, "orc_ewald.c"), os.path.join(HERE, "orc_trans.c")]
    deps = srcs + ours + [os.path.join(HERE, "orc.h")]
    if force or _newer(out, deps):
        objs = []
        for src in srcs + ours[:2]:
            obj = os.path.join(out_dir, os.path.basename(src) + ".o")
            inc = ["-I", shim, "-I", qdir] if src not in ours[:1] else ["-I", HERE]
            subprocess.check_call(["gcc", "-std=gnu11", "-O2", "-fPIC", "-DLATTICESUMS32", "-w", "-c"] + inc +
                                  [src, "-o", obj])
            objs.append(obj)
        subprocess.check_call(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-fopenmp", "-I", HERE, "-o", out] +
                              objs + ours[2:] + ["-lm"])
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    print(build_ref_lib(force="--force" in sys.argv))
