"""Build the reference's own WFS module (``cent``) into ``oracle/_ref/`` --
TEST INFRASTRUCTURE ONLY.

Recipe
------
1. Stage: copy ``cmod/src/centmodule.c`` and ``cmod/src/qsort.h`` byte for
   byte from the reference tree (``/root/reference`` unless ``DASP_REFERENCE``
   names another) into ``oracle/_ref/src/`` with their SHA-256 digests.  The
   staged copy is a build output (``oracle/_ref/`` is git-ignored) and lets a
   machine without the reference tree rebuild the module from it; the digests
   are checked before every compile.  Nothing is edited.
2. Compile the unmodified ``centmodule.c`` with gcc against Python 3 and
   numpy, force-including ``refbuild/py2compat.h`` (PyInt_* and Py_InitModule
   mapped onto Python 3), with ``refbuild/shim`` on the include path in place
   of the FFTW3 and GSL headers, plus ``refbuild/fft_shim.c``,
   ``refbuild/gsl_shim.c`` (the FFTW/GSL subsets, written from the published
   algorithms) and ``refbuild/pyinit.c`` (the PyInit_cent entry).
   Flags follow a distutils build of the module (cmod/src/setup.py:55-63:
   ``-pthread``, Python's default ``-O2 -fwrapv -fno-strict-aliasing``), with
   ``-ffp-contract=off`` so the floating-point results do not depend on
   whether the host ISA has fused multiply-add.
3. Output: ``oracle/_ref/cent.so`` (imported by ``oracle/ref_cent.py``).

What is the reference's code and what is not: every line of
``centroidsFromPhase``/``centroidsFromImage``, the crop, PSF convolution
arithmetic, binning, normalisation, PCG32 + rk_poisson, readCCD, threshold,
centroiding, fits, calibration, the thread partition and the Python entry
points is the reference's, unmodified.  The FFTs (FFTW is a system library
the reference does not ship) and GSL's MT19937 / gaussian / 6x6 LU are the
shims'.  Read noise therefore matches GSL only as far as the shim restates
GSL's documented algorithm.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
REFBUILD = os.path.join(HERE, "refbuild")
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
SO = os.path.join(OUT, "cent.so")
FILES = ("centmodule.c", "qsort.h")
SHIMS = ("fft_shim.c", "gsl_shim.c", "pyinit.c")
CFLAGS = ["-O2", "-fwrapv", "-fno-strict-aliasing", "-ffp-contract=off", "-DNDEBUG", "-fPIC", "-pthread",
          "-w"]


def reference_dir() -> str:
    return os.path.join(os.environ.get("DASP_REFERENCE", "/root/reference"), "cmod", "src")


def _sha(path: str) -> str:
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def stage() -> bool:
    """Copy the two reference files into oracle/_ref/src (when the reference
    tree is present).  Returns True when a staged copy exists afterwards."""
    ref = reference_dir()
    if all(os.path.isfile(os.path.join(ref, f)) for f in FILES):
        os.makedirs(SRC, exist_ok=True)
        lines = []
        for f in FILES:
            dst = os.path.join(SRC, f)
            src = os.path.join(ref, f)
            if not os.path.isfile(dst) or _sha(dst) != _sha(src):
                shutil.copyfile(src, dst)
            lines.append("%s  %s\n" % (_sha(src), f))
        with open(os.path.join(SRC, "SHA256SUMS"), "w") as fh:
            fh.writelines(lines)
    return all(os.path.isfile(os.path.join(SRC, f)) for f in FILES + ("SHA256SUMS",))


def _check_digests() -> None:
    with open(os.path.join(SRC, "SHA256SUMS")) as fh:
        for line in fh:
            digest, name = line.split()
            if _sha(os.path.join(SRC, name)) != digest:
                raise RuntimeError("staged reference file %s does not match its recorded digest" % name)


def _inputs_digest() -> str:
    h = hashlib.sha256()
    for p in [os.path.join(SRC, f) for f in FILES] + [os.path.join(REFBUILD, f) for f in SHIMS] + [
            os.path.join(REFBUILD, "py2compat.h")]:
        h.update(open(p, "rb").read())
    for root, _, files in sorted(os.walk(os.path.join(REFBUILD, "shim"))):
        for f in sorted(files):
            h.update(open(os.path.join(root, f), "rb").read())
    h.update(" ".join(CFLAGS).encode())
    h.update(sys.version.encode())
    import numpy
    h.update(numpy.__version__.encode())
    return h.hexdigest()


def available() -> bool:
    return os.path.isfile(SO) or stage()


def build(force: bool = False, verbose: bool = False) -> str:
    """Stage (if the reference tree is here) and compile oracle/_ref/cent.so."""
    if not stage():
        raise FileNotFoundError("reference sources not found (neither %s nor a staged copy in %s)"
                                % (reference_dir(), SRC))
    _check_digests()
    stamp = os.path.join(OUT, "cent.sha256")
    digest = _inputs_digest()
    if not force and os.path.isfile(SO) and os.path.isfile(stamp) and open(stamp).read().strip() == digest:
        return SO
    import numpy
    # numpy 2 headers expose PyArray_Descr.elsize (read at centmodule.c:2144)
    # only when compiling for the 2.x API; numpy 1.x headers always do.
    npdef = ["-DNPY_TARGET_VERSION=NPY_2_0_API_VERSION"] if int(numpy.__version__.split(".")[0]) >= 2 else []
    inc = [sysconfig.get_paths()["include"], numpy.get_include(), os.path.join(REFBUILD, "shim"), REFBUILD]
    tmp = SO + ".%d.tmp" % os.getpid()
    cmd = (["gcc"] + CFLAGS + npdef + ["-include", os.path.join(REFBUILD, "py2compat.h")] + ["-I" + d for d in inc]
           + ["-shared", "-o", tmp, os.path.join(SRC, "centmodule.c")]
           + [os.path.join(REFBUILD, f) for f in SHIMS] + ["-lm", "-lpthread"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n%s\n%s" % (r.stdout, r.stderr[-4000:]))
    os.replace(tmp, SO)
    with open(stamp, "w") as fh:
        fh.write(digest)
    if verbose:
        print("built", SO)
    return SO


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
