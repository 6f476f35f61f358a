"""Loading the golden fixtures of tests/golden/ (inputs and the reference's
own outputs; see tests/golden/make_golden.py) as ``Case`` objects."""
from __future__ import annotations

import glob
import json
import os

import numpy as np

from tests.wfs_cases import Case

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    """(spec, arrays) of one fixture."""
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        d = {k: z[k] for k in z.files}
    return json.loads(str(d.pop("spec"))), d


def case_of(spec, d):
    """The fixture's configuration with its exact inputs: the stored PSF,
    array parameters and first phase frame replace the generated ones."""
    kw = dict(spec["case"])
    if "psf" in d:
        kw["psf"] = d["psf"]
    for k in spec["arrays"]:
        kw[k] = d["param_" + k]
    c = Case(**kw)
    if "phs" in d:
        c.phs = np.ascontiguousarray(d["phs"][0], dtype=np.float32)
    return c


def compare(c, spec, cents, bimg, ref_cents, ref_bimg, lit_only=False, cent_tol=None, img_rtol=None):
    """Centroids within the fixture's tolerance (px) and images within its
    fraction of the frame's peak pixel; returns the two differences."""
    cent_tol = spec["cent_tol"] if cent_tol is None else cent_tol
    img_rtol = spec["img_rtol"] if img_rtol is None else img_rtol
    ec, rc = np.asarray(cents).reshape(-1, 2), np.asarray(ref_cents).reshape(-1, 2)
    eb, rb = np.asarray(bimg).reshape(c.nsubaps, -1), np.asarray(ref_bimg).reshape(c.nsubaps, -1)
    if lit_only:
        sel = c.lit()
        ec, rc, eb, rb = ec[sel], rc[sel], eb[sel], rb[sel]
    peak = max(float(np.abs(rb).max()), 1e-30)
    di, dc = float(np.abs(eb - rb).max()), float(np.abs(ec - rc).max())
    assert di <= img_rtol * peak, "image mismatch %g (peak %g)" % (di, peak)
    assert dc <= cent_tol, "centroid mismatch %g px" % dc
    return dc, di
