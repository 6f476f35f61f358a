"""The CUDA engine against the golden fixtures: outputs of the reference's own
module (cmod/src/centmodule.c, unmodified) stored with their exact inputs in
tests/golden/, through the C ABI (dasp_gb300.centcmod -> libshwfs.so).  Needs
no reference sources on the machine.

Tolerances: the FP32 form within the fixture's own (centroids 1e-5 px, 1e-4
px for the fits and threshold type 1; images 1e-4 of the frame's peak, 3e-4
with pixel power 2); the FP16 tensor-core form within its stated accuracy,
1e-3 px on the lit subapertures, images within 5e-3 of the peak.  The noisy
fixture (the reference's own noise draws) is the oracle's test only.
"""
import numpy as np
import pytest

from tests import golden_cases as gc

pytestmark = pytest.mark.gpu

NAMES = [n for n in gc.names() if gc.load(n)[0]["gpu"]]
TC_NAMES = [n for n in gc.names() if gc.load(n)[0]["tc"]]


def _engine_frames(spec, d, form=None):
    c = gc.case_of(spec, d)
    cents = np.full(c.nsubaps * 2, spec["init_cents"], np.float32)
    if spec["input"] == "phase":
        phs = np.ascontiguousarray(d["phs"][0], dtype=np.float32)
        eng = c.engine(phs=phs, cents=cents)
    else:
        eng = c.engine(cents=cents, inputImage=np.ascontiguousarray(d["image"]))
    try:
        if form:
            eng.set_form(form)
            assert eng.info()["form_active"] != 0, "tensor-core form did not engage"
        for f in range(spec["frames"]):
            if spec["input"] == "phase":
                phs[...] = d["phs"][f]
                eng.run(c.params["calsource"])
            else:
                eng.runSlope(0)
            yield c, f
    finally:
        eng.free()


@pytest.mark.parametrize("name", NAMES)
def test_fp32_form_matches_reference_fixture(name):
    spec, d = gc.load(name)
    for c, f in _engine_frames(spec, d):
        gc.compare(c, spec, c.cents, c.bimg, d["cents"][f], d["bimg"][f])


@pytest.mark.parametrize("name", TC_NAMES)
def test_fp16_form_matches_reference_fixture(name):
    spec, d = gc.load(name)
    for c, f in _engine_frames(spec, d, form="fp16"):
        gc.compare(c, spec, c.cents, c.bimg, d["cents"][f], d["bimg"][f], lit_only=True, cent_tol=1e-3,
                   img_rtol=5e-3)
