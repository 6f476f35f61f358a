"""Many WFSs per launch (CUDA-graph batches) and the tile autotuner.

A batched readout frame must give bit-identical images and centroids to the
same handle configuration run on its own (``run_batch`` with one frame): the
graph replays the same kernels, and each handle's noise frame index advances
on the device exactly as its host counter does."""
import numpy as np
import pytest

from tests.wfs_cases import Case

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

NOISY = dict(sig=2e3, skybrightness=5.0, readnoise=2.0, addPoisson=1, noiseFloor=1.0)
GEOMS = [dict(nsubx=8, p=8, N=16, C=16, m=8), dict(nsubx=12, p=10, N=20, C=20, m=10, psf="gauss"),
         dict(nsubx=6, p=8, N=24, C=24, m=12)]


class DevEngine:
    """An engine whose phase and outputs live in CUDA tensors."""

    def __init__(self, case, form="fp32"):
        self.c = case
        self.eng = case.engine()
        self.phs = torch.from_numpy(case.phs.copy()).cuda()
        self.cents = torch.zeros(case.nsubaps * 2, device="cuda")
        self.bimg = torch.zeros(case.nsubaps, case.m, case.m, device="cuda")
        self.eng.set_io(self.phs, self.cents, self.bimg)
        if form != "fp32":
            self.eng.set_form(form)
        torch.cuda.synchronize()  # the engine's streams do not wait on torch's

    def run_alone(self):
        self.eng.run_batch(self.phs[None], self.cents[None], self.bimg[None])

    def outputs(self):
        torch.cuda.synchronize()
        return self.cents.cpu().numpy().copy(), self.bimg.cpu().numpy().copy()


def _pairs(forms=None):
    forms = forms or ["fp32"] * len(GEOMS)
    a = [DevEngine(Case(**g, **NOISY), f) for g, f in zip(GEOMS, forms)]
    b = [DevEngine(Case(**g, **NOISY), f) for g, f in zip(GEOMS, forms)]
    return a, b


def _same(x, y):
    for (c0, b0), (c1, b1) in zip(x, y):
        np.testing.assert_array_equal(c0, c1)
        np.testing.assert_array_equal(b0, b1)


def _new_phase(pairs, seed):
    for k, (x, y) in enumerate(pairs):
        ph = torch.from_numpy(np.ascontiguousarray(x.c.new_phase(seed + k), np.float32)).cuda()
        x.phs.copy_(ph)
        y.phs.copy_(ph)
    torch.cuda.synchronize()


def test_batch_equals_individual_runs():
    from dasp_gb300.batch import WfsBatch
    a, b = _pairs()
    batch = WfsBatch([x.eng for x in a])
    for f in range(3):
        _new_phase(list(zip(a, b)), 50 + 10 * f)
        batch.run()
        for y in b:
            y.run_alone()
        _same([x.outputs() for x in a], [y.outputs() for y in b])
        assert all(x.eng.info()["frames_read"] == f + 1 for x in a)
    # noise really changes between frames
    c0, _ = a[0].outputs()
    batch.run()
    c1, _ = a[0].outputs()
    assert not np.array_equal(c0, c1)
    batch.free()


def test_batch_recaptures_after_update_and_solo_runs():
    from dasp_gb300.batch import WfsBatch
    from dasp_gb300.centcmod import SIG
    a, b = _pairs()
    batch = WfsBatch([x.eng for x in a])
    batch.run()
    for y in b:
        y.run_alone()
    # an update changes a captured argument: the batch re-captures
    a[1].eng.update(SIG, 3.5e3)
    b[1].eng.update(SIG, 3.5e3)
    # a handle run on its own advances its frame index outside the graph
    a[2].run_alone()
    b[2].run_alone()
    torch.cuda.synchronize()
    for _ in range(2):
        batch.run(torch.cuda.current_stream())
        for y in b:
            y.run_alone()
    _same([x.outputs() for x in a], [y.outputs() for y in b])
    batch.free()


def test_batch_with_tensor_core_form():
    from dasp_gb300.batch import WfsBatch
    a, b = _pairs(["bf16x3", "fp32", "bf16x3"])
    assert a[0].eng.info()["form_active"] == 2
    batch = WfsBatch([x.eng for x in a])
    for f in range(2):
        _new_phase(list(zip(a, b)), 80 + 10 * f)
        batch.run()
        for y in b:
            y.run_alone()
    _same([x.outputs() for x in a], [y.outputs() for y in b])
    batch.free()


def test_batch_rejects_host_io_and_duplicates():
    from dasp_gb300.batch import WfsBatch
    c = Case(nsubx=8, **NOISY)
    host = c.engine()
    with pytest.raises(ValueError):
        WfsBatch([host])
    d = DevEngine(Case(nsubx=8, **NOISY))
    with pytest.raises(ValueError):
        WfsBatch([d.eng, d.eng])
    host.free()


def test_autotune_keeps_results():
    base = DevEngine(Case(nsubx=16, p=10, N=20, C=20, m=10, psf="gauss", **NOISY))
    tuned = DevEngine(Case(nsubx=16, p=10, N=20, C=20, m=10, psf="gauss", **NOISY))
    ts = tuned.eng.autotune()
    assert ts == tuned.eng.info()["tile_subaps"] and 1 <= ts <= 64
    assert tuned.eng.info()["frames_read"] == 0
    for _ in range(2):
        base.run_alone()
        tuned.run_alone()
    _same([base.outputs()], [tuned.outputs()])


@pytest.mark.parametrize("form", ["fp16", "bf16x3", "tf32"])
def test_autotune_gemm_staging_keeps_results(form):
    """The tensor-core forms' autotuner times every staging of the GEMM
    kernel and keeps one; the MMAs see the same k-steps in the same order
    (GEMM2's K padding beyond the crop only adds zeros), so the outputs stay
    bit-identical to the default staging."""
    kw = dict(nsubx=16, p=10, N=20, C=20, m=10, psf="gauss", **NOISY)
    base = DevEngine(Case(**kw), form)
    tuned = DevEngine(Case(**kw), form)
    d = base.eng.info()
    assert d["form_active"] != 0 and d["gemm_kcb"] in (64, 128)
    tuned.eng.autotune()
    t = tuned.eng.info()
    assert t["gemm_kcb"] in (64, 128) and t["gemm_nw"] >= 2 and t["gemm_nk"] in (1, 2) and 0 <= t["gemm_dbuf"] <= 3
    assert d["gemm_cw"] == 80 and t["gemm_cw"] in (64, 80)  # 20 x 20 crop: 5 chunks of 80 (default) or 7 of 64
    assert t["frames_read"] == 0
    for k in range(2):
        if k:
            _new_phase([(base, tuned)], 40)
        base.run_alone()
        tuned.run_alone()
        _same([base.outputs()], [tuned.outputs()])


@pytest.mark.parametrize("form", ["fp16", "bf16x3", "tf32"])
def test_every_gemm_staging_gives_the_same_results(form):
    """Every staging the tensor-core forms can run (SHWFS_GEMMSTAGING; output
    chunks of 64 or 80 complex outputs for the 20 x 20 crop, W2 chunk width,
    operand double buffering, ring depths) gives bit-identical images and
    centroids."""
    from dasp_gb300.centcmod import GEMMSTAGING
    kw = dict(nsubx=16, p=10, N=20, C=20, m=10, psf="gauss", **NOISY)
    base = DevEngine(Case(**kw), form)
    n = base.eng.info()["gemm_candidates"]
    assert n >= 2
    base.run_alone()
    ref = base.outputs()
    cws = set()
    for i in range(1, n):
        e = DevEngine(Case(**kw), form)
        e.eng.update(GEMMSTAGING, i)
        inf = e.eng.info()
        assert inf["gemm_staging"] == i
        cws.add(inf["gemm_cw"])
        e.run_alone()
        _same([ref], [e.outputs()])
        e.eng.free()
    assert 64 in cws
    with pytest.raises(Exception):
        base.eng.update(GEMMSTAGING, n)


def test_multi_handle_kernel_equals_individual_runs():
    """FP32-form handles of one kernel instantiation (fftsize 16, no PSF;
    8x8 to 20x20 subapertures, different signal, noise and seeds) run as one
    persistent multi-handle kernel in the batch graph, beside a handle of
    another instantiation and a tensor-core one; every handle's images and
    centroids equal its run on its own, frame after frame."""
    from dasp_gb300.batch import WfsBatch
    same = [dict(nsubx=n, p=8, N=16, C=16, m=8, sig=s, skybrightness=sk, readnoise=rn, addPoisson=1, noiseFloor=1.0,
                 seed=sd)
            for n, s, sk, rn, sd in ((8, 2e3, 5.0, 2.0, 3), (12, 4e3, 1.0, 1.0, 4), (20, 1e3, 8.0, 3.0, 5),
                                     (16, 3e3, 0.0, 0.5, 6))]
    other = [dict(nsubx=12, p=10, N=20, C=20, m=10, psf="gauss", **NOISY)]
    geoms = same + other + [dict(nsubx=12, p=10, N=20, C=20, m=10, psf="gauss", **NOISY)]
    forms = ["fp32"] * (len(same) + 1) + ["fp16"]
    a = [DevEngine(Case(**g), f) for g, f in zip(geoms, forms)]
    b = [DevEngine(Case(**g), f) for g, f in zip(geoms, forms)]
    batch = WfsBatch([x.eng for x in a])
    assert batch.multi_launches() == 0  # off by default
    batch.set_multi(True)
    assert batch.multi_launches() == 1
    for f in range(3):
        _new_phase(list(zip(a, b)), 120 + 10 * f)
        batch.run()
        for y in b:
            y.run_alone()
        _same([x.outputs() for x in a], [y.outputs() for y in b])
    batch.free()
    # more handles of one instantiation than one launch takes: several launches
    many = [DevEngine(Case(**dict(same[k % 4], seed=30 + k))) for k in range(10)]
    solo = [DevEngine(Case(**dict(same[k % 4], seed=30 + k))) for k in range(10)]
    batch = WfsBatch([x.eng for x in many], multi=True)
    assert batch.multi_launches() == 2
    batch.run()
    for y in solo:
        y.run_alone()
    _same([x.outputs() for x in many], [y.outputs() for y in solo])
    batch.free()
