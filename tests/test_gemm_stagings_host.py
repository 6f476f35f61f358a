"""Host-only checks of the tensor-core GEMM kernel's stagings (no GPU).

``shwfs_gemm_stagings`` enumerates the stagings the GEMM-DFT kernel can use
for a geometry, in the order the GEMMSTAGING update code and the autotuner
index them.  Every staging it offers must keep the kernel inside the
hardware's budgets -- a CTA's shared memory, the 512 tensor-memory columns,
the MMA shape limits and the 16-byte alignment of bulk copies -- since a
staging outside them would fault or corrupt on the device.  These tests
restate the budgets independently and check every row over a sweep of
geometries, and pin the documented coverage limits (no tensor-core form at
fftsize 64; no TF32 or BF16x3 at fftsize 32).
"""
import pytest

from dasp_gb300 import centcmod

# a CTA's dynamic shared memory: 227 KB less 4 KB kept for the kernel's static
# shared memory (3,072 bytes: the phase-offset table and the mbarriers)
SMEM_LIMIT = 227 * 1024 - 4096
TMEM_COLS = 512
MAX_NW = 8
FORMS = ("bf16", "bf16x3", "fp16", "tf32")


def _round(x, m):
    return (x + m - 1) // m * m


def _esz(form):
    return 4 if form == "tf32" else 2


def _smem(form, s):
    """Dynamic shared memory of a staging: field tile(s), |F|^2 tile(s), the W2
    ring and the Kc ring, each region starting on a 1024-byte boundary."""
    esz, hl = _esz(form), (2 if form == "bf16x3" else 1)
    a1 = 128 * s["k1"] * esz * hl * (2 if s["dbuf"] else 1)
    a2 = 128 * s["cw"] * esz * hl * (2 if s["dbuf_a2"] else 1)
    w_stage = 2 * s["cw"] * s["kcb"] * hl
    k_stage = s["n2"] * s["cw"] * esz * hl
    off = _round(a1, 1024)
    off = _round(off + a2, 1024)
    off = _round(off + s["nw"] * w_stage, 1024)
    return off + s["nk"] * k_stage, w_stage, k_stage


def _tmem_ranges(s):
    """Column ranges [start, end) of the GEMM1 accumulator buffers and of D2."""
    w1 = 2 * s["cw"]
    if s["nd1"] == 3:
        d1 = [(0, 128), (128, 256), (384, 512)]
        d2 = (256, 256 + s["n2"])
    else:
        d1 = [(b * w1, (b + 1) * w1) for b in range(s["nd1"])]
        d2 = (s["nd1"] * w1, s["nd1"] * w1 + s["n2"])
    return d1, d2


def _check_staging(form, p, crop, nimg, s):
    esz = _esz(form)
    cc = crop * crop
    k1 = _round(2 * _round(p * p, 8), 16)
    assert s["k1"] == k1
    assert s["n2"] == _round(nimg * nimg, 16) and s["n2"] <= 256
    # GEMM1: M = 128, N = 2 CW (a multiple of 16 up to 256); the chunks cover the crop
    assert s["cw"] % 16 == 0 and 64 <= s["cw"] and 2 * s["cw"] <= 256
    assert s["noc"] * s["cw"] >= cc > (s["noc"] - 1) * s["cw"]
    # streamed W2 chunks: whole 32-byte k-steps covering GEMM1's K
    assert s["kcb"] in (64, 128) and s["kcb"] % 32 == 0
    assert s["nkc"] * s["kcb"] >= k1 * esz > (s["nkc"] - 1) * s["kcb"]
    if form == "bf16x3":
        assert s["kcb"] == 64
    # field double buffering only for the one-pass 16-bit formats
    if s["dbuf"]:
        assert form in ("bf16", "fp16")
    # rings deep enough for the producer to run ahead, within the barrier arrays
    assert 1 <= s["nk"] <= 2 and 2 <= s["nw"] <= MAX_NW
    if s["nk"] == 2:
        assert s["nw"] >= 3
    # shared memory: the restated layout, within a CTA's limit; bulk-copy
    # stages are whole 16-byte units
    total, w_stage, k_stage = _smem(form, s)
    assert s["smem"] == total <= SMEM_LIMIT
    assert w_stage % 16 == 0 and k_stage % 16 == 0
    # the W2 ring could not hold one more stage (the ring is as deep as
    # shared memory allows, up to the barrier arrays)
    if s["nw"] < MAX_NW:
        assert total + w_stage > SMEM_LIMIT
    # tensor memory: three 128-column GEMM1 buffers only with 64-wide chunks
    # and a narrow GEMM2; every accumulator inside the 512 columns, none overlapping
    assert (s["nd1"] == 3) == (s["cw"] == 64 and s["n2"] <= 128)
    d1, d2 = _tmem_ranges(s)
    ranges = sorted(d1 + [d2])
    for (a0, a1), (b0, _) in zip(ranges, ranges[1:]):
        assert a1 <= b0
    assert max(e for _, e in ranges) == s["tmem"] <= TMEM_COLS
    for a0, a1 in d1:
        assert a1 - a0 == 2 * s["cw"]


GEOMS = [(p, crop, nimg) for p in (4, 6, 8, 10, 12, 14, 16)
         for crop in (8, 12, 16, 20, 24, 28, 32) if crop >= p
         for nimg in (2, 4, 6, 8, 10, 12, 14, 16)]


@pytest.mark.parametrize("form", FORMS)
def test_every_staging_fits_the_kernel_budgets(form):
    offered = 0
    for p, crop, nimg in GEOMS:
        rows = centcmod.gemm_stagings(form, p, crop, nimg)
        keys = set()
        for s in rows:
            _check_staging(form, p, crop, nimg, s)
            key = (s["cw"], s["kcb"], s["dbuf"], s["dbuf_a2"], s["nk"], s["nw"])
            assert key not in keys, "staging offered twice"
            keys.add(key)
        if rows:
            offered += 1
            # the default has the fewest GEMM1 output chunks of any staging
            assert rows[0]["noc"] == min(s["noc"] for s in rows)
            # 64-wide chunks are always among the candidates
            assert any(s["cw"] == 64 for s in rows)
    assert offered > 0


def test_default_staging_of_the_74x74_workload():
    # phasesize 10, fftsize 20 (crop 20 x 20 = 400 outputs), 10 x 10 images:
    # five 80-wide GEMM1 output chunks instead of seven 64-wide ones
    rows = centcmod.gemm_stagings("fp16", 10, 20, 10)
    assert len(rows) > 1
    assert rows[0]["cw"] == 80 and rows[0]["noc"] == 5
    assert rows[0]["k1"] == 208 and rows[0]["n2"] == 112
    assert any(s["cw"] == 64 and s["noc"] == 7 for s in rows)


@pytest.mark.parametrize("form", FORMS)
def test_fftsize_64_has_no_tensor_core_form(form):
    # p = 32: GEMM1's K (2 p^2 = 2048) needs a 512 KB field tile
    assert centcmod.gemm_stagings(form, 32, 64, 16) == []
    assert centcmod.gemm_stagings(form, 17, 34, 8) == []


def test_fftsize_32_formats():
    # p = 16: the 16-bit one-pass formats fit, TF32 (4-byte field) and BF16x3
    # (hi and lo fields) do not
    for form in ("fp16", "bf16"):
        assert centcmod.gemm_stagings(form, 16, 32, 8), form
    for form in ("tf32", "bf16x3"):
        assert centcmod.gemm_stagings(form, 16, 32, 8) == [], form


def test_images_wider_than_16_pixels_have_no_tensor_core_form():
    # GEMM2's N (nimg^2 rounded up to 16) is at most 256
    assert centcmod.gemm_stagings("fp16", 8, 16, 16)
    assert centcmod.gemm_stagings("fp16", 8, 16, 17) == []


def test_bad_staging_queries_are_rejected():
    for args in (("fp32", 8, 16, 8), (5, 8, 16, 8), ("fp16", 0, 16, 8), ("fp16", 8, 0, 8), ("fp16", 8, 16, 0)):
        with pytest.raises(ValueError, match="bad staging query"):
            centcmod.gemm_stagings(*args)
