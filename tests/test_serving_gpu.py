"""Serving loop: continuous batching across systems, HBM-budget admission,
and results that do not depend on what else is being served.

Each system's noise streams are keyed by (seed, frame index of that system,
subaperture, pixel), and each system's frames run in submission order, so a
system's centroids are bit-identical whether it is served alone or mixed with
other systems' requests arriving at random times."""
import numpy as np
import pytest

from tests.wfs_cases import Case

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

NOISY = dict(sig=2e3, skybrightness=5.0, readnoise=2.0, addPoisson=1, noiseFloor=1.0)


def _kw(c: Case, **over):
    p = dict(c.params)
    p.update(over)
    return dict(nthreads=p["nthreads"], nsubx=c.nsubx, ncen=c.ncen, fftsize=c.N, clipsize=c.C, nimg=c.m,
                phasesize=c.p, readnoise=p["readnoise"], readbg=p["readbg"], addPoisson=p["addPoisson"],
                noiseFloor=p["noiseFloor"], sig=p["sig"], skybrightness=p["skybrightness"], calsource=p["calsource"],
                pxlPower=p["pxlPower"], nintegrations=p["nintegrations"], nlatency=p["nlatency"], seed=p["seed"],
                phs=c.phs, pup=c.pup, spotpsf=c.psf, cents=np.zeros(c.nsubaps * 2, np.float32),
                bimg=np.zeros((c.nsubaps, c.m, c.m), np.float32), minarea=p["minarea"],
                opticalBinning=p["opticalBinning"], centWeight=p["centWeight"],
                correlationCentroiding=p["correlationCentroiding"], corrThresh=p["corrThresh"],
                corrPattern=p["corrPattern"], corrimg=p["corrimg"], threshType=p["threshType"],
                imageOnly=p["imageOnly"], useBrightest=p["useBrightest"], preBinningFactor=p["preBinningFactor"],
                parabolicFit=p["parabolicFit"], gaussianFitVals=p["gaussianFitVals"])


def _phases(c: Case, n, seed0):
    return [torch.from_numpy(np.ascontiguousarray(c.new_phase(seed0 + k), np.float32)).cuda() for k in range(n)]


def test_results_same_alone_and_in_mix():
    from dasp_gb300.serving import WfsServer
    a = Case(nsubx=12, p=10, N=20, C=20, m=10, psf="gauss", seed=21, **NOISY)
    ph = _phases(a, 6, 300)
    # alone
    srv = WfsServer(8 << 30, max_inflight=8)
    sid = srv.add_system(form="fp16", **_kw(a))
    alone = [np.zeros(a.nsubaps * 2, np.float32) for _ in ph]
    for k, p in enumerate(ph):
        srv.submit(sid, p, out=alone[k])
    done = srv.drain(60)
    assert all(c["status"] == 0 and c["readout"] == 1 for c in done)
    srv.close()
    # in a mix of other systems (different sizes, forms, seeds), random release times
    others = [Case(nsubx=8, p=8, N=16, seed=3, **NOISY), Case(nsubx=20, p=10, N=20, seed=4, **NOISY),
              Case(nsubx=16, p=8, N=16, psf="gauss", seed=5, **NOISY)]
    srv = WfsServer(8 << 30, max_inflight=4)
    ids = [srv.add_system(form=f, **_kw(c)) for c, f in zip(others, ["fp32", "bf16x3", "fp16"])]
    sid = srv.add_system(form="fp16", **_kw(a))
    oph = [_phases(c, 3, 700 + 10 * k) for k, c in enumerate(others)]
    mixed = [np.zeros(a.nsubaps * 2, np.float32) for _ in ph]
    rng = np.random.default_rng(0)
    t0 = srv.clock() + 0.02
    for k, p in enumerate(ph):
        srv.submit(sid, p, out=mixed[k], release_s=t0 + 0.002 * k)
        for j, i in enumerate(ids):
            srv.submit(i, oph[j][k % 3], release_s=t0 + rng.uniform(0, 0.012))
    done = srv.drain(60)
    assert all(c["status"] == 0 for c in done)
    srv.close()
    for x, y in zip(alone, mixed):
        np.testing.assert_array_equal(x, y)
    assert not np.array_equal(alone[0], alone[1])


def test_server_matches_standalone_engine():
    from dasp_gb300.serving import WfsServer
    c = Case(nsubx=10, p=8, N=16, C=16, m=8, seed=8, **NOISY)
    ph = _phases(c, 3, 40)
    eng = c.engine()
    dc = torch.zeros((1, c.nsubaps * 2), device="cuda")
    db = torch.zeros((1, c.nsubaps, c.m, c.m), device="cuda")
    ref = []
    for p in ph:
        eng.run_batch(p[None], dc, db)
        torch.cuda.synchronize()
        ref.append(dc[0].cpu().numpy().copy())
    eng.free()
    srv = WfsServer(1 << 30)
    sid = srv.add_system(**_kw(c))
    got = [np.zeros(c.nsubaps * 2, np.float32) for _ in ph]
    for k, p in enumerate(ph):
        srv.submit(sid, p, out=got[k])
    srv.drain(60)
    srv.close()
    for x, y in zip(ref, got):
        np.testing.assert_array_equal(x, y)


def test_admission_by_hbm_budget():
    from dasp_gb300.serving import WfsServer
    cs = [Case(nsubx=20, p=10, N=20, seed=s, **NOISY) for s in range(3)]
    probe = WfsServer(8 << 30)
    probe.add_system(**_kw(cs[0]))
    probe.drain(10)
    import time
    for _ in range(200):
        st = probe.stats()
        if st["admitted"] == 1:
            break
        time.sleep(0.01)
    one = probe.stats()["used_bytes"]
    probe.close()
    assert one > 0
    srv = WfsServer(int(one * 2.5))  # room for two systems
    ids = [srv.add_system(**_kw(c)) for c in cs]
    for _ in range(500):
        st = srv.stats()
        if st["admitted"] == 2:
            break
        time.sleep(0.01)
    assert st["admitted"] == 2 and st["pending"] == 1, st
    ph = _phases(cs[2], 1, 5)[0]
    out = np.zeros(cs[2].nsubaps * 2, np.float32)
    srv.submit(ids[2], ph, out=out)
    time.sleep(0.2)
    assert srv.poll() == []  # the third system is not admitted yet
    srv.remove_system(ids[0])
    done = srv.drain(30)
    assert len(done) == 1 and done[0]["status"] == 0 and done[0]["system"] == ids[2]
    assert np.abs(out).sum() > 0
    assert srv.stats()["admitted"] == 2
    srv.close()


def test_integration_frames():
    from dasp_gb300.serving import WfsServer
    c = Case(nsubx=8, p=8, N=16, nintegrations=2, **NOISY)
    srv = WfsServer(1 << 30)
    sid = srv.add_system(**_kw(c))
    ph = _phases(c, 1, 9)[0]
    for _ in range(4):
        srv.submit(sid, ph)
    done = sorted(srv.drain(30), key=lambda d: d["request"])
    srv.close()
    assert [d["readout"] for d in done] == [0, 1, 0, 1]


def test_poisson_load_latency_and_throughput():
    from dasp_gb300.serving import WfsServer, poisson_schedule, run_schedule
    cs = [Case(nsubx=n, p=8, N=16, seed=n, **NOISY) for n in (8, 16, 24, 32)]
    srv = WfsServer(8 << 30, max_inflight=8)
    ids = [srv.add_system(form="fp16", **_kw(c)) for c in cs]
    phases = [_phases(c, 2, 11 * k) for k, c in enumerate(cs)]
    sched = poisson_schedule([500.0, 1000.0, 1500.0, 2000.0], 0.2, seed=1)
    r = run_schedule(srv, ids, phases, sched)
    srv.close()
    assert r["errors"] == 0 and r["requests"] == len(sched)
    assert r["latency_ms"]["p99"] < 50.0


def test_removed_system_completes_every_queued_request():
    # requests still queued when their system is removed complete with
    # SHWFS_ERR_STATE (5); nothing stays pending
    from dasp_gb300.serving import WfsServer
    a = Case(nsubx=8, p=8, N=16, seed=2, **NOISY)
    ph = _phases(a, 2, 50)
    srv = WfsServer(4 << 30, max_inflight=2)
    sid = srv.add_system(form="fp32", **_kw(a))
    far = srv.clock() + 30.0
    ids = [srv.submit(sid, ph[k % 2], release_s=far) for k in range(5)]
    srv.remove_system(sid)
    done = srv.drain(10)
    assert sorted(c["request"] for c in done) == sorted(ids)
    assert all(c["status"] == 5 for c in done)
    assert srv.stats()["completed"] == srv.stats()["submitted"]
    srv.close()


def test_systems_added_while_the_dispatcher_runs():
    # add_system grows the server's system list while the dispatcher walks it
    from dasp_gb300.serving import WfsServer
    srv = WfsServer(8 << 30, max_inflight=8)
    cases = [Case(nsubx=8, p=8, N=16, seed=30 + k, **NOISY) for k in range(24)]
    ph = _phases(cases[0], 2, 90)
    outs = []
    for k, c in enumerate(cases):
        sid = srv.add_system(form="fp32", **_kw(c))
        for j in range(2):
            o = np.zeros(c.nsubaps * 2, np.float32)
            outs.append(o)
            srv.submit(sid, ph[j], out=o)
    done = srv.drain(60)
    assert len(done) == 48 and all(c["status"] == 0 for c in done)
    srv.close()
