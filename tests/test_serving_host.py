"""Host-side logic of the serving loop, without a GPU: argument checks,
budget rejection, and requests of systems whose engine cannot be created
(no device here) completing with an error instead of hanging."""
import numpy as np
import pytest

from tests.wfs_cases import Case


def _server(budget=1 << 30):
    from dasp_gb300.serving import WfsServer
    return WfsServer(budget, max_inflight=4)


def _kw(c):
    from tests.test_serving_gpu import _kw as kw
    return kw(c)


def test_rejects_bad_config():
    from dasp_gb300.serving import WfsServer
    with pytest.raises(ValueError):
        WfsServer(0)
    with pytest.raises(ValueError):
        WfsServer(1 << 20, max_inflight=0)


def test_system_larger_than_budget_is_refused():
    from dasp_gb300._lib import ShwfsError
    srv = _server(budget=1 << 16)
    with pytest.raises(ShwfsError):
        srv.add_system(**_kw(Case(nsubx=16, p=8, N=16)))
    srv.close()


def test_requests_complete_with_error_when_engine_cannot_start():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("needs a machine without a GPU")
    from dasp_gb300._lib import ShwfsError
    c = Case(nsubx=8, p=8, N=16)
    srv = _server()
    sid = srv.add_system(**_kw(c))
    out = np.zeros(c.nsubaps * 2, np.float32)
    accepted = 0
    for _ in range(2):
        try:
            srv.submit(sid, c.phs, out=out)
            accepted += 1
        except ShwfsError as e:  # the engine already failed to start
            assert "could not be started" in str(e)
    done = srv.drain(20)
    assert len(done) == accepted and all(d["status"] != 0 for d in done)
    with pytest.raises(ShwfsError):
        srv.submit(sid, c.phs)
    st = srv.stats()
    assert st["admitted"] == 0 and st["submitted"] == accepted and st["completed"] == accepted
    srv.close()


def test_poisson_schedule_rates():
    from dasp_gb300.serving import poisson_schedule
    ev = poisson_schedule([1000.0, 250.0], 4.0, seed=3)
    n0 = sum(1 for _, k in ev if k == 0)
    n1 = sum(1 for _, k in ev if k == 1)
    assert abs(n0 - 4000) < 5 * np.sqrt(4000) and abs(n1 - 1000) < 5 * np.sqrt(1000)
    assert all(ev[i][0] <= ev[i + 1][0] for i in range(len(ev) - 1))
