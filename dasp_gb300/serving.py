"""Serving loop for many simulated AO systems on one GPU.

Python face of the native server (``shwfs_server_*`` in include/shwfs.h,
dasp_gb300/csrc/shwfs_server.cu): a dispatcher thread inside the library
keeps each admitted system's WFS state resident on the device, admits
systems against a fixed HBM budget, and launches each released WFS-frame
request as soon as its system is idle and a device slot is free -- frames of
different systems overlap on the device (continuous batching).  Latency is
measured by the server from each request's release time to the moment its
centroids are on the host.

The reference has no counterpart: each WFS of a DASP simulation is a
``wfscent`` object stepped by the simulation's own scheduler
(science/wfscent.py:585-683) around one ``centcmod`` handle.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib
from ._lib import ShwfsCompletion, ShwfsServerConfig, ShwfsServerStats, check
from .centcmod import FORMS, _is_array, centcmod


class _SystemSpec(centcmod):
    """centcmod's argument handling without creating a handle: the server
    creates the engine when the system is admitted."""

    def _create(self, ini):
        self.centstruct = None


class WfsServer:
    def __init__(self, hbm_budget_bytes: int, max_inflight: int = 32, device: int = 0, integration: str = "compat"):
        """integration: "compat" (the reference's: only the readout frame's
        phase reaches the image) or "physical" (each system's sub-exposures
        averaged on the device; see centcmod.set_integration_mode)."""
        cfg = ShwfsServerConfig(int(hbm_budget_bytes), int(max_inflight), int(device),
                                {"compat": 0, "physical": 1}[integration])
        s = ctypes.c_void_p()
        check(_lib.lib().shwfs_server_create(ctypes.byref(cfg), ctypes.byref(s)), "server_create")
        self._s = s
        self._specs = {}
        self._pending = {}  # request id -> objects kept alive until completion
        self.lit = {}

    # -- systems --
    def add_system(self, form: str = "fp32", **kw) -> int:
        """Register a WFS; ``kw`` are ``centcmod``'s constructor arguments
        (``phs``, ``cents`` and ``bimg`` only give shapes)."""
        spec = _SystemSpec(**kw)
        sid = ctypes.c_int(-1)
        check(_lib.lib().shwfs_server_add_system(self._s, ctypes.byref(spec._ini), FORMS[form], ctypes.byref(sid)),
              "server_add_system")
        self._specs[sid.value] = spec
        self.lit[sid.value] = int(np.count_nonzero(spec.subflag))
        return sid.value

    def remove_system(self, sid: int) -> None:
        check(_lib.lib().shwfs_server_remove_system(self._s, int(sid)), "server_remove_system")

    # -- requests --
    def submit(self, sid: int, phase, out=None, release_s: float | None = None) -> int:
        """One WFS frame of system ``sid``.  ``phase``: CUDA tensor (used in
        place) or float32 numpy array; ``out``: optional float32 numpy array of
        nsubaps*2 centroids, written before the completion is reported."""
        dev = _is_array(phase) and getattr(phase, "is_cuda", False)
        if dev:
            ptr = phase.data_ptr()
        else:
            phase = np.ascontiguousarray(phase, dtype=np.float32)
            ptr = phase.ctypes.data
        optr = None
        if out is not None:
            if not (isinstance(out, np.ndarray) and out.dtype == np.float32 and out.flags.c_contiguous
                    and out.size >= 2 * self._specs[sid].nsubaps):
                raise ValueError("out must be a contiguous float32 numpy array of nsubaps*2 values")
            optr = out.ctypes.data
        rid = ctypes.c_uint64(0)
        check(_lib.lib().shwfs_server_submit(self._s, int(sid), ptr, int(dev), optr,
                                             float(release_s) if release_s is not None else 0.0,
                                             ctypes.byref(rid)), "server_submit")
        self._pending[rid.value] = (phase, out)
        return rid.value

    def poll(self, max_n: int = 4096) -> list:
        buf = (ShwfsCompletion * max_n)()
        n = ctypes.c_int(0)
        check(_lib.lib().shwfs_server_poll(self._s, buf, max_n, ctypes.byref(n)), "server_poll")
        out = []
        for k in range(n.value):
            c = buf[k]
            self._pending.pop(c.request, None)
            out.append({"request": c.request, "system": c.system, "status": c.status, "readout": c.readout,
                        "latency_s": c.latency_s, "done_s": c.done_s})
        return out

    def drain(self, timeout_s: float = 60.0) -> list:
        """Poll until every submitted request has completed."""
        got = []
        t_end = time.time() + timeout_s
        while self._pending:
            got.extend(self.poll())
            if not self._pending:
                break
            if time.time() > t_end:
                raise TimeoutError("%d requests still pending" % len(self._pending))
            time.sleep(2e-4)
        return got

    def stats(self) -> dict:
        st = ShwfsServerStats()
        check(_lib.lib().shwfs_server_get_stats(self._s, ctypes.byref(st)), "server_get_stats")
        return {f: getattr(st, f) for f, _ in ShwfsServerStats._fields_}

    def clock(self) -> float:
        return float(_lib.lib().shwfs_server_clock(self._s))

    def close(self) -> None:
        if getattr(self, "_s", None) is not None:
            _lib.lib().shwfs_server_destroy(self._s)
            self._s = None
            self._pending.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_schedule(rates_hz, duration_s: float, seed: int = 0):
    """Arrival times of independent Poisson request streams, one per system:
    a list of (time_s, system_index) sorted by time."""
    rng = np.random.default_rng(seed)
    ev = []
    for k, r in enumerate(rates_hz):
        t = rng.exponential(1.0 / r)
        while t < duration_s:
            ev.append((t, k))
            t += rng.exponential(1.0 / r)
    ev.sort()
    return ev


def run_schedule(server: WfsServer, sids, phases, schedule, lead_s: float | None = None, timeout_s: float = 120.0):
    """Submit a whole arrival schedule (released on the server clock from now
    + lead_s, by default long enough for the submissions themselves), drain
    it, and summarise latency and throughput.  ``phases[k]`` is a list of
    device phase frames of system k, used round-robin."""
    if lead_s is None:
        lead_s = 0.05 + 3e-5 * len(schedule)
    t0 = server.clock() + lead_s
    nph = [0] * len(sids)
    for t, k in schedule:
        ph = phases[k][nph[k] % len(phases[k])]
        nph[k] += 1
        server.submit(sids[k], ph, release_s=t0 + t)
    done = server.drain(timeout_s)
    bad = [c for c in done if c["status"] != 0]
    lat = np.array([c["latency_s"] for c in done]) * 1e3
    ro = [c for c in done if c["readout"]]
    span = max(c["done_s"] for c in done) - t0 if done else 0.0
    work = sum(server.lit[c["system"]] for c in ro)
    return {"requests": len(done), "errors": len(bad), "readout_frames": len(ro),
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "max": float(lat.max()), "mean": float(lat.mean())} if len(lat) else {},
            "makespan_s": span, "subap_frames_per_s": work / span if span > 0 else 0.0}
