"""Several wavefront sensors per launch: one CUDA graph per readout frame.

The reference serves several WFSs of a simulation by giving each its own
``centcmod`` object and running them one after another from
``science/wfscent.py`` (resource sharing, science/wfscent.py:585-598).  A
:class:`WfsBatch` captures one readout frame of every handle into a CUDA graph,
each handle's kernels on their own branch so that sensors of different sizes
share the GPU (optionally, handles on the FP32 form that share a kernel
instantiation as one persistent multi-handle kernel), and replays it with
one launch per frame.  Every handle must
have its ``phs``, ``cents`` and ``bimg`` bound to CUDA tensors (``set_io``);
the noise frame index of each handle advances on the device between replays,
so a batched frame gives the same images and centroids as ``run_batch`` with
one frame on that handle alone.
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import check


class WfsBatch:
    def __init__(self, engines, multi=False):
        """``multi``: run the FP32-form handles that share a kernel
        instantiation as one persistent multi-handle kernel (see
        :meth:`set_multi`)."""
        self.engines = list(engines)
        if not self.engines:
            raise ValueError("a batch needs at least one engine")
        arr = (ctypes.c_void_p * len(self.engines))(*[e.centstruct for e in self.engines])
        b = ctypes.c_void_p()
        check(_lib.lib().shwfs_batch_create(arr, len(self.engines), ctypes.byref(b)), "batch_create")
        self._b = b
        if multi:
            self.set_multi(True)

    def set_multi(self, on=True):
        """Group FP32-form handles of one kernel instantiation and shared-memory
        footprint into persistent multi-handle kernel launches (off by
        default: concurrent per-handle launches measured as fast or faster);
        results are identical either way.  Re-captures the graph."""
        check(_lib.lib().shwfs_batch_set_multi(self._b, 1 if on else 0), "batch_set_multi")

    def run(self, stream=None):
        """One readout frame of every engine.  With ``stream`` (torch stream
        or raw handle) the graph is queued and not waited for; without, the
        call waits and checks the kernels' status."""
        s = getattr(stream, "cuda_stream", stream)
        check(_lib.lib().shwfs_batch_run(self._b, s), "batch_run")

    def multi_launches(self) -> int:
        """Multi-handle fused-kernel launches in the captured graph: handles on
        the FP32 form that share a kernel instantiation run as one persistent
        kernel over all their tiles."""
        n = ctypes.c_int(0)
        check(_lib.lib().shwfs_batch_multi_launches(self._b, ctypes.byref(n)), "batch_multi_launches")
        return n.value

    def free(self):
        if getattr(self, "_b", None) is not None:
            _lib.lib().shwfs_batch_free(self._b)
            self._b = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
