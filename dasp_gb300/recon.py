"""Reconstructor step on the device: the consumer of the centroids.

DASP's tomoRecon turns slopes into actuator commands each iteration: decay
the previous commands (science/tomoRecon.py:1089-1107) and subtract the
gain-weighted reconstructor product (:1196-1223,
``outputData -= gains * dot(reconmx, data)``).  :class:`Reconstructor` keeps
the reconstructor, gains, decay and commands in HBM and does the step in one
HBM-bound kernel (``shwfs_mvm_update``), so centroids from the engine's
device-resident ``cents`` feed it without a host round trip.
"""
from __future__ import annotations

import numpy as np

from . import _lib


class Reconstructor:
    def __init__(self, reconmx, gains=0.5, decay=1.0):
        import torch
        r = torch.as_tensor(np.asarray(reconmx, np.float32) if not isinstance(reconmx, torch.Tensor) else reconmx)
        self.R = r.to(device="cuda", dtype=torch.float32).contiguous()
        self.nacts, self.ncents = self.R.shape
        self._gain_vec = self._vec(gains)
        self._decay_vec = self._vec(decay)
        self.gain = float(gains) if self._gain_vec is None else 0.0
        self.decay = float(decay) if self._decay_vec is None else 0.0
        self.act = torch.zeros(self.nacts, device="cuda", dtype=torch.float32)

    def _vec(self, v):
        import torch
        if np.ndim(v) == 0:
            return None
        t = torch.as_tensor(np.asarray(v, np.float32)).cuda().contiguous()
        if t.numel() != self.nacts:
            raise ValueError("per-actuator gains/decay need nacts values")
        return t

    def step(self, slopes, stream=None):
        """One iteration with the slope vector ``slopes`` (CUDA tensor of
        ncents float32); returns the updated command tensor."""
        if not (slopes.is_cuda and slopes.is_contiguous() and slopes.numel() == self.ncents
                and str(slopes.dtype) == "torch.float32"):
            raise ValueError("slopes must be a contiguous float32 CUDA tensor of ncents values")
        s = getattr(stream, "cuda_stream", stream)
        gp = None if self._gain_vec is None else self._gain_vec.data_ptr()
        dp = None if self._decay_vec is None else self._decay_vec.data_ptr()
        _lib.check(_lib.lib().shwfs_mvm_update(self.nacts, self.ncents, self.R.data_ptr(), slopes.data_ptr(), gp,
                                               self.gain, dp, self.decay, self.act.data_ptr(), s), "mvm_update")
        return self.act
