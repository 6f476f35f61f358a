"""ctypes binding of the C ABI in ``include/shwfs.h``.

Loads the in-tree ``dasp_gb300/_build/libshwfs.so`` and nothing else: if the
library has not been built the import of the engine fails loudly instead of
falling back to any CPU code.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libshwfs.so")

SHWFS_OK = 0
SHWFS_ERR_INVALID = 1
SHWFS_ERR_UNSUPPORTED = 2
SHWFS_ERR_CUDA = 3
SHWFS_ERR_NOMEM = 4
SHWFS_ERR_STATE = 5

SHWFS_F32 = 0
SHWFS_I32 = 1

VAL_NONE, VAL_INT, VAL_FLOAT, VAL_ARRAY, VAL_TUPLE3 = 0, 1, 2, 3, 4

NOISE_COUNTER = 0
NOISE_REFERENCE = 1
NOISEMODE = 100

# every entry point declared in include/shwfs.h
EXPORTS = ("shwfs_initialise", "shwfs_run", "shwfs_run_slope", "shwfs_update", "shwfs_free",
           "shwfs_last_error", "shwfs_run_async", "shwfs_run_batch", "shwfs_set_io",
           "shwfs_get_info", "shwfs_version", "shwfs_image_centroids_noalloc",
           "shwfs_batch_create", "shwfs_batch_run", "shwfs_batch_free", "shwfs_batch_set_multi",
           "shwfs_batch_multi_launches", "shwfs_autotune", "shwfs_gemm_stagings",
           "shwfs_sample_noise", "shwfs_set_split_event", "shwfs_server_create", "shwfs_server_add_system",
           "shwfs_server_remove_system", "shwfs_server_submit", "shwfs_server_poll", "shwfs_server_get_stats",
           "shwfs_server_clock", "shwfs_server_destroy", "shwfs_selftest_bounded_wait",
           "shwfs_screen_create", "shwfs_screen_add", "shwfs_screen_window", "shwfs_screen_read",
           "shwfs_screen_free", "shwfs_mvm_update", "shwfs_test_correlation", "shwfs_run_prenoise",
           "shwfs_screens_pupil_phase")

NOALLOC_MAX_SUBAPS = 65536


class ShwfsServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_int64), ("max_inflight", ctypes.c_int), ("device", ctypes.c_int),
                ("integration_mode", ctypes.c_int)]


class ShwfsCompletion(ctypes.Structure):
    _fields_ = [("request", ctypes.c_uint64), ("system", ctypes.c_int), ("status", ctypes.c_int),
                ("readout", ctypes.c_int), ("latency_s", ctypes.c_double), ("done_s", ctypes.c_double)]


class ShwfsServerStats(ctypes.Structure):
    _fields_ = [("systems", ctypes.c_int), ("admitted", ctypes.c_int), ("pending", ctypes.c_int),
                ("used_bytes", ctypes.c_int64), ("budget_bytes", ctypes.c_int64), ("inflight", ctypes.c_int),
                ("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64)]


class ShwfsImageJob(ctypes.Structure):
    """shwfs_image_job: arguments of the allocation-free image centroiding call."""
    _fields_ = [("nsubx", ctypes.c_int), ("nimg", ctypes.c_int), ("ncen", ctypes.c_int),
                ("image_ndim", ctypes.c_int), ("image_rows", ctypes.c_int64), ("image_cols", ctypes.c_int64),
                ("image", ctypes.c_void_p), ("subflag", ctypes.c_void_p), ("refCents", ctypes.c_void_p),
                ("noiseFloor", ctypes.c_float), ("threshType", ctypes.c_int), ("calsource", ctypes.c_int),
                ("useBrightest", ctypes.c_int), ("pxlPower", ctypes.c_float), ("imageOnly", ctypes.c_int),
                ("readNoise", ctypes.c_float), ("readBg", ctypes.c_float), ("seed", ctypes.c_uint64),
                ("frame", ctypes.c_uint64), ("cents", ctypes.c_void_p), ("bimg", ctypes.c_void_p)]


class ShwfsArray(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("ndim", ctypes.c_int), ("shape", ctypes.c_int64 * 4),
                ("dtype", ctypes.c_int), ("on_device", ctypes.c_int)]


class ShwfsInit(ctypes.Structure):
    _fields_ = [
        ("nthreads", ctypes.c_int), ("nsubaps", ctypes.c_int), ("ncen", ctypes.c_int),
        ("fftsize", ctypes.c_int), ("clipsize", ctypes.c_int), ("nimg", ctypes.c_int),
        ("phasesize", ctypes.c_int), ("readnoise", ctypes.c_float), ("readbg", ctypes.c_float),
        ("addPoisson", ctypes.c_int), ("noiseFloor", ctypes.c_float), ("sig", ctypes.c_double),
        ("sigArr", ShwfsArray), ("skybrightness", ctypes.c_double), ("skybrightnessArr", ShwfsArray),
        ("calsource", ctypes.c_int), ("pxlPower", ctypes.c_float), ("nintegrations", ctypes.c_int),
        ("nlatency", ctypes.c_int), ("seed", ctypes.c_uint64), ("phs", ShwfsArray), ("pupfn", ShwfsArray),
        ("spotpsf", ShwfsArray), ("cents", ShwfsArray), ("subflag", ShwfsArray), ("bimg", ShwfsArray),
        ("fracSubArea", ShwfsArray), ("opticalBinning", ctypes.c_int), ("centWeight", ShwfsArray),
        ("correlationCentroiding", ctypes.c_int), ("corrThresh", ctypes.c_float),
        ("corrPattern", ShwfsArray), ("corrimg", ShwfsArray), ("threshType", ctypes.c_int),
        ("imageOnly", ctypes.c_int), ("useBrightest", ctypes.c_int), ("useBrightestArr", ShwfsArray),
        ("preBinningFactor", ctypes.c_int), ("parabolicFit", ctypes.c_int), ("gaussianFit", ctypes.c_int),
        ("gaussianMinVal", ctypes.c_float), ("gaussianReplaceVal", ctypes.c_float),
        ("inputImage", ShwfsArray), ("subapLocation", ShwfsArray),
    ]


class ShwfsValue(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("ival", ctypes.c_int64), ("dval", ctypes.c_double),
                ("arr", ShwfsArray * 3)]


class ShwfsInfo(ctypes.Structure):
    _fields_ = [("nsubx", ctypes.c_int), ("nsubaps", ctypes.c_int), ("nlit", ctypes.c_int),
                ("fftsize", ctypes.c_int), ("psfsize", ctypes.c_int), ("clipsize", ctypes.c_int),
                ("nimg", ctypes.c_int), ("phasesize", ctypes.c_int), ("tile_subaps", ctypes.c_int),
                ("smem_bytes", ctypes.c_int), ("grid_ctas", ctypes.c_int), ("noise_mode", ctypes.c_int),
                ("cur_integ", ctypes.c_int), ("frames_read", ctypes.c_uint64), ("form", ctypes.c_int),
                ("form_active", ctypes.c_int), ("host_io_direct", ctypes.c_int),
                ("gemm_kcb", ctypes.c_int), ("gemm_nw", ctypes.c_int), ("gemm_nk", ctypes.c_int),
                ("gemm_dbuf", ctypes.c_int), ("gemm_cw", ctypes.c_int), ("gemm_staging", ctypes.c_int),
                ("gemm_candidates", ctypes.c_int)]


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libshwfs.so is not built (%s); run `python -m dasp_gb300.build` or "
                               "__graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        vp = ctypes.c_void_p
        L.shwfs_initialise.argtypes = [P(ShwfsInit), P(vp)]
        L.shwfs_run.argtypes = [vp, P(ctypes.c_float)]
        L.shwfs_run_slope.argtypes = [vp, P(ctypes.c_float)]
        L.shwfs_update.argtypes = [vp, ctypes.c_int, P(ShwfsValue)]
        L.shwfs_free.argtypes = [vp]
        L.shwfs_last_error.restype = ctypes.c_char_p
        L.shwfs_last_error.argtypes = []
        L.shwfs_run_async.argtypes = [vp, vp]
        L.shwfs_run_prenoise.argtypes = [vp, P(ShwfsArray), P(ShwfsArray), P(ShwfsArray), P(ctypes.c_float)]
        L.shwfs_run_batch.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int64, vp, vp, vp]
        L.shwfs_set_io.argtypes = [vp, P(ShwfsArray), P(ShwfsArray), P(ShwfsArray)]
        L.shwfs_get_info.argtypes = [vp, P(ShwfsInfo)]
        L.shwfs_version.restype = ctypes.c_char_p
        L.shwfs_version.argtypes = []
        L.shwfs_image_centroids_noalloc.argtypes = [P(ShwfsImageJob), vp, ctypes.c_char_p, ctypes.c_size_t]
        L.shwfs_batch_create.argtypes = [P(vp), ctypes.c_int, P(vp)]
        L.shwfs_batch_run.argtypes = [vp, vp]
        L.shwfs_batch_free.argtypes = [vp]
        L.shwfs_batch_multi_launches.argtypes = [vp, P(ctypes.c_int)]
        L.shwfs_batch_set_multi.argtypes = [vp, ctypes.c_int]
        L.shwfs_autotune.argtypes = [vp, P(ctypes.c_int)]
        L.shwfs_gemm_stagings.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          P(ctypes.c_int), ctypes.c_int, P(ctypes.c_int)]
        L.shwfs_set_split_event.argtypes = [vp, vp]
        L.shwfs_server_create.argtypes = [P(ShwfsServerConfig), P(vp)]
        L.shwfs_server_add_system.argtypes = [vp, P(ShwfsInit), ctypes.c_int, P(ctypes.c_int)]
        L.shwfs_server_remove_system.argtypes = [vp, ctypes.c_int]
        L.shwfs_server_submit.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, vp, ctypes.c_double,
                                          P(ctypes.c_uint64)]
        L.shwfs_server_poll.argtypes = [vp, P(ShwfsCompletion), ctypes.c_int, P(ctypes.c_int)]
        L.shwfs_server_get_stats.argtypes = [vp, P(ShwfsServerStats)]
        L.shwfs_server_clock.argtypes = [vp]
        L.shwfs_server_destroy.argtypes = [vp]
        L.shwfs_server_clock.restype = ctypes.c_double
        L.shwfs_sample_noise.argtypes = [ctypes.c_int, vp, ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint64, vp, vp]
        L.shwfs_test_correlation.argtypes = [ctypes.c_int, vp, vp]
        L.shwfs_selftest_bounded_wait.argtypes = [ctypes.c_int64, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.shwfs_screen_create.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_uint64,
                                          ctypes.POINTER(ctypes.c_void_p)]
        L.shwfs_screen_add.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, vp, vp]
        L.shwfs_screen_window.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp,
                                          ctypes.c_int64, vp]
        L.shwfs_screen_read.argtypes = [vp, vp]
        L.shwfs_screens_pupil_phase.argtypes = [P(vp), ctypes.c_int, P(ctypes.c_int), P(ctypes.c_int),
                                                P(ctypes.c_float), P(ctypes.c_float), ctypes.c_int, vp,
                                                ctypes.c_double, ctypes.c_int, ctypes.c_float, vp, vp]
        L.shwfs_screen_free.argtypes = [vp]
        L.shwfs_mvm_update.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, vp, ctypes.c_float, vp, ctypes.c_float, vp,
                                       vp]
        for name in EXPORTS:
            if name not in ("shwfs_last_error", "shwfs_version", "shwfs_server_clock"):
                getattr(L, name).restype = ctypes.c_int
        _lib = L
    return _lib


class ShwfsError(RuntimeError):
    """A failed engine call; ``status`` holds the shwfs_status code."""

    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


def check(status: int, what: str) -> None:
    if status != SHWFS_OK:
        msg = lib().shwfs_last_error().decode(errors="replace")
        text = "%s: %s" % (what, msg)
        if status in (SHWFS_ERR_INVALID,):
            raise ValueError(text)
        if status == SHWFS_ERR_UNSUPPORTED:
            raise NotImplementedError(text)
        raise ShwfsError(status, text)


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def as_array(x, dtype: str, name: str, keep: list) -> ShwfsArray:
    """Describe ``x`` (None, numpy array, torch tensor) as a shwfs_array.

    Arrays must already be C-contiguous with the right dtype, as the
    reference's checkFloatContigArr/checkIntContigArr require
    (cmod/src/centmodule.c:2132-2149); nothing is converted silently.
    """
    a = ShwfsArray()
    if x is None:
        return a
    code = SHWFS_F32 if dtype == "f" else SHWFS_I32
    if _is_torch(x):
        import torch
        want = torch.float32 if dtype == "f" else torch.int32
        if x.dtype != want or not x.is_contiguous():
            raise ValueError("%s must be %s and contiguous" % (name, "float32" if dtype == "f" else "int32"))
        if x.dim() > 4:
            raise ValueError("%s has too many dimensions" % name)
        if x.is_cuda:
            a.data = x.data_ptr()
            a.on_device = 1
        else:
            arr = x.numpy()
            a.data = arr.ctypes.data
            a.on_device = 0
        a.ndim = x.dim()
        for i, s in enumerate(x.shape):
            a.shape[i] = s
        a.dtype = code
        keep.append(x)
        return a
    if not isinstance(x, np.ndarray):
        raise ValueError("%s must be an array" % name)
    ok = (x.dtype == np.float32) if dtype == "f" else (x.dtype.kind == "i" and x.dtype.itemsize == 4)
    if not ok or not x.flags.c_contiguous:
        raise ValueError("%s must be %s and contiguous" % (name, "float32" if dtype == "f" else "int32"))
    if x.ndim > 4:
        raise ValueError("%s has too many dimensions" % name)
    a.data = x.ctypes.data if x.size else None
    a.ndim = x.ndim
    for i, s in enumerate(x.shape):
        a.shape[i] = s
    a.dtype = code
    a.on_device = 0
    keep.append(x)
    return a
