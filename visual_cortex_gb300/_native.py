"""ctypes binding of the C ABI declared in include/patchv1_gb300.h.

The native library is the product: there is no Python or CPU fallback for the hot path.  The
library is loaded (and built if it is out of date) on the first use of `lib`; if it is missing
and cannot be built, that first use raises ImportError.  Importing this module alone (for the
ctypes structures of the model objects) maps nothing.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import library_path

MAX_NTYPE = 2
MAX_NG = 2

PV1_OK = 0
ERRORS = {-1: "bad argument", -2: "CUDA error", -3: "call out of order", -4: "unsupported option",
          -5: "device error word", -6: "out of device memory"}

REC_RAW, REC_LGN_SP, REC_LGN_FR, REC_SPIKES = 1, 2, 4, 8
ST = dict(v=0, w=1, tBack=2, dep=3, gFF=4, hFF=5, gE=6, hE=7, gI=8, hI=9, sInfo=10,
          lgn_ltr=11, lgn_lnl=12, lgn_sInfo=13, farPull=14, lgn_rng=15, v1_rng_cond=16,
          v1_rng_noisy=17, sLGN=18, ff_post=19, ff_pre=20, total_ff=21)

_f2 = C.c_float * MAX_NG
_t2 = C.c_float * MAX_NTYPE
_t4 = C.c_float * (MAX_NTYPE * MAX_NG)
_tt = C.c_float * (MAX_NTYPE * MAX_NTYPE)


class V1Config(C.Structure):
    _fields_ = [
        ("nblock", C.c_uint32), ("blockSize", C.c_uint32), ("nType", C.c_uint32),
        ("nTypeE", C.c_uint32), ("typeAcc", C.c_uint32 * MAX_NTYPE),
        ("ngFF", C.c_uint32), ("ngE", C.c_uint32), ("ngI", C.c_uint32), ("dt", C.c_float),
        ("riseFF", _f2), ("decayFF", _f2), ("riseE", _f2), ("decayE", _f2),
        ("riseI", _f2), ("decayI", _f2),
        ("vE", C.c_float), ("vI", C.c_float), ("vL", C.c_float),
        ("vR", _t2), ("vThres", _t2), ("gL", _t2), ("C", _t2), ("tRef", _t2), ("vT", _t2),
        ("deltaT", _t2), ("tau_w", _t2), ("a", _t2), ("b", _t2),
        ("pFF", _t4), ("pE", _t4), ("pI", _t4), ("synFail", _tt), ("synPerCon", _tt),
        ("synFailFF", _t2), ("synPerConFF", _t2), ("noisyDep", _t2),
        ("tau_noise", C.c_float), ("noiseOnTonic", C.c_int32), ("iModel", C.c_int32),
        ("noDelay", C.c_int32), ("noFarDelay", C.c_int32), ("speedOfThought", C.c_float),
        ("hWrite", C.c_int32),
    ]


class FFLearning(C.Structure):
    """pv1_ff_learning: the cfg values of LGN->V1 plasticity (learning 1-4)."""
    _fields_ = [("learning", C.c_int32), ("tauLTP", C.c_float), ("tauLTD", C.c_float), ("tauTrip", C.c_float),
                ("tauAvg", C.c_float), ("targetFR", C.c_float), ("A_LGN", C.c_float), ("r_LTD", C.c_float),
                ("gmaxLGN", C.c_float), ("gminLGN", C.c_float), ("sRatioLGN", C.c_float),
                ("decayTimeHomeoFF", C.c_float), ("FF_InfRatio", C.c_float), ("applyHomeo", C.c_int32),
                ("symmetricHomeo", C.c_int32), ("rebound", C.c_int32), ("nLearnTypeFF_E", C.c_int32),
                ("nLearnTypeFF_I", C.c_int32), ("tauLTP_I", C.c_float), ("tauLTD_I", C.c_float),
                ("tauTrip_I", C.c_float), ("tauAvg_I", C.c_float), ("targetFR_I", C.c_float), ("A_LGN_I", C.c_float),
                ("r_LTD_I", C.c_float), ("gmaxLGN_I", C.c_float), ("gminLGN_I", C.c_float),
                ("sRatioLGN_I", C.c_float), ("tauAvgCortical", C.c_float)]


class LgnConfig(C.Structure):
    _fields_ = [
        ("nLGN", C.c_uint32), ("nParvo_I", C.c_uint32), ("nMagno_I", C.c_uint32),
        ("nParvo_C", C.c_uint32), ("nMagno_C", C.c_uint32), ("mSample1D", C.c_uint32),
        ("nKernelSample", C.c_uint32), ("kernelSampleInterval", C.c_uint32),
        ("iKernelSampleT0", C.c_uint32), ("denorm", C.c_uint32), ("ntPerFrame", C.c_uint32),
        ("maxFrame", C.c_uint32), ("magnoComp", C.c_uint32), ("frameOffset", C.c_uint32),
        ("dt", C.c_float), ("kernelSampleDt", C.c_float), ("kernelSampleT0", C.c_float),
        ("convolRatio", C.c_float), ("frRatio", C.c_float), ("normViewDistance", C.c_float),
        ("L_x0", C.c_float), ("L_y0", C.c_float), ("R_x0", C.c_float), ("R_y0", C.c_float),
        ("nsig", C.c_float), ("flat_retina", C.c_int32),
    ]


class LgnParvoConfig(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("nSample1D", "nKernelSample", "kernelSampleInterval",
                                          "iKernelSampleT0", "parvoComp", "frameOffset")] + \
               [("kernelSampleDt", C.c_float), ("kernelSampleT0", C.c_float)]


_FP = C.POINTER(C.c_float)
_UP = C.POINTER(C.c_uint32)


class LgnParams(C.Structure):
    _fields_ = [(n, _FP) for n in ("polar", "ecc", "rw", "rh", "orient", "k", "ratio", "tauR",
                                   "tauD", "nR", "nD", "delay", "spont", "c50", "sharpness")] + \
               [("coneType", _UP)]


class InitRecord(C.Structure):
    _fields_ = [("uniforms", _FP), ("nUniform", _UP), ("normals", _FP), ("nNormal", _UP),
                ("normalCap", C.c_uint32), ("history", _FP)]


def _load() -> C.CDLL:
    import os
    from .build import build_native
    override = os.environ.get("PV1_LIBRARY")
    try:
        # PV1_LIBRARY: an already built library with this ABI; otherwise the in-tree build
        # (a no-op when the library is newer than its sources)
        path = override if override else build_native()
    except RuntimeError as e:
        path = library_path()
        if not Path(path).exists():
            raise ImportError(f"native library {path} is missing and cannot be built: {e}") from e
    lib = C.CDLL(str(path))
    P = C.c_void_p
    sig = {
        "pv1_abi_version": ([], C.c_int),
        "pv1_set_device": ([C.c_int], C.c_int),
        "pv1_host_alloc": ([C.c_uint64, C.POINTER(C.c_void_p)], C.c_int),
        "pv1_run_spikes_to_host": ([P, C.c_uint32, _FP], C.c_int),
        "pv1_host_free": ([C.c_void_p], None),
        "pv1_plan_create": ([C.POINTER(V1Config), C.POINTER(P)], C.c_int),
        "pv1_plan_destroy": ([P], None),
        "pv1_last_error": ([P], C.c_char_p),
        "pv1_lgn_setup": ([P, C.POINTER(LgnConfig), C.POINTER(LgnParams), C.c_uint64], C.c_int),
        "pv1_lgn_get_tables": ([P, _FP, _FP, _FP, _FP], C.c_int),
        "pv1_stimulus_load": ([P, C.c_uint32, C.c_uint32, C.c_uint32, _FP, _FP], C.c_int),
        "pv1_lgn_get_spatial": ([P, _FP], C.c_int),
        "pv1_lgn_setup_parvo": ([P, C.POINTER(LgnConfig), C.POINTER(LgnParvoConfig), C.POINTER(LgnParams), _FP,
                                 C.c_uint64], C.c_int),
        "pv1_lgn_get_parvo_tables": ([P, _FP, _FP, _FP], C.c_int),
        "pv1_lgn_get_parvo_spatial": ([P, _FP], C.c_int),
        "pv1_v1_set_lgn_synapses": ([P, C.c_uint32, _UP, _UP, _FP], C.c_int),
        "pv1_v1_set_near": ([P, C.c_uint32, _UP, _UP, _FP], C.c_int),
        "pv1_v1_set_far": ([P, _UP, _UP, _FP, _FP], C.c_int),
        "pv1_v1_set_near_delayed": ([P, C.c_uint32, _UP, _UP, _FP, _FP], C.c_int),
        "pv1_v1_set_state": ([P, _FP, _FP, _FP, _FP, _FP, _FP, _FP, _FP, _FP], C.c_int),
        "pv1_v1_init_rng": ([P, C.c_uint64, C.c_uint32], C.c_int),
        "pv1_v1_far_failure_engines": ([P, C.c_uint64, C.c_uint32], C.c_int),
        "pv1_sample_ids": ([C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _UP, C.POINTER(C.c_uint32)],
                           C.c_int),
        "pv1_frames_setup": ([P, C.c_uint32, C.c_uint32, _UP, _UP, C.c_uint32, C.c_float], C.c_int),
        "pv1_frames_collect": ([P, C.c_uint64, C.c_uint32, _FP, C.POINTER(C.c_uint32)], C.c_int),
        "pv1_checkpoint_size": ([P, C.POINTER(C.c_uint64)], C.c_int),
        "pv1_checkpoint_save": ([P, C.c_void_p, C.c_uint64], C.c_int),
        "pv1_checkpoint_load": ([P, C.c_void_p, C.c_uint64], C.c_int),
        "pv1_set_step": ([P, C.c_int64], C.c_int),
        "pv1_v1_init_spikes": ([P, C.c_uint64, C.c_uint32, _FP, C.c_uint32, C.POINTER(InitRecord)], C.c_int),
        "pv1_host_init_state": ([C.POINTER(V1Config), C.c_uint64, _FP, _UP, C.c_int, C.c_float,
                                 _FP, _FP, _FP, _FP, _FP, _FP, _FP, _FP, _FP, _FP, _FP, _FP],
                                C.c_int),
        "pv1_set_record": ([P, C.c_int, C.c_uint32], C.c_int),
        "pv1_raw_record_floats": ([P], C.c_int64),
        "pv1_run": ([P, C.c_uint32, C.c_int], C.c_int),
        "pv1_fetch_records": ([P, C.c_uint64, C.c_uint32, _FP, _FP, _FP], C.c_int),
        "pv1_get_state": ([P, C.c_int, _FP], C.c_int),
        "pv1_put_state": ([P, C.c_int, _FP], C.c_int),
        "pv1_set_draw_record": ([P, C.c_uint32, C.c_uint32], C.c_int),
        "pv1_fetch_draws": ([P, C.c_int, _FP, C.POINTER(C.c_int32)], C.c_int),
        "pv1_last_launch_count": ([P], C.c_int64),
        "pv1_fetch_spikes": ([P, C.c_uint64, C.c_uint32, _FP], C.c_int),
        "pv1_run_timed": ([P, C.c_uint32, C.c_uint64, _FP], C.c_int),
        "pv1_time_kernels": ([P, C.c_uint32, _FP, _FP, C.POINTER(C.c_int)], C.c_int),
        "pv1_persistent_mode": ([P, C.c_int], C.c_int),
        "pv1_set_wait_limit": ([P, C.c_int64], C.c_int),
        "pv1_set_ff_learning": ([P, C.POINTER(FFLearning)], C.c_int),
        "pv1_set_lgn_source": ([P, C.c_void_p, C.c_int64, C.c_int64], C.c_int),
        "pv1_lgn_tc_device_spikes": ([P], C.c_void_p),
        "pv1_ff_learning_rates": ([C.POINTER(FFLearning), C.c_float, _FP], C.c_int),
        "pv1_lgn_spikes_noalloc": ([P, C.c_uint32, _FP, _FP], C.c_int),
        "pv1_batch_create": ([C.POINTER(P), C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(P)], C.c_int),
        "pv1_batch_destroy": ([P], None),
        "pv1_batch_last_error": ([P], C.c_char_p),
        "pv1_batch_run": ([P, C.c_uint64, _FP], C.c_int64),
        "pv1_batch_autotune": ([P, C.c_int], C.c_int),
        "pv1_batch_tuning": ([P, C.POINTER(C.c_int), C.POINTER(C.c_int), _FP], C.c_int),
        "pv1_batch_stats": ([P, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                             C.POINTER(C.c_double)], C.c_int),
        "pv1_batch_launch_count": ([P], C.c_int64),
        "pv1_batch_sweep": ([P, _FP], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


_LIB = None


def _lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = _load()
    return _LIB


def __getattr__(name):
    # `N.lib` loads the library on first access (PEP 562)
    if name == "lib":
        return _lib()
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")


def loaded() -> bool:
    """Whether this process has mapped the native library."""
    return _LIB is not None


class NativeError(RuntimeError):
    pass


def fptr(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_FP)


def uptr(a):
    if a is None:
        return None
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(_UP)


def check(plan, rc: int, what: str):
    if rc != PV1_OK:
        msg = _lib().pv1_last_error(plan).decode() if plan else ""
        raise NativeError(f"{what} failed ({ERRORS.get(rc, rc)}): {msg}")


class _PinnedBlock:
    """Owner of one page-locked host allocation (freed when the last array view goes)."""

    def __init__(self, nbytes: int):
        ptr = C.c_void_p()
        rc = _lib().pv1_host_alloc(nbytes, C.byref(ptr))
        if rc != 0 or not ptr.value:
            raise MemoryError(f"pv1_host_alloc({nbytes}) failed: {rc}")
        self.ptr = ptr.value
        self.nbytes = nbytes

    def __del__(self):
        if getattr(self, "ptr", None):
            _lib().pv1_host_free(C.c_void_p(self.ptr))
            self.ptr = None


def pinned_empty(shape, dtype=np.float32) -> np.ndarray:
    """A numpy array in page-locked host memory: the library's copies to and from it (stimulus
    frames in, records out) run asynchronously at the full host-link bandwidth."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape))
    block = _PinnedBlock(max(n * dtype.itemsize, 1))
    buf = (C.c_char * block.nbytes).from_address(block.ptr)
    buf.owner = block        # the allocation lives as long as any view of the array
    return np.frombuffer(buf, dtype=dtype, count=n).reshape(shape)
