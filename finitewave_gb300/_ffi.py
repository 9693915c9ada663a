"""ctypes binding of libfwgpu.so (the C ABI declared in include/fwgpu.h).

The structures below mirror fwgpu.h field for field; ``load()`` checks their
sizes against the library's own ``fw_struct_size`` before any call is made.
Every non-OK status is turned into an exception carrying
``fw_last_error()``.  There is no fallback: if the library cannot be loaded
(no CUDA toolkit to build it, no GPU to run it) the calls raise.
"""
import ctypes
import os
import threading

from . import _build

FW_OK = 0
FW_ERR_ARG = -1
FW_ERR_CUDA = -2
FW_ERR_UNSUPPORTED = -3

FW_DEV_LAT_OVERFLOW = 1
FW_DEV_PROBE_OVERFLOW = 2
FW_DEV_BATCH_FAULT = 4
FW_DEV_TIMEOUT = 8
FW_DEV_TIP_OVERFLOW = 16
FW_DEV_NONFINITE = 32

FW_DEBUG_FORCE_TIMEOUT = 1

MODEL_AP, MODEL_MS, MODEL_FK, MODEL_TP06, MODEL_CRN = 1, 2, 3, 4, 5
MODEL_BK, MODEL_BO, MODEL_LR91 = 6, 7, 8
ISO5, ANISO9, ISO7, ANISO19, SYM9, ANISO19_XY = 1, 2, 3, 4, 5, 6
F64, F32 = 0, 1
FORM_PLAIN, FORM_FUSED = 0, 1
STIM_VOLTAGE, STIM_CURRENT = 0, 1

MAX_STATE = 24
MAX_PARAMS = 64
MAX_STIMS = 16
MAX_AT = 4
MAX_LAT = 2
MAX_PROBE = 4
MAX_PROBE_VARS = 8
MAX_ECG = 2
MAX_TIP = 1
MAX_ECG_LEADS = 8
MAX_FUSED_STATE = 4

STENCIL_NW = {ISO5: 5, ANISO9: 9, ISO7: 7, ANISO19: 19, SYM9: 9,
              ANISO19_XY: 19}
# weight planes of the 19-point stencil that in-plane fibers leave at zero
ANISO19_XY_ZERO = (9, 10, 13, 14, 15, 16, 17, 18)

_i32, _i64, _f64, _vp = (ctypes.c_int32, ctypes.c_int64, ctypes.c_double,
                         ctypes.c_void_p)


class Window(ctypes.Structure):
    _fields_ = [("first", _i64), ("last", _i64), ("stride", _i64)]


class Stim(ctypes.Structure):
    _fields_ = [("kind", _i32), ("has_umax", _i32), ("first", _i64),
                ("last", _i64), ("value", _f64), ("u_max", _f64),
                ("lo", _i64 * 3), ("hi", _i64 * 3), ("mask", _vp)]


class AtTracker(ctypes.Structure):
    _fields_ = [("win", Window), ("threshold", _f64), ("act_step", _vp)]


class LatTracker(ctypes.Structure):
    _fields_ = [("win", Window), ("threshold", _f64), ("activated", _vp),
                ("cross_steps", _vp), ("cross_count", _vp),
                ("capacity", _i32)]


class ProbeTracker(ctypes.Structure):
    _fields_ = [("win", Window), ("n_cells", _i32), ("n_vars", _i32),
                ("var_ids", _i32 * MAX_PROBE_VARS), ("cells", _vp),
                ("out", _vp), ("sample_offset", _i64), ("capacity", _i64)]


class EcgTracker(ctypes.Structure):
    _fields_ = [("win", Window), ("n_leads", _i32), ("reserved", _i32),
                ("coords", (_f64 * 3) * MAX_ECG_LEADS), ("dr", _f64),
                ("out", _vp), ("sample_offset", _i64), ("capacity", _i64)]


class Tip(ctypes.Structure):
    _fields_ = [("sample", _i32), ("k", _i32), ("i", _i32), ("j", _i32),
                ("x", _f64), ("y", _f64)]


class TipTracker(ctypes.Structure):
    _fields_ = [("win", Window), ("threshold", _f64), ("u_prev", _vp),
                ("out", _vp), ("count", _vp), ("capacity", _i64),
                ("sample_offset", _i64)]


class StepArgs(ctypes.Structure):
    _fields_ = [("model", _i32), ("stencil", _i32), ("precision", _i32),
                ("form", _i32), ("ni", _i64), ("nj", _i64), ("nk", _i64),
                ("mesh", _vp), ("myo", _vp), ("weights", _vp),
                ("u", _vp * 2), ("state", _vp * MAX_STATE),
                ("params", _f64 * MAX_PARAMS), ("dt", _f64),
                ("n_stims", _i32), ("n_at", _i32), ("n_lat", _i32),
                ("n_probe", _i32),
                ("stims", Stim * MAX_STIMS), ("at", AtTracker * MAX_AT),
                ("lat", LatTracker * MAX_LAT),
                ("probe", ProbeTracker * MAX_PROBE),
                ("status", _vp), ("fused_k", _i32),
                ("fused_variant", _i32), ("weights_packed", _vp),
                ("n_ecg", _i32), ("n_tip", _i32),
                ("ecg", EcgTracker * MAX_ECG),
                ("tip", TipTracker * MAX_TIP),
                ("debug_flags", _i32), ("reserved2", _i32),
                ("pitch", _i64), ("state_b", _vp * MAX_FUSED_STATE),
                ("fibers_f32", _vp), ("fly_D_al", _f64), ("fly_D_ac", _f64),
                ("fly_cond", _f64), ("fly_scale", _f64),
                ("weight_rows", _vp), ("weight_row_index", _vp)]


class Batch(ctypes.Structure):
    _fields_ = [("plan", _vp), ("n_tissues", _i32), ("n_tiles", _i32),
                ("ksteps", _i32), ("grid", _i32), ("kernel", _i32),
                ("reserved", _i32), ("group_end", _i32 * 6)]


class FwError(RuntimeError):
    """A non-OK status from libfwgpu."""

    def __init__(self, fn, code, msg):
        super().__init__(f"{fn} failed ({code}): {msg}")
        self.code = code


_lib = None
_lock = threading.Lock()

_SIGS = {
    "fw_version": ([], _i32),
    "fw_launch_count": ([], _i64),
    "fw_struct_size": ([_i32], ctypes.c_size_t),
    "fw_last_error": ([], ctypes.c_char_p),
    "fw_model_info": ([_i32, ctypes.POINTER(_i32), ctypes.POINTER(_i32)],
                      _i32),
    "fw_state_is_f64": ([_i32, _i32, _i32], _i32),
    "fw_state_is_pair": ([_i32, _i32, _i32], _i32),
    "fw_build_weights": ([_i32, _i32, _vp, _vp, _f64, _vp, _f64, _f64, _f64,
                          _f64, _f64, _i64, _i64, _i64, _vp, _vp], _i32),
    "fw_diffuse": ([_i32, _i32, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64,
                    _vp], _i32),
    "fw_ionic": ([_i32, _i32, _vp, _vp, _vp, _vp, _i64, _f64, _vp, _vp],
                 _i32),
    "fw_step": ([ctypes.POINTER(StepArgs), _i64, _i64, _vp], _i32),
    "fw_pack_weights": ([_i32, _vp, _i64, _vp, _vp], _i32),
    "fw_ecg": ([_i32, _i32, _vp, _vp, _vp, _i64, _i64, _i64, _vp, _i32, _f64,
                _vp, _vp], _i32),
    "fw_batch_plan_size": ([_vp, _i32, ctypes.POINTER(_i64)], _i32),
    "fw_batch_plan": ([_vp, _i32, _vp, _vp, _i64, ctypes.POINTER(Batch),
                       _vp], _i32),
    "fw_batch_scratch_size": ([ctypes.POINTER(_i64)], _i32),
    "fw_batch_run": ([ctypes.POINTER(Batch), _vp, _i64, _i64, _vp], _i32),
    "fw_batch_run_noalloc": ([ctypes.POINTER(Batch), _i64, _i64, _vp], _i32),
}

# symbol -> ctypes structure whose size must match the library's
_STRUCTS = {0: StepArgs, 1: Stim, 2: AtTracker, 3: LatTracker,
            4: ProbeTracker, 5: Window, 6: Batch, 7: EcgTracker,
            8: TipTracker, 9: Tip}


def load(path=None):
    """Load (building first if needed) libfwgpu.so and return the handle.
    The environment variable FWGPU_LIBRARY names a prebuilt library to load
    instead."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if path is None:
            path = os.environ.get("FWGPU_LIBRARY") or _build.build()
        if not os.path.exists(path):
            raise OSError(f"libfwgpu not found at {path}")
        L = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        for which, struct in _STRUCTS.items():
            got = L.fw_struct_size(which)
            if got != ctypes.sizeof(struct):
                raise RuntimeError(
                    f"ABI mismatch for {struct.__name__}: library "
                    f"{got} bytes, binding {ctypes.sizeof(struct)} bytes")
        _lib = L
        return _lib


def check(fn, rc):
    if rc != FW_OK:
        msg = load().fw_last_error()
        raise FwError(fn, rc, msg.decode() if msg else "")
    return rc


def call(name, *args):
    return check(name, getattr(load(), name)(*args))


def model_info(model):
    ns, npar = _i32(), _i32()
    call("fw_model_info", model, ctypes.byref(ns), ctypes.byref(npar))
    return ns.value, npar.value


def state_is_f64(model, precision, index):
    return bool(load().fw_state_is_f64(model, precision, index))


def state_is_pair(model, precision, index):
    """True when the state variable is a compensated float32 pair (hi, lo)
    per node."""
    return bool(load().fw_state_is_pair(model, precision, index))
