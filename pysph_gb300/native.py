"""ctypes binding of the C ABI declared in ``include/pysph_gb300.h``.

The library is ``pysph_gb300/_native/libpysph_gb300.so`` (built by
``python -m pysph_gb300.build``).  There is no fallback: if the library or a
CUDA device is missing, :func:`lib` raises.
"""
import ctypes
import os
import threading

from . import build as _build

SPH_OK = 0
SPH_ERR_ARG = -1
SPH_ERR_CUDA = -2
SPH_ERR_GRID = -3
SPH_ERR_JUMP = -4
SPH_ERR_STATE = -5
SPH_ERR_NOTSUP = -6

TERM_PGRAD = 1
TERM_AVISC = 2
TERM_XSPH = 4
TERM_BFORCE = 8
TERM_DRHO = 16
TERM_VDIV = 32

MAX_SOURCES = 8
MAX_AXPY_LINES = 12

VIEW_FIELDS = ("x", "y", "z", "u", "v", "w", "m", "h", "rho", "p", "cs",
               "nx", "ny", "nz", "tx", "ty", "tz")

# Every symbol include/pysph_gb300.h declares (checked by the CPU tests).
EXPORTS = (
    "sph_ctx_create", "sph_ctx_destroy", "sph_ctx_set_stream", "sph_last_error",
    "sph_version", "sph_nnps_build", "sph_nnps_count", "sph_nnps_fill",
    "sph_refresh_state", "sph_density", "sph_rates", "sph_tait", "sph_const_rates",
    "sph_adke_smoothing", "sph_adke_conduction",
    "sph_integrate", "sph_invariants", "sph_error_word", "sph_mean_neighbours",
    "sph_launch_count", "sph_invariants_noalloc", "sph_selftest_conversions", "sph_nbr_lists",
    "sph_batch_create", "sph_batch_destroy", "sph_batch_setup", "sph_batch_step",
    "sph_batch_sync", "sph_batch_error_word", "sph_batch_stream",
    "sph_batch_pair_counts", "sph_batch_stats", "sph_ctx_set_skin", "sph_nnps_update", "sph_nnps_stats",
    "sph_ctx_set_symmetric", "sph_ctx_set_periodic", "sph_ctx_set_deferred",
    "sph_nnps_deferred_stats", "sph_ctx_set_bricks", "sph_pair_pass_stats",
    "sph_step_begin", "sph_step_end", "sph_step_run", "sph_step_stats", "sph_step_destroy",
    "sph_mlp_features", "sph_mlp_sync", "sph_mlp_forward", "sph_mlp_backward_scratch",
    "sph_mlp_backward", "sph_mlp_adam", "sph_mlp_apply", "sph_mlp_targets",
)

# learned momentum closure (include/pysph_gb300.h SPH_MLP_*)
MLP_NIN, MLP_NH, MLP_NOUT = 192, 128, 2
MLP_NNBR, MLP_NCH = 32, 6
MLP_OFF_W1 = 0
MLP_OFF_B1 = MLP_OFF_W1 + MLP_NH * MLP_NIN
MLP_OFF_W2 = MLP_OFF_B1 + MLP_NH
MLP_OFF_B2 = MLP_OFF_W2 + MLP_NH * MLP_NH
MLP_OFF_W3 = MLP_OFF_B2 + MLP_NH
MLP_OFF_B3 = MLP_OFF_W3 + MLP_NOUT * MLP_NH
MLP_NPARAM = MLP_OFF_B3 + MLP_NOUT
SPH_EFLAG_TIMEOUT = 8


class MlpModel(ctypes.Structure):
    _fields_ = [("params", ctypes.c_void_p), ("w1", ctypes.c_void_p), ("w2", ctypes.c_void_p),
                ("w2t", ctypes.c_void_p), ("w3", ctypes.c_void_p)]


class MlpFeatureParams(ctypes.Structure):
    _fields_ = [("c0", ctypes.c_double), ("mean", ctypes.c_float * MLP_NCH),
                ("inv_std", ctypes.c_float * MLP_NCH)]


class ArrayView(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64)] + [(f, ctypes.c_void_p) for f in VIEW_FIELDS] + [
        ("tag", ctypes.c_void_p)]


class SourceTerm(ctypes.Structure):
    _fields_ = [("src", ctypes.c_int), ("flags", ctypes.c_uint32),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
                ("eta", ctypes.c_double), ("eps", ctypes.c_double),
                ("delp", ctypes.c_double)]


class DensityParams(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("tait", ctypes.c_int), ("co", ctypes.c_double),
                ("ro", ctypes.c_double), ("gamma", ctypes.c_double), ("h0", ctypes.c_double)]


class RatesParams(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("add_velocity", ctypes.c_int),
                ("gx", ctypes.c_double), ("gy", ctypes.c_double), ("gz", ctypes.c_double),
                ("add_gravity", ctypes.c_int), ("drho_out", ctypes.c_void_p)]


class AxpyLine(ctypes.Structure):
    _fields_ = [("out", ctypes.c_void_p), ("save", ctypes.c_void_p),
                ("base", ctypes.c_void_p), ("k1", ctypes.c_void_p),
                ("k2", ctypes.c_void_p), ("c1", ctypes.c_double), ("mode", ctypes.c_int),
                ("k3", ctypes.c_void_p), ("k4", ctypes.c_void_p)]


class BatchInstance(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_int64), ("n", ctypes.c_int64),
                ("cell_size", ctypes.c_double), ("lo", ctypes.c_double * 3),
                ("hi", ctypes.c_double * 3), ("uniform_h", ctypes.c_int),
                ("subdiv", ctypes.c_int)]


class BatchRecipe(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("subdiv", ctypes.c_int), ("scheme", ctypes.c_int),
                ("list_cap", ctypes.c_int), ("radius_scale", ctypes.c_double),
                ("dt", ctypes.c_double), ("density", DensityParams), ("term", SourceTerm),
                ("rates", RatesParams), ("margin", ctypes.c_double)]


SPH_EFLAG_JUMP = 1
SPH_EFLAG_BOX = 4


class NativeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


_lock = threading.Lock()
_lib = None


def library_path():
    return _build.LIB


def load_library(build_if_missing=True):
    """Load the shared library (building it if stale) without touching CUDA."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError("pysph_gb300 native library missing: %s "
                               "(run python -m pysph_gb300.build)" % path)
        L = ctypes.CDLL(path)
        vp, i32, i64, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
        P = ctypes.POINTER
        L.sph_ctx_create.argtypes = [i32, P(vp)]
        L.sph_ctx_destroy.argtypes = [vp]
        L.sph_ctx_set_stream.argtypes = [vp, vp]
        L.sph_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
        L.sph_version.argtypes = []
        L.sph_nnps_build.argtypes = [vp, P(ArrayView), i32, d, d, i32, i32]
        L.sph_nnps_count.argtypes = [vp, i32, i32, d, vp]
        L.sph_ctx_set_skin.argtypes = [vp, d]
        L.sph_ctx_set_symmetric.argtypes = [vp, i32]
        L.sph_ctx_set_periodic.argtypes = [vp, i32, d, d]
        L.sph_ctx_set_deferred.argtypes = [vp, i32]
        L.sph_ctx_set_bricks.argtypes = [vp, i32]
        L.sph_step_begin.argtypes = [vp]
        L.sph_step_end.argtypes = [vp, P(vp)]
        L.sph_step_run.argtypes = [vp, i32]
        L.sph_step_stats.argtypes = [vp, P(i64)]
        L.sph_step_destroy.argtypes = [vp]
        L.sph_pair_pass_stats.argtypes = [vp, P(i64)]
        L.sph_nnps_update.argtypes = [vp, P(ArrayView), i32, d, d, i32, i32, P(i32)]
        L.sph_nnps_stats.argtypes = [vp, P(i64)]
        L.sph_nnps_deferred_stats.argtypes = [vp, P(i64)]
        L.sph_nnps_fill.argtypes = [vp, i32, i32, d, vp, vp]
        L.sph_refresh_state.argtypes = [vp, i32, P(ArrayView)]
        L.sph_nbr_lists.argtypes = [vp, i32, P(i32), i32]
        L.sph_batch_create.argtypes = [P(vp)]
        L.sph_batch_destroy.argtypes = [vp]
        L.sph_batch_setup.argtypes = [vp, P(ArrayView), P(BatchInstance), i32, P(BatchRecipe)]
        L.sph_batch_step.argtypes = [vp, i32, i32]
        L.sph_batch_sync.argtypes = [vp]
        L.sph_batch_stream.argtypes = [vp, P(vp)]
        L.sph_batch_pair_counts.argtypes = [vp, P(ctypes.c_uint64)]
        L.sph_batch_error_word.argtypes = [vp, P(ctypes.c_uint32)]
        L.sph_batch_stats.argtypes = [vp, P(ctypes.c_int64)]
        L.sph_density.argtypes = [vp, i32, P(i32), i32, P(DensityParams), vp, vp, vp]
        L.sph_rates.argtypes = [vp, i32, P(SourceTerm), i32, P(RatesParams), P(vp), P(vp), i32]
        L.sph_tait.argtypes = [vp, i64, vp, vp, d, d, d, vp, vp]
        L.sph_adke_smoothing.argtypes = [vp, i64, i64, vp, vp, d, d, d, vp]
        L.sph_adke_conduction.argtypes = [vp, i64, vp, vp, vp, vp, d, d, vp]
        L.sph_const_rates.argtypes = [vp, i32, i64, vp, P(d), vp, vp, vp, i32, P(vp)]
        L.sph_integrate.argtypes = [vp, i64, P(AxpyLine), i32]
        L.sph_invariants.argtypes = [vp, P(ArrayView), P(d)]
        L.sph_error_word.argtypes = [vp, P(ctypes.c_uint32)]
        L.sph_mean_neighbours.argtypes = [vp, i32, i32, P(d)]
        L.sph_launch_count.argtypes = [P(i64)]
        L.sph_invariants_noalloc.argtypes = [P(ArrayView), P(d), vp]
        L.sph_selftest_conversions.argtypes = [i64, P(i64)]
        f32 = ctypes.c_float
        L.sph_mlp_features.argtypes = [vp, i32, i32, P(MlpFeatureParams), vp, vp]
        L.sph_mlp_sync.argtypes = [P(MlpModel), vp]
        L.sph_mlp_forward.argtypes = [P(MlpModel), vp, i64, vp, vp, vp, vp, vp, vp, vp]
        L.sph_mlp_backward_scratch.argtypes = [i64, P(i64)]
        L.sph_mlp_backward.argtypes = [P(MlpModel), vp, vp, vp, vp, vp, vp, vp, i64, f32, vp, vp,
                                       vp, vp, vp]
        L.sph_mlp_adam.argtypes = [P(MlpModel), vp, vp, vp, f32, f32, f32, f32, i32, vp]
        L.sph_mlp_apply.argtypes = [vp, i32, vp, d, P(d), P(d), P(vp), i32]
        L.sph_mlp_targets.argtypes = [i64, vp, vp, vp, d, P(d), P(d), vp, vp]
        for name in EXPORTS:
            getattr(L, name).restype = ctypes.c_int
        _lib = L
        return L


def lib():
    """The loaded library; raises unless a CUDA device is present."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("pysph_gb300 needs a CUDA device (GB300, sm_103a); "
                           "there is no CPU fallback")
    return load_library()


def last_error():
    buf = ctypes.create_string_buffer(2048)
    load_library(False).sph_last_error(buf, 2048)
    return buf.value.decode(errors="replace")


_EXC = {
    SPH_ERR_ARG: ValueError,
    SPH_ERR_JUMP: RuntimeError,
    SPH_ERR_NOTSUP: NotImplementedError,
}


def check(rc, what=""):
    if rc == SPH_OK:
        return
    msg = last_error()
    if what:
        msg = "%s: %s" % (what, msg)
    exc = _EXC.get(rc)
    if exc is not None:
        raise exc(msg)
    raise NativeError(rc, msg)


def launch_count():
    """Kernels launched by the library so far in this process."""
    out = ctypes.c_int64()
    check(load_library(False).sph_launch_count(ctypes.byref(out)), "launch count")
    return out.value


def ptr(t):
    """Device pointer of a torch tensor (None for None)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())
