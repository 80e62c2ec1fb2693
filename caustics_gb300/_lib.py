"""ctypes binding of libcaustics_gb300.so (the C ABI in include/caustics_gb300.h).

The library is built in-tree (``caustics_gb300.build``).  There is no CPU or
pure-PyTorch fallback: if the library is missing or no CUDA device is present
every compute call raises.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcaustics_gb300.so")

CGB_OK = 0
CGB_ERR_INVALID = 1
CGB_ERR_CUDA = 2
CGB_ERR_UNSUPPORTED = 3

PREC_FP64 = 0
PREC_MIXED = 1
PREC_FP64_COMP = 2

ST_NOCONV = 1
ST_AMBIGUOUS = 2
ST_FALLBACK = 4
ST_MERGE = 8
ST_CAPACITY = 16
ST_INVALID = 32


class LensParams(ctypes.Structure):
    _fields_ = [("nlenses", ctypes.c_int32), ("s", ctypes.c_double), ("q", ctypes.c_double),
                ("q3", ctypes.c_double), ("r3", ctypes.c_double), ("psi", ctypes.c_double)]


class EsOptions(ctypes.Structure):
    _fields_ = [("npts_limb", ctypes.c_int32), ("limb_darkening", ctypes.c_int32), ("u1", ctypes.c_double),
                ("npts_ld", ctypes.c_int32), ("roots_itmax", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("grid", ctypes.c_int32), ("queue_chunk", ctypes.c_int32), ("ld_group", ctypes.c_int32),
                ("labelling", ctypes.c_int32), ("grad_fp64_above", ctypes.c_double),
                ("triple_routing", ctypes.c_int32), ("cta_threads", ctypes.c_int32),
                ("point_lanes", ctypes.c_int32)]


class CurveParams(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("s", "q", "rho", "u1", "u0", "alpha", "t0", "tE")]


# name -> (restype, argtypes); every symbol the public header declares
_P = ctypes.c_void_p
SIGNATURES = {
    "cgb_last_error": (ctypes.c_char_p, []),
    "cgb_abi_version": (ctypes.c_int32, []),
    "cgb_gauss_legendre": (ctypes.c_int, [ctypes.c_int32, _P, _P]),
    "cgb_ea_solve": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P, _P]),
    "gpu_ehrlich_aberth": (None, [_P, _P, ctypes.c_char_p, ctypes.c_size_t]),
    "cgb_lens_polynomial": (ctypes.c_int, [_P, _P, ctypes.c_int64, LensParams, _P]),
    "cgb_parallax_trajectory": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_int64, _P, ctypes.c_int64, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _P,
                                               _P, _P]),
    "cgb_marginalized_log_likelihood": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int64, _P, _P, _P, _P, _P, _P,
                                                       _P, _P]),
    "cgb_critical_curves_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int32, ctypes.c_int32]),
    "cgb_critical_and_caustic_curves": (ctypes.c_int, [ctypes.c_int32, LensParams, ctypes.c_int32, _P, _P, _P, _P,
                                                       ctypes.c_size_t, _P]),
    "cgb_ea_roots_jvp": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int64, ctypes.c_int32, _P]),
    "cgb_ea_roots_vjp": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, _P]),
    "cgb_mag_point_source": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int64, LensParams, ctypes.c_int32,
                                            ctypes.c_int32, _P, _P]),
    "cgb_mag_extended_source": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.c_double, LensParams,
                                               ctypes.POINTER(EsOptions), _P, _P]),
    "cgb_mag": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_double, LensParams, ctypes.POINTER(EsOptions),
                               _P, _P]),
    "cgb_mag_extended_source_grad": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_double, LensParams,
                                                    ctypes.POINTER(EsOptions), _P, _P]),
    "cgb_mag_extended_source_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int64]),
    "cgb_mag_extended_source_ws": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.c_double, LensParams,
                                                  ctypes.POINTER(EsOptions), _P, _P, ctypes.c_size_t, _P]),
    "cgb_mag_extended_source_grad_ws": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_double, LensParams,
                                                       ctypes.POINTER(EsOptions), _P, _P, ctypes.c_size_t, _P]),
    "cgb_mag_ws": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_double, LensParams, ctypes.POINTER(EsOptions),
                                  _P, _P, ctypes.c_size_t, _P]),
    "cgb_debug_extended_source": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.c_double, LensParams,
                                                 ctypes.POINTER(EsOptions), _P, _P, _P]),
    "cgb_debug_record_len": (ctypes.c_int64, [ctypes.c_int32]),
    "cgb_mag_lc_batched_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int64]),
    "cgb_mag_lc_batched_vjp_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int64]),
    "cgb_mag_lc_batched_noalloc": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int64, _P, _P, _P,
                                                  ctypes.POINTER(EsOptions), _P]),
    "cgb_mag_lc_batched": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int64, _P, _P, _P,
                                          ctypes.POINTER(EsOptions), _P, ctypes.c_size_t, _P]),
    "cgb_mag_lc_batched_vjp": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int64, _P, _P, _P, _P, _P,
                                              ctypes.POINTER(EsOptions), _P, ctypes.c_size_t, _P]),
    "cgb_mag_lc_batched_triple": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int64, _P, _P, _P,
                                                 ctypes.POINTER(EsOptions), _P, ctypes.c_size_t, _P]),
    "cgb_mag_lc_batched_triple_vjp": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int64, _P, _P, _P, _P, _P,
                                                     ctypes.POINTER(EsOptions), _P, ctypes.c_size_t, _P]),
    "cgb_mag_lc_batched_triple_vjp_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int64]),
}

_lock = threading.Lock()
_lib = None


class CausticsError(RuntimeError):
    pass


def lib():
    """The loaded library; raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise CausticsError(
                    f"{LIB_PATH} is missing: build it with `python -m caustics_gb300.build` "
                    "(the magnification kernels have no CPU fallback)")
            h = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(h, name)
                f.restype = res
                f.argtypes = args
            _lib = h
    return _lib


def check(rc, what):
    if rc != CGB_OK:
        msg = lib().cgb_last_error().decode(errors="replace")
        raise CausticsError(f"{what} failed ({rc}): {msg}")


def lens_params(nlenses, params):
    if nlenses == 2:
        return LensParams(2, float(params["s"]), float(params["q"]), 0.0, 0.0, 0.0)
    if nlenses == 3:
        return LensParams(3, float(params["s"]), float(params["q"]), float(params["q3"]), float(params["r3"]),
                          float(params["psi"]))
    raise ValueError("`nlenses` has to be 2 or 3.")
