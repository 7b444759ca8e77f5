"""ctypes binding of libdpfehm_gpu.so (the C ABI declared in include/dpfehm_gpu.h).

The shared library must have been built (``build.build()``); loading fails
loudly otherwise -- there is no CPU implementation behind this package.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdpfehm_gpu.so")

DPF_OK, DPF_BAD_INPUT, DPF_NOT_CONVERGED, DPF_NAN, DPF_OOM, DPF_CUDA, DPF_NO_DEVICE, DPF_STATE, DPF_UNSUPPORTED, DPF_TIMEOUT = range(10)
STATUS_NAMES = {
    0: "DPF_OK", 1: "DPF_BAD_INPUT", 2: "DPF_NOT_CONVERGED", 3: "DPF_NAN", 4: "DPF_OOM", 5: "DPF_CUDA",
    6: "DPF_NO_DEVICE", 7: "DPF_STATE", 8: "DPF_UNSUPPORTED", 9: "DPF_TIMEOUT",
}
MEAN_GEOMETRIC, MEAN_HARMONIC = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
SOLVER_CG, SOLVER_CHOLESKY = 0, 1


class Options(ctypes.Structure):
    _fields_ = [
        ("reltol", ctypes.c_double),
        ("maxiter", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("cheb_degree", ctypes.c_int),
        ("cheb_lo", ctypes.c_double),
        ("coarse_scale", ctypes.c_double),
        ("max_coarse", ctypes.c_int),
        ("max_outer", ctypes.c_int),
        ("use_graphs", ctypes.c_int),
        ("check_every", ctypes.c_int),
        ("blocks_per_sm", ctypes.c_int),
        ("tail_cells", ctypes.c_int),
        ("plane", ctypes.c_int),
        ("plane_cells", ctypes.c_int),
        ("plane_blocks_per_sm", ctypes.c_int),
        ("df_plane_cells", ctypes.c_int),
        ("df_plane_blocks_per_sm", ctypes.c_int),
        ("tail_cluster", ctypes.c_int),
        ("plane_levels", ctypes.c_int),
        ("streams", ctypes.c_int),
        ("fuse", ctypes.c_int),
        ("solver", ctypes.c_int),
    ]


_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes); pointer arguments are passed as c_void_p so that
# host (numpy) and device (torch CUDA) buffers go through the same binding.
SIGNATURES = {
    "dpf_default_options": (None, [ctypes.POINTER(Options)]),
    "dpf_create": (ctypes.c_int, [_i64, _i64, _vp, _vp, _vp, _vp, _i64, _vp, ctypes.POINTER(Options),
                                  ctypes.POINTER(_vp)]),
    "dpf_create_regular3d": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, _i64, _vp,
                                            ctypes.POINTER(Options), ctypes.POINTER(_vp)]),
    "dpf_detect_regular3d": (ctypes.c_int, [_i64, _i64, _vp, _vp, _vp, _vp, _vp]),
    "dpf_destroy": (None, [_vp]),
    "dpf_last_error": (ctypes.c_char_p, [_vp]),
    "dpf_info": (ctypes.c_int, [_vp, _i64p, _i64p, _i64p, _ip, _ip]),
    "dpf_last_stats": (ctypes.c_int, [_vp, _ip, _ip, _f64p]),
    "dpf_steady_forward": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "dpf_steady_adjoint": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "dpf_logk_to_faces": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp]),
    "dpf_logk_to_faces_vjp": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, _vp]),
    "dpf_steady_forward_logk": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, _vp, _vp]),
    "dpf_steady_adjoint_logk": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "dpf_transient_forward": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_double, ctypes.c_int, _vp,
                                             ctypes.c_int, _vp, _vp]),
    "dpf_transient_adjoint": (ctypes.c_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "dpf_batch_autotune": (ctypes.c_int, [ctypes.c_int, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(Options), _vp,
                                           ctypes.c_int, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.POINTER(Options),
                                           ctypes.POINTER(ctypes.c_double)]),
    "dpf_batch_create": (ctypes.c_int, [ctypes.c_int, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(Options),
                                        ctypes.POINTER(_vp)]),
    "dpf_batch_offsets": (ctypes.c_int, [_vp, ctypes.c_int, _i64p, _i64p]),
    "dpf_batch_solve_grad_logk": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "dpf_batch_sample_logk": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp]),
    "dpf_solve_grad_logk": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, _vp, _i64, _vp, _vp, _vp]),
    "dpf_apply_operator": (ctypes.c_int, [_vp, _vp, _vp]),
    "dpf_profile": (ctypes.c_int, [_vp, ctypes.c_int]),
    "dpf_profile_report": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                          ctypes.POINTER(ctypes.c_longlong), _f64p,
                                          ctypes.POINTER(ctypes.c_longlong)]),
    "dpf_launch_count": (ctypes.c_longlong, [_vp]),
    "dpf_set_stream": (ctypes.c_int, [_vp, _vp]),
    "dpf_create_general": (ctypes.c_int, [_i64, _i64, _vp, _vp, _vp, _vp, _i64, _vp, ctypes.POINTER(Options),
                                          ctypes.POINTER(_vp)]),
    "dpf_richards_steady": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_double, ctypes.c_int,
                                           _vp]),
    "dpf_richards_adjoint": (ctypes.c_int, [_vp, _vp, ctypes.c_double, ctypes.c_int, _vp, _vp, _vp, _vp, _vp]),
    "dpf_richards_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), _f64p]),
    "dpf_richards_transient_forward": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_double,
                                                      ctypes.c_int, ctypes.c_double, ctypes.c_int, _vp, _vp]),
    "dpf_richards_transient_adjoint": (ctypes.c_int, [_vp, _i64, _vp, _vp, _vp, ctypes.c_double, ctypes.c_int, _vp,
                                                      _vp, _vp, _vp, _vp, _vp]),
    "dpf_logk_to_faces_regular_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_int,
                                                         _vp]),
    "dpf_debug_fail_alloc": (None, [ctypes.c_int64]),
    "dpf_debug_alloc_stats": (None, [ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "dpf_debug_expired_wait": (ctypes.c_int, [_f64p]),
    "dpf_debug_split48": (ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "dpf_debug_band_order_graph": (ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p]),
    "dpf_debug_band_order_grids": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "dpf_debug_check_report": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
}

_lib = None


def load(path=None):
    """Load the library (once). Raises OSError if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("DPFEHM_GPU_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise OSError("libdpfehm_gpu.so not found at %s: build it first (dpfehm.jl_gb300/build.py or "
                      "__graft_entry__.build()); there is no CPU fallback" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def default_options(**kw):
    o = Options()
    load().dpf_default_options(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError("unknown option %r" % k)
        setattr(o, k, v)
    return o
