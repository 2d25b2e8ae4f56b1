"""ctypes binding of libopyx.so (the C ABI declared in include/opyx.h).

This module replaces the reference's PyCUDA glue (opymize/tools/gpu.py:39-80):
instead of compiling kernels at run time from preprocessor constants, every
operator calls a precompiled sm_103a entry point with run-time shapes.  The
library is loaded from the package directory; if it is missing or cannot be
loaded, every GPU operation raises ``OpyxLibraryError`` -- there is no CPU
fallback.
"""

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libopyx.so")

OPYX_OK = 0
OPYX_ERR_ARG = 1
OPYX_ERR_LAUNCH = 2
OPYX_ERR_UNSUPPORTED = 3
OPYX_ERR_WORKSPACE = 4
OPYX_ERR_NOT_CONVERGED = 5
OPYX_ERR_SCRATCH_LIMIT = 6
OPYX_F32, OPYX_F64 = 0, 1
SCHEME = {"forward": 0, "centered": 1}
BC = {"neumann": 0, "curvature": 1, "second-order": 2}
NORM = {"frobenius": 0, "spectral": 1}
STEPS = {"const": 0, "adaptive": 1, "precond": 2}
MAX_DIMS = 6
ROF_MAX_C = 4


class OpyxLibraryError(RuntimeError):
    pass


class OpyxError(RuntimeError):
    def __init__(self, fn, status, msg):
        RuntimeError.__init__(self, "%s failed with status %d (%s)" % (fn, status, msg))
        self.status = status


class opyx_grid(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("nchannels", C.c_int32),
                ("dims", C.c_int64 * MAX_DIMS), ("h", C.c_double * MAX_DIMS)]


class opyx_step(C.Structure):
    _fields_ = [("vec", C.c_void_p), ("dev", C.c_void_p), ("value", C.c_double)]


class opyx_adaptive_state(C.Structure):
    _fields_ = [("tau", C.c_double), ("sigma", C.c_double), ("alpha", C.c_double),
                ("eta", C.c_double), ("Delta", C.c_double), ("theta", C.c_double),
                ("eps", C.c_double * 4), ("sums", C.c_double * 4),
                ("resp", C.c_double), ("resd", C.c_double), ("epsp", C.c_double),
                ("epsd", C.c_double), ("xsize", C.c_double), ("ysize", C.c_double)]


FCT = {name: i for i, name in enumerate(
    ["ssd", "l1norms", "l1norms_conj", "huber", "huber_conj", "quadepi_ind", "quadepi_supp",
     "huber_persp", "truncquad_ind", "positivity", "negativity", "affine", "indicator",
     "constrain", "masked_affine"])}


class opyx_fct(C.Structure):
    _fields_ = [("kind", C.c_int32), ("matrixnorm", C.c_int32), ("ngroups", C.c_int64),
                ("m1", C.c_int32), ("m2", C.c_int32), ("lbd", C.c_double),
                ("alpha", C.c_double), ("a", C.c_double), ("scalar0", C.c_double),
                ("scalar1", C.c_double), ("v0", C.c_void_p), ("v1", C.c_void_p),
                ("vol", C.c_void_p), ("mask", C.c_void_p)]


class opyx_epigraph(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("nsubpoints", C.c_int32), ("nfuns", C.c_int64),
                ("nregions", C.c_int64), ("npoints", C.c_int64), ("I", C.c_void_p),
                ("J", C.c_void_p), ("v", C.c_void_p), ("b", C.c_void_p),
                ("eq_off", C.c_void_p), ("eqns", C.c_void_p), ("checks", C.c_void_p),
                ("bt", C.c_void_p), ("It", C.c_void_p)]


class opyx_sublabel(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("L", C.c_int32), ("nsub", C.c_int32), ("pad", C.c_int32),
                ("H", C.c_int64), ("W", C.c_int64), ("xk", C.c_void_p), ("xkp1", C.c_void_p),
                ("xbar", C.c_void_p), ("yk", C.c_void_p), ("ykp1", C.c_void_p),
                ("t", C.c_double * 32), ("B", C.c_double * 124), ("tau_u", C.c_double * 32),
                ("tau_mu", C.c_double * 62), ("sig_q", C.c_double * 32),
                ("sig_z", C.c_double * 62), ("sig_e", C.c_double), ("sig_s", C.c_double),
                ("tau_g", C.c_void_p), ("sig_p", C.c_void_p), ("tau_g0", C.c_double),
                ("sig_p0", C.c_double), ("lbd", C.c_double), ("theta", C.c_double),
                ("v", C.c_void_p), ("bt", C.c_void_p), ("It", C.c_void_p), ("J", C.c_void_p),
                ("sorted", C.c_int32), ("perm", C.c_uint8 * (31 * 16)),
                ("vsorted", C.c_double * (31 * 16)), ("hull", C.c_void_p)]


class opyx_rof_problem(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("ndim", C.c_int32), ("nchannels", C.c_int32),
                ("steps", C.c_int32), ("dims", C.c_int64 * 3), ("h", C.c_double * 3),
                ("weights", C.c_double * ROF_MAX_C), ("vol", C.c_double * ROF_MAX_C),
                ("ssd_shift", C.c_double), ("lbd", C.c_double), ("huber_alpha", C.c_double),
                ("tau", C.c_double), ("sigma", C.c_double), ("theta", C.c_double),
                ("alpha0", C.c_double), ("eta", C.c_double), ("Delta", C.c_double),
                ("eps", C.c_double * 4), ("term_relgap", C.c_double),
                ("term_infeas", C.c_double), ("term_mode", C.c_int32),
                ("rows_per_thread", C.c_int32), ("flags", C.c_int32),
                ("reserved", C.c_int32)]


class opyx_rof_buffers(C.Structure):
    _fields_ = [("x", C.c_void_p), ("xbar", C.c_void_p), ("y", C.c_void_p),
                ("f", C.c_void_p), ("mask", C.c_void_p), ("xgrad", C.c_void_p),
                ("gp", C.c_void_p), ("ws", C.c_void_p), ("y2", C.c_void_p)]


class opyx_rof_info(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("objp", "objd", "infeasp", "infeasd", "gap", "relgap", "tau", "sigma",
                 "alpha", "resp", "resd", "epsp", "epsd", "checks", "done", "fault")]


ROF_INFO_FIELDS = [n for n, _ in opyx_rof_info._fields_]

OPYX_CONV_GELU, OPYX_CONV_F32, OPYX_CONV_BF16 = 0, 1, 2


class opyx_conv3x3_desc(C.Structure):
    _fields_ = [("batch", C.c_int32), ("height", C.c_int32), ("width", C.c_int32),
                ("in_channels", C.c_int32), ("in_stride", C.c_int32), ("in_offset", C.c_int32),
                ("out_channels", C.c_int32), ("out_stride", C.c_int32), ("out_offset", C.c_int32),
                ("epilogue", C.c_int32), ("accumulate", C.c_int32),
                ("x", C.c_void_p), ("w", C.c_void_p), ("bias", C.c_void_p),
                ("y", C.c_void_p), ("z", C.c_void_p)]


vp, i32, i64, f64, sz = C.c_void_p, C.c_int, C.c_int64, C.c_double, C.c_size_t
P = C.POINTER

# name -> (restype, argtypes); the order and types follow include/opyx.h
SIGNATURES = {
    "opyx_version": (i32, []),
    "opyx_status_string": (C.c_char_p, [i32]),
    "opyx_sm_count": (i32, []),
    "opyx_fill": (i32, [i32, vp, i64, f64, vp]),
    "opyx_axpby": (i32, [i32, i64, f64, vp, f64, vp, vp]),
    "opyx_abs": (i32, [i32, i64, vp, vp, vp]),
    "opyx_recip_positive": (i32, [i32, i64, vp, f64, vp]),
    "opyx_cast": (i32, [i32, i32, i64, vp, vp, vp]),
    "opyx_broadcast_mid": (i32, [i32, vp, i64, i64, i64, vp, i32, vp]),
    "opyx_reduce_workspace_size": (sz, []),
    "opyx_norms": (i32, [i32, i64, vp, vp, vp, vp]),
    "opyx_dot": (i32, [i32, i64, vp, vp, vp, vp, vp]),
    "opyx_l1normsproj_jac": (i32, [i32, i64, i32, f64, vp, vp, vp, vp]),
    "opyx_l12proj_jacobian": (i32, [i32, i64, i32, vp, vp, vp, vp, i32, vp]),
    "opyx_gradient": (i32, [P(opyx_grid), i32, vp, i32, vp, vp, i32, vp]),
    "opyx_divergence": (i32, [P(opyx_grid), i32, vp, i32, vp, vp, i32, vp]),
    "opyx_gradient_rowlp": (i32, [P(opyx_grid), i32, vp, i32, f64, i32, vp, i32, vp]),
    "opyx_laplacian": (i32, [P(opyx_grid), i32, i32, i32, vp, vp, i32, vp]),
    "opyx_laplacian_rowlp": (i32, [P(opyx_grid), i32, i32, f64, i32, vp, i32, vp]),
    "opyx_matrixmult": (i32, [i32, i64, i32, i32, vp, i32, vp, vp, i32, vp]),
    "opyx_matrixmultr": (i32, [i32, i64, i32, i32, vp, i32, vp, vp, i32, vp]),
    "opyx_matrixmultr_batched": (i32, [i32, i32, i64, i32, i32, vp, i32, vp, vp, i32, vp]),
    "opyx_tangled_matrixmultr": (i32, [i32, i32, i64, i32, i32, i32, vp, i32, vp, vp, i32, vp]),
    "opyx_diag_matrixmultr": (i32, [i32, i64, i32, vp, vp, vp, i32, vp]),
    "opyx_indexedmult": (i32, [i32, i32, i64, i32, i32, i32, vp, vp, vp, vp, i32, vp]),
    "opyx_indexedmult_adj": (i32, [i32, i32, i64, i32, i32, i32, vp, vp, vp, vp, i32, vp]),
    "opyx_shiftscale": (i32, [i32, i64, vp, f64, vp, f64, vp, f64, vp, vp, i32, vp]),
    "opyx_affine_prox": (i32, [i32, i64, vp, f64, vp, f64, opyx_step, vp, vp, vp]),
    "opyx_ssd_prox": (i32, [i32, i64, i32, vp, vp, vp, opyx_step, vp, vp, vp]),
    "opyx_posproj": (i32, [i32, i64, vp, vp, i32, vp]),
    "opyx_negproj": (i32, [i32, i64, vp, vp, i32, vp]),
    "opyx_constrain": (i32, [i32, i64, i32, vp, vp, vp, vp, i32, vp]),
    "opyx_l1normsproj": (i32, [i32, i64, i32, i32, f64, i32, vp, vp]),
    "opyx_huber_conj_prox": (i32, [i32, i64, i32, f64, f64, opyx_step, vp, vp]),
    "opyx_quadepiproj": (i32, [i32, i64, i32, f64, vp, f64, vp, vp]),
    "opyx_take_step": (i32, [i32, i64, vp, vp, i32, opyx_step, vp, vp]),
    "opyx_dual_step": (i32, [i32, i64, vp, vp, opyx_step, f64, vp, vp, vp]),
    "opyx_residual_pair": (i32, [i32, i64, opyx_step, vp, vp, f64, vp, f64, f64, vp,
                                 vp, vp, vp]),
    "opyx_adaptive_update": (i32, [vp, vp]),
    "opyx_fct_eval": (i32, [P(opyx_fct), i32, vp, vp, vp, vp]),
    "opyx_epigraph_proj": (i32, [P(opyx_epigraph), i32, vp, vp, i32, f64, vp, vp]),
    "opyx_epigraph_eval": (i32, [P(opyx_epigraph), i32, i32, vp, vp, vp, vp]),
    "opyx_convexify_max_faces": (i32, [i32, i32]),
    "opyx_convexify": (i32, [i32, i64, vp, i64, vp, i64, i32, vp, vp, vp, vp, i32, i32]),
    "opyx_rof_workspace_size": (sz, []),
    "opyx_rof_info_offset": (sz, []),
    "opyx_rof_init": (i32, [P(opyx_rof_problem), P(opyx_rof_buffers), vp]),
    "opyx_rof_iterate": (i32, [P(opyx_rof_problem), P(opyx_rof_buffers), i32, vp]),
    "opyx_rof_gap": (i32, [P(opyx_rof_problem), P(opyx_rof_buffers), vp]),
    "opyx_rof_gap_iterate": (i32, [P(opyx_rof_problem), P(opyx_rof_buffers), i32, vp]),
    "opyx_rof_pass": (i32, [P(opyx_rof_problem), P(opyx_rof_buffers), i32, vp]),
    "opyx_rof_uses_sweep": (i32, [P(opyx_rof_problem), P(opyx_rof_buffers)]),
    "opyx_rof_iterate_noalloc": (i32, [P(opyx_rof_problem), vp, vp, vp, vp, i32, vp, vp]),
    "opyx_rof_batch_record_bytes": (sz, []),
    "opyx_rof_batch_desc_bytes": (sz, [i32, i32]),
    "opyx_rof_batch_describe": (i32, [P(opyx_rof_problem), P(opyx_rof_buffers), i32, vp, vp, i32,
                                      vp, sz, P(C.c_int)]),
    "opyx_rof_batch_init": (i32, [vp, vp, vp]),
    "opyx_rof_batch_iterate": (i32, [vp, vp, i32, vp]),
    "opyx_rof_batch_iterate_class": (i32, [vp, vp, i32, i32, vp]),
    "opyx_rof_batch_gap": (i32, [vp, vp, vp, vp]),
    "opyx_rof_batch_persist_ws_bytes": (sz, [vp]),
    "opyx_rof_batch_persist": (i32, [vp, vp, vp, i32, i32, vp]),
    "opyx_sublabel_pass": (i32, [P(opyx_sublabel), i32, vp]),
    "opyx_conv3x3": (i32, [P(opyx_conv3x3_desc), vp]),
    "opyx_conv3x3_wgrad_workspace": (sz, [P(opyx_conv3x3_desc)]),
    "opyx_conv3x3_wgrad": (i32, [P(opyx_conv3x3_desc), vp, vp, i32, vp, sz, vp]),
    "opyx_net_fault": (i32, [P(C.c_uint)]),
    "opyx_gelu_bwd_workspace": (sz, [i64, i32]),
    "opyx_gelu_bwd": (i32, [i64, i32, vp, i32, i32, vp, vp, vp, i32, vp, sz, vp]),
    "opyx_pool2": (i32, [i32, i32, i32, i32, vp, i32, i32, vp, vp]),
    "opyx_pool2_bwd": (i32, [i32, i32, i32, i32, vp, vp, i32, i32, i32, vp]),
    "opyx_up2": (i32, [i32, i32, i32, i32, vp, vp, i32, i32, vp]),
    "opyx_up2_bwd": (i32, [i32, i32, i32, i32, vp, i32, i32, vp, vp]),
    "opyx_pack_input": (i32, [i32, i64, vp, vp, f64, vp, vp]),
    "opyx_pack_input_state": (i32, [i32, i64, vp, vp, f64, vp, vp, vp, vp]),
    "opyx_warm_unpack_rel": (i32, [i32, i64, vp, vp, vp, vp, vp, vp, vp]),
    "opyx_head": (i32, [i64, i32, vp, vp, vp, vp, vp]),
    "opyx_head_bwd_workspace": (sz, [i64, i32]),
    "opyx_head_bwd": (i32, [i64, i32, vp, vp, vp, vp, vp, vp, vp, sz, vp]),
    "opyx_mse": (i32, [i64, i32, vp, vp, vp, vp, vp, i32, vp]),
    "opyx_warm_loss": (i32, [i32, i32, i32, vp, vp, vp, f64, f64, f64, f64, vp, vp, vp, i32, vp]),
    "opyx_warm_unpack": (i32, [i32, i64, vp, vp, vp, vp, vp, vp]),
    "opyx_adam": (i32, [i64, vp, vp, vp, vp, f64, f64, f64, f64, i32, vp, vp, i32, i32, vp]),
    "opyx_conv_weights": (i32, [i32, i32, vp, vp, vp, vp]),
}

_lib = None


def load(path=LIB_PATH):
    """Load libopyx.so and bind every exported entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OpyxLibraryError(
            "libopyx.so not found at %s: build it first "
            "(python -m opymize_gb300.build); there is no CPU fallback" % path)
    try:
        lib = C.CDLL(path)
    except OSError as e:
        raise OpyxLibraryError("cannot load %s: %s" % (path, e))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(status):
    return load().opyx_status_string(status).decode()


def call(name, *args):
    """Call an int-status entry point and raise OpyxError unless it is OK."""
    fn = getattr(load(), name)
    st = fn(*args)
    if st != OPYX_OK:
        raise OpyxError(name, st, status_string(st))
    return st
