"""ctypes binding of ``libbssn_gb300.so`` (C ABI in ``include/bssn_gb300.h``).

The structs below mirror the header field for field.  Every call returns an
int status; non-zero raises ``ValueError`` for validation failures (the
reference raises ValueError from its host-side validators) and
``RuntimeError`` otherwise, carrying ``bssn_last_error()``.

There is no fallback: importing this module on a machine without the built
library, or calling into it without a CUDA device, fails loudly.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

from .build import LIBRARY

c_double_p = ctypes.POINTER(ctypes.c_double)

BSSN_OK = 0
BSSN_ERR_INVALID = 1
BSSN_ERR_WORKSPACE = 2
BSSN_ERR_CUDA = 3
BSSN_ERR_NONFINITE = 4
BSSN_ERR_NOT_CONVERGED = 6

PRECISION_F64 = 0
PRECISION_F32 = 1
PRECISION_F32_PAIRED = 2

OP_RHS = 1
OP_RK4 = 2
OP_CONSTRAINTS = 3
OP_RHS_MATTER = 4


class BssnParams(ctypes.Structure):
    _fields_ = [
        ("eta", ctypes.c_double), ("kappa", ctypes.c_double), ("nu", ctypes.c_double),
        ("g", ctypes.c_double), ("dx", ctypes.c_double), ("dt", ctypes.c_double),
        ("zero_shift", ctypes.c_int32), ("gauge", ctypes.c_int32),
        ("bc", ctypes.c_int32 * 6),
        ("xmin", ctypes.c_double * 3),
        ("mad_q", ctypes.c_double),
        ("guard_cells", ctypes.c_int32),
        ("owned_shape", ctypes.c_int32 * 3),
        ("owned_faces", ctypes.c_int32 * 6),
        ("reduced_axes", ctypes.c_int32 * 3),
        ("precision", ctypes.c_int32),
    ]


class BssnBox(ctypes.Structure):
    _fields_ = [("src", ctypes.c_void_p), ("shape", ctypes.c_int32 * 3), ("lo", ctypes.c_int32 * 3),
                ("extent", ctypes.c_int32 * 3)]


MAX_GATHER_BOXES = 32


class BssnFields(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in (
        "conformal_metric", "conformal_factor", "traceless_K", "trace_K",
        "conformal_connection", "lapse", "shift")]


class BssnMatter(ctypes.Structure):
    _fields_ = [("energy_density", ctypes.c_void_p), ("momentum_density", ctypes.c_void_p),
                ("spatial_stress", ctypes.c_void_p)]


class BssnFmrPatch(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32 * 3), ("parent", ctypes.c_int32),
                ("coarse_lo", ctypes.c_int32 * 3), ("coarse_hi", ctypes.c_int32 * 3)]


class BssnPatch(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32 * 3), ("ghost", ctypes.c_int32)]


Shape3 = ctypes.c_int32 * 3

class BssnHorizonGeometry(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_void_p), ("curvature", ctypes.c_void_p), ("dims", ctypes.c_int32),
                ("size", ctypes.c_int32 * 3), ("origin", ctypes.c_double * 3), ("spacing", ctypes.c_double * 3),
                ("margin", ctypes.c_int32)]


# name -> (restype, argtypes)
SIGNATURES = {
    "bssn_last_error": (ctypes.c_char_p, []),
    "bssn_abi_version": (ctypes.c_int, []),
    "bssn_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int, Shape3, ctypes.POINTER(BssnParams)]),
    "bssn_rhs": (ctypes.c_int, [ctypes.POINTER(BssnFields), ctypes.POINTER(BssnFields), Shape3,
                                ctypes.POINTER(BssnParams), ctypes.POINTER(BssnMatter),
                                ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_rhs_noalloc": (ctypes.c_int, [ctypes.POINTER(BssnFields), ctypes.POINTER(BssnFields), Shape3,
                                        ctypes.POINTER(BssnParams), ctypes.c_void_p]),
    "bssn_project": (ctypes.c_int, [ctypes.POINTER(BssnFields), Shape3, ctypes.c_void_p]),
    "bssn_rk4_step": (ctypes.c_int, [ctypes.POINTER(BssnFields), Shape3, ctypes.POINTER(BssnParams),
                                     ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_constraints": (ctypes.c_int, [ctypes.POINTER(BssnFields), Shape3, ctypes.POINTER(BssnParams),
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_patch_values": (ctypes.c_size_t, [ctypes.POINTER(BssnPatch)]),
    "bssn_patch_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(BssnPatch), ctypes.POINTER(BssnParams)]),
    "bssn_patch_import": (ctypes.c_int, [ctypes.POINTER(BssnFields), ctypes.c_void_p,
                                         ctypes.POINTER(BssnPatch), ctypes.c_void_p]),
    "bssn_patch_export": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnFields),
                                         ctypes.POINTER(BssnPatch), ctypes.c_void_p]),
    "bssn_patch_fill_periodic": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnPatch), ctypes.c_void_p]),
    "bssn_patch_rk4": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnPatch), ctypes.POINTER(BssnParams),
                                      ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_patch_check_finite": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnPatch),
                                               ctypes.c_void_p, ctypes.c_void_p]),
    "bssn_batch_values": (ctypes.c_size_t, [ctypes.POINTER(BssnPatch), ctypes.c_int32]),
    "bssn_batch_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(BssnPatch), ctypes.c_int32,
                                                      ctypes.POINTER(BssnParams)]),
    "bssn_batch_import": (ctypes.c_int, [ctypes.POINTER(BssnFields), ctypes.c_void_p, ctypes.POINTER(BssnPatch),
                                         ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "bssn_batch_export": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnFields), ctypes.POINTER(BssnPatch),
                                         ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "bssn_batch_fill_periodic": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnPatch), ctypes.c_int32,
                                                ctypes.c_void_p]),
    "bssn_batch_rk4": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnPatch), ctypes.c_int32,
                                      ctypes.POINTER(BssnParams), ctypes.c_int32, ctypes.c_void_p,
                                      ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_batch_check_finite": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnPatch), ctypes.c_int32,
                                               ctypes.c_void_p, ctypes.c_void_p]),
    "bssn_rhs_vjp_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(BssnPatch), ctypes.c_int32]),
    "bssn_rhs_vjp": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(BssnPatch),
                                    ctypes.c_int32, ctypes.POINTER(BssnParams), ctypes.c_void_p, ctypes.c_size_t,
                                    ctypes.c_void_p]),
    "bssn_adjoint_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(BssnPatch), ctypes.c_int32,
                                                        ctypes.POINTER(BssnParams), ctypes.c_int32, ctypes.c_int32,
                                                        ctypes.c_int32]),
    "bssn_adjoint_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnPatch), ctypes.c_int32,
                                            ctypes.POINTER(BssnParams), ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_adjoint_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnPatch), ctypes.c_int32,
                                             ctypes.POINTER(BssnParams), ctypes.c_int32, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_batch_rk4_monitored": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnPatch), ctypes.c_int32,
                                                ctypes.POINTER(BssnParams), ctypes.c_int32, ctypes.c_int32,
                                                ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p,
                                                ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_set_tma": (ctypes.c_int, [ctypes.c_int32]),
    "bssn_tma_status": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64)]),
    "bssn_tune_patch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnPatch), ctypes.c_int32,
                                       ctypes.POINTER(BssnParams), ctypes.c_float, ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_fields_to_components": (ctypes.c_int, [ctypes.POINTER(BssnFields), ctypes.c_void_p, Shape3,
                                                 ctypes.c_void_p]),
    "bssn_components_to_fields": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BssnFields), Shape3,
                                                 ctypes.c_void_p]),
    "bssn_fmr_workspace_bytes": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "bssn_fmr_refresh": (ctypes.c_int, [ctypes.c_void_p, Shape3, ctypes.c_void_p, ctypes.c_void_p]),
    "bssn_fmr_prolong": (ctypes.c_int, [ctypes.c_void_p, Shape3, ctypes.c_void_p, Shape3, Shape3,
                                        ctypes.c_void_p]),
    "bssn_fmr_inject": (ctypes.c_int, [ctypes.c_void_p, Shape3, ctypes.c_void_p, Shape3, Shape3,
                                       ctypes.c_void_p]),
    "bssn_fmr_prepare": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_void_p]),
    "bssn_fmr_stage_rhs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_fmr_rk4_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                         ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_fmr_constraint_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_cartoon_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int32, Shape3, ctypes.POINTER(BssnParams)]),
    "bssn_cartoon_fill_ghosts": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, Shape3, ctypes.c_void_p]),
    "bssn_cartoon_reconstruct": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, Shape3,
                                                ctypes.POINTER(BssnParams), ctypes.c_void_p]),
    "bssn_cartoon_rhs": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, Shape3,
                                        ctypes.POINTER(BssnParams), ctypes.c_void_p, ctypes.c_size_t,
                                        ctypes.c_void_p]),
    "bssn_cartoon_rk4_step": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, Shape3, ctypes.POINTER(BssnParams),
                                             ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_cartoon_constraints": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, Shape3,
                                                ctypes.POINTER(BssnParams), ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_probe_fma_peak": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]),
    "bssn_check_div6": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                       ctypes.c_void_p]),
    "bssn_h_plus": (ctypes.c_int, [ctypes.POINTER(BssnFields), Shape3, ctypes.c_void_p, ctypes.c_void_p]),
    "bssn_wave_norm_workspace_bytes": (ctypes.c_size_t, []),
    "bssn_wave_norm_sums": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           Shape3, ctypes.c_void_p, ctypes.c_int32, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_puncture_fields": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, c_double_p, c_double_p, c_double_p,
                                            ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p]),
    "bssn_puncture_operator": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              Shape3, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_puncture_workspace_bytes": (ctypes.c_size_t, [Shape3, ctypes.c_int32]),
    "bssn_puncture_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, Shape3, ctypes.c_double, ctypes.c_int32,
                                           ctypes.c_double, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                                           ctypes.c_void_p, ctypes.c_void_p, c_double_p,
                                           ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                           ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_horizon_sample": (ctypes.c_int, [ctypes.POINTER(BssnHorizonGeometry), ctypes.c_void_p, ctypes.c_int64,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "bssn_horizon_angular_derivatives": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                                        ctypes.c_void_p, ctypes.c_void_p]),
    "bssn_horizon_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int32, ctypes.c_int32]),
    "bssn_horizon_surface": (ctypes.c_int, [ctypes.POINTER(BssnHorizonGeometry), c_double_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_horizon_jacobian": (ctypes.c_int, [ctypes.POINTER(BssnHorizonGeometry), c_double_p, ctypes.c_void_p,
                                             ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "bssn_horizon_newton_direction": (ctypes.c_int, [ctypes.POINTER(BssnHorizonGeometry), c_double_p,
                                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                                     ctypes.c_int32, ctypes.c_double, ctypes.c_void_p,
                                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                     ctypes.c_void_p]),
    "bssn_horizon_regrid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "bssn_gather_boxes": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "bssn_launch_count": (ctypes.c_longlong, []),
    "bssn_profile_enable": (None, [ctypes.c_int]),
    "bssn_profile_reset": (None, []),
    "bssn_profile_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
}

KERNEL_CLASSES = ("fill", "first_derivs", "rhs_gauge", "rhs_kgt", "rhs_at", "mom_derived", "mom_damping",
                  "sommerfeld", "rk4_stage", "project", "import", "export", "constraints", "fmr_transfer",
                  "cartoon", "convert", "other", "rhs_curv", "solve_newton", "solve_apply", "solve_update", "horizon_surface",
                  "horizon_solve", "adjoint_point", "adjoint_stencil", "adjoint_stage")


def profile_read() -> dict:
    """{class: (milliseconds, launches)} accumulated since bssn_profile_reset."""
    lib = load()
    n = len(KERNEL_CLASSES)
    ms = (ctypes.c_double * n)()
    counts = (ctypes.c_longlong * n)()
    lib.bssn_profile_read(ctypes.cast(ms, ctypes.c_void_p), ctypes.cast(counts, ctypes.c_void_p), n)
    return {name: (ms[i], counts[i]) for i, name in enumerate(KERNEL_CLASSES) if counts[i]}

_lib = None


def library_path() -> Path:
    return LIBRARY


def load(path: Path | None = None):
    """Load the CUDA library once; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = Path(path or LIBRARY)
    if not path.exists():
        raise RuntimeError(
            f"{path} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(str(path))
    for name, (restype, argtypes) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    if path == LIBRARY:
        _lib = lib
    return lib


def last_error() -> str:
    return load().bssn_last_error().decode(errors="replace")


def check(status: int, what: str) -> None:
    if status == BSSN_OK:
        return
    message = f"{what}: {last_error()}"
    if status in (BSSN_ERR_INVALID, BSSN_ERR_WORKSPACE):
        raise ValueError(message)
    raise RuntimeError(message)


def fma_peak_gflops(precision: int) -> float:
    """Measured FMA throughput (GFLOP/s) of the current GPU, FP64 or FP32."""
    lib = load()
    out = ctypes.c_double(0.0)
    check(lib.bssn_probe_fma_peak(int(precision), ctypes.byref(out)), "bssn_probe_fma_peak")
    return out.value


def tune_launch_shapes(state_ptr: int, shape, instances: int, cparams: BssnParams, device,
                       workspace=None, margin: float = 0.98) -> str:
    """Autotune the RHS launch shapes of a padded (ghost 4) batch state in
    place (bssn_tune_patch): a slot takes the fastest candidate block size when
    it times below ``margin`` x the current shapes; returns the report."""
    import torch
    from . import _device
    lib = load()
    patch = BssnPatch()
    for d in range(3):
        patch.n[d] = int(shape[d])
    patch.ghost = 4
    nbytes = lib.bssn_batch_workspace_bytes(patch, int(instances), cparams)
    if workspace is None or workspace.numel() < nbytes:
        workspace = torch.empty(nbytes, dtype=torch.uint8, device=device)
    report = ctypes.create_string_buffer(4096)
    check(lib.bssn_tune_patch(state_ptr, patch, int(instances), cparams, float(margin), workspace.data_ptr(),
                              workspace.numel(),
                              report, 4096, _device.stream_handle()), "bssn_tune_patch")
    return report.value.decode()


TMA_GAUGE, TMA_DERIVS, TMA_AT, TMA_KGT, TMA_ALL = 1, 2, 4, 8, 15
TMA_DEFAULT = TMA_ALL


def set_tma(kernels) -> None:
    """The float forms' TMA-staged kernels to use (bssn_set_tma): a mask of
    TMA_GAUGE, TMA_DERIVS, TMA_AT and TMA_KGT; True is the library's default
    (TMA_DEFAULT) and False the generic kernels everywhere."""
    mask = TMA_DEFAULT if kernels is True else (0 if kernels is False else int(kernels))
    check(load().bssn_set_tma(mask), "bssn_set_tma")


def tma_status() -> tuple:
    """(TMA tile waits that gave up since the last call, TMA launches so far)
    (bssn_tma_status)."""
    timeouts, launches = ctypes.c_int32(0), ctypes.c_int64(0)
    check(load().bssn_tma_status(ctypes.byref(timeouts), ctypes.byref(launches)), "bssn_tma_status")
    return timeouts.value, launches.value
