"""ctypes binding of libptyg.so (the C ABI in include/ptyg.h).

Only plain pointers and sizes cross the boundary.  Statuses map to the
exceptions PtyLab raises on the same conditions: invalid switches ->
ValueError (PtyLab/Engines/BaseEngine.py:376-403), unsupported branches ->
NotImplementedError, no usable GPU -> ImportError (BaseEngine.py:617-621).
There is no fallback: if the library is missing or no sm_103a device is
present, every entry point raises.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libptyg.so"

PTYG_OK = 0
PTYG_ERR_INVALID = -1
PTYG_ERR_UNSUPPORTED = -2
PTYG_ERR_OOM = -3
PTYG_ERR_CUDA = -4
PTYG_ERR_TIMEOUT = -5
PTYG_ERR_DEVICE = -6

ENGINES = {"ePIE": 0, "mPIE": 1, "qNewton": 2, "e3PIE": 3, "mqNewton": 4}
MOMENTUM_METHODS = {"momentum": 0, "ADAM": 1, "NADAM": 2}
INTENSITY_CONSTRAINTS = {"standard": 0, "poission": 1, "exponential": 2, "fluctuation": 3, "interferometric": 4}
# the engines' propagators: polychromeASP is the ASP kernel with one table per wavelength
PROPAGATORS = {"fraunhofer": 0, "fresnel": 1, "asp": 2, "polychromeasp": 2}
# ptyg_propagate_sets (include/ptyg.h enum ptyg_propagator)
SET_PROPAGATORS = {"polychromeasp": 3, "scaledasp": 4, "scaledpolychromeasp": 5, "twosteppolychrome": 6, "identity": 7}

_EXC = {
    PTYG_ERR_INVALID: ValueError,
    PTYG_ERR_UNSUPPORTED: NotImplementedError,
    PTYG_ERR_OOM: MemoryError,
    PTYG_ERR_CUDA: RuntimeError,
    PTYG_ERR_TIMEOUT: TimeoutError,
    PTYG_ERR_DEVICE: ImportError,
}


class Geometry(C.Structure):
    _fields_ = [
        ("Np", C.c_int32),
        ("No", C.c_int32),
        ("nosm", C.c_int32),
        ("npsm", C.c_int32),
        ("nslice", C.c_int32),
        ("num_frames", C.c_int32),
        ("num_scans", C.c_int32),
        ("engine", C.c_int32),
        ("propagator", C.c_int32),
        ("fftshift", C.c_int32),
        ("fpm", C.c_int32),
        ("cluster", C.c_int32),
        ("throughput", C.c_int32),
        ("nlambda", C.c_int32),
        ("threads", C.c_int32),
        ("probe_in_smem", C.c_int32),
        ("asp_table_in_smem", C.c_int32),
    ]


class UpdateParams(C.Structure):
    _fields_ = [
        ("beta_object", C.c_float),
        ("beta_probe", C.c_float),
        ("alpha_object", C.c_float),
        ("alpha_probe", C.c_float),
        ("reg_object", C.c_float),
        ("reg_probe", C.c_float),
        ("friction", C.c_float),
        ("feedback", C.c_float),
        ("probe_weight", C.c_float),
        ("slice_beta", C.c_float),
        ("momentum_method", C.c_int32),
        ("beta1", C.c_double),
        ("beta2", C.c_double),
        ("beta1_scale", C.c_float),
        ("beta2_scale", C.c_float),
        ("beta_object_m", C.c_float),
        ("beta_probe_m", C.c_float),
    ]


class Projection(C.Structure):
    _fields_ = [
        ("intensity_constraint", C.c_int32),
        ("adaptive_denoising", C.c_int32),
        ("background_mode", C.c_int32),
        ("fourier_mask", C.c_int32),
        ("intensity_mask", C.c_int32),
    ]


class ScanBuffers(C.Structure):
    _fields_ = [
        ("object", C.c_void_p),
        ("probe", C.c_void_p),
        ("positions", C.c_void_p),
        ("order", C.c_void_p),
        ("momentum_flags", C.c_void_p),
        ("object_buffer", C.c_void_p),
        ("object_momentum", C.c_void_p),
        ("probe_buffer", C.c_void_p),
        ("probe_momentum", C.c_void_p),
        ("second_moment", C.c_void_p),
    ]


class Multislice(C.Structure):
    _fields_ = [
        ("Np", C.c_int32),
        ("No", C.c_int32),
        ("npsm", C.c_int32),
        ("nslice", C.c_int32),
        ("num_frames", C.c_int32),
        ("chunk", C.c_int32),
    ]


# name -> argtypes; every function returns an int status unless listed in _RESTYPES
_SIGNATURES = {
    "ptyg_version": [],
    "ptyg_last_error": None,
    "ptyg_device_init": [C.c_int],
    "ptyg_propagate": [
        C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
    ],
    "ptyg_propagate_noalloc": [
        C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
    ],
    "ptyg_nn_conv3_path": [C.c_int],
    "ptyg_nn_set_wait_policy": [C.c_longlong, C.c_int],
    "ptyg_calib_spectra": [C.c_int, C.c_int] + [C.c_void_p] * 8,
    "ptyg_calib_normalise": [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p],
    "ptyg_calib_gaussian": [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
    "ptyg_calib_arcs": [
        C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
        C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
    ],
    "ptyg_calib_rms": [
        C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
    ],
    "ptyg_stitch": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
    "ptyg_propagate_sets": [
        C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
    ],
    "ptyg_plan_create": [C.POINTER(Geometry), C.POINTER(C.c_void_p)],
    "ptyg_plan_destroy": [C.c_void_p],
    "ptyg_plan_set_tables": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
    "ptyg_plan_bind_scan": [C.c_void_p, C.c_int, C.POINTER(ScanBuffers), C.c_void_p, C.c_void_p],
    "ptyg_plan_run": [C.c_void_p, C.POINTER(UpdateParams), C.c_int, C.c_int, C.c_int, C.c_void_p],
    "ptyg_plan_set_order": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p],
    "ptyg_plan_info": [
        C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
    ],
    "ptyg_plan_frame_errors": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "ptyg_plan_frame_errors_device": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "ptyg_plan_frame_errors_all_device": [C.c_void_p, C.c_void_p, C.c_void_p],
    "ptyg_plan_detector_error": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "ptyg_plan_status": [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_void_p],
    "ptyg_plan_set_projection": [C.c_void_p, C.POINTER(Projection), C.c_void_p, C.c_void_p, C.c_void_p],
    "ptyg_plan_set_background": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "ptyg_plan_get_reference": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "ptyg_plan_get_background": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "ptyg_plan_intensity_scaling": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "ptyg_multislice_workspace_bytes": [C.POINTER(Multislice)],
    "ptyg_multislice_forward": [
        C.POINTER(Multislice), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
        C.c_void_p,
    ],
    "ptyg_multislice_adjoint": [
        C.POINTER(Multislice), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
        C.c_void_p, C.c_size_t, C.c_void_p,
    ],
    "ptyg_multislice_amplitude_gradient": [
        C.POINTER(Multislice), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
    ],
    "ptyg_qn_step": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int64, C.c_float, C.c_float, C.c_void_p,
                     C.c_void_p],
    "ptyg_nn_gemm": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                     C.c_int, C.c_void_p, C.c_void_p],
    "ptyg_nn_conv3": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "ptyg_nn_conv3_wgrad": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                            C.c_int, C.c_void_p, C.c_void_p, C.c_void_p],
    "ptyg_nn_dense_wgrad": [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                            C.c_void_p],
    "ptyg_nn_reduce_splits": [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p],
    "ptyg_nn_im2col_t": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                         C.c_void_p],
    "ptyg_nn_im2col1": [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p],
    "ptyg_nn_transpose": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p],
    "ptyg_nn_flip_weights": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p],
    "ptyg_nn_relu_bwd": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p],
    "ptyg_nn_col_sum": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p],
    "ptyg_nn_pool2": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p],
    "ptyg_nn_pool2_bwd": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p],
    "ptyg_nn_up2": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p],
    "ptyg_nn_up2_bwd": [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p],
    "ptyg_nn_slice_add": [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int64, C.c_int, C.c_void_p],
    "ptyg_nn_cast_bf16": [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p],
    "ptyg_nn_adam": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.c_float,
                     C.c_float, C.c_float, C.c_int, C.c_float, C.c_void_p],
    "ptyg_mul_window": [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p],
    "ptyg_gram": [C.c_void_p, C.c_int, C.c_int64, C.c_void_p, C.c_void_p],
    "ptyg_mix_modes": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int64, C.c_void_p],
}

_RESTYPES = {"ptyg_last_error": C.c_char_p, "ptyg_multislice_workspace_bytes": C.c_size_t}

_lock = threading.Lock()
_lib = None
_device_ready = set()


def load_library(path: Path | str | None = None):
    """Load libptyg.so and declare its prototypes (no device needed)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else LIB_PATH
        if not p.exists():
            raise ImportError(
                f"{p} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                "or `python -m ptylab_gb300._build`"
            )
        lib = C.CDLL(str(p))
        for name, args in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = _RESTYPES.get(name, C.c_int)
            fn.argtypes = args if args is not None else []
        if path is None:
            _lib = lib
        return lib


def check(status: int, what: str = "") -> None:
    if status == PTYG_OK:
        return
    lib = load_library()
    msg = lib.ptyg_last_error().decode(errors="replace")
    exc = _EXC.get(status, RuntimeError)
    raise exc(f"{what}: {msg}" if what else msg)


def require(device: int = 0):
    """Return the library once `device` is initialised; raise ImportError if unusable."""
    lib = load_library()
    if device not in _device_ready:
        check(lib.ptyg_device_init(int(device)), "ptyg_device_init")
        _device_ready.add(device)
    return lib


def available(device: int = 0) -> bool:
    """True when the library loads and `device` is an sm_103a GPU (gpuSwitch check)."""
    try:
        import torch

        if not torch.cuda.is_available():
            return False
        require(device)
        return True
    except Exception:
        return False


def exported_symbols() -> list[str]:
    return sorted(_SIGNATURES)
