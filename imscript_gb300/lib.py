"""ctypes binding of libsimpois_gpu.so (include/simpois_gpu.h).

There is no CPU fallback: if the library is missing or cannot be loaded, every
call raises.  Build it with ``python -m imscript_gb300._build`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

OK, EINVAL, ENOMEM, NOT_CONVERGED, BREAKDOWN, ECUDA, ENODEV, SINGULAR = range(8)
FLAG_NO_MG, FLAG_NO_GRAPH, FLAG_OUT_RESID, FLAG_UNFUSED, FLAG_KTIMER = 0x1, 0x2, 0x4, 0x8, 0x10
FLAG_MINI = 0x20
FLAG_TMA = 0x40

STATUS_NAMES = {OK: "ok", EINVAL: "einval", ENOMEM: "enomem", NOT_CONVERGED: "not_converged",
                BREAKDOWN: "breakdown", ECUDA: "ecuda", ENODEV: "enodev", SINGULAR: "singular"}


class Params(ctypes.Structure):
    _fields_ = [
        ("tstep", ctypes.c_float),
        ("niter", ctypes.c_int),
        ("scale", ctypes.c_int),
        ("cgit", ctypes.c_int),
        ("pmsfac", ctypes.c_double),
        ("ponlit", ctypes.c_double),
        ("cg_eps", ctypes.c_double),
        ("rtol", ctypes.c_double),
        ("max_iter", ctypes.c_int),
        ("flags", ctypes.c_int),
    ]


class Report(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int),
        ("unknowns", ctypes.c_int),
        ("iterations", ctypes.c_int),
        ("refinements", ctypes.c_int),
        ("rel_residual", ctypes.c_double),
        ("rel_residual_out", ctypes.c_double),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


def report_dicts(reps, n=None):
    """The first n records of a Report array as dicts (as Report.as_dict),
    read through one numpy view: a batch's hundreds of records convert in a
    fraction of the per-field ctypes reads."""
    import numpy as np
    n = len(reps) if n is None else n
    rows = np.frombuffer(reps, dtype=REPORT_DTYPE, count=n).tolist()
    return [{"status": a, "unknowns": b, "iterations": c, "refinements": d, "rel_residual": e,
             "rel_residual_out": f} for a, b, c, d, e, f in rows]


class Image(ctypes.Structure):
    _fields_ = [
        ("inp", ctypes.c_void_p),
        ("dat", ctypes.c_void_p),
        ("out", ctypes.c_void_p),
        ("w", ctypes.c_int),
        ("h", ctypes.c_int),
        ("pd", ctypes.c_int),
        ("tstep", ctypes.c_float),
        ("rtol", ctypes.c_double),
    ]


def _np_dtypes():
    import numpy as np
    img = np.dtype([("inp", np.uint64), ("dat", np.uint64), ("out", np.uint64), ("w", np.int32),
                    ("h", np.int32), ("pd", np.int32), ("tstep", np.float32), ("rtol", np.float64)], align=True)
    rep = np.dtype([("status", np.int32), ("unknowns", np.int32), ("iterations", np.int32),
                    ("refinements", np.int32), ("rel_residual", np.float64), ("rel_residual_out", np.float64)],
                   align=True)
    assert img.itemsize == ctypes.sizeof(Image) and rep.itemsize == ctypes.sizeof(Report)
    return img, rep


# numpy views of simpois_image and simpois_report (the batch entry points fill
# and read hundreds of them per call)
IMAGE_DTYPE, REPORT_DTYPE = _np_dtypes()


def image_array(rows):
    """A simpois_image array from (in, dat, out, w, h, pd, tstep, rtol) rows
    (pointers as ints, 0 for none); returns (numpy array, ctypes pointer)."""
    import numpy as np
    a = np.array(rows, dtype=IMAGE_DTYPE)
    return a, a.ctypes.data_as(ctypes.POINTER(Image))


# every symbol include/simpois_gpu.h declares
EXPORTS = [
    "simpois_default_params", "simpois_params_from_env", "simpois_create", "simpois_destroy",
    "simpois_strerror", "simpois_last_error", "simpois_solve", "simpois_solve_device",
    "simpois_solve_batch", "simpois_solve_batch_host", "simpois_residual_device", "simpois_residual_device_noalloc",
    "simpois_adjoint_device", "simpois_autotune", "simpois_autotune_ex", "simpois_set_coarse_max",
    "simpois_set_sweeps", "simpois_set_memory_limit", "simpois_set_tune_cache",
    "simpois_amle_device", "simpois_amle", "amle",
    "simpois_launch_count", "simpois_reset_launch_count", "simpois_kernel_stats",
    "simpois_reset_kernel_stats",
    "poisson_solver_separable", "poisson_rec", "poisson_recursive",
]

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load the library (and declare the prototypes); raises if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"libsimpois_gpu.so is not built ({path}); run "
                                   "`python -m imscript_gb300._build`")
            _build.build_library()
        L = ctypes.CDLL(path)
        vp, ip, fp = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        P = ctypes.POINTER(Params)
        R = ctypes.POINTER(Report)
        L.simpois_default_params.argtypes = [P]
        L.simpois_default_params.restype = None
        L.simpois_params_from_env.argtypes = [P]
        L.simpois_params_from_env.restype = None
        L.simpois_create.argtypes = [ctypes.POINTER(vp), ip, vp]
        L.simpois_destroy.argtypes = [vp]
        L.simpois_strerror.argtypes = [ip]
        L.simpois_strerror.restype = ctypes.c_char_p
        L.simpois_last_error.argtypes = [vp]
        L.simpois_last_error.restype = ctypes.c_char_p
        L.simpois_solve.argtypes = [vp, vp, vp, vp, ip, ip, ip, P, R]
        L.simpois_solve_device.argtypes = [vp, vp, vp, vp, ip, ip, ip, P, R]
        L.simpois_solve_batch.argtypes = [vp, ctypes.POINTER(Image), ip, P, R]
        L.simpois_solve_batch_host.argtypes = [vp, ctypes.POINTER(Image), ip, P, R]
        L.simpois_residual_device.argtypes = [vp, vp, vp, vp, ip, ip, ip, ip,
                                              ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_double)]
        L.simpois_residual_device_noalloc.argtypes = L.simpois_residual_device.argtypes
        L.simpois_adjoint_device.argtypes = [vp, vp, vp, ip, ip, ip, vp, vp, P, R]
        L.simpois_autotune.argtypes = [vp, ctypes.POINTER(Image), ip, P, R, ctypes.POINTER(ip)]
        L.simpois_autotune_ex.argtypes = [vp, ctypes.POINTER(Image), ip, P, R, ctypes.POINTER(ip),
                                          ctypes.POINTER(ip)]
        L.simpois_set_coarse_max.argtypes = [vp, ip]
        L.simpois_set_sweeps.argtypes = [vp, ip]
        L.simpois_set_memory_limit.argtypes = [vp, ctypes.c_size_t]
        L.simpois_set_tune_cache.argtypes = [vp, ctypes.c_char_p]
        dp = ctypes.POINTER(ctypes.c_double)
        L.simpois_amle_device.argtypes = [vp, vp, vp, ip, ip, ip, ip, ip, vp, dp]
        L.simpois_amle.argtypes = [vp, vp, vp, ip, ip, ip, ip, ip, vp, dp]
        L.amle.argtypes = [vp, vp, ip, ip]
        L.amle.restype = None
        L.simpois_launch_count.argtypes = [vp]
        L.simpois_launch_count.restype = ctypes.c_longlong
        L.simpois_reset_launch_count.argtypes = [vp]
        L.simpois_reset_launch_count.restype = None
        L.simpois_kernel_stats.argtypes = [vp]
        L.simpois_kernel_stats.restype = ctypes.c_char_p
        L.simpois_reset_kernel_stats.argtypes = [vp]
        L.simpois_reset_kernel_stats.restype = None
        L.poisson_solver_separable.argtypes = [vp, vp, vp, ip, ip, ip, fp, ip, ip, fp]
        L.poisson_solver_separable.restype = None
        L.poisson_rec.argtypes = [vp, vp, vp, ip, ip, fp, ip, ip, ip]
        L.poisson_rec.restype = None
        L.poisson_recursive.argtypes = [vp, vp, vp, ip, ip, fp, ip, ip]
        L.poisson_recursive.restype = None
        _lib = L
        return L


class SimpoisError(RuntimeError):
    def __init__(self, status, message=""):
        self.status = status
        name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"simpois: {name}" + (f": {message}" if message else ""))


def default_params(**kw) -> Params:
    p = Params()
    load().simpois_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise TypeError(f"unknown parameter {k}")
        setattr(p, k, v)
    return p


class Context:
    """A solver context bound to one device and one CUDA stream."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._lib = load()
        self.device = device
        self.stream = stream or 0
        h = ctypes.c_void_p()
        rc = self._lib.simpois_create(ctypes.byref(h), device, ctypes.c_void_p(self.stream))
        if rc:
            raise SimpoisError(rc, self._lib.simpois_strerror(rc).decode())
        self.handle = h

    def launches(self) -> int:
        return int(self._lib.simpois_launch_count(self.handle))

    def reset_launches(self):
        self._lib.simpois_reset_launch_count(self.handle)

    def kernel_stats(self) -> dict:
        import json
        return json.loads(self._lib.simpois_kernel_stats(self.handle).decode())

    def reset_kernel_stats(self):
        self._lib.simpois_reset_kernel_stats(self.handle)

    def set_coarse_max(self, coarse_max: int):
        """Fix the fused V-cycle's hand-over size (8..128; 0: tuned or default)."""
        self.check(self._lib.simpois_set_coarse_max(self.handle, int(coarse_max)))

    def set_sweeps(self, sweeps: int):
        """Fix the tile kernels' smoothing sweeps per side (1..3; 0: tuned or default)."""
        self.check(self._lib.simpois_set_sweeps(self.handle, int(sweeps)))

    def set_memory_limit(self, nbytes: int):
        """Largest device arena this context may hold (0: no limit); a solve
        that needs more returns ENOMEM before it touches anything."""
        self.check(self._lib.simpois_set_memory_limit(self.handle, int(nbytes)))

    def set_tune_cache(self, path):
        """Keep the autotuner's choices in the file ``path`` (None: stop); the
        choices it holds for this device are loaded now, and a batch shape
        whose choice is known is not timed again."""
        self.check(self._lib.simpois_set_tune_cache(self.handle, None if path is None else str(path).encode()))

    def last_error(self) -> str:
        return self._lib.simpois_last_error(self.handle).decode()

    def check(self, rc, allow=(OK,)):
        if rc not in allow:
            raise SimpoisError(rc, self.last_error())
        return rc

    def close(self):
        if getattr(self, "handle", None):
            self._lib.simpois_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
