"""CPU oracle for the simpois hole-filling path.

TEST INFRASTRUCTURE ONLY: the checker used by ``tests/``, by
``__graft_entry__.smoke()`` and by the CPU-baseline leg of ``bench.py``.  The
product (``imscript_gb300``) never imports this module.

Three checkers live here:

* ``poisson_solver_separable`` -- ctypes binding of ``simpois_oracle.c``, a C
  restatement of ``poisson_solver_separable`` (simpois.c:288) and everything
  below it.  ``order="raster"`` reproduces the reference bit for bit;
  ``order="colour"`` sweeps the colour classes the GPU sweeps, so its result is
  the exact CPU image of the GPU's Gauss-Seidel path.
* ``run_reference`` -- runs the reference ``simpois`` binary built from its own
  sources into ``oracle/_ref/`` (present only where the reference tree was).
* ``rel_residual`` -- the FP64 relative residual of the CG operators
  (cleant_cgpois.c:67-121, 226-233) on a float output.

Images are planar float32 arrays of shape (pd, h, w): sample (l, j, i) is at
``x[w*h*l + j*w + i]`` exactly as in iio's split layout (iio.h:42-43).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_simpois.so")
REF_BIN = os.path.join(HERE, "_ref", "simpois")
MINI_BIN = os.path.join(HERE, "_ref", "minisimpois")
AMLE_BIN = os.path.join(HERE, "_ref", "amle")

ORDER = {"raster": 0, "colour": 1}


class _Opts(ctypes.Structure):
    _fields_ = [
        ("pmsfac", ctypes.c_double),
        ("ponlit", ctypes.c_double),
        ("cg_eps", ctypes.c_double),
        ("order", ctypes.c_int),
        ("cg_log", ctypes.c_int),
    ]


_lib = None


def build(reference: bool | None = None, tree: str | None = None) -> None:
    """Compile the restatement, and the reference binaries from the reference
    tree ``tree`` (default: the SIMPOIS_REFERENCE_TREE environment variable)
    when its sources are there."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref_src = tree or os.environ.get("SIMPOIS_REFERENCE_TREE", "")
    if reference is None:
        reference = bool(ref_src) and os.path.isfile(os.path.join(ref_src, "src", "simpois.c"))
    if reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE={ref_src}"], check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or any(
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, src))
            for src in ("simpois_oracle.c", "amle_oracle.c")
        ):
            build(reference=False)
        L = ctypes.CDLL(LIB_PATH)
        fp = ctypes.POINTER(ctypes.c_float)
        op = ctypes.POINTER(_Opts)
        L.oracle_poisson_solver_separable.argtypes = [
            fp, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
            ctypes.c_int, ctypes.c_int, ctypes.c_float, op]
        L.oracle_poisson_solver_separable.restype = None
        L.oracle_rel_residual.argtypes = [fp, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_double)]
        L.oracle_rel_residual.restype = ctypes.c_double
        L.oracle_rhs_norm.argtypes = [fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_rhs_norm.restype = ctypes.c_double
        L.oracle_restrict.argtypes = [fp, ctypes.c_int, ctypes.c_int, fp, ctypes.c_int, ctypes.c_int]
        L.oracle_prolong.argtypes = [fp, ctypes.c_int, ctypes.c_int, fp, ctypes.c_int, ctypes.c_int]
        L.oracle_gs.argtypes = [fp, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                ctypes.c_int, fp, ctypes.c_int]
        L.oracle_cg_extension.argtypes = [fp, fp, fp, ctypes.c_int, ctypes.c_int, fp, ctypes.c_int,
                                          ctypes.c_int, op, ctypes.POINTER(ctypes.c_double)]
        L.oracle_cg_extension.restype = ctypes.c_int
        L.oracle_apply_mask.argtypes = [fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_poisson_recursive.argtypes = [fp, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                               ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.amle_oracle.argtypes = [fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp,
                                  ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.amle_oracle.restype = ctypes.c_int
        L.amle_oracle_colouring.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int)]
        L.amle_oracle_colouring.restype = None
        _lib = L
    return _lib


def _fptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _planar(a, name):
    a = np.asarray(a)
    if a.ndim == 2:
        a = a[None]
    if a.ndim != 3:
        raise ValueError(f"{name}: expected (pd,h,w) or (h,w), got {a.shape}")
    return np.ascontiguousarray(a, dtype=np.float32)


def opts(order="raster", pmsfac=3.0, ponlit=0.0, cg_eps=-1.0, cg_log=False) -> _Opts:
    return _Opts(float(pmsfac), float(ponlit), float(cg_eps), ORDER[order], int(cg_log))


def poisson_solver_separable(inp, dat=None, tstep=0.25, niter=10, scale=99, cgrad=0.0,
                             order="raster", pmsfac=3.0, ponlit=0.0, cg_eps=-1.0):
    """Restatement of simpois.c:288 on planar (pd,h,w) float32 input."""
    g = _planar(inp, "inp")
    pd, h, w = g.shape
    f = None if dat is None else _planar(dat, "dat")
    if f is not None and f.shape != g.shape:
        raise ValueError("dat shape mismatch")
    out = np.empty_like(g)
    o = opts(order, pmsfac, ponlit, cg_eps)
    lib().oracle_poisson_solver_separable(_fptr(out), _fptr(g), _fptr(f), w, h, pd,
                                          float(tstep), int(niter), int(scale), float(cgrad),
                                          ctypes.byref(o))
    return out


def poisson_recursive(inp, dat=None, tstep=0.45, niter=10, scale=99, order="raster"):
    """Restatement of ftr/minisimpois.c:127-162 (GS only) on planar input."""
    g = _planar(inp, "inp")
    pd, h, w = g.shape
    f = None if dat is None else _planar(dat, "dat")
    out = np.empty_like(g)
    for l in range(pd):
        lib().oracle_poisson_recursive(_fptr(out[l]), _fptr(g[l]), None if f is None else _fptr(f[l]),
                                       w, h, float(tstep), int(niter), int(scale), ORDER[order])
    return out


def apply_mask(img, mask):
    """NaN where mask > 0 in every channel (simpois.c:421-424)."""
    g = _planar(img, "img").copy()
    m = np.ascontiguousarray(np.asarray(mask, dtype=np.float32).reshape(g.shape[1:]))
    lib().oracle_apply_mask(_fptr(g), _fptr(m), g.shape[2], g.shape[1], g.shape[0])
    return g


def rel_residual(u, g, f=None, kind=0):
    """Per-channel FP64 relative residual; kind 0 = -Lap (5-pt), 1 = 13-pt bilaplacian.

    Returns (rel[pd], bnorm[pd]).
    """
    u = _planar(u, "u")
    g = _planar(g, "g")
    f = None if f is None else _planar(f, "f")
    pd, h, w = g.shape
    rel = np.zeros(pd)
    bn = np.zeros(pd)
    for l in range(pd):
        b = ctypes.c_double(0)
        rel[l] = lib().oracle_rel_residual(_fptr(u[l]), _fptr(g[l]),
                                           None if f is None else _fptr(f[l]), w, h, kind,
                                           ctypes.byref(b))
        bn[l] = b.value
    return rel, bn


def rhs_norm(g, f=None, kind=0):
    return rel_residual(g, g, f, kind)[1]


def restrict(img, ow, oh):
    a = np.ascontiguousarray(img, dtype=np.float32)
    out = np.empty((oh, ow), np.float32)
    lib().oracle_restrict(_fptr(out), ow, oh, _fptr(a), a.shape[1], a.shape[0])
    return out


def prolong(img, ow, oh):
    a = np.ascontiguousarray(img, dtype=np.float32)
    out = np.empty((oh, ow), np.float32)
    lib().oracle_prolong(_fptr(out), ow, oh, _fptr(a), a.shape[1], a.shape[0])
    return out


def cg_extension(g, f=None, init=None, maxit=-1, kind=0, cg_eps=-1.0):
    """The CG branch alone on one channel (cleant_cgpois.c:197-278)."""
    g = np.ascontiguousarray(g, dtype=np.float32)
    h, w = g.shape
    f = None if f is None else np.ascontiguousarray(f, dtype=np.float32)
    init = np.zeros_like(g) if init is None else np.ascontiguousarray(init, dtype=np.float32)
    out = np.empty_like(g)
    o = opts("raster", cg_eps=cg_eps)
    rr = ctypes.c_double(0)
    it = lib().oracle_cg_extension(_fptr(out), _fptr(g), _fptr(f), w, h, _fptr(init), int(maxit),
                                   int(kind), ctypes.byref(o), ctypes.byref(rr))
    return out, it, rr.value


# ---------------------------------------------------------------- reference binary

def have_reference() -> bool:
    return os.path.isfile(REF_BIN) and os.access(REF_BIN, os.X_OK)


def to_hwc(planar):
    """planar (pd,h,w) -> interleaved (h,w,pd), the npy layout iio writes."""
    return np.ascontiguousarray(np.moveaxis(np.asarray(planar), 0, -1))


def from_hwc(a):
    a = np.asarray(a)
    if a.ndim == 2:
        a = a[..., None]
    return np.ascontiguousarray(np.moveaxis(a, -1, 0), dtype=np.float32)


def run_reference(inp=None, dat=None, mask=None, args=(), env=None, timeout=600,
                  input_via_stdin=False, binary=None):
    """Run the reference binary on planar inputs; returns the planar output."""
    binary = binary or REF_BIN
    if not os.path.isfile(binary):
        raise FileNotFoundError(binary)
    with tempfile.TemporaryDirectory() as td:
        cmd = [binary]
        stdin = None
        if inp is not None:
            p = os.path.join(td, "in.npy")
            np.save(p, to_hwc(_planar(inp, "inp")))
            if input_via_stdin:
                stdin = open(p, "rb")
            else:
                cmd += ["-i", p]
        if dat is not None:
            p = os.path.join(td, "f.npy")
            np.save(p, to_hwc(_planar(dat, "dat")))
            cmd += ["-f", p]
        if mask is not None:
            p = os.path.join(td, "m.npy")
            np.save(p, np.asarray(mask, dtype=np.float32))
            cmd += ["-m", p]
        out = os.path.join(td, "out.npy")
        cmd += list(args) + ["-o", out]
        e = dict(os.environ)
        for k in ("PMSFAC", "PONLIT", "CG_EPS"):
            e.pop(k, None)
        if env:
            e.update({k: str(v) for k, v in env.items()})
        try:
            subprocess.run(cmd, env=e, check=True, timeout=timeout, stdin=stdin,
                           stderr=subprocess.DEVNULL)
        finally:
            if stdin is not None:
                stdin.close()
        return from_hwc(np.load(out))


# ------------------------------------------------------------------ AMLE (src/amle.c)

def amle(inp, nn=4, niter=100, init=None, order="raster", gaps=False):
    """AMLE fill of every channel of a planar (pd, h, w) float32 image (NaN =
    unknown), as src/amle.c:196-246 does for one channel; init (same shape)
    replaces the upper start at the unknowns.  order "raster" is the
    reference's sweep (bit-exact), "colour" the GPU's.  With gaps, also the
    per-channel (max, mean) of |tinf - tsup| over the unknowns."""
    x = _planar(inp, "inp")
    pd, h, w = x.shape
    ini = None if init is None else _planar(init, "init")
    out = np.empty_like(x)
    g = np.zeros((pd, 2))
    L = lib()
    for c in range(pd):
        y = np.empty((h, w), np.float32)
        gp = (ctypes.c_double * 2)()
        rc = L.amle_oracle(_fptr(y), _fptr(np.ascontiguousarray(x[c])), w, h, int(nn), int(niter),
                           None if ini is None else _fptr(np.ascontiguousarray(ini[c])),
                           0 if order == "raster" else 1, gp)
        if rc:
            raise MemoryError("amle oracle")
        out[c] = y
        g[c] = (gp[0], gp[1])
    return (out, g) if gaps else out


def amle_colouring(nn):
    """(m, k): the colour classes (i + k j) mod m of the parallel AMLE sweep."""
    m, k = ctypes.c_int(), ctypes.c_int()
    lib().amle_oracle_colouring(int(nn), ctypes.byref(m), ctypes.byref(k))
    return m.value, k.value


def run_reference_amle(inp, mask=None, env=None, timeout=600):
    """Run the reference amle binary (`amle in mask out`, src/amle.c:330-367)
    on one channel (h, w); returns the (h, w) output."""
    if not os.path.isfile(AMLE_BIN):
        raise FileNotFoundError(AMLE_BIN)
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "in.npy")
        np.save(p, np.asarray(inp, np.float32))
        pm = ""
        if mask is not None:
            pm = os.path.join(td, "m.npy")
            np.save(pm, np.asarray(mask, np.float32))
        out = os.path.join(td, "out.npy")
        e = dict(os.environ)
        for k in ("AMLE_NN", "AMLE_NITER", "AMLE_INIT", "AMLE_TAU"):
            e.pop(k, None)
        if env:
            e.update({k: str(v) for k, v in env.items()})
        subprocess.run([AMLE_BIN, p, pm, out], env=e, check=True, timeout=timeout,
                       stderr=subprocess.DEVNULL)
        y = np.load(out)
        return y.reshape(y.shape[0], y.shape[1])
