"""Python mirror of the simpois solver interface over the C ABI.

``poisson_solver_separable`` keeps the argument meaning of the reference's
``poisson_solver_separable(out, in, dat, w, h, pd, tstep, niter, scale,
cgrad)`` (simpois.c:288-290): planar channels, NaN = unknown, ``dat`` the
optional data term, ``tstep``/``niter``/``scale``/``cgrad`` the -t/-n/-s/-c
options.  Two additions: ``rtol`` > 0 selects the converged schedule (solve to
an FP64 relative residual), and the call returns per-channel reports.

Inputs may be numpy arrays (host memory: the copies in and out are part of the
call) or CUDA torch tensors (device memory, issued on the current stream).
Images are float32 (pd, h, w) or (h, w).
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import lib as _lib

_ctx_lock = threading.Lock()
_contexts: dict = {}


def context(device: int = 0, stream: int | None = None) -> _lib.Context:
    """The cached context of (device, stream)."""
    key = (device, stream or 0)
    with _ctx_lock:
        c = _contexts.get(key)
        if c is None:
            c = _contexts[key] = _lib.Context(device, stream)
        return c


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _params(tstep, niter, scale, cgrad, rtol, pmsfac, ponlit, cg_eps, max_iter, flags):
    return _lib.default_params(tstep=float(tstep), niter=int(niter), scale=int(scale),
                               cgit=int(cgrad), rtol=float(rtol), pmsfac=float(pmsfac),
                               ponlit=float(ponlit), cg_eps=float(cg_eps), max_iter=int(max_iter),
                               flags=int(flags))


def _shape3(x):
    shp = tuple(x.shape)
    if len(shp) == 2:
        return 1, shp[0], shp[1]
    if len(shp) == 3:
        return shp
    raise ValueError(f"expected (pd,h,w) or (h,w), got {shp}")


def _torch_stream(t):
    import torch
    return torch.cuda.current_stream(t.device).cuda_stream


def poisson_solver_separable(inp, dat=None, tstep=0.25, niter=10, scale=99, cgrad=0.0, *,
                             rtol=0.0, pmsfac=3.0, ponlit=0.0, cg_eps=-1.0, max_iter=0,
                             flags=0, out=None, allow=(_lib.OK,)):
    """Fill the NaN pixels of every channel; returns (out, reports)."""
    pd, h, w = _shape3(inp)
    prm = _params(tstep, niter, scale, cgrad, rtol, pmsfac, ponlit, cg_eps, max_iter, flags)
    reps = (_lib.Report * pd)()
    if _is_torch(inp):
        import torch
        if not inp.is_cuda:
            inp = inp.numpy()
        else:
            g = inp.contiguous()
            if g.dtype != torch.float32:
                raise TypeError("float32 input expected")
            f = None
            if dat is not None:
                f = dat.contiguous()
                if f.shape != g.shape or f.dtype != torch.float32 or f.device != g.device:
                    raise ValueError("dat must match inp (shape, float32, device)")
            o = torch.empty_like(g) if out is None else out
            ctx = context(g.device.index or 0, _torch_stream(g))
            rc = _lib.load().simpois_solve_device(ctx.handle, o.data_ptr(), g.data_ptr(),
                                                  f.data_ptr() if f is not None else None,
                                                  w, h, pd, ctypes.byref(prm), reps)
            ctx.check(rc, allow)
            return o, [r.as_dict() for r in reps]
    g = np.ascontiguousarray(inp, dtype=np.float32)
    f = None if dat is None else np.ascontiguousarray(dat, dtype=np.float32)
    if f is not None and f.shape != g.shape:
        raise ValueError("dat shape mismatch")
    o = np.empty_like(g) if out is None else out
    ctx = context(0)
    rc = _lib.load().simpois_solve(ctx.handle, o.ctypes.data, g.ctypes.data,
                                   None if f is None else f.ctypes.data, w, h, pd,
                                   ctypes.byref(prm), reps)
    ctx.check(rc, allow)
    return o, [r.as_dict() for r in reps]


def poisson_rec(g, f=None, tstep=0.25, niter=10, scale=99, cgit=0, **kw):
    """One channel (simpois.c:247-248)."""
    out, reps = poisson_solver_separable(g, f, tstep, niter, scale, cgit, **kw)
    return out, reps[0]


def solve(g, f=None, *, tstep=0.25, rtol=1e-6, **kw):
    """Converged fill of CUDA tensors (or numpy arrays) to ``rtol``."""
    return poisson_solver_separable(g, f, tstep, rtol=rtol, **kw)


def solve_batch(images, *, rtol=1e-6, tstep=0.25, max_iter=0, flags=0, allow=(_lib.OK,), outs=None):
    """Batched converged solve of CUDA tensors of different sizes.

    ``images`` is a list of ``g`` tensors or of ``(g, f)`` / ``(g, f, tstep)``
    tuples.  Returns (outputs, reports) with one report per channel.
    """
    outs, reps, _ = _batch(images, rtol, tstep, max_iter, flags, allow, outs, False)
    return outs, reps


def solve_batch_host(images, *, rtol=1e-6, tstep=0.25, max_iter=0, flags=0, allow=(_lib.OK,), outs=None,
                     device=0):
    """Batched converged solve of numpy images in host memory (page-locked
    ones move fastest) through simpois_solve_batch_host: the copies to and
    from the device are part of the call.  ``images`` as in ``solve_batch``;
    returns (outputs, reports)."""
    items = []
    for k, it in enumerate(images):
        if isinstance(it, (tuple, list)):
            g, f = it[0], (it[1] if len(it) > 1 else None)
            t = it[2] if len(it) > 2 else tstep
        else:
            g, f, t = it, None, tstep
        if not (isinstance(g, np.ndarray) and g.dtype == np.float32 and g.flags.c_contiguous):
            raise ValueError(f"image {k}: contiguous float32 numpy array expected")
        if f is not None and (f.shape != g.shape or f.dtype != np.float32 or not f.flags.c_contiguous):
            raise ValueError(f"image {k}: data term must match the image")
        items.append((g, f, t))
    if outs is None:
        outs = [np.empty_like(g) for g, _, _ in items]
    rows = []
    total = 0
    for k, (g, f, t) in enumerate(items):
        pd, h, w = _shape3(g)
        if outs[k].shape != g.shape or outs[k].dtype != np.float32 or not outs[k].flags.c_contiguous:
            raise ValueError(f"output {k} must match image {k}")
        rows.append((g.ctypes.data, f.ctypes.data if f is not None else 0, outs[k].ctypes.data, w, h, pd, t, rtol))
        total += pd
    keep, arr = _lib.image_array(rows)
    reps = (_lib.Report * max(1, total))()
    prm = _lib.default_params(rtol=float(rtol), max_iter=int(max_iter), flags=int(flags), tstep=float(tstep))
    ctx = context(device)
    rc = _lib.load().simpois_solve_batch_host(ctx.handle, arr, len(items), ctypes.byref(prm), reps)
    ctx.check(rc, allow)
    return outs, _lib.report_dicts(reps, total)


def autotune(images, *, rtol=1e-6, tstep=0.25, max_iter=0, flags=0, allow=(_lib.OK,), outs=None):
    """``solve_batch`` that also times the fused V-cycle's launch choices --
    the hand-over size (no bit of a result depends on it), then the smoothing
    sweeps per side of the tile kernels (1, 2 or 3) -- and keeps the fastest
    pair for later batches of the same shapes on this context.

    Returns (outputs, reports, {"coarse_max": .., "sweeps": ..}); the outputs
    are those of the chosen pair."""
    return _batch(images, rtol, tstep, max_iter, flags, allow, outs, True)


def _batch(images, rtol, tstep, max_iter, flags, allow, outs, tune):
    import torch
    items = []
    for k, it in enumerate(images):
        if isinstance(it, (tuple, list)):
            g, f = it[0], (it[1] if len(it) > 1 else None)
            t = it[2] if len(it) > 2 else tstep
        else:
            g, f, t = it, None, tstep
        if not (g.is_cuda and g.dtype == torch.float32 and g.is_contiguous()):
            raise ValueError(f"image {k}: contiguous float32 CUDA tensor expected")
        if f is not None and (f.shape != g.shape or not f.is_contiguous()):
            raise ValueError(f"image {k}: data term must match the image")
        items.append((g, f, t))
    if not items:
        return [], [], None
    dev = items[0][0].device
    outs = [torch.empty_like(g) for g, _, _ in items] if outs is None else outs
    rows = []
    total = 0
    for k, (g, f, t) in enumerate(items):
        pd, h, w = _shape3(g)
        rows.append((g.data_ptr(), f.data_ptr() if f is not None else 0, outs[k].data_ptr(), w, h, pd, t, rtol))
        total += pd
    keep, arr = _lib.image_array(rows)
    reps = (_lib.Report * total)()
    prm = _lib.default_params(rtol=float(rtol), max_iter=int(max_iter), flags=int(flags),
                              tstep=float(tstep))
    ctx = context(dev.index or 0, _torch_stream(items[0][0]))
    tuned = None
    if tune:
        cm, nu = ctypes.c_int(0), ctypes.c_int(0)
        rc = _lib.load().simpois_autotune_ex(ctx.handle, arr, len(items), ctypes.byref(prm), reps,
                                             ctypes.byref(cm), ctypes.byref(nu))
        tuned = {"coarse_max": cm.value, "sweeps": nu.value}
    else:
        rc = _lib.load().simpois_solve_batch(ctx.handle, arr, len(items), ctypes.byref(prm), reps)
    ctx.check(rc, allow)
    return outs, _lib.report_dicts(reps), tuned


def residual(u, g, f=None, kind=0):
    """FP64 relative residual of a float output per channel (CUDA tensors)."""
    import torch
    pd, h, w = _shape3(g)
    for name, t in (("u", u), ("g", g), ("f", f)):
        if t is None:
            continue
        if not t.is_cuda or t.device != g.device:
            raise ValueError(f"residual: {name} must be a CUDA tensor on {g.device}")
        if t.dtype != torch.float32:
            raise TypeError(f"residual: {name} must be float32, got {t.dtype}")
        if tuple(t.shape[-2:]) != (h, w) or t.numel() != pd * h * w:
            raise ValueError(f"residual: {name} has shape {tuple(t.shape)}, expected {(pd, h, w)}")
    u, g = u.contiguous(), g.contiguous()
    f = f.contiguous() if f is not None else None
    rel = (ctypes.c_double * pd)()
    bn = (ctypes.c_double * pd)()
    ctx = context(g.device.index or 0, _torch_stream(g))
    rc = _lib.load().simpois_residual_device(ctx.handle, u.data_ptr(), g.data_ptr(),
                                             f.data_ptr() if f is not None else None, w, h, pd,
                                             int(kind), rel, bn)
    ctx.check(rc)
    return list(rel), list(bn)


def adjoint(grad_out, g, *, rtol=1e-6, max_iter=0, flags=0, want_dat=True, allow=(_lib.OK,)):
    """Adjoint of the converged 5-point fill (CUDA tensors).

    Returns (grad_in, grad_dat, reports): grad_in is grad_out plus the adjoint
    solution scattered to the known 5-neighbours (0 at the unknowns); grad_dat
    is minus the adjoint solution at the unknowns (0 elsewhere)."""
    import torch
    pd, h, w = _shape3(g)
    go = grad_out.contiguous().to(torch.float32)
    gi = torch.empty_like(g)
    gd = torch.empty_like(g) if want_dat else None
    reps = (_lib.Report * pd)()
    prm = _lib.default_params(rtol=float(rtol), max_iter=int(max_iter), flags=int(flags))
    ctx = context(g.device.index or 0, _torch_stream(g))
    rc = _lib.load().simpois_adjoint_device(ctx.handle, go.data_ptr(), g.data_ptr(), w, h, pd,
                                            gi.data_ptr(), gd.data_ptr() if gd is not None else None,
                                            ctypes.byref(prm), reps)
    ctx.check(rc, allow)
    return gi, gd, [r.as_dict() for r in reps]


def amle(inp, nn=4, niter=100, init=None, *, out=None):
    """AMLE fill of every channel (src/amle.c:196-246): ``nn`` neighbours
    (AMLE_NN), ``niter`` iterations (AMLE_NITER), ``init`` the start of the
    upper iterate at the unknowns (AMLE_INIT; same shape as ``inp``).  Returns
    (out, gaps) with gaps[c] = (max, mean) of |lower - upper| over channel c's
    unknowns after the last iteration.  numpy arrays or CUDA tensors."""
    pd, h, w = _shape3(inp)
    gaps = (ctypes.c_double * (2 * pd))()
    if _is_torch(inp) and inp.is_cuda:
        import torch
        g = inp.contiguous()
        if g.dtype != torch.float32:
            raise TypeError("float32 input expected")
        ini = None
        if init is not None:
            ini = init.contiguous()
            if ini.shape != g.shape or ini.dtype != torch.float32 or ini.device != g.device:
                raise ValueError("init must match inp (shape, float32, device)")
        o = torch.empty_like(g) if out is None else out
        ctx = context(g.device.index or 0, _torch_stream(g))
        rc = _lib.load().simpois_amle_device(ctx.handle, o.data_ptr(), g.data_ptr(), w, h, pd, int(nn),
                                             int(niter), None if ini is None else ini.data_ptr(), gaps)
    else:
        if _is_torch(inp):
            inp = inp.numpy()
        g = np.ascontiguousarray(inp, dtype=np.float32)
        ini = None if init is None else np.ascontiguousarray(init, dtype=np.float32)
        if ini is not None and ini.shape != g.shape:
            raise ValueError("init shape mismatch")
        o = np.empty_like(g) if out is None else out
        ctx = context(0)
        rc = _lib.load().simpois_amle(ctx.handle, o.ctypes.data, g.ctypes.data, w, h, pd, int(nn), int(niter),
                                      None if ini is None else ini.ctypes.data, gaps)
    ctx.check(rc)
    return o, [(gaps[2 * c], gaps[2 * c + 1]) for c in range(pd)]
