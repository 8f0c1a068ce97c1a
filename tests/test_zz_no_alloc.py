"""simpois_residual_device_noalloc through the C ABI.

The allocation-free entry point serves callers that may not allocate device
memory where they check a result (a device budget reserved up front, a path
that must not enter an allocator).  It must give the numbers of the regular
entry point, simpois_residual_device, which takes its scratch from the
allocator; both sum the same FP64 partials in the same order, so the test
holds them to 1e-12 relative.  Two calls in a row with different inputs check
that what the first call leaves in the shared scratch array does not leak
into the second.  This file is collected last (pytest orders files by name).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-12


def _case(seed, pd, h, w, with_f):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((pd, h, w)).astype(np.float32)
    g[:, rng.random((h, w)) < 0.3] = np.nan
    u = np.where(np.isnan(g), rng.standard_normal(g.shape).astype(np.float32), g)
    f = (rng.standard_normal(g.shape) * 0.1).astype(np.float32) if with_f else None
    return g, u, f


def _call(L, name, ctx, u, g, f, kind):
    pd, h, w = g.shape
    rel = (ctypes.c_double * pd)()
    bn = (ctypes.c_double * pd)()
    rc = getattr(L, name)(ctx.handle, u.data_ptr(), g.data_ptr(),
                          None if f is None else f.data_ptr(), w, h, pd, kind, rel, bn)
    return rc, np.array(rel), np.array(bn)


def test_noalloc_residual_matches_allocating_entry_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from imscript_gb300 import lib
    L = lib.load()
    ctx = lib.Context(0)
    cases = [(_case(1, 3, 97, 131, True), 0), (_case(2, 2, 64, 50, False), 1)]
    for (g, u, f), kind in cases:
        tg, tu = torch.from_numpy(g).cuda(), torch.from_numpy(u).cuda()
        tf = None if f is None else torch.from_numpy(f).cuda()
        torch.cuda.synchronize()
        rc0, rel0, bn0 = _call(L, "simpois_residual_device", ctx, tu, tg, tf, kind)
        rc1, rel1, bn1 = _call(L, "simpois_residual_device_noalloc", ctx, tu, tg, tf, kind)
        assert rc0 == 0 and rc1 == 0, ctx.last_error()
        assert np.all(rel0 > 0) and np.all(bn0 > 0)
        np.testing.assert_allclose(rel1, rel0, rtol=TOL, atol=0)
        np.testing.assert_allclose(bn1, bn0, rtol=TOL, atol=0)
    ctx.close()


def test_noalloc_residual_rejects_oversize_requests():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from imscript_gb300 import lib
    L = lib.load()
    ctx = lib.Context(0)
    tiny = torch.zeros(16, device="cuda")
    rel = (ctypes.c_double * 1)()
    # rejected on the host before any work is issued: 4097 x 4096 pixels
    rc = L.simpois_residual_device_noalloc(ctx.handle, tiny.data_ptr(), tiny.data_ptr(), None,
                                           4097, 4096, 1, 0, rel, None)
    assert rc == lib.EINVAL and "exceeds the limit" in ctx.last_error()
    rc = L.simpois_residual_device_noalloc(ctx.handle, tiny.data_ptr(), tiny.data_ptr(), None,
                                           4, 4, 65, 0, (ctypes.c_double * 65)(), None)
    assert rc == lib.EINVAL
    ctx.close()
