"""The host entry point with page-locked buffers (direct I/O: the output's
known pixels go back during the solve, f and the output move only in 4-pixel
groups holding an unknown) writes the same bits as with pageable buffers
(whole-buffer copies); unaligned buffers and sizes that are not a multiple of
4 take the whole-buffer path."""
import numpy as np
import pytest

from imscript_gb300 import simpois, synth

pytestmark = pytest.mark.gpu


def _case(seed, pd, h, w, guided):
    rng = np.random.default_rng(seed)
    g = np.stack([synth.gaussian_field(rng, h, w, 6) for _ in range(pd)]).astype(np.float32)
    m = synth.disk_mask(rng, h, w, 0.25, rmin=2, rmax=8)
    g[:, m] = np.nan
    f = None
    if guided:
        f = np.stack([synth.guidance(synth.gaussian_field(rng, h, w, 6))[2] for _ in range(pd)])
        f = f.astype(np.float32)
    return g, f


def _pinned(a, offset=0):
    """A numpy view of page-locked memory holding a, `offset` floats in."""
    import torch
    t = torch.empty(a.size + offset, dtype=torch.float32).pin_memory()
    v = t.numpy()[offset:offset + a.size].reshape(a.shape)
    v[...] = a
    return t, v


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("guided", [False, True])
@pytest.mark.parametrize("shape,offset", [((3, 96, 128), 0), ((1, 77, 52), 0), ((2, 64, 80), 1),
                                          ((1, 33, 31), 0), ((1, 250, 300), 0)])
def test_direct_io_same_bits(shape, offset, guided):
    pd, h, w = shape
    g, f = _case(11 + h, pd, h, w, guided)
    want, rw = simpois.poisson_solver_separable(g, f, 0.25, rtol=1e-6)   # pageable buffers
    keep = []
    tg, hg = _pinned(g, offset)
    hf = None
    if f is not None:
        tf, hf = _pinned(f, offset)
        keep.append(tf)
    to, ho = _pinned(np.full_like(g, 7.0), offset)   # stale values must all be replaced
    ctx = simpois.context(0)
    ctx.reset_launches()
    got, rg = simpois.poisson_solver_separable(hg, hf, 0.25, rtol=1e-6, out=ho)
    n_direct = ctx.launches()
    ctx.reset_launches()
    simpois.poisson_solver_separable(g, f, 0.25, rtol=1e-6)
    n_copy = ctx.launches()
    assert np.array_equal(_bits(got), _bits(want))
    assert [r["iterations"] for r in rg] == [r["iterations"] for r in rw]
    direct = offset == 0 and g.size % 4 == 0
    # the direct path adds k_put_unknowns, and k_fetch_rhs with a data term
    assert n_direct - n_copy == ((1 + (f is not None)) if direct else 0)
    del keep, tg, to


def test_direct_io_all_known_and_all_unknown():
    g, f = _case(5, 1, 40, 48, True)
    for img in (np.nan_to_num(g, nan=1.0), np.full_like(g, np.nan)):
        want, _ = simpois.poisson_solver_separable(img, f, 0.25, rtol=1e-6,
                                                   allow=(0, simpois._lib.NOT_CONVERGED))
        _, hg = _pinned(img)
        _, hf = _pinned(f)
        _, ho = _pinned(np.zeros_like(img))
        got, _ = simpois.poisson_solver_separable(hg, hf, 0.25, rtol=1e-6, out=ho,
                                                  allow=(0, simpois._lib.NOT_CONVERGED))
        assert np.array_equal(_bits(got), _bits(want))


def test_batch_host_entry_point_gives_the_device_batch_bits():
    """simpois_solve_batch_host (host buffers, page-locked or pageable) gives
    the bits of simpois_solve_batch on the same images in device memory."""
    import torch
    from imscript_gb300 import simpois, synth
    insts = synth.config3(seed=3, n=6, smax=256)
    dev = [(torch.from_numpy(i.g).cuda(), None if i.f is None else torch.from_numpy(i.f).cuda(), i.tstep)
           for i in insts]
    douts, dreps = simpois.solve_batch(dev, rtol=1e-6)
    for pinned in (True, False):
        if pinned:
            hg = [torch.from_numpy(i.g).pin_memory().numpy() for i in insts]
            hf = [None if i.f is None else torch.from_numpy(i.f).pin_memory().numpy() for i in insts]
        else:
            hg = [i.g.copy() for i in insts]
            hf = [None if i.f is None else i.f.copy() for i in insts]
        houts, hreps = simpois.solve_batch_host(list(zip(hg, hf, [i.tstep for i in insts])), rtol=1e-6)
        for d, h in zip(douts, houts):
            assert np.array_equal(d.cpu().numpy().view(np.uint32), h.view(np.uint32))
        assert [r["iterations"] for r in hreps] == [r["iterations"] for r in dreps]
