"""GPU parity of the AMLE fill (src/amle.c) through the C ABI: bit for bit
the colour-ordered oracle on the reference's own fixtures and on random
cases; with the 4-neighbourhood run to its fixed point, the reference's
raster-order result."""
import ctypes

import numpy as np
import pytest

from golden_cases import amle_inputs, cases, load, same_bits_or_nan

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def sp():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from imscript_gb300 import simpois
    return simpois


def _cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


@pytest.mark.parametrize("path", cases("amle_"), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_amle_fixture_matches_colour_oracle(sp, oracle_mod, path):
    d = load(path)
    x, nn, niter, init = amle_inputs(d)
    want, wg = oracle_mod.amle(x, nn=nn, niter=niter, init=init, order="colour", gaps=True)
    got, gaps = sp.amle(_cuda(x), nn=nn, niter=niter, init=None if init is None else _cuda(init))
    assert same_bits_or_nan(got.cpu().numpy(), want)
    if np.isfinite(wg[0, 0]):
        assert gaps[0][0] == pytest.approx(wg[0, 0], rel=0, abs=0)


@pytest.mark.parametrize("nn", [0, 1, 4, 5, 6, 8, 16, 24, 32, 40])
def test_amle_random_multichannel(sp, oracle_mod, nn):
    from imscript_gb300 import synth
    rng = np.random.default_rng(100 + nn)
    pd, h, w = 3, 45, 70
    x = np.stack([synth.gaussian_field(rng, h, w, 4) for _ in range(pd)])
    x[:, synth.disk_mask(rng, h, w, 0.3, rmin=2, rmax=12)] = np.nan
    x[1, rng.random((h, w)) < 0.1] = np.nan     # channels with different holes
    for niter in (1, 6):
        want = oracle_mod.amle(x, nn=nn, niter=niter, order="colour")
        got, _ = sp.amle(_cuda(x), nn=nn, niter=niter)
        assert same_bits_or_nan(got.cpu().numpy(), want), (nn, niter)
        host, _ = sp.amle(x, nn=nn, niter=niter)   # host entry point
        assert same_bits_or_nan(host, want)


def test_amle_reaches_reference_fixed_point(sp, oracle_mod):
    """4 neighbours, run to the fixed point: the reference's raster sweep and
    the GPU's colour sweep meet (lower and upper iterates too)."""
    from imscript_gb300 import synth
    rng = np.random.default_rng(31)
    x = synth.gaussian_field(rng, 40, 52, 3)[None]
    x[0, 8:30, 10:40] = np.nan
    ref = oracle_mod.amle(x, nn=4, niter=1500, order="raster")
    got, gaps = sp.amle(_cuda(x), nn=4, niter=1500)
    assert np.abs(got.cpu().numpy() - ref).max() < 1e-5
    assert gaps[0][0] < 1e-5


def test_amle_dropin_symbol(sp, oracle_mod, monkeypatch):
    """amle(y, x, w, h) with AMLE_NN / AMLE_NITER from the environment."""
    from imscript_gb300 import lib
    rng = np.random.default_rng(2)
    x = rng.standard_normal((30, 41)).astype(np.float32)
    x[rng.random(x.shape) < 0.3] = np.nan
    monkeypatch.setenv("AMLE_NN", "8")
    monkeypatch.setenv("AMLE_NITER", "7")
    y = np.empty_like(x)
    L = lib.load()
    L.amle(y.ctypes.data, x.ctypes.data, 41, 30)
    want = oracle_mod.amle(x[None], nn=8, niter=7, order="colour")[0]
    assert same_bits_or_nan(y, want)
