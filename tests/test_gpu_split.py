"""Biharmonic channels split into their hole components.  Groups of unknowns
that no stencil couples (no 8 x 8 pixel blocks holding them touch) are solved
as separate problems, each in a crop of the channel, and retire on their own;
the channel's output is the FP64 direct solve of the whole channel within
1e-4, its known pixels are its input's, and its report sums the unknowns,
takes the largest iteration count of its components and combines their
residuals into the channel's (|r|^2 and |b|^2 summed over the components)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def sp():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from imscript_gb300 import simpois
    return simpois


def _holes(rng, h, w):
    from imscript_gb300 import synth
    m = np.zeros((h, w), bool)
    m[50:130, 60:140] = True                       # a square hole
    m[200:203, 20:380] = True                      # an L-shaped scratch whose bounding box
    m[20:203, 376:379] = True                      # holds the square and a small disk
    yy, xx = np.mgrid[0:h, 0:w]
    m |= (yy - 100) ** 2 + (xx - 300) ** 2 <= 36   # the disk
    m |= synth.scratch_mask(rng, h, w, 3, lmin=20, lmax=60) & (yy > 230)
    m[h - 2:, w - 40:w - 10] = True                # a hole on the image side (the clamp)
    return m


@pytest.mark.parametrize("pd", [1, 2])
def test_components_match_the_whole_channel_fp64_solve(sp, pd):
    from imscript_gb300 import synth
    from oracle import fp64
    rng = np.random.default_rng(17)
    h, w = 260, 400
    g = np.stack([synth.gaussian_field(rng, h, w, 12) for _ in range(pd)]).astype(np.float32)
    masks = [_holes(rng, h, w) for _ in range(pd)]
    for l in range(pd):
        g[l][masks[l]] = np.nan
    out, reps = sp.solve(torch.from_numpy(g).cuda(), None, tstep=-0.08, rtol=1e-8)
    out = out.cpu().numpy()
    for l in range(pd):
        m = masks[l]
        assert reps[l]["status"] == 0 and reps[l]["rel_residual"] <= 1e-8, reps[l]
        assert reps[l]["unknowns"] == int(m.sum())
        np.testing.assert_array_equal(out[l][~m].view(np.int32), g[l][~m].view(np.int32))
        x = fp64.solve(g[l], None, 1)
        err = np.abs(out[l][m] - x[m]).max() / np.abs(x[m]).max()
        assert err <= 1e-4, err


def test_split_solves_repeat_bit_for_bit(sp):
    from imscript_gb300 import synth
    rng = np.random.default_rng(23)
    h, w = 260, 400
    g = synth.gaussian_field(rng, h, w, 12).astype(np.float32)
    g[_holes(rng, h, w)] = np.nan
    gt = torch.from_numpy(g[None]).cuda()
    a, ra = sp.solve(gt, None, tstep=-0.08, rtol=1e-6)
    b, rb = sp.solve(gt, None, tstep=-0.08, rtol=1e-6)
    assert ra == rb
    assert torch.equal(a.view(torch.int32), b.view(torch.int32))


def test_a_channel_splits_the_same_in_a_batch(sp):
    """Whether and how a channel is split depends on the channel alone: in a
    batch with other biharmonic images it gives the bits it gives alone."""
    from imscript_gb300 import synth
    rng = np.random.default_rng(29)
    h, w = 260, 400
    imgs = []
    for k in range(3):
        g = synth.gaussian_field(rng, h, w, 12).astype(np.float32)
        g[_holes(rng, h, w) if k != 1 else synth.disk_mask(rng, h, w, 0.2, rmin=3, rmax=12)] = np.nan
        imgs.append(torch.from_numpy(g[None]).cuda())
    outs, reps = sp.solve_batch([(g, None, -0.08) for g in imgs], rtol=1e-6)
    for k, g in enumerate(imgs):
        one, r1 = sp.solve(g, None, tstep=-0.08, rtol=1e-6)
        assert r1[0] == reps[k]
        assert torch.equal(one.view(torch.int32), outs[k].view(torch.int32)), k


def test_data_term_and_many_components(sp):
    """A biharmonic image with a data term is split like one without (the
    crops carry their part of f); a channel with more than 256 hole
    components is solved whole; both within 1e-4 of the FP64 solve."""
    from imscript_gb300 import synth
    from oracle import fp64
    rng = np.random.default_rng(41)
    cases = []
    h, w = 260, 400
    g = synth.gaussian_field(rng, h, w, 10).astype(np.float32)
    f = (0.01 * synth.gaussian_field(rng, h, w, 10)).astype(np.float32)
    m = _holes(rng, h, w)
    cases.append((g, f, m))
    # 400 single-pixel holes 20 pixels apart (no two in touching 8 x 8 blocks)
    # and a rectangle: more components than a channel is split into
    h, w = 400, 400
    g = synth.gaussian_field(rng, h, w, 10).astype(np.float32)
    m = np.zeros((h, w), bool)
    m[5::20, 5::20] = True
    m[100:140, 100:160] = True
    cases.append((g, None, m))
    for g, f, m in cases:
        g = g.copy()
        g[m] = np.nan
        gt = torch.from_numpy(g[None]).cuda()
        ft = None if f is None else torch.from_numpy(f[None]).cuda()
        out, reps = sp.solve(gt, ft, tstep=-0.08, rtol=1e-8)
        assert reps[0]["status"] == 0 and reps[0]["unknowns"] == int(m.sum()), reps
        o = out[0].cpu().numpy()
        x = fp64.solve(g, f, 1)
        err = np.abs(o[m] - x[m]).max() / np.abs(x[m]).max()
        assert err <= 1e-4, err
