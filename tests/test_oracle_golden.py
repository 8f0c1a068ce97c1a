"""The oracle restatement against the reference's own outputs (CPU)."""
import numpy as np
import pytest

from golden_cases import amle_inputs, cases, load, parse_args, same_bits_or_nan


@pytest.mark.parametrize("path", cases("pin_"), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_oracle_reproduces_reference_bit_exact(oracle_mod, path):
    d = load(path)
    kw = parse_args(d["args"], d["env"])
    g = d["g"]
    if d["mask"] is not None:
        g = oracle_mod.apply_mask(g, d["mask"])
    out = oracle_mod.poisson_solver_separable(g, d["f"], order="raster", **kw)
    assert out.shape == d["out"].shape
    assert np.array_equal(out.view(np.uint32), d["out"].view(np.uint32))


@pytest.mark.parametrize("path", cases("conv_"), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_converged_fixture_against_fp64(oracle_mod, path):
    """The converged reference output is within its stated residual and close
    to the FP64 direct solve; the residual evaluator agrees with scipy's."""
    from oracle import fp64
    d = load(path)
    kind = d["extra"]["kind"]
    g, f, out = d["g"][0], None if d["f"] is None else d["f"][0], d["out"][0]
    rel = oracle_mod.rel_residual(out, g, f, kind)[0][0]
    assert rel < 1e-6
    assert abs(rel - fp64.rel_residual64(out, g, f, kind)) < 1e-9
    x = fp64.solve(g, f, kind)
    unk = np.isnan(g)
    err = np.abs(out[unk] - x[unk]).max() / np.abs(x[unk]).max()
    assert err < 1e-4
    assert np.array_equal(out[~unk].view(np.uint32), g[~unk].view(np.uint32))


def test_colour_order_converges_to_same_fixed_point(oracle_mod):
    """Raster and colour-ordered Gauss-Seidel share the fixed point."""
    rng = np.random.default_rng(3)
    g = rng.standard_normal((1, 20, 24)).astype(np.float32)
    g[0, 5:12, 6:15] = np.nan
    a = oracle_mod.poisson_solver_separable(g, niter=3000, scale=1, order="raster")
    b = oracle_mod.poisson_solver_separable(g, niter=3000, scale=1, order="colour")
    assert np.abs(a - b).max() < 1e-5


def test_live_reference_matches_oracle_random(oracle_mod):
    """Extra random cases against the live reference binary, where it exists."""
    if not oracle_mod.have_reference():
        pytest.skip("reference binary not built here")
    rng = np.random.default_rng(11)
    for k in range(6):
        pd, h, w = int(rng.integers(1, 4)), int(rng.integers(1, 30)), int(rng.integers(2, 30))
        g = rng.standard_normal((pd, h, w)).astype(np.float32)
        g[:, rng.random((h, w)) < 0.4] = np.nan
        args = [["-n", "9"], ["-c", "7", "-s", "3"], ["-t", "-0.05", "-n", "6"]][k % 3]
        ref = oracle_mod.run_reference(g, args=args)
        out = oracle_mod.poisson_solver_separable(g, **{k2: v for k2, v in parse_args(args, {}).items()})
        assert np.array_equal(ref.view(np.uint32), out.view(np.uint32))


def _mini_kw(args):
    opt = {"t": "0.45", "n": "10", "s": "99"}
    for k in range(0, len(args), 2):
        opt[args[k][1:]] = args[k + 1]
    return dict(tstep=float(np.float32(float(opt["t"]))), niter=int(float(opt["n"])),
                scale=int(float(opt["s"])))


@pytest.mark.parametrize("path", cases("mini_"), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_oracle_reproduces_minisimpois_bit_exact(oracle_mod, path):
    d = load(path)
    out = oracle_mod.poisson_recursive(d["g"], d["f"], order="raster", **_mini_kw(d["args"]))
    assert np.array_equal(out.view(np.uint32), d["out"].view(np.uint32))


@pytest.mark.parametrize("path", cases("amle_"), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_amle_oracle_reproduces_reference_bit_exact(oracle_mod, path):
    d = load(path)
    x, nn, niter, init = amle_inputs(d)
    out = oracle_mod.amle(x, nn=nn, niter=niter, init=init, order="raster")
    assert same_bits_or_nan(out, d["out"])


def test_amle_colourings_separate_every_neighbour(oracle_mod):
    """No neighbour offset of the first nn falls in the pixel's own class, so
    a class updates in parallel (the GPU sweep)."""
    offsets = [(1, 0), (0, 1), (-1, 0), (0, -1), (1, 1), (-1, -1), (-1, 1), (1, -1),
               (2, 1), (1, 2), (2, -1), (1, -2), (-2, -1), (-1, -2), (-2, 1), (-1, 2),
               (3, 1), (1, 3), (3, -1), (1, -3), (-3, -1), (-1, -3), (-3, 1), (-1, 3),
               (3, 2), (2, 3), (3, -2), (2, -3), (-3, -2), (-2, -3), (-3, 2), (-2, 3)]
    for nn in range(1, 33):
        m, k = oracle_mod.amle_colouring(nn)
        assert all((a + k * b) % m != 0 for a, b in offsets[:nn]), nn
    assert oracle_mod.amle_colouring(4) == (2, 1)


def test_amle_colour_order_converges_with_raster(oracle_mod):
    """With the 4-neighbourhood both sweep orders reach the same fixed point
    (and tinf meets tsup).  With 8 or more neighbours the weighted min/max
    iteration stalls with tinf and tsup apart (the reference's own gap stays
    ~0.04 here), so the two orders stop at different points: only the
    colour-ordered restatement is a bit-exact target for the GPU there."""
    rng = np.random.default_rng(8)
    from imscript_gb300 import synth
    x = synth.gaussian_field(rng, 24, 30, 3)[None]
    x[0, 6:18, 8:22] = np.nan
    a, ga = oracle_mod.amle(x, nn=4, niter=400, order="raster", gaps=True)
    b, gb = oracle_mod.amle(x, nn=4, niter=400, order="colour", gaps=True)
    assert np.abs(a - b).max() < 1e-5 and ga[0, 0] < 1e-5 and gb[0, 0] < 1e-5
