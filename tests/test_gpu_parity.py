"""GPU parity: the CUDA path (through the C ABI) against the oracle.

* reference schedule: bit-exact against the oracle's colour-ordered
  restatement (same float operations, same sweep classes), within 1e-5 where
  the FP64 CG runs (its dot products are summed in another order);
* converged schedule: within 1e-4 relative max-abs of the reference's own
  converged output (golden fixtures) and of the FP64 direct solve, FP64
  relative residual <= rtol, known pixels bit-exact.
"""
import numpy as np
import pytest

from golden_cases import cases, load, parse_args

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def sp():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from imscript_gb300 import simpois
    return simpois


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _run_ref_schedule(sp, g, f, kw, device):
    kw = dict(kw)
    opts = dict(tstep=kw.pop("tstep"), niter=kw.pop("niter"), scale=kw.pop("scale"),
                cgrad=kw.pop("cgrad"), pmsfac=kw.pop("pmsfac"), ponlit=kw.pop("ponlit"),
                cg_eps=kw.pop("cg_eps"))
    allow = (0, 4)
    if device:
        out, reps = sp.poisson_solver_separable(_cuda(g), None if f is None else _cuda(f), **opts,
                                                allow=allow)
        return out.cpu().numpy(), reps
    return sp.poisson_solver_separable(g, f, **opts, allow=allow)


@pytest.mark.parametrize("path", cases("pin_"), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_reference_schedule_matches_colour_oracle(sp, oracle_mod, path):
    d = load(path)
    kw = parse_args(d["args"], d["env"])
    g = d["g"]
    if d["mask"] is not None:
        g = oracle_mod.apply_mask(g, d["mask"])
    want = oracle_mod.poisson_solver_separable(g, d["f"], order="colour", **kw)
    got, reps = _run_ref_schedule(sp, g, d["f"], kw, device=True)
    if kw["cgrad"] == 0 or int(kw["cgrad"]) < -1:
        assert np.array_equal(_bits(got), _bits(want)), "GS/pyramid path must be bit-exact"
    else:
        fin = np.isfinite(want)
        scale = max(1.0, float(np.abs(want[fin]).max())) if fin.any() else 1.0
        assert np.array_equal(fin, np.isfinite(got))
        assert np.array_equal(_bits(got[~fin]), _bits(want[~fin]))
        assert np.allclose(got[fin], want[fin], rtol=0, atol=1e-5 * scale)
        known = ~np.isnan(g)
        assert np.array_equal(_bits(got[known]), _bits(g[known]))


def test_reference_schedule_host_entry_equals_device_entry(sp, oracle_mod):
    rng = np.random.default_rng(7)
    g = rng.standard_normal((2, 45, 61)).astype(np.float32)
    g[:, rng.random((45, 61)) < 0.3] = np.nan
    kw = parse_args(["-n", "17"], {})
    a, _ = _run_ref_schedule(sp, g, None, kw, device=False)
    b, _ = _run_ref_schedule(sp, g, None, kw, device=True)
    assert np.array_equal(_bits(a), _bits(b))
    want = oracle_mod.poisson_solver_separable(g, None, order="colour", **kw)
    assert np.array_equal(_bits(a), _bits(want))


@pytest.mark.parametrize("path", cases("conv_"), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_converged_matches_reference_converged(sp, oracle_mod, path):
    from oracle import fp64
    d = load(path)
    kind = d["extra"]["kind"]
    g, f, ref = d["g"], d["f"], d["out"]
    tstep = -0.08 if kind else 0.25
    out, reps = sp.poisson_solver_separable(_cuda(g), None if f is None else _cuda(f), tstep,
                                            rtol=1e-6)
    out = out.cpu().numpy()
    unk = np.isnan(g)
    assert np.array_equal(_bits(out[~unk]), _bits(g[~unk])), "known pixels must be bit-exact"
    r = reps[0]
    assert r["status"] == 0 and r["rel_residual"] <= 1e-6
    scale = np.abs(ref[unk]).max()
    assert np.abs(out[unk] - ref[unk]).max() <= 1e-4 * scale
    x = fp64.solve(g[0], None if f is None else f[0], kind)
    assert np.abs(out[0][unk[0]] - x[unk[0]]).max() <= 1e-4 * np.abs(x[unk[0]]).max()
    rel = oracle_mod.rel_residual(out, g, f, kind)[0][0]
    assert rel < 2e-6, "FP32 output stays near the storage floor"


def _random_case(rng, h, w, frac, rmax, with_f, kind):
    from imscript_gb300 import synth
    img = synth.gaussian_field(rng, h, w, 8)
    m = synth.disk_mask(rng, h, w, frac, rmin=1.5, rmax=rmax)
    img[m] = np.nan
    f = None
    if with_f:
        f = synth.guidance(synth.gaussian_field(rng, h, w, 8))[2][None]
    return img[None], f


@pytest.mark.parametrize("kind,h,w,frac,rmax,with_f", [
    (0, 96, 128, 0.3, 14, False), (0, 130, 77, 0.5, 20, True), (0, 33, 300, 0.2, 9, True),
    (0, 1, 200, 0.4, 3, False), (0, 200, 1, 0.4, 3, True), (0, 7, 5, 0.5, 2, False),
    (1, 64, 80, 0.15, 6, False), (1, 71, 53, 0.2, 5, True),
])
def test_converged_random_vs_fp64(sp, oracle_mod, kind, h, w, frac, rmax, with_f):
    from oracle import fp64
    rng = np.random.default_rng(h * 1000 + w + kind)
    g, f = _random_case(rng, h, w, frac, rmax, with_f, kind)
    if not np.isnan(g).any() or np.isnan(g).all():
        pytest.skip("degenerate draw")
    tstep = -0.08 if kind else 0.25
    out, reps = sp.poisson_solver_separable(_cuda(g), None if f is None else _cuda(f), tstep,
                                            rtol=1e-6, flags=4)
    out = out.cpu().numpy()
    r = reps[0]
    assert r["status"] == 0, r
    assert r["rel_residual"] <= 1e-6
    unk = np.isnan(g[0])
    x = fp64.solve(g[0], None if f is None else f[0], kind)
    err = np.abs(out[0][unk] - x[unk]).max() / max(np.abs(x[unk]).max(), 1e-30)
    assert err <= 1e-4
    rel_cpu = oracle_mod.rel_residual(out, g, f, kind)[0][0]
    assert abs(rel_cpu - r["rel_residual_out"]) <= 1e-3 * rel_cpu + 1e-12


def test_batched_equals_plain_bit_exact(sp):
    """Each problem of a batch computes exactly what it computes alone."""
    from imscript_gb300 import synth
    insts = synth.config3(seed=5, n=6, smin=40, smax=150)
    imgs = [(_cuda(i.g), None if i.f is None else _cuda(i.f)) for i in insts]
    outs, reps = sp.solve_batch(imgs, rtol=1e-6)
    k = 0
    for (g, f), o in zip(imgs, outs):
        solo, r1 = sp.solve(g, f, rtol=1e-6)
        assert torch.equal(o.view(torch.int32), solo.view(torch.int32))
        for rr in r1:
            assert reps[k]["iterations"] == rr["iterations"]
            assert reps[k]["rel_residual"] <= 1e-6
            k += 1


@pytest.mark.parametrize("h,w,pd", [(300, 260, 2), (129, 517, 1)])
def test_fused_cycle_equals_per_sweep_kernels(sp, h, w, pd):
    """The fused tile kernels compute what the one-launch-per-sweep kernels
    compute, bit for bit (images wider than the shared-memory coarse levels)."""
    from imscript_gb300 import lib, synth
    rng = np.random.default_rng(h + w)
    g = np.stack([synth.gaussian_field(rng, h, w, 8) for _ in range(pd)])
    m = synth.disk_mask(rng, h, w, 0.3, rmin=3, rmax=25)
    g[:, m] = np.nan
    f = np.stack([synth.guidance(synth.gaussian_field(rng, h, w, 8))[2] for _ in range(pd)])
    a, ra = sp.solve(_cuda(g), _cuda(f), rtol=1e-6)
    b, rb = sp.solve(_cuda(g), _cuda(f), rtol=1e-6, flags=lib.FLAG_UNFUSED)
    assert [r["iterations"] for r in ra] == [r["iterations"] for r in rb]
    assert torch.equal(a.view(torch.int32), b.view(torch.int32))


def test_kernel_timer_replay_is_identical(sp):
    """SIMPOIS_FLAG_KTIMER issues the same kernels eagerly with CUDA events
    around them: same bits as the graph-launched solve, and per-kernel stats."""
    from imscript_gb300 import lib, synth
    inst = synth.config1(seed=3, size=300, channels=2)
    g, f = _cuda(inst.g), _cuda(inst.f)
    ctx = sp.context(0, torch.cuda.current_stream().cuda_stream)
    ctx.reset_kernel_stats()
    a, ra = sp.solve(g, f, rtol=1e-6)
    b, rb = sp.solve(g, f, rtol=1e-6, flags=lib.FLAG_KTIMER)
    assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    st = ctx.kernel_stats()
    for name in ("k_pre5", "k_post5", "k_coarse5", "k_spmv5", "k_resid5"):
        assert st[name]["launches"] > 0 and st[name]["ms"] > 0 and st[name]["bytes"] > 0, name


def test_fused_small_problems_close_to_per_sweep(sp):
    """Images no wider than the shared-memory coarse levels: same answer
    (only the order of one FP64 sum differs)."""
    from imscript_gb300 import lib
    rng = np.random.default_rng(4)
    g, f = _random_case(rng, 100, 120, 0.3, 10, True, 0)
    a, ra = sp.solve(_cuda(g), _cuda(f), rtol=1e-6)
    b, rb = sp.solve(_cuda(g), _cuda(f), rtol=1e-6, flags=lib.FLAG_UNFUSED)
    assert ra[0]["rel_residual"] <= 1e-6 and rb[0]["rel_residual"] <= 1e-6
    a, b = a.cpu().numpy(), b.cpu().numpy()
    assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max()


def test_all_known_and_all_unknown(sp, oracle_mod):
    rng = np.random.default_rng(1)
    g = rng.standard_normal((1, 20, 30)).astype(np.float32)
    out, reps = sp.poisson_solver_separable(_cuda(g), rtol=1e-6)
    assert np.array_equal(_bits(out.cpu().numpy()), _bits(g))
    assert reps[0]["unknowns"] == 0 and reps[0]["rel_residual"] == 0
    # no known pixel: singular; the reference schedule's answer is returned
    gn = np.full((1, 12, 9), np.nan, np.float32)
    f = (rng.standard_normal(gn.shape) * 0.1).astype(np.float32)
    out, reps = sp.poisson_solver_separable(_cuda(gn), _cuda(f), rtol=1e-6)
    assert reps[0]["status"] == 7
    want = oracle_mod.poisson_solver_separable(gn, f, order="colour")
    assert np.array_equal(_bits(out.cpu().numpy()), _bits(want))


def test_residual_entry_matches_oracle(sp, oracle_mod):
    rng = np.random.default_rng(3)
    g, f = _random_case(rng, 60, 70, 0.3, 8, True, 0)
    u = np.where(np.isnan(g), rng.standard_normal(g.shape).astype(np.float32), g)
    for kind in (0, 1):
        rel, bn = sp.residual(_cuda(u), _cuda(g), _cuda(f), kind)
        want, wbn = oracle_mod.rel_residual(u, g, f, kind)
        assert abs(rel[0] - want[0]) <= 1e-9 * want[0]
        assert abs(bn[0] - wbn[0]) <= 1e-9 * wbn[0]


def test_dropin_symbol_matches_oracle(sp, oracle_mod):
    """poisson_solver_separable with the reference's exact signature."""
    import ctypes
    from imscript_gb300 import lib
    L = lib.load()
    rng = np.random.default_rng(9)
    g = rng.standard_normal((3, 23, 31)).astype(np.float32)
    g[:, rng.random((23, 31)) < 0.35] = np.nan
    out = np.zeros_like(g)
    L.poisson_solver_separable(out.ctypes.data, g.ctypes.data, None, 31, 23, 3,
                               ctypes.c_float(0.25), 25, 99, ctypes.c_float(0))
    want = oracle_mod.poisson_solver_separable(g, None, niter=25, order="colour")
    assert np.array_equal(_bits(out), _bits(want))


@pytest.mark.parametrize("path", cases("mini_"), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_minisimpois_variant_matches_colour_oracle(sp, oracle_mod, path):
    """The ftr viewers' GS-only pyramid (SIMPOIS_FLAG_MINI), bit for bit."""
    from imscript_gb300 import lib
    from test_oracle_golden import _mini_kw
    d = load(path)
    kw = _mini_kw(d["args"])
    want = oracle_mod.poisson_recursive(d["g"], d["f"], order="colour", **kw)
    got, _ = sp.poisson_solver_separable(_cuda(d["g"]), None if d["f"] is None else _cuda(d["f"]),
                                         kw["tstep"], kw["niter"], kw["scale"], 0, flags=lib.FLAG_MINI)
    assert np.array_equal(_bits(got.cpu().numpy()), _bits(want))


def test_poisson_recursive_dropin_in_place(sp, oracle_mod):
    """poisson_recursive(strip, strip, 0, w, h, 0.25, 10, 99) as ftr/vnav.c:855 calls it."""
    import ctypes
    from imscript_gb300 import lib
    rng = np.random.default_rng(12)
    g = rng.standard_normal((40, 33)).astype(np.float32)
    g[rng.random((40, 33)) < 0.3] = np.nan
    want = oracle_mod.poisson_recursive(g, None, 0.25, 10, 99, order="colour")[0]
    strip = g.copy()
    lib.load().poisson_recursive(strip.ctypes.data, strip.ctypes.data, None, 33, 40,
                                 ctypes.c_float(0.25), 10, 99)
    assert np.array_equal(_bits(strip), _bits(want))


@pytest.mark.parametrize("h,w,seed", [(50, 64, 1), (50, 65, 12), (64, 64, 12), (40, 40, 12), (40, 40, 1),
                                      (20, 30, 12)])
def test_biharmonic_small_images_converge(sp, h, w, seed):
    """Small biharmonic fills whose holes run into the border: the FP64 PCG
    with the squared 5-point V-cycle as FP32 preconditioner takes the
    flexible beta and converges in one refinement step (the classical
    r.z / rho_old stalled here for thousands of iterations)."""
    from imscript_gb300 import synth
    rng = np.random.default_rng(seed)
    g = synth.gaussian_field(rng, h, w, 8)[None]
    m = synth.disk_mask(rng, h, w, 0.2, rmin=3, rmax=20)
    g[:, m] = np.nan
    out, reps = sp.solve_batch([(_cuda(g), None, -0.08)], rtol=1e-6, max_iter=3000)
    r = reps[0]
    assert r["status"] == 0 and r["rel_residual"] <= 1e-6
    assert r["iterations"] <= 200 and r["refinements"] == 1, r
    o = out[0].cpu().numpy()
    assert np.array_equal(_bits(o[:, ~m]), _bits(g[:, ~m]))


def test_unaligned_caller_buffers(sp):
    """Input and output planes that start 4 bytes past a 16-byte boundary (a
    width that is a multiple of 4 would otherwise take the vector path): the
    same bits as aligned buffers."""
    from imscript_gb300 import synth
    rng = np.random.default_rng(21)
    h, w = 200, 256
    g = synth.gaussian_field(rng, h, w, 8)[None]
    g[:, synth.disk_mask(rng, h, w, 0.3, rmin=3, rmax=25)] = np.nan
    a, ra = sp.solve_batch([_cuda(g)], rtol=1e-6)
    buf = torch.empty(h * w + 8, dtype=torch.float32, device="cuda")
    gin = buf[1:1 + h * w].view(1, h, w)
    gin.copy_(_cuda(g))
    obuf = torch.empty(h * w + 8, dtype=torch.float32, device="cuda")
    out = obuf[3:3 + h * w].view(1, h, w)
    b, rb = sp.solve_batch([gin], rtol=1e-6, outs=[out])
    assert ra[0]["iterations"] == rb[0]["iterations"]
    assert torch.equal(a[0].view(torch.int32), b[0].view(torch.int32))


@pytest.mark.parametrize("h,w", [(1, 300), (300, 1), (2, 2), (3, 1000), (1000, 3), (65, 1)])
def test_converged_thin_images(sp, h, w):
    """Rows, columns and tiny images on the converged schedule: FP64
    residual <= rtol, close to the FP64 direct solve, knowns bit-exact."""
    from oracle import fp64
    rng = np.random.default_rng(h * 7 + w)
    g = (rng.standard_normal((1, h, w)) * 0.3 + 1).astype(np.float32)
    m = rng.random((h, w)) < 0.5
    m.flat[0] = False           # at least one known pixel
    g[:, m] = np.nan
    f = (rng.standard_normal((1, h, w)) * 0.01).astype(np.float32)
    for kind, t in ((0, 0.25), (1, -0.08)):
        out, reps = sp.solve(_cuda(g), _cuda(f) if kind == 0 else None, tstep=t, rtol=1e-6, max_iter=5000)
        r = reps[0]
        assert r["status"] == 0 and r["rel_residual"] <= 1e-6, (kind, r)
        o = out.cpu().numpy()[0]
        x = fp64.solve(g[0], f[0] if kind == 0 else None, kind)
        assert np.abs(o[m] - x[m]).max() <= 1e-4 * max(1.0, np.abs(x[m]).max())
        assert np.array_equal(_bits(o[~m]), _bits(g[0][~m]))


@pytest.mark.parametrize("h,w,pd", [(384, 512, 2), (330, 640, 1), (200, 520, 1)])
def test_tma_region_loads_same_bits(sp, h, w, pd):
    """SIMPOIS_FLAG_TMA: the tile kernels load their regions through the
    tensor memory accelerator where a level's rows are 16-byte multiples;
    the result is the same bits as the vector loads' (and as the unfused
    kernels')."""
    from imscript_gb300 import lib, synth
    rng = np.random.default_rng(h + w + pd)
    g = np.stack([synth.gaussian_field(rng, h, w, 8) for _ in range(pd)])
    g[:, synth.disk_mask(rng, h, w, 0.25, rmin=3, rmax=30)] = np.nan
    f = np.stack([synth.guidance(synth.gaussian_field(rng, h, w, 8))[2] for _ in range(pd)])
    a, ra = sp.solve(_cuda(g), _cuda(f), rtol=1e-6)
    b, rb = sp.solve(_cuda(g), _cuda(f), rtol=1e-6, flags=lib.FLAG_TMA)
    c, rc = sp.solve(_cuda(g), _cuda(f), rtol=1e-6, flags=lib.FLAG_UNFUSED)
    assert [r["iterations"] for r in ra] == [r["iterations"] for r in rb] == [r["iterations"] for r in rc]
    assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    assert torch.equal(a.view(torch.int32), c.view(torch.int32))
