"""The autotuner's knobs.  The fused V-cycle's hand-over size (levels wider
than it run in the 32 x 32 tile kernels, the others in one shared-memory block
per channel) moves work between kernels without changing any result bit.  The
smoothing sweeps per side (1, 2 or 3; the tile kernels' halo is 4 or 8)
change the preconditioner: each count gives the bits of the per-sweep kernels
with that count, and meets the FP64 direct solve within 1e-4.  The tuner
picks one of the timed candidates and later solves reuse it."""
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


def _cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _images(seed, biharmonic=False):
    from imscript_gb300 import synth
    rng = np.random.default_rng(seed)
    out = []
    # a wide image (level 0 in the tile kernels), a 64 x 50 one (level 0 in
    # the shared-memory kernel whatever the hand-over) and a 300 x 140 one
    for (h, w, pd) in [(520, 610, 2), (50, 64, 1), (140, 300, 1)]:
        g = np.stack([synth.gaussian_field(rng, h, w, 8) for _ in range(pd)])
        m = synth.disk_mask(rng, h, w, 0.2 if biharmonic else 0.3, rmin=3, rmax=20 if biharmonic else 40)
        g[:, m] = np.nan
        if biharmonic:
            out.append((_cuda(g), None, -0.08))
        else:
            f = np.stack([synth.guidance(synth.gaussian_field(rng, h, w, 8))[2] for _ in range(pd)])
            out.append((_cuda(g), _cuda(f), 0.25))
    return out


def _ctx(sp):
    return sp.context(0, torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("biharmonic", [False, True])
def test_handover_size_changes_no_bit(sp, biharmonic):
    imgs = _images(11 + biharmonic, biharmonic)
    ctx = _ctx(sp)
    base = None
    try:
        for cm in (8, 32, 64, 128):
            ctx.set_coarse_max(cm)
            outs, reps = sp.solve_batch(imgs, rtol=1e-6, max_iter=4000)
            bits = [o.view(torch.int32).cpu() for o in outs]
            its = [r["iterations"] for r in reps]
            assert all(r["status"] == 0 and r["rel_residual"] <= 1e-6 for r in reps), reps
            if base is None:
                base = (bits, its)
                continue
            assert its == base[1], cm
            for a, b in zip(bits, base[0]):
                assert torch.equal(a, b), cm
    finally:
        ctx.set_coarse_max(0)


def test_handover_size_range_is_checked(sp):
    from imscript_gb300 import lib
    ctx = _ctx(sp)
    with pytest.raises(lib.SimpoisError):
        ctx.set_coarse_max(4)
    with pytest.raises(lib.SimpoisError):
        ctx.set_coarse_max(256)
    ctx.set_coarse_max(0)


def test_autotune_picks_a_candidate_and_keeps_the_bits(sp):
    imgs = _images(5)
    a, ra, tuned = sp.autotune(imgs, rtol=1e-6)
    cm = tuned["coarse_max"]
    assert cm in (32, 64, 128) and tuned["sweeps"] in (1, 2, 3)
    assert all(r["status"] == 0 and r["rel_residual"] <= 1e-6 for r in ra)
    b, rb = sp.solve_batch(imgs, rtol=1e-6)   # uses the tuned hand-over
    assert [r["iterations"] for r in ra] == [r["iterations"] for r in rb]
    for x, y in zip(a, b):
        assert torch.equal(x.view(torch.int32), y.view(torch.int32))
    # a fixed hand-over overrides the tuned one and is what autotune reports
    ctx = _ctx(sp)
    try:
        ctx.set_coarse_max(32)
        ctx.set_sweeps(tuned["sweeps"])
        c, rc, t2 = sp.autotune(imgs, rtol=1e-6)
        assert t2 == {"coarse_max": 32, "sweeps": tuned["sweeps"]}
        for x, y in zip(a, c):
            assert torch.equal(x.view(torch.int32), y.view(torch.int32))
    finally:
        ctx.set_coarse_max(0)
        ctx.set_sweeps(0)


def test_sweeps_range_is_checked(sp):
    from imscript_gb300 import lib
    ctx = _ctx(sp)
    with pytest.raises(lib.SimpoisError):
        ctx.set_sweeps(4)
    with pytest.raises(lib.SimpoisError):
        ctx.set_sweeps(-1)
    ctx.set_sweeps(0)


@pytest.mark.parametrize("sweeps", [1, 2, 3])
def test_every_sweep_count_equals_the_per_sweep_kernels(sp, sweeps):
    """The fused tile kernels with 1, 2 or 3 sweeps per side compute what the
    one-launch-per-sweep kernels with that count compute, bit for bit (widths
    that are and are not multiples of 4, small and large images)."""
    from imscript_gb300 import lib
    imgs = _images(23)
    ctx = _ctx(sp)
    try:
        ctx.set_sweeps(sweeps)
        a, ra = sp.solve_batch(imgs, rtol=1e-6)
        b, rb = sp.solve_batch(imgs, rtol=1e-6, flags=lib.FLAG_UNFUSED)
    finally:
        ctx.set_sweeps(0)
    assert [r["iterations"] for r in ra] == [r["iterations"] for r in rb]
    assert all(r["status"] == 0 and r["rel_residual"] <= 1e-6 for r in ra)
    for x, y in zip(a, b):
        assert torch.equal(x.view(torch.int32), y.view(torch.int32))


@pytest.mark.parametrize("sweeps", [1, 2, 3])
def test_every_candidate_meets_the_fp64_solve(sp, sweeps):
    """Every (hand-over, sweeps) candidate of the autotuner on uneven
    instances of the batched workload and a guided Poisson image: within 1e-4
    of the FP64 direct solve at rtol 1e-6."""
    from imscript_gb300 import synth
    from oracle import fp64
    insts = synth.config3(seed=7, n=12, smax=512) + [synth.config1(seed=3, size=384, channels=1)]
    ctx = _ctx(sp)
    try:
        ctx.set_sweeps(sweeps)
        for cm in (32, 64, 128):
            ctx.set_coarse_max(cm)
            outs, reps = sp.solve_batch([(_cuda(i.g), None if i.f is None else _cuda(i.f), i.tstep)
                                         for i in insts], rtol=1e-6)
            assert all(r["status"] == 0 and r["rel_residual"] <= 1e-6 for r in reps)
            if cm != 64:
                continue   # the hand-over changes no bit: one FP64 comparison per sweep count
            for inst, o in zip(insts, outs):
                o = o.cpu().numpy()
                for l in range(inst.g.shape[0]):
                    m = np.isnan(inst.g[l])
                    if not m.any():
                        continue
                    x = fp64.solve(inst.g[l], None if inst.f is None else inst.f[l], 0)
                    err = np.abs(o[l][m] - x[m]).max() / np.abs(x[m]).max()
                    assert err <= 1e-4, (sweeps, inst.meta, err)
    finally:
        ctx.set_sweeps(0)
        ctx.set_coarse_max(0)


_STREAMS = []


def _on_new_stream(fn):
    """Run fn on a stream of its own: simpois.context caches one context per
    stream, so this gives a context that has not tuned anything yet."""
    s = torch.cuda.Stream()
    _STREAMS.append(s)   # the cached context keeps the handle: keep the stream
    with torch.cuda.stream(s):
        out = fn()
    torch.cuda.synchronize()
    return out


def test_tuning_file_keeps_the_choice_across_contexts(sp, tmp_path):
    """A context with a tuning file writes its choice there; a new context
    reading the file solves the same shapes with the file's choice without
    timing (a choice planted in the file is the one reported and used)."""
    from imscript_gb300 import lib
    imgs = _images(31)
    path = tmp_path / "tune.txt"

    def first():
        sp.context(0, torch.cuda.current_stream().cuda_stream).set_tune_cache(path)
        return sp.autotune(imgs, rtol=1e-6)
    _, ra, tuned = _on_new_stream(first)
    assert all(r["status"] == 0 for r in ra)
    lines = path.read_text().splitlines()
    assert lines[0] == "simpois-tune 1" and lines[1].startswith("device ") and len(lines) == 3
    cm, nu, key = lines[2].split(" ", 2)
    assert (int(cm), int(nu)) == (tuned["coarse_max"], tuned["sweeps"])
    # plant another choice for the same shapes
    path.write_text("\n".join(lines[:2] + [f"32 3 {key}"]) + "\n")

    def second():
        ctx = sp.context(0, torch.cuda.current_stream().cuda_stream)
        ctx.set_tune_cache(path)
        outs, reps, t2 = sp.autotune(imgs, rtol=1e-6)
        ctx.set_coarse_max(32)
        ctx.set_sweeps(3)
        try:
            ref, _ = sp.solve_batch(imgs, rtol=1e-6)
        finally:
            ctx.set_coarse_max(0)
            ctx.set_sweeps(0)
        return outs, reps, t2, ref
    outs, reps, t2, ref = _on_new_stream(second)
    assert t2 == {"coarse_max": 32, "sweeps": 3}
    assert all(r["status"] == 0 and r["rel_residual"] <= 1e-6 for r in reps)
    for x, y in zip(outs, ref):
        assert torch.equal(x.view(torch.int32), y.view(torch.int32))


def test_tuning_file_errors(sp, tmp_path):
    """Not a tuning file, or a malformed choice: SIMPOIS_EINVAL and no file on
    the context; another device model's file reads as empty and is rewritten
    with this device's choice."""
    from imscript_gb300 import lib
    ctx = _ctx(sp)
    bad = tmp_path / "bad.txt"
    bad.write_text("hello\n")
    with pytest.raises(lib.SimpoisError):
        ctx.set_tune_cache(bad)
    dev = None
    good = tmp_path / "t.txt"
    imgs = _images(37)

    def tune():
        c = sp.context(0, torch.cuda.current_stream().cuda_stream)
        c.set_tune_cache(good)
        return sp.autotune(imgs, rtol=1e-6)
    _on_new_stream(tune)
    lines = good.read_text().splitlines()
    dev = lines[1]
    bad.write_text(f"simpois-tune 1\n{dev}\n32 x 0fm|10x10\n")
    with pytest.raises(lib.SimpoisError):
        ctx.set_tune_cache(bad)
    other = tmp_path / "other.txt"
    other.write_text("simpois-tune 1\ndevice 1.0 1 another GPU\n32 3 " + lines[2].split(" ", 2)[2] + "\n")

    def retune():
        c = sp.context(0, torch.cuda.current_stream().cuda_stream)
        c.set_tune_cache(other)
        return sp.autotune(imgs, rtol=1e-6)
    _, reps, t3 = _on_new_stream(retune)
    assert all(r["status"] == 0 for r in reps)
    rewritten = other.read_text().splitlines()
    assert rewritten[1] == dev and len(rewritten) == 3
    assert rewritten[2].split(" ", 2)[:2] == [str(t3["coarse_max"]), str(t3["sweeps"])]
    ctx.set_tune_cache(None)
