"""The converged schedule on the benchmark workloads at their full sizes,
against the FP64 converged solve (oracle/fp64.py: the system the reference's
CG solves, cleant_cgpois.c:197-264, factorised in float64) and against the
reference's own converged CG output (the oracle's bit-exact restatement of
`CG_EPS=rtol*|b| simpois -s 1 -c -1`, cleant_cgpois.c:197-278 over
minicg.c:24-56).

Bar: max |u_gpu - u_fp64| over the filled pixels <= 1e-4 * max |u_fp64| there,
per channel and per instance; known pixels bit for bit.  Each test prints the
errors it measured (``pytest -s``).

The FP64 solves run in a process pool started with `spawn` (a pool forked
after CUDA is initialised would hang)."""
import multiprocessing as mp
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-4


def _fp64_job(args):
    g, f, kind = args
    from oracle import fp64
    return fp64.solve(g, f, kind)


def _cg_job(args):
    g, f, rtol = args
    from oracle import oracle
    bn = float(oracle.rhs_norm(g[None], None if f is None else f[None], 0)[0])
    out, it, _ = oracle.cg_extension(g, f, init=np.zeros_like(g), maxit=-1, kind=0, cg_eps=rtol * bn)
    return out, it


@pytest.fixture(scope="module")
def pool():
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as p:
        yield p


def _dev(a):
    import torch
    return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _err(u, x, m):
    """max-abs error at the filled pixels relative to the FP64 solution's max there"""
    return float(np.abs(u[m].astype(np.float64) - x[m]).max() / max(np.abs(x[m]).max(), 1e-30))


def _check_known(out, g):
    known = ~np.isnan(g)
    assert np.array_equal(out[known].view(np.uint32), g[known].view(np.uint32))
    assert not np.isnan(out).any()


def test_poisson_guided_2048x2048x3_against_fp64(pool):
    from imscript_gb300 import simpois, synth
    inst = synth.config1(seed=0, rtol=1e-6)
    pd = inst.g.shape[0]
    jobs = pool.map_async(_fp64_job, [(inst.g[l], inst.f[l], 0) for l in range(pd)])
    out, reps = simpois.solve(_dev(inst.g), _dev(inst.f), tstep=inst.tstep, rtol=1e-6)
    out = out.cpu().numpy()
    _check_known(out, inst.g)
    errs = []
    for l, x in enumerate(jobs.get()):
        m = np.isnan(inst.g[l])
        assert reps[l]["status"] == 0 and reps[l]["rel_residual"] <= 1e-6
        errs.append(_err(out[l], x, m))
    print(f"\n2048x2048x3 guided Poisson, rtol 1e-6: max rel. error vs FP64 per channel {errs}")
    assert max(errs) <= REL, errs


def test_poisson_guided_2048_channel_against_reference_converged_cg(pool):
    """One whole 2048^2 channel against the reference's converged CG output
    (CG_EPS = 1e-7 |b|): the two converged solvers agree within 1e-4."""
    from imscript_gb300 import simpois, synth
    inst = synth.config1(seed=0, rtol=1e-6)
    g, f = inst.g[0], inst.f[0]
    job = pool.apply_async(_cg_job, ((g, f, 1e-7),))
    out, reps = simpois.solve(_dev(g[None]), _dev(f[None]), tstep=inst.tstep, rtol=1e-6)
    out = out.cpu().numpy()[0]
    ref, it = job.get()
    m = np.isnan(g)
    e = _err(out, ref.astype(np.float64), m)
    print(f"\n2048x2048 channel vs the reference's converged CG ({it} iterations): max rel. error {e:.3e}")
    assert np.array_equal(ref[~m].view(np.uint32), g[~m].view(np.uint32))
    assert e <= REL


def test_batch_of_256_uneven_instances_against_fp64(pool):
    from imscript_gb300 import simpois, synth
    insts = synth.config3(seed=0)
    chans = [(i.g[l], None if i.f is None else i.f[l], 0 if i.tstep > 0 else 1)
             for i in insts for l in range(i.g.shape[0])]
    jobs = pool.map_async(_fp64_job, chans, chunksize=1)
    outs, reps = simpois.solve_batch([(_dev(i.g), _dev(i.f), i.tstep) for i in insts], rtol=1e-6)
    outs = [o.cpu().numpy() for o in outs]
    xs = jobs.get()
    errs = []
    k = 0
    for n, inst in enumerate(insts):
        _check_known(outs[n], inst.g)
        for l in range(inst.g.shape[0]):
            assert reps[k]["status"] == 0 and reps[k]["rel_residual"] <= 1e-6, (n, l, reps[k])
            m = np.isnan(inst.g[l])
            if m.any():
                errs.append(_err(outs[n][l], xs[k], m))
            k += 1
    errs = np.array(errs)
    print(f"\n256 uneven instances ({len(errs)} channels), rtol 1e-6: max rel. error vs FP64 "
          f"{errs.max():.3e}, median {np.median(errs):.3e}")
    assert errs.max() <= REL


def test_biharmonic_4096x4096_against_fp64(pool):
    """The 13-point system of 1.23M unknowns (a 1024^2 square and 200
    scratches): the FP64 factorisation takes about a minute and 14 GB.

    The workload's own target, a relative residual of 1e-6, leaves an error
    of about 6e-4 against the FP64 solve: the operator's condition number is
    about 1e11 (its smallest eigenvalue ~ (pi/1024)^4), so a residual does not
    bound the error as it does for the 5-point systems.  That error is
    measured and bounded here; the 1e-4 agreement of two converged solvers is
    asserted on the solve to rtol 1e-8."""
    from imscript_gb300 import simpois, synth
    inst = synth.config2(seed=0)
    job = pool.apply_async(_fp64_job, ((inst.g[0], None, 1),))
    m = np.isnan(inst.g[0])
    errs = {}
    for rtol in (1e-6, 1e-8):
        out, reps = simpois.solve(_dev(inst.g), None, tstep=inst.tstep, rtol=rtol)
        out = out.cpu().numpy()
        _check_known(out, inst.g)
        assert reps[0]["status"] == 0 and reps[0]["rel_residual"] <= rtol, reps
        errs[rtol] = (out[0], reps[0]["iterations"])
    x = job.get()
    e6, e8 = (_err(errs[r][0], x, m) for r in (1e-6, 1e-8))
    print(f"\n4096x4096 biharmonic: max rel. error vs FP64 {e6:.3e} at rtol 1e-6 ({errs[1e-6][1]} PCG "
          f"iterations), {e8:.3e} at rtol 1e-8 ({errs[1e-8][1]} iterations)")
    assert e6 <= 2e-3
    assert e8 <= REL


def test_laplace_512x512_against_fp64(pool):
    from imscript_gb300 import simpois, synth
    inst = synth.config0(seed=0)
    x = pool.apply(_fp64_job, ((inst.g[0], None, 0),))
    out, reps = simpois.solve(_dev(inst.g), None, rtol=1e-6)
    out = out.cpu().numpy()
    _check_known(out, inst.g)
    e = _err(out[0], x, np.isnan(inst.g[0]))
    print(f"\n512x512 Laplace, rtol 1e-6: max rel. error vs FP64 {e:.3e}")
    assert e <= REL
