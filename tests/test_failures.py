"""Failure paths, made on the host: none of these faults, traps or hangs a GPU.

* CG breakdown.  The reference's CG (minicg.c:24-56) divides r.r by p.Ap with
  no guard: when the initial residual is exactly 0 -- here an all-zero image
  with a hole, so b = 0 and the start x0 = 0 -- alpha = 0/0 and every unknown
  of the output is NaN (the reference binary does this; the oracle, its
  restatement, too).  The GPU's reference schedule stops with
  SIMPOIS_BREAKDOWN and keeps the last (finite) iterate.
* A solve that cannot reach its tolerance within max_iter iterations ends
  with SIMPOIS_NOT_CONVERGED and a finite output.
* A context whose device-memory limit is below a solve's working set returns
  SIMPOIS_ENOMEM before it touches anything, and stays usable.
* The command on a truncated, corrupt or zero-sized npy file: the reference's
  warning for a short file (iio.c, "npy file smaller than expected"), a
  nonzero exit with a message for the others (the reference aborts on a bad
  magic and exits through xmalloc on a zero size, simpois.c:10-19).
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _zero_image_with_hole():
    g = np.zeros((1, 20, 24), np.float32)
    g[0, 5:12, 6:15] = np.nan
    return g


def test_oracle_breakdown_fills_nan_like_the_reference():
    from oracle import oracle
    g = _zero_image_with_hole()
    out = oracle.poisson_solver_separable(g, None, 0.25, 10, 1, -1)
    m = np.isnan(g)
    assert np.isnan(out[m]).all()
    assert np.array_equal(out[~m], g[~m])
    ref = os.path.join(ROOT, "oracle", "_ref", "simpois")
    if os.path.exists(ref):   # the reference binary itself, where it was built
        import tempfile
        with tempfile.TemporaryDirectory() as td:
            a, o = os.path.join(td, "a.npy"), os.path.join(td, "o.npy")
            np.save(a, g[0])
            subprocess.run([ref, "-i", a, "-c", "-1", "-s", "1", "-o", o], check=True,
                           capture_output=True)
            r = np.load(o)[..., 0]
            assert np.isnan(r[m[0]]).all()


@pytest.fixture(scope="module")
def cli():
    from imscript_gb300 import _build
    _build.build()
    return _build.CLI_BIN


def _npy_bytes(a):
    import io
    b = io.BytesIO()
    np.save(b, a)
    return b.getvalue()


def test_cli_corrupt_npy_exits_nonzero_with_a_message(cli, tmp_path):
    p = tmp_path / "bad.npy"
    p.write_bytes(b"\x00" * len(_npy_bytes(np.zeros((8, 9), np.float32))))
    r = subprocess.run([cli, "-i", str(p), "-o", str(tmp_path / "o.npy")], capture_output=True, text=True)
    assert r.returncode != 0
    assert "could not read image" in r.stderr


def test_cli_zero_sized_npy_exits_nonzero_with_a_message(cli, tmp_path):
    p = tmp_path / "zero.npy"
    np.save(p, np.zeros((0, 5), np.float32))
    r = subprocess.run([cli, "-i", str(p), "-o", str(tmp_path / "o.npy")], capture_output=True, text=True)
    assert r.returncode != 0
    assert "badly formed npy header" in r.stderr


def test_cli_negative_shape_npy_exits_nonzero(cli, tmp_path):
    b = bytearray(_npy_bytes(np.zeros((8, 9), np.float32)))
    hdr = bytes(b[10:10 + b[8] + 256 * b[9]])
    new = hdr.replace(b"(8, 9)", b"(-8, 9)")
    assert new.endswith(b" \n")
    new = new[:-2] + b"\n"   # one padding space less: the header keeps its length
    b[10:10 + len(hdr)] = new
    p = tmp_path / "neg.npy"
    p.write_bytes(bytes(b))
    r = subprocess.run([cli, "-i", str(p), "-o", str(tmp_path / "o.npy")], capture_output=True, text=True)
    assert r.returncode != 0


def test_cli_truncated_npy_warns_like_the_reference(cli, tmp_path):
    b = _npy_bytes(np.zeros((8, 9), np.float32))
    p = tmp_path / "trunc.npy"
    p.write_bytes(b[:-20])
    r = subprocess.run([cli, "-i", str(p), "-o", str(tmp_path / "o.npy")], capture_output=True, text=True)
    assert "npy file smaller than expected" in r.stderr


# ------------------------------------------------------------------ GPU

def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.gpu
def test_reference_schedule_breakdown_returns_status_and_finite_output():
    from imscript_gb300 import lib, simpois
    g = _zero_image_with_hole()
    out, reps = simpois.poisson_solver_separable(_dev(g), None, 0.25, 10, 1, -1,
                                                 allow=(lib.OK, lib.BREAKDOWN))
    o = out.cpu().numpy()
    assert reps[0]["status"] == lib.BREAKDOWN
    assert np.isfinite(o).all()
    m = np.isnan(g)
    assert np.array_equal(o[~m].view(np.uint32), g[~m].view(np.uint32))
    assert (o[m] == 0).all()   # the last iterate: the start, which is exact here
    # the host entry point reports it as the call's status
    ho, hreps = simpois.poisson_solver_separable(g, None, 0.25, 10, 1, -1, allow=(lib.OK, lib.BREAKDOWN))
    assert hreps[0]["status"] == lib.BREAKDOWN and np.isfinite(ho).all()


@pytest.mark.gpu
def test_converged_schedule_not_converged_within_max_iter():
    from imscript_gb300 import lib, simpois, synth
    inst = synth.config0(seed=0)
    out, reps = simpois.solve(_dev(inst.g), None, rtol=1e-6, max_iter=2,
                              allow=(lib.OK, lib.NOT_CONVERGED))
    assert reps[0]["status"] == lib.NOT_CONVERGED, reps
    assert reps[0]["iterations"] <= 2
    assert reps[0]["rel_residual"] > 1e-6
    assert np.isfinite(out.cpu().numpy()).all()


@pytest.mark.gpu
def test_memory_limit_returns_enomem_and_the_context_stays_usable():
    import torch
    from imscript_gb300 import lib, simpois, synth
    inst = synth.config0(seed=0)
    g = _dev(inst.g)
    out = torch.full_like(g, 7.0)
    # a private context on its own stream, so no cached arena is reused
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx = simpois.context(0, s.cuda_stream)
        ctx.set_memory_limit(1 << 20)
        with pytest.raises(lib.SimpoisError) as e:
            simpois.solve(g, None, rtol=1e-6, out=out)
        assert e.value.status == lib.ENOMEM
        assert "limit" in ctx.last_error()
        torch.cuda.synchronize()
        assert (out == 7.0).all()   # untouched
        ctx.set_memory_limit(0)
        out2, reps = simpois.solve(g, None, rtol=1e-6, out=out)
        torch.cuda.synchronize()
        assert reps[0]["status"] == lib.OK and reps[0]["rel_residual"] <= 1e-6


@pytest.mark.gpu
def test_cli_breakdown_warns_and_writes_a_finite_image(cli, tmp_path):
    g = _zero_image_with_hole()[0]
    a, o = str(tmp_path / "a.npy"), str(tmp_path / "o.npy")
    np.save(a, g)
    r = subprocess.run([cli, "-i", a, "-c", "-1", "-s", "1", "-o", o], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "breakdown" in r.stderr.lower()
    assert np.isfinite(np.load(o)).all()


@pytest.mark.gpu
def test_cli_truncated_npy_is_solved_like_the_reference(cli, tmp_path):
    b = _npy_bytes(np.zeros((8, 9), np.float32))
    p = tmp_path / "trunc.npy"
    p.write_bytes(b[:-20])
    r = subprocess.run([cli, "-i", str(p), "-o", str(tmp_path / "o.npy")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "npy file smaller than expected" in r.stderr
    assert np.load(tmp_path / "o.npy").shape[:2] == (8, 9)
