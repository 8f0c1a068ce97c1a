"""Adjoint kernel and torch.autograd.Function against FP64 references.

The loss is L = 0.5 * sum((u - T)^2) of the converged Poisson fill u of known
pixels g and guidance G (f = div G).  References: the FP64 adjoint formula
through a sparse FP64 factorisation, FP64 central finite differences on 64
coordinates (on a whole 1024 x 1024 image of the differentiation workload,
and on a 64 x 64 one), and torch autograd through a dense FP64 solve (64 x 64
crops).  Forward and adjoint solves run at rtol 1e-6, the setting the
benchmark and autograd.fill use.  Tolerance: 1e-5 of the gradient's largest
magnitude.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

REL = 1e-5


@pytest.fixture(scope="module")
def ag():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from imscript_gb300 import autograd
    return autograd


def _instance(seed, h, w):
    from imscript_gb300 import synth
    rng = np.random.default_rng(seed)
    base = synth.gaussian_field(rng, h, w, 8)
    gx, gy, _ = synth.guidance(synth.gaussian_field(rng, h, w, 8))
    m = synth.disk_mask(rng, h, w, 0.2, rmin=2, rmax=9)
    T = synth.gaussian_field(rng, h, w, 8)
    return base, m, gx, gy, T


def _fp64_loss(base, m, gx, gy, T):
    from oracle import fp64
    g = base.astype(np.float32).copy()
    g[m] = np.nan
    F = gx.astype(np.float64).copy()
    F[:, 1:] -= gx[:, :-1]
    F += gy
    F[1:, :] -= gy[:-1, :]
    A, b, idx = fp64.build_system(g, None, 0)
    b = b - F.ravel()[idx]
    import scipy.sparse.linalg as spla
    x = spla.spsolve(A.tocsc(), b)
    u = base.astype(np.float64).ravel().copy()
    u[idx] = x
    return 0.5 * np.sum((u - T.ravel()) ** 2), u, A, idx


def _gpu_grads(ag, base, m, gx, gy, T, rtol=1e-6):
    dev = "cuda"
    img = torch.tensor(base, device=dev, requires_grad=True)
    Gx = torch.tensor(gx, device=dev, requires_grad=True)
    Gy = torch.tensor(gy, device=dev, requires_grad=True)
    mask = torch.tensor(m, device=dev)
    g = torch.where(mask, torch.full_like(img, float("nan")), img)[None]
    f = ag.divergence(Gx, Gy)[None]
    u = ag.fill(g, f, rtol=rtol)
    loss = 0.5 * ((u[0] - torch.tensor(T, device=dev)) ** 2).sum()
    loss.backward()
    return (loss.item(), u.detach().cpu().numpy()[0], img.grad.cpu().numpy().astype(np.float64),
            Gx.grad.cpu().numpy().astype(np.float64), Gy.grad.cpu().numpy().astype(np.float64))


def test_adjoint_against_fp64_formula(ag):
    import scipy.sparse.linalg as spla
    base, m, gx, gy, T = _instance(0, 72, 90)
    L, u, A, idx = _fp64_loss(base, m, gx, gy, T)
    _, u_gpu, g_img, _, _ = _gpu_grads(ag, base, m, gx, gy, T)
    assert np.abs(u_gpu.ravel() - u).max() <= 1e-5 * np.abs(u).max()
    # FP64 adjoint: lambda = A^-1 (u - T)_U
    r = (u - T.ravel())
    lam = spla.spsolve(A.tocsc(), r[idx])
    h, w = base.shape
    lamimg = np.zeros(h * w)
    lamimg[idx] = lam
    lamimg = lamimg.reshape(h, w)
    want = r.reshape(h, w).copy()
    want[m] = 0
    nb = np.zeros_like(want)
    nb[:, :-1] += lamimg[:, 1:]
    nb[:, 1:] += lamimg[:, :-1]
    nb[:-1, :] += lamimg[1:, :]
    nb[1:, :] += lamimg[:-1, :]
    want[~m] += nb[~m]
    err = np.abs(g_img - want).max() / np.abs(want).max()
    assert err <= REL


def test_adjoint_against_central_differences(ag):
    base, m, gx, gy, T = _instance(1, 64, 64)
    _, _, g_img, g_gx, g_gy = _gpu_grads(ag, base, m, gx, gy, T)
    rng = np.random.default_rng(2)
    known = np.argwhere(~m)
    eps = 1e-3
    worst = 0.0
    scale = max(np.abs(g_img).max(), np.abs(g_gx).max(), np.abs(g_gy).max())
    for n in range(64):
        which = n % 3
        if which == 0:
            j, i = known[rng.integers(len(known))]
            arrs = [base, gx, gy]
            k = 0
        else:
            j, i = rng.integers(64), rng.integers(63 if which == 1 else 64)
            if which == 2:
                j = rng.integers(63)
            arrs = [base, gx, gy]
            k = which
        plus = [a.astype(np.float64).copy() for a in arrs]
        minus = [a.astype(np.float64).copy() for a in arrs]
        plus[k][j, i] += eps
        minus[k][j, i] -= eps
        Lp = _fp64_loss(plus[0], m, plus[1], plus[2], T)[0]
        Lm = _fp64_loss(minus[0], m, minus[1], minus[2], T)[0]
        fd = (Lp - Lm) / (2 * eps)
        got = [g_img, g_gx, g_gy][k][j, i]
        worst = max(worst, abs(fd - got) / scale)
    assert worst <= REL


def test_autograd_against_dense_fp64_solve(ag):
    """64x64 crop: torch autograd through a dense FP64 solve."""
    from oracle import fp64
    base, m, gx, gy, T = _instance(3, 64, 64)
    _, _, g_img, g_gx, g_gy = _gpu_grads(ag, base, m, gx, gy, T)
    g32 = base.astype(np.float32).copy()
    g32[m] = np.nan
    A, _, idx = fp64.build_system(g32, None, 0)
    Ad = torch.tensor(A.toarray(), dtype=torch.float64)
    img = torch.tensor(base, dtype=torch.float64, requires_grad=True)
    Gx = torch.tensor(gx, dtype=torch.float64, requires_grad=True)
    Gy = torch.tensor(gy, dtype=torch.float64, requires_grad=True)
    mask = torch.tensor(m)
    kimg = torch.where(mask, torch.zeros_like(img), img)
    # b = -f_U + sum of the known 5-neighbours (clamped border)
    from imscript_gb300.autograd import divergence
    f = divergence(Gx, Gy)
    nb = torch.zeros_like(kimg)
    nb[:, :-1] += kimg[:, 1:]
    nb[:, 1:] += kimg[:, :-1]
    nb[:-1, :] += kimg[1:, :]
    nb[1:, :] += kimg[:-1, :]
    tidx = torch.tensor(idx)
    b = (-f + nb).reshape(-1)[tidx]
    x = torch.linalg.solve(Ad, b)
    u = img.reshape(-1).clone()
    u = u.index_put((tidx,), x)
    loss = 0.5 * ((u - torch.tensor(T, dtype=torch.float64).reshape(-1)) ** 2).sum()
    loss.backward()
    for got, want in ((g_img, img.grad.numpy()), (g_gx, Gx.grad.numpy()), (g_gy, Gy.grad.numpy())):
        assert np.abs(got - want).max() <= REL * np.abs(want).max()


def _div64(gx, gy):
    F = gx.astype(np.float64).copy()
    F[:, 1:] -= gx[:, :-1]
    F += gy
    F[1:, :] -= gy[:-1, :]
    return F


def test_adjoint_1024_against_central_differences(ag):
    """A whole 1024 x 1024 image of the differentiation workload (15 % holes
    as blobs, 157k unknowns): 64 central differences of the FP64 loss, each
    two solves with one FP64 factorisation.  The loss is quadratic in the
    inputs, so the central difference is exact up to rounding for any step."""
    import scipy.sparse.linalg as spla
    from imscript_gb300 import synth
    from oracle import fp64
    insts, targets, guid = synth.config4(seed=5, n=1)
    g32 = insts[0].g[0]
    m = np.isnan(g32)
    base = np.nan_to_num(g32, nan=0.0)
    gx, gy = guid[0]
    T = targets[0]
    _, _, g_img, g_gx, g_gy = _gpu_grads(ag, base, m, gx, gy, T, rtol=1e-6)
    A, _, idx = fp64.build_system(g32, None, 0)
    p = fp64.nested_dissection(idx % g32.shape[1], idx // g32.shape[1], 1)
    lu = spla.splu(A[p][:, p].tocsc(), permc_spec="NATURAL", diag_pivot_thresh=0.0,
                   options=dict(SymmetricMode=True))

    def loss(img, Gx, Gy):
        gg = img.astype(np.float32).copy()
        gg[m] = np.nan
        _, b, _ = fp64.build_system(gg, None, 0)
        b = b - _div64(Gx, Gy).ravel()[idx]
        x = np.empty(idx.size)
        x[p] = lu.solve(b[p])
        u = img.astype(np.float64).ravel().copy()
        u[idx] = x
        return 0.5 * np.sum((u - T.ravel()) ** 2)

    # coordinates where the gradient goes through the solve: known pixels with
    # an unknown 4-neighbour, guidance samples whose divergence reaches an
    # unknown pixel; every third one anywhere
    h, w = m.shape
    near = np.zeros_like(m)
    near[:, :-1] |= m[:, 1:]
    near[:, 1:] |= m[:, :-1]
    near[:-1, :] |= m[1:, :]
    near[1:, :] |= m[:-1, :]
    rng = np.random.default_rng(11)
    scale = max(np.abs(g_img).max(), np.abs(g_gx).max(), np.abs(g_gy).max())
    eps = 0.25
    worst = 0.0
    for n in range(64):
        k = n % 3
        if k == 0:
            cand = np.argwhere(near & ~m) if n % 2 == 0 else np.argwhere(~m)
        else:
            cand = np.argwhere(m) if n % 2 == 0 else np.argwhere(np.ones_like(m))
        j, i = cand[rng.integers(len(cand))]
        arrs = [base.astype(np.float64), gx.astype(np.float64), gy.astype(np.float64)]
        plus = [a.copy() for a in arrs]
        minus = [a.copy() for a in arrs]
        plus[k][j, i] += eps
        minus[k][j, i] -= eps
        fd = (loss(*plus) - loss(*minus)) / (2 * eps)
        got = [g_img, g_gx, g_gy][k][j, i]
        worst = max(worst, abs(fd - got) / scale)
    print(f"\n1024x1024 adjoint at rtol 1e-6: worst |FD - adjoint| / max|grad| over 64 coordinates "
          f"{worst:.3e}")
    assert worst <= REL
