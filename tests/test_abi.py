"""CPU checks of the C-ABI library: it loads without a GPU, exports every
function include/simpois_gpu.h declares, and fails loudly (no CPU fallback)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def libmod():
    from imscript_gb300 import _build, lib
    _build.build_library()
    return lib


def header_functions():
    src = open(os.path.join(ROOT, "include", "simpois_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?(?:int|void|char|double|long long)\s*\*?\s*(\w+)\s*\(", src,
                       flags=re.M)
    return sorted(set(names))


def test_header_declares_the_expected_entry_points(libmod):
    assert set(header_functions()) == set(libmod.EXPORTS)


def test_library_exports_every_declared_symbol(libmod):
    L = ctypes.CDLL(libmod.library_path())
    for name in header_functions():
        assert hasattr(L, name), name


def test_defaults_match_the_reference_options(libmod):
    p = libmod.default_params()
    assert (p.tstep, p.niter, p.scale, p.cgit) == (np.float32(0.25), 10, 99, 0)
    assert (p.pmsfac, p.ponlit, p.cg_eps, p.rtol) == (3.0, 0.0, -1.0, 0.0)


def test_params_from_env(libmod, monkeypatch):
    monkeypatch.setenv("PMSFAC", "2.5")
    monkeypatch.setenv("PONLIT", "64")
    monkeypatch.setenv("CG_EPS", "1e-3")
    monkeypatch.setenv("SIMPOIS_RTOL", "1e-7")
    p = libmod.default_params()
    libmod.load().simpois_params_from_env(ctypes.byref(p))
    assert (p.pmsfac, p.ponlit, p.cg_eps, p.rtol) == (2.5, 64.0, 1e-3, 1e-7)
    monkeypatch.setenv("PMSFAC", "junk")
    q = libmod.default_params()
    libmod.load().simpois_params_from_env(ctypes.byref(q))
    assert q.pmsfac == 3.0


def test_strerror_covers_every_status(libmod):
    L = libmod.load()
    for st in range(8):
        assert L.simpois_strerror(st).decode() not in ("", "unknown status")


def test_no_cpu_fallback_without_gpu(libmod):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(libmod.SimpoisError):
        libmod.Context(0)
    from imscript_gb300 import simpois
    g = np.zeros((1, 4, 4), np.float32)
    with pytest.raises(libmod.SimpoisError):
        simpois.poisson_solver_separable(g)
