"""The simpois command: texts, argument handling, exit codes and image I/O
against the reference command's own behaviour (fixtures from the reference
binary, tests/golden/cli.json and io.json); end-to-end solves on the GPU."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def cli():
    from imscript_gb300 import _build
    _build.build()
    return _build.CLI_BIN


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("h") / "imageio_harness")
    cli_dir = os.path.join(ROOT, "imscript_gb300", "cli")
    subprocess.run(["gcc", "-O1", "-std=gnu99", "-I", cli_dir, os.path.join(ROOT, "tests", "imageio_harness.c"),
                    os.path.join(cli_dir, "imageio.c"), "-o", out, "-lm"], check=True)
    return out


def _fixtures(name):
    with open(os.path.join(GOLDEN, name)) as fh:
        return json.load(fh)


@pytest.mark.parametrize("arg", ["-h", "--help", "--version", "-?"])
def test_help_texts(cli, arg):
    want = _fixtures("cli.json")[arg]
    r = subprocess.run([cli, arg], capture_output=True, text=True)
    assert (r.stdout, r.stderr, r.returncode) == (want["stdout"], want["stderr"], want["rc"])


def test_stray_argument_prints_usage_and_fails(cli):
    want = _fixtures("cli.json")["stray"]
    r = subprocess.run([cli, "-n", "3", "stray"], capture_output=True, text=True)
    assert r.returncode == want["rc"] == 1
    assert r.stderr.replace(cli, "ARGV0") == want["stderr"]


@pytest.mark.parametrize("which,flag", [("mismatch_if", "-f"), ("mismatch_im", "-m")])
def test_size_mismatch_exit_codes(cli, tmp_path, which, flag):
    want = _fixtures("cli.json")[which]
    a, b = str(tmp_path / "a.npy"), str(tmp_path / "b.npy")
    np.save(a, np.zeros((4, 5, 1), np.float32))
    np.save(b, np.zeros((4, 6, 1), np.float32))
    r = subprocess.run([cli, "-i", a, flag, b, "-o", str(tmp_path / "o.npy")], capture_output=True,
                       text=True)
    assert (r.stderr, r.returncode) == (want["stderr"], want["rc"])


IO = None


def _io():
    global IO
    if IO is None:
        IO = _fixtures("io.json")
    return IO


@pytest.mark.parametrize("tag", ["c3", "c1"])
@pytest.mark.parametrize("ext", ["npy", "pfm", "ppm", "pgm", "asc", "tif", "txt"])
def test_writers_match_reference_bytes(harness, tmp_path, tag, ext):
    rng = np.random.default_rng(77)
    img3 = (rng.random((5, 7, 3)) * 200).astype(np.float32)
    img1 = (rng.random((6, 4, 1)) * 200).astype(np.float32)
    src = str(tmp_path / "src.npy")
    np.save(src, img3 if tag == "c3" else img1)
    dst = str(tmp_path / f"out.{ext}")
    subprocess.run([harness, "write", src, dst], check=True)
    assert list(open(dst, "rb").read()) == _io()[f"write_{tag}_{ext}"]


@pytest.mark.parametrize("key", ["u8_hw", "i16_hwc", "f8_hwc", "u2_hw", "p2", "p5", "p6"])
def test_readers_match_reference(harness, tmp_path, key):
    d = _io()[f"read_{key}"]
    src = str(tmp_path / ("in.npy" if "_" in key else key))
    open(src, "wb").write(bytes(d["in"]))
    dst = str(tmp_path / "o.npy")
    subprocess.run([harness, "read", src, dst], check=True)
    assert list(open(dst, "rb").read()) == d["out"]


def test_gray_mask_conversion_matches_reference(harness, tmp_path):
    d = _io()["mask_rgb"]
    mp = str(tmp_path / "m.ppm")
    open(mp, "wb").write(bytes(d["mask"]))
    dst = str(tmp_path / "m.npy")
    subprocess.run([harness, "gray", mp, dst], check=True)
    gray = np.load(dst)[..., 0]
    g = np.array(d["g"], np.float32).reshape(gray.shape)
    ref = np.frombuffer(bytes(d["out"]), np.uint8)
    out = np.load(dst.replace("m.npy", "m.npy"))
    want = np.where(gray > 0, np.nan, g)
    # the reference (-n 0) filled nothing: NaN where the gray mask is > 0
    import io
    refimg = np.load(io.BytesIO(bytes(d["out"])))[..., 0]
    assert np.array_equal(np.isnan(refimg), np.isnan(want))
    assert ref.size > 0 and out.size > 0


@pytest.mark.gpu
def test_cli_end_to_end_matches_oracle(cli, tmp_path, oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rng = np.random.default_rng(5)
    g = rng.standard_normal((2, 40, 52)).astype(np.float32)
    g[:, rng.random((40, 52)) < 0.3] = np.nan
    f = (rng.standard_normal(g.shape) * 0.1).astype(np.float32)
    pi, pf, po = str(tmp_path / "i.npy"), str(tmp_path / "f.npy"), str(tmp_path / "o.npy")
    np.save(pi, oracle_mod.to_hwc(g))
    np.save(pf, oracle_mod.to_hwc(f))
    env = {k: v for k, v in os.environ.items() if k not in ("PMSFAC", "PONLIT", "CG_EPS", "SIMPOIS_RTOL")}
    subprocess.run([cli, "-i", pi, "-f", pf, "-n", "12", "-o", po], check=True, env=env)
    got = oracle_mod.from_hwc(np.load(po))
    want = oracle_mod.poisson_solver_separable(g, f, niter=12, order="colour")
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # stdin -> stdout, mask file, converged schedule through SIMPOIS_RTOL
    pm = str(tmp_path / "m.npy")
    m = (rng.random((40, 52)) < 0.2).astype(np.float32)
    np.save(pm, m)
    env2 = dict(env, SIMPOIS_RTOL="1e-6")
    r = subprocess.run([cli, "-m", pm], input=open(pi, "rb").read(), capture_output=True, env=env2,
                       check=True)
    import io
    out = oracle_mod.from_hwc(np.load(io.BytesIO(r.stdout)))
    gm = oracle_mod.apply_mask(g, m)
    rel, _ = oracle_mod.rel_residual(out, gm, None, 0)
    assert np.all(rel < 2e-6)
    known = ~np.isnan(gm)
    assert np.array_equal(out[known].view(np.uint32), gm[known].view(np.uint32))


# ------------------------------------------------------------------ the amle command

@pytest.fixture(scope="module")
def amle_cli():
    from imscript_gb300 import _build
    _build.build()
    return _build.AMLE_BIN


@pytest.mark.parametrize("arg", ["-h", "--help", "--version", "-?"])
def test_amle_help_texts(amle_cli, arg):
    want = _fixtures("amle_cli.json")[arg]
    r = subprocess.run([amle_cli, arg], capture_output=True, text=True)
    assert (r.stdout, r.stderr, r.returncode) == (want["stdout"], want["stderr"], want["rc"])


def test_amle_extra_arguments_print_usage(amle_cli):
    want = _fixtures("amle_cli.json")["extra_args"]
    r = subprocess.run([amle_cli, "a", "b", "c", "d"], capture_output=True, text=True)
    assert (r.stderr.replace(amle_cli, "ARGV0"), r.returncode) == (want["stderr"], want["rc"])


def test_amle_mask_size_mismatch_fails(amle_cli, tmp_path):
    want = _fixtures("amle_cli.json")["mask_mismatch"]
    a, b = str(tmp_path / "a.npy"), str(tmp_path / "b.npy")
    np.save(a, np.zeros((4, 5, 1), np.float32))
    np.save(b, np.zeros((4, 6, 1), np.float32))
    r = subprocess.run([amle_cli, a, b, str(tmp_path / "o.npy")], capture_output=True, text=True)
    assert r.returncode == want["rc"] == 255
    assert r.stderr.strip().endswith(want["tail"])


@pytest.mark.gpu
def test_amle_command_writes_the_reference_bytes(amle_cli, tmp_path):
    want = _fixtures("amle_cli.json")["file"]
    x = np.array(want["in"], np.float32).reshape(4, 5)
    a, o = str(tmp_path / "a.npy"), str(tmp_path / "o.npy")
    np.save(a, x)
    env = dict(os.environ, AMLE_NITER="1")
    subprocess.run([amle_cli, a, "", o], check=True, env=env, capture_output=True)
    assert list(open(o, "rb").read()) == want["out_bytes"]


@pytest.mark.parametrize("name,shape,value", [("zero:6x4,3", (4, 6, 3), 0.0), ("one:3x2", (2, 3, 1), 1.0),
                                              ("constant:1.5:7x5", (5, 7, 1), 1.5),
                                              ("constant:-2e-3:2x9", (9, 2, 1), np.float32(-2e-3))])
def test_semantic_image_names(harness, tmp_path, name, shape, value):
    """iio's semantic names read as images (iio.c:5604-5633); where the
    reference binary is built here, its reading of the same name agrees."""
    dst = str(tmp_path / "o.npy")
    subprocess.run([harness, "read", name, dst], check=True)
    got = np.load(dst)
    assert got.reshape(shape[0], shape[1], -1).shape == shape
    assert np.all(got == np.float32(value))
    from oracle import oracle as O
    if O.have_reference():
        ref = str(tmp_path / "r.npy")
        subprocess.run([O.REF_BIN, "-i", name, "-n", "0", "-o", ref], check=True, capture_output=True)
        assert open(ref, "rb").read() == open(dst, "rb").read()


def test_bad_semantic_name_fails(harness, tmp_path):
    r = subprocess.run([harness, "read", "zero:axb", str(tmp_path / "o.npy")], capture_output=True, text=True)
    assert r.returncode != 0 and "bad semantical name" in r.stderr


# iio's transformations on reading (iio.c:3796-3884, 5677-5705); the
# reference command filled the cells a negative trim pads (NaN here), so those
# are compared by position only
_PADDED = {"x=-2": 30, "y=-1,h=7": 42, "w=9": 30}


def _read_with(harness, tmp_path, name, env_list):
    dst = str(tmp_path / "o.npy")
    env = {k: v for k, v in os.environ.items() if k != "IIO_TRANS"}
    if env_list:
        env["IIO_TRANS"] = env_list
    subprocess.run([harness, "read", name, dst], check=True, env=env)
    return np.load(dst)


def _trans_src(tmp_path):
    d = _fixtures("trans.json")
    src = str(tmp_path / "in.npy")
    np.save(src, np.array(d["in"], np.float32).reshape(d["shape"]))
    return d, src


def _same_where_known(got, want, padded):
    nan = np.isnan(got)
    assert int(nan.sum()) == padded
    assert np.array_equal(got[~nan], want[~nan])


@pytest.mark.parametrize("lst", json.load(open(os.path.join(GOLDEN, "trans.json")))["env"].keys())
def test_iio_trans_matches_reference(harness, tmp_path, lst):
    d, src = _trans_src(tmp_path)
    want = d["env"][lst]
    got = _read_with(harness, tmp_path, src, lst)
    assert list(got.shape) == want["shape"]
    _same_where_known(got, np.array(want["out"], np.float32).reshape(want["shape"]), _PADDED.get(lst, 0))


@pytest.mark.parametrize("key", json.load(open(os.path.join(GOLDEN, "trans.json")))["prefix"].keys())
def test_trans_prefix_matches_reference(harness, tmp_path, key):
    """TRANS[list]:name, alone and with IIO_TRANS (applied to the inner read
    and again to the outer one)."""
    d, src = _trans_src(tmp_path)
    lst, env = key.split("|")
    want = d["prefix"][key]
    got = _read_with(harness, tmp_path, f"TRANS[{lst}]:{src}", env)
    assert list(got.shape) == want["shape"]
    assert np.array_equal(got, np.array(want["out"], np.float32).reshape(want["shape"]))


def test_iio_trans_errors(harness, tmp_path):
    _, src = _trans_src(tmp_path)
    for lst in ("flip=XYZ", "x=7", "h=0"):
        env = dict(os.environ, IIO_TRANS=lst)
        r = subprocess.run([harness, "read", src, str(tmp_path / "o.npy")], capture_output=True, text=True, env=env)
        assert r.returncode != 0, lst
    # a failing pipe leaves the image as it was
    got = _read_with(harness, tmp_path, src, "pipe=false")
    d = _fixtures("trans.json")
    assert np.array_equal(got, np.array(d["in"], np.float32).reshape(d["shape"]))


@pytest.mark.parametrize("key", json.load(open(os.path.join(GOLDEN, "text.json"))).keys())
def test_text_formats_match_reference(harness, tmp_path, key):
    """CSV, TXT and an ASC-looking TXT read as the reference reads them
    (iio.c:2992-3071, 5260-5400)."""
    d = _fixtures("text.json")[key]
    src = str(tmp_path / key)
    open(src, "w").write(d["text"])
    if d.get("env"):   # IIO_TXT: every file read as TXT
        dst = str(tmp_path / "o.npy")
        env = {k: v for k, v in os.environ.items() if k not in ("IIO_RAW", "IIO_TRANS", "IIO_TXT")}
        env.update(d["env"])
        subprocess.run([harness, "read", src, dst], check=True, env=env)
        got = np.load(dst)
    else:
        got = _read_with(harness, tmp_path, src, "")
    assert list(got.shape) == d["shape"]
    assert np.array_equal(got.view(np.uint32), np.array(d["out"], np.float32).reshape(d["shape"]).view(np.uint32))


@pytest.mark.parametrize("ext", ["csv", "txt", "asc"])
def test_text_writers_read_back(harness, tmp_path, ext):
    rng = np.random.default_rng(3)
    a = (rng.standard_normal((12, 9, 1)) * 30).astype(np.float32)
    src, dst, back = str(tmp_path / "a.npy"), str(tmp_path / f"a.{ext}"), str(tmp_path / "b.npy")
    np.save(src, a)
    subprocess.run([harness, "write", src, dst], check=True)
    subprocess.run([harness, "read", dst, back], check=True)
    assert np.array_equal(np.load(back).reshape(a.shape), a)


@pytest.mark.parametrize("key", json.load(open(os.path.join(GOLDEN, "raw.json"))).keys())
def test_raw_images_match_reference(harness, tmp_path, key):
    """Headerless binary images, RAW[fields]:file or IIO_RAW (iio.c:3597-3795):
    sizes, header, sample types, byte swaps, orientation, image index and
    fields read from the file, as the reference reads them."""
    d = _fixtures("raw.json")[key]
    src = str(tmp_path / "img.bin")
    open(src, "wb").write(bytes(d["data"]))
    dst = str(tmp_path / "o.npy")
    env = {k: v for k, v in os.environ.items() if k not in ("IIO_RAW", "IIO_TRANS", "IIO_TXT")}
    if d.get("env"):
        env["IIO_RAW"] = d["env"]
        name = src
    else:
        name = f"RAW[{d['spec']}]:{src}"
    subprocess.run([harness, "read", name, dst], check=True, env=env)
    got = np.load(dst)
    assert list(got.shape) == d["shape"]
    assert np.array_equal(got.view(np.uint32), np.array(d["out"], np.float32).reshape(d["shape"]).view(np.uint32))


def test_raw_too_small_fails(harness, tmp_path):
    src = str(tmp_path / "img.bin")
    open(src, "wb").write(bytes(10))
    r = subprocess.run([harness, "read", f"RAW[w4,h4,tfloat,o0]:{src}", str(tmp_path / "o.npy")],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "not large enough" in r.stderr


_MORE_SHAPES = {"img2": (5, 6, 2), "img3": (4, 5, 3), "img1": (3, 7, 1)}


@pytest.mark.parametrize("key", ["uv", "flo", "raw", "txt_prefix", "raw_prefix", "mw"])
def test_more_writers_match_reference_bytes(harness, tmp_path, key):
    """.uv and .flo (two channels), .raw, and the TXT: and RAW: name prefixes
    (iio.c:4110-4148, 4277-4334, 6166-6307), byte for byte."""
    d = _fixtures("io_more.json")
    w = d["write"][key]
    src = str(tmp_path / "src.npy")
    np.save(src, np.array(d[w["tag"]], np.float32).reshape(_MORE_SHAPES[w["tag"]]))
    prefix, fname = (w["name"].split(":", 1) + [""])[:2] if ":" in w["name"] else ("", w["name"])
    path = str(tmp_path / fname)
    subprocess.run([harness, "write", src, (prefix + ":" if prefix else "") + path], check=True)
    assert list(open(path, "rb").read()) == w["bytes"]


@pytest.mark.parametrize("key", ["uv", "flo"])
def test_flow_formats_read_like_reference(harness, tmp_path, key):
    d = _fixtures("io_more.json")
    src = str(tmp_path / ("in." + key))
    open(src, "wb").write(bytes(d["write"][key]["bytes"]))
    got = _read_with(harness, tmp_path, src, "")
    want = d["read"][key]
    assert list(got.shape) == want["shape"]
    assert np.array_equal(got.view(np.uint32), np.array(want["out"], np.float32).reshape(want["shape"]).view(np.uint32))


@pytest.mark.parametrize("key", ["ffd", "pcm", "p7", "p9", "p9_16", "p2_float", "lum", "lum12", "rim_ir",
                                 "rim_mi", "rim_im", "rim_we", "rim_vi", "rat", "fit_f32", "fit_i16_3ch",
                                 "fit_f64_long", "pds_f32", "pds_u16_flips_prefix", "pds_undefined", "vic_real",
                                 "vic_half_high_nbb_nlb", "vic_byte_2bands", "ccsd"])
def test_farbfeld_and_pcm_read_like_reference(harness, tmp_path, key):
    """farbfeld, PCM, iio's n-channel PNM variants P7/P9 and ASCII PNM
    samples read as floats, as the reference reads them."""
    want = _fixtures("io_more.json")["read"][key]
    src = str(tmp_path / ("in." + key))
    open(src, "wb").write(bytes(want["bytes"]))
    got = _read_with(harness, tmp_path, src, "")
    assert list(got.shape) == want["shape"]
    assert np.array_equal(got.view(np.uint32), np.array(want["out"], np.float32).reshape(want["shape"]).view(np.uint32))


def test_rim_swapped_float_image_reads_as_its_twin(harness, tmp_path):
    """An "RI" float image (bytes swapped) reads as the "IR" one with the same
    samples (the reference aborts on "RI" files, so this case is not pinned)."""
    d = _fixtures("io_more.json")["read"]["rim_ir"]
    ir = bytes(d["bytes"])
    w = int.from_bytes(ir[4:6], "big")
    h = int.from_bytes(ir[6:8], "big")
    body = np.frombuffer(ir[8 + 56 + 3:], "<f4")
    ri = (b"RI" + (3).to_bytes(2, "little") + w.to_bytes(2, "little") + h.to_bytes(2, "little") + bytes(56) + b"abc"
          + body.astype(">f4").tobytes())
    src = str(tmp_path / "in.rim")
    open(src, "wb").write(ri)
    got = _read_with(harness, tmp_path, src, "")
    assert np.array_equal(got.view(np.uint32), np.array(d["out"], np.float32).reshape(d["shape"]).view(np.uint32))


def test_vrt_mosaic_reads_like_reference(harness, tmp_path):
    """A GDAL VRT pasting three tiles (gray float, colour float, bytes) read
    from its directory (iio.c:3085-3160), as the reference reads it."""
    d = _fixtures("io_more.json")["vrt"]
    vd = tmp_path / "vrt"
    vd.mkdir()
    for fname, data in d["tiles"].items():
        open(vd / fname, "wb").write(bytes(data))
    open(vd / "m.vrt", "w").write(d["text"])
    got = _read_with(harness, tmp_path, str(vd / "m.vrt"), "")
    assert list(got.shape) == d["shape"]
    assert np.array_equal(got.view(np.uint32), np.array(d["out"], np.float32).reshape(d["shape"]).view(np.uint32))
