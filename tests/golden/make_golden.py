"""Generate the golden fixtures under tests/golden/ from the reference binary.

Run in a tree where the reference sources are present (the binary is built
from them by ``oracle/Makefile`` into ``oracle/_ref/``):

    python tests/golden/make_golden.py

Each fixture is one ``.npz`` holding the planar inputs (``g`` with NaN holes,
optional ``f`` data term, optional ``mask``), the command-line arguments and
environment the reference ran with, and its planar output ``out``.

* ``pin_*``   small cases across every option, env var and edge case; the
              oracle restatement must reproduce them bit for bit.
* ``conv_*``  single-channel cases run to convergence with the reference
              recipe ``CG_EPS=rtol*||b|| simpois -s 1 -c -1`` (rtol 1e-7); the
              GPU solver must agree within 1e-4 relative max-abs.
* ``trans.json`` iio's transformations on reading (IIO_TRANS, TRANS[...]:)
              applied by the reference command to an all-known image.
* ``text.json`` CSV / TXT / ASC-looking text images as the reference reads them.
* ``raw.json``  headerless binary images (RAW[...]:file, IIO_RAW) as the reference
              reads them.
* ``io_more.json`` the .uv, .flo, .raw, TXT: and RAW: writers, byte for byte,
              and the reading of .flo and .uv.
* ``amle_*``  the reference ``amle`` (src/amle.c) on one channel: neighbourhood
              sizes (AMLE_NN), iteration counts (AMLE_NITER), a mask file, an
              AMLE_INIT start image, all-known, all-NaN and 1-pixel images.

``python tests/golden/make_golden.py amle`` regenerates only the AMLE group.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from imscript_gb300 import synth  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def save(name, g, f=None, mask=None, args=(), env=None, out=None, extra=None, init=None):
    d = {"g": g, "args": np.array(json.dumps(list(args))),
         "env": np.array(json.dumps(env or {})), "out": out}
    if init is not None:
        d["init"] = init
    if f is not None:
        d["f"] = f
    if mask is not None:
        d["mask"] = mask
    if extra:
        d["extra"] = np.array(json.dumps(extra))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **d)


def noisy(rng, pd, h, w, frac):
    x = (rng.standard_normal((pd, h, w)) * 0.5).astype(np.float32)
    x += synth.gaussian_field(rng, h, w, 3)[None]
    m = rng.random((h, w)) < frac
    x[:, m] = np.nan
    return x


def pin_cases(rng):
    shapes = [(1, 17, 23), (3, 12, 9), (1, 1, 40), (1, 33, 1), (1, 1, 1), (1, 2, 3), (2, 16, 16)]
    argsets = [
        [], ["-n", "40"], ["-n", "3", "-s", "1"], ["-s", "2", "-n", "7"],
        ["-t", "-0.08", "-n", "30"], ["-t", "-1000.01", "-n", "3", "-s", "2"],
        ["-c", "25"], ["-s", "1", "-c", "-1"], ["-t", "-0.08", "-s", "2", "-c", "30"],
        ["-t", "0.1", "-n", "12", "-s", "3", "-c", "5"],
    ]
    k = 0
    for (pd, h, w) in shapes:
        for a in argsets:
            g = noisy(rng, pd, h, w, 0.35)
            f = None
            if k % 2 == 1:
                f = (rng.standard_normal(g.shape) * 0.05).astype(np.float32)
            out = O.run_reference(g, f, args=a)
            save(f"pin_{k:03d}", g, f, args=a, out=out)
            k += 1
    # environment smart parameters (smapa.h:44-60)
    g = noisy(rng, 1, 24, 20, 0.3)
    f = (rng.standard_normal(g.shape) * 0.05).astype(np.float32)
    for env, a in [({"PMSFAC": "1.5"}, ["-n", "20"]), ({"PONLIT": "12"}, ["-n", "20"]),
                   ({"PONLIT": "24"}, ["-n", "20", "-c", "10"]), ({"CG_EPS": "0.01"}, ["-c", "-1"]),
                   ({"PMSFAC": "2.7", "CG_EPS": "1e-3"}, ["-c", "50", "-s", "3"])]:
        out = O.run_reference(g, f, args=a, env=env)
        save(f"pin_{k:03d}", g, f, args=a, env=env, out=out)
        k += 1
    # mask image (applied to every channel), including all-known/all-unknown
    g = noisy(rng, 2, 14, 18, 0.0)
    mk = (rng.random((14, 18)) < 0.3).astype(np.float32) * 2 - 0.5
    out = O.run_reference(g, None, mask=mk, args=["-n", "15"])
    save(f"pin_{k:03d}", g, None, mask=mk, args=["-n", "15"], out=out)
    k += 1
    out = O.run_reference(g, None, args=["-n", "5"])  # nothing to fill
    save(f"pin_{k:03d}", g, None, args=["-n", "5"], out=out)
    k += 1
    gall = np.full((1, 9, 11), np.nan, np.float32)
    fall = (rng.standard_normal(gall.shape) * 0.1).astype(np.float32)
    out = O.run_reference(gall, fall, args=["-n", "10"])
    save(f"pin_{k:03d}", gall, fall, args=["-n", "10"], out=out)
    k += 1
    # +-Inf known pixels: overwritten by init during the sweeps, restored at the end
    g = noisy(rng, 1, 15, 15, 0.3)
    g[0, 3, 4] = np.inf
    g[0, 10, 2] = -np.inf
    for a in (["-n", "10"], ["-c", "10"]):
        out = O.run_reference(g, None, args=a)
        save(f"pin_{k:03d}", g, None, args=a, out=out)
        k += 1
    return k


def conv_cases(rng):
    k = 0
    specs = [("lap", 64, 64, 0.25, False), ("lap", 80, 48, 0.25, False),
             ("poi", 64, 64, 0.25, True), ("poi", 57, 71, 0.25, True),
             ("bih", 40, 40, -0.08, False), ("bih", 36, 44, -0.08, True)]
    for kind, h, w, t, with_f in specs:
        img = synth.gaussian_field(rng, h, w, 6)
        m = synth.disk_mask(rng, h, w, 0.2, rmin=2, rmax=8 if kind == "bih" else 12)
        img[m] = np.nan
        g = img[None]
        f = None
        if with_f:
            f = synth.guidance(synth.gaussian_field(rng, h, w, 6))[2][None] * 0.5
        ckind = 1 if t < 0 else 0
        bn = float(O.rhs_norm(g, f, ckind)[0])
        rtol = 1e-7
        args = ["-s", "1", "-c", "-1", "-t", str(t)]
        env = {"CG_EPS": repr(rtol * bn)}
        out = O.run_reference(g, f, args=args, env=env, timeout=3000)
        rel = float(O.rel_residual(out, g, f, ckind)[0][0])
        save(f"conv_{kind}_{k:02d}", g, f, args=args, env=env, out=out,
             extra={"rel_residual": rel, "bnorm": bn, "kind": ckind})
        print(f"conv_{kind}_{k:02d}: {w}x{h} n={int(np.isnan(g).sum())} rel={rel:.2e}")
        k += 1
    return k


def cli_cases():
    """Texts and exit codes of the reference command (no image work)."""
    import subprocess
    import tempfile
    res = {}
    for a in (["-h"], ["--help"], ["--version"], ["-?"]):
        r = subprocess.run([O.REF_BIN] + a, capture_output=True, text=True)
        res[" ".join(a)] = {"stdout": r.stdout, "stderr": r.stderr, "rc": r.returncode}
    r = subprocess.run([O.REF_BIN, "-n", "3", "stray"], capture_output=True, text=True)
    res["stray"] = {"stdout": r.stdout, "stderr": r.stderr.replace(O.REF_BIN, "ARGV0"),
                    "rc": r.returncode}
    with tempfile.TemporaryDirectory() as td:
        a = os.path.join(td, "a.npy")
        b = os.path.join(td, "b.npy")
        np.save(a, np.zeros((4, 5, 1), np.float32))
        np.save(b, np.zeros((4, 6, 1), np.float32))
        r = subprocess.run([O.REF_BIN, "-i", a, "-f", b, "-o", os.path.join(td, "o.npy")],
                           capture_output=True, text=True)
        res["mismatch_if"] = {"stdout": r.stdout, "stderr": r.stderr, "rc": r.returncode}
        r = subprocess.run([O.REF_BIN, "-i", a, "-m", b, "-o", os.path.join(td, "o.npy")],
                           capture_output=True, text=True)
        res["mismatch_im"] = {"stdout": r.stdout, "stderr": r.stderr, "rc": r.returncode}
    with open(os.path.join(OUT, "cli.json"), "w") as fh:
        json.dump(res, fh, indent=1)
    return len(res)


def io_cases():
    """How the reference reads and writes each format: an all-known image
    (nothing to fill) read from format X and written as npy, and read from
    npy and written as format Y."""
    import subprocess
    import tempfile
    rng = np.random.default_rng(77)
    res = {}
    img3 = (rng.random((5, 7, 3)) * 200).astype(np.float32)
    img1 = (rng.random((6, 4, 1)) * 200).astype(np.float32)
    with tempfile.TemporaryDirectory() as td:
        for tag, img in (("c3", img3), ("c1", img1)):
            src = os.path.join(td, f"{tag}.npy")
            np.save(src, img)
            for ext in ("npy", "pfm", "ppm", "pgm", "asc", "tif", "txt"):
                dst = os.path.join(td, f"{tag}_out.{ext}")
                subprocess.run([O.REF_BIN, "-i", src, "-o", dst], check=True)
                res[f"write_{tag}_{ext}"] = list(open(dst, "rb").read())
        # readers: npy dtypes, 2-D npy, pnm (ascii, binary), asc
        cases = {}
        cases["u8_hw"] = np.arange(20, dtype=np.uint8).reshape(4, 5)
        cases["i16_hwc"] = (np.arange(24, dtype=np.int16) - 7).reshape(2, 4, 3)
        cases["f8_hwc"] = rng.standard_normal((3, 2, 2))
        cases["u2_hw"] = (np.arange(6, dtype=np.uint16) * 1000).reshape(2, 3)
        for k, a in cases.items():
            p = os.path.join(td, k + ".npy")
            np.save(p, a)
            o = os.path.join(td, k + "_o.npy")
            subprocess.run([O.REF_BIN, "-i", p, "-o", o], check=True)
            res[f"read_{k}"] = {"in": list(open(p, "rb").read()), "out": list(open(o, "rb").read())}
        texts = {"p2": b"P2\n3 2\n255\n0 1 2\n3 4 255\n", "p5": b"P5\n2 2\n255\n\x00\x10\x20\xff",
                 "p6": b"P6\n1 2\n255\n\x01\x02\x03\x04\x05\x06"}
        for k, t in texts.items():
            p = os.path.join(td, k)
            open(p, "wb").write(t)
            o = os.path.join(td, k + "_o.npy")
            subprocess.run([O.REF_BIN, "-i", p, "-o", o], check=True)
            res[f"read_{k}"] = {"in": list(t), "out": list(open(o, "rb").read())}
        # mask: RGB uint8 ppm turned gray by the reference's weights
        img = synth.gaussian_field(rng, 4, 6, 2)[None]
        np.save(os.path.join(td, "g.npy"), O.to_hwc(img))
        mk = b"P6\n6 4\n255\n" + bytes(rng.integers(0, 2, 72, dtype=np.uint8).tolist())
        open(os.path.join(td, "m.ppm"), "wb").write(mk)
        o = os.path.join(td, "gm.npy")
        subprocess.run([O.REF_BIN, "-i", os.path.join(td, "g.npy"), "-m", os.path.join(td, "m.ppm"),
                        "-n", "0", "-o", o], check=True)
        res["mask_rgb"] = {"g": O.to_hwc(img).ravel().tolist(), "mask": list(mk),
                           "out": list(open(o, "rb").read())}
    with open(os.path.join(OUT, "io.json"), "w") as fh:
        json.dump(res, fh)
    return len(res)


TRANS_LISTS = ["flip=leftright", "flip=topdown", "flip=transpose", "flip=r90", "flip=r180", "flip=r270",
               "flip=posetrans", "flip=Xy", "flip=yX", "flip=YX", "flip=xyz", "flip=yxz", "flip=zxy", "flip=zyx",
               "flip=xzy", "flip=yzx", "x=2", "y=1", "w=4", "h=3", "x=1,y=1,w=3,h=2", "x=-2", "y=-1,h=7",
               "flip=leftright,x=2,flip=transpose", "w=9", "pipe=cat", "bogus=3,flip=nothing"]


def trans_cases():
    """iio's transformations on reading (IIO_TRANS and the TRANS[...]:
    prefix): an all-known image read by the reference command under each
    list, with nothing to fill, written as npy (tests/golden/trans.json)."""
    import subprocess
    import tempfile
    rng = np.random.default_rng(99)
    img = (rng.random((5, 7, 3)) * 100).astype(np.float32)
    res = {"in": img.ravel().tolist(), "shape": list(img.shape), "env": {}, "prefix": {}}
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "in.npy")
        np.save(src, img)
        o = os.path.join(td, "o.npy")
        e0 = {k: v for k, v in os.environ.items() if k not in ("PMSFAC", "PONLIT", "CG_EPS", "IIO_TRANS")}
        for lst in TRANS_LISTS:
            subprocess.run([O.REF_BIN, "-i", src, "-n", "0", "-o", o], env=dict(e0, IIO_TRANS=lst), check=True,
                           capture_output=True)
            a = np.load(o)
            res["env"][lst] = {"shape": list(a.shape), "out": a.ravel().tolist()}
        # the prefix, alone and together with IIO_TRANS (applied inside and outside)
        for lst, env in (("flip=topdown", ""), ("x=1,w=5", ""), ("flip=leftright", "flip=transpose")):
            ee = dict(e0, IIO_TRANS=env) if env else e0
            subprocess.run([O.REF_BIN, "-i", f"TRANS[{lst}]:{src}", "-n", "0", "-o", o], env=ee, check=True,
                           capture_output=True)
            a = np.load(o)
            res["prefix"][f"{lst}|{env}"] = {"shape": list(a.shape), "out": a.ravel().tolist()}
    with open(os.path.join(OUT, "trans.json"), "w") as fh:
        json.dump(res, fh)
    return len(res["env"]) + len(res["prefix"])


def text_cases():
    """Text images as the reference command reads them (CSV, TXT, and a TXT
    whose first line looks like an ASC header), all-known, nothing to fill,
    written as npy (tests/golden/text.json).  Every file is at least 256
    bytes: the reference's format sniffing reads that many."""
    import subprocess
    import tempfile
    rng = np.random.default_rng(31)
    a = (rng.standard_normal((9, 7)) * 50).astype(np.float32)
    files = {
        "csv": "\n".join(",".join(f"{v:.6g}" for v in row) for row in a) + "\n",
        "txt": "\n".join(" ".join(f"{v:.6g}" for v in row) for row in a) + "\n",
        "txt_like_asc": "3 5 1 2\n" + "\n".join(" ".join(f"{v:.5g}" for v in row[:4]) for row in a) + "\n",
        "csv_exp": "\n".join(",".join(f"{v:.3e}" for v in row) for row in a) + "\n",
        "txt_uneven": "\n".join(" ".join(f"{v:.6g}" for v in row[: 7 - (k % 2)]) for k, row in enumerate(a)) + "\n",
    }
    res = {}
    with tempfile.TemporaryDirectory() as td:
        o = os.path.join(td, "o.npy")
        env0 = {k: v for k, v in os.environ.items() if k not in ("IIO_RAW", "IIO_TRANS", "IIO_TXT")}
        for k, text in files.items():
            assert len(text) >= 256, (k, len(text))
            src = os.path.join(td, k)
            open(src, "w").write(text)
            subprocess.run([O.REF_BIN, "-i", src, "-n", "0", "-o", o], check=True, capture_output=True, env=env0)
            out = np.load(o)
            res[k] = {"text": text, "shape": list(out.shape), "out": out.ravel().tolist()}
        # IIO_TXT: a CSV file read as TXT (one number a line: atof stops at the comma)
        src = os.path.join(td, "csv_as_txt")
        open(src, "w").write(files["csv"])
        subprocess.run([O.REF_BIN, "-i", src, "-n", "0", "-o", o], check=True, capture_output=True,
                       env=dict(env0, IIO_TXT="1"))
        out = np.load(o)
        res["csv_as_txt"] = {"text": files["csv"], "env": {"IIO_TXT": "1"}, "shape": list(out.shape),
                             "out": out.ravel().tolist()}
    with open(os.path.join(OUT, "text.json"), "w") as fh:
        json.dump(res, fh)
    return len(res)


def raw_cases():
    """Headerless binary images named RAW[...]:file, and read through
    IIO_RAW, as the reference command reads them (all-known, nothing to
    fill, written as npy: tests/golden/raw.json)."""
    import subprocess
    import tempfile
    rng = np.random.default_rng(17)
    f32 = (rng.standard_normal(7 * 5) * 40).astype("<f4").tobytes()
    u8 = rng.integers(0, 256, 7 * 5 * 3, dtype=np.uint8).tobytes()
    u16be = rng.integers(0, 65536, 6 * 4, dtype=np.uint16).astype(">u2").tobytes()
    i16 = bytes(range(16)) + rng.integers(-3000, 3000, 4 * 3, dtype=np.int16).astype("<i2").tobytes()
    i32 = bytes(8) + rng.integers(-99999, 99999, 6 * 5, dtype=np.int32).astype("<i4").tobytes()
    f64 = (rng.standard_normal(5 * 4 * 2) * 9).astype("<f8").tobytes()
    stack = (rng.standard_normal(3 * 2 * 3) * 5).astype("<f4").tobytes()
    fields = np.array([6, 5], "<u2").tobytes() + bytes(4) + rng.integers(0, 256, 30, dtype=np.uint8).tobytes()
    f32be = (rng.standard_normal(4 * 3) * 7).astype(">f4").tobytes()
    cases = [("f32", "w7,h5,tfloat", f32), ("u8_rgb", "w7,h5,p3,tuint8", u8),
             ("u16_be_h_estimated", "w6,tuint16,e1", u16be), ("i16_header", "w4,h3,o16,tint16", i16),
             ("i32_w_estimated", "h5,o8,tint32", i32), ("f64_2ch", "w5,h4,p2,tdouble", f64),
             ("u8_orient", "w7,h5,p3,tUINT8,rYx", u8), ("f32_stack_index", "w3,h2,o0,tfloat,i2", stack),
             ("fields_from_file", "w@0/2,h@2/2,o8,tuint8", fields), ("f32_be", "w4,h3,tfloat,e1", f32be)]
    res = {}
    with tempfile.TemporaryDirectory() as td:
        o = os.path.join(td, "o.npy")
        env0 = {k: v for k, v in os.environ.items() if k not in ("IIO_RAW", "IIO_TRANS", "IIO_TXT")}
        for key, spec, data in cases:
            src = os.path.join(td, key + ".bin")
            open(src, "wb").write(data)
            subprocess.run([O.REF_BIN, "-i", f"RAW[{spec}]:{src}", "-n", "0", "-o", o], check=True,
                           capture_output=True, env=env0)
            out = np.load(o)
            res[key] = {"spec": spec, "data": list(data), "shape": list(out.shape), "out": out.ravel().tolist()}
        # IIO_RAW: a plain file name read as raw
        src = os.path.join(td, "plain.bin")
        open(src, "wb").write(f32)
        subprocess.run([O.REF_BIN, "-i", src, "-n", "0", "-o", o], check=True, capture_output=True,
                       env=dict(env0, IIO_RAW="w5,h7,tfloat"))
        out = np.load(o)
        res["iio_raw_env"] = {"spec": "", "env": "w5,h7,tfloat", "data": list(f32), "shape": list(out.shape),
                              "out": out.ravel().tolist()}
    with open(os.path.join(OUT, "raw.json"), "w") as fh:
        json.dump(res, fh)
    return len(res)


def io_more_cases():
    """Writers the reference command picks by name -- .uv and .flo (two
    channels), .raw, the TXT: and RAW: prefixes -- byte for byte, and its
    reading back of .flo and .uv (tests/golden/io_more.json)."""
    import subprocess
    import tempfile
    rng = np.random.default_rng(23)
    img2 = (rng.standard_normal((5, 6, 2)) * 3).astype(np.float32)
    img3 = (rng.standard_normal((4, 5, 3)) * 3).astype(np.float32)
    img1 = (rng.standard_normal((3, 7, 1)) * 3).astype(np.float32)
    res = {"img2": img2.ravel().tolist(), "img3": img3.ravel().tolist(), "img1": img1.ravel().tolist(),
           "write": {}, "read": {}}
    with tempfile.TemporaryDirectory() as td:
        srcs = {}
        for tag, a in (("img2", img2), ("img3", img3), ("img1", img1)):
            srcs[tag] = os.path.join(td, tag + ".npy")
            np.save(srcs[tag], a)
        for key, tag, prefix, fname in (("uv", "img2", "", "o.uv"), ("flo", "img2", "", "o.flo"),
                                        ("raw", "img3", "", "o.raw"), ("txt_prefix", "img1", "TXT:", "o.dat"),
                                        ("raw_prefix", "img3", "RAW:", "o.bin"), ("mw", "img1", "", "o.mw")):
            path = os.path.join(td, fname)
            subprocess.run([O.REF_BIN, "-i", srcs[tag], "-n", "0", "-o", prefix + path], check=True,
                           capture_output=True)
            name = prefix + fname
            res["write"][key] = {"tag": tag, "name": name, "bytes": list(open(path, "rb").read())}
        for key in ("uv", "flo"):
            src = os.path.join(td, "o." + key)
            o = os.path.join(td, "back.npy")
            subprocess.run([O.REF_BIN, "-i", src, "-n", "0", "-o", o], check=True, capture_output=True)
            a = np.load(o)
            res["read"][key] = {"shape": list(a.shape), "out": a.ravel().tolist()}
        # farbfeld (RGBA, 16-bit big-endian) and PCM (two float channels)
        ffd = (b"farbfeld" + np.array([5, 3], ">u4").tobytes()
               + rng.integers(0, 65536, 5 * 3 * 4, dtype=np.uint16).astype(">u2").tobytes())
        pcm = b"PC 4 3 1.5\n" + (rng.standard_normal(4 * 3 * 2) * 2).astype("<f4").tobytes()
        # iio's n-channel PNM variants and ASCII samples read as floats
        p7 = b"P7\n3 2\n2\n255\n" + " ".join(f"{v:.3f}" for v in rng.standard_normal(12) * 9).encode() + b"\n"
        p9 = b"P9 3 2 2 255\n" + rng.integers(0, 256, 12, dtype=np.uint8).tobytes()
        p9_16 = b"P9 2 2 3 65535\n" + rng.integers(0, 65536, 12, dtype=np.uint16).astype(">u2").tobytes()
        p2f = b"P2\n3 2\n255\n0.5 -1 2.25\n3 4e1 5\n"
        # LUM: big-endian floats after a 3988-byte header, or 12-bit samples after 11968 bytes
        hd = bytearray(0xf94)
        hd[2:4] = (5).to_bytes(2, "big")
        hd[6:8] = (3).to_bytes(2, "big")
        hd[8:12] = b"FLOA"
        lum = bytes(hd) + (rng.standard_normal(15) * 4).astype(">f4").tobytes()
        hd12 = bytearray(11968)
        hd12[0:4] = (6).to_bytes(4, "little")   # (4 would read as the RAT magic)
        hd12[4:8] = (3).to_bytes(4, "little")
        hd12[8:12] = b"12LI"
        lum12 = bytes(hd12) + rng.integers(0, 4096, 18, dtype=np.uint16).astype("<u2").tobytes()
        # MegaWave RIM: float and byte images in both byte orders, planar ccimage and cfimage
        def rim_head(tag, w, h, little):
            sh = (lambda v: v.to_bytes(2, "little" if little else "big"))
            return tag + sh(3) + sh(w) + sh(h) + bytes(56) + b"abc"
        fl = (rng.standard_normal(4 * 3) * 6).astype(np.float32)
        rim_ir = rim_head(b"IR", 4, 3, False) + fl.astype("<f4").tobytes()
        rim_ri = rim_head(b"RI", 4, 3, True) + fl.astype(">f4").tobytes()
        by = rng.integers(0, 256, 5 * 2, dtype=np.uint8).tobytes()
        rim_mi = rim_head(b"MI", 5, 2, False) + by
        rim_im = rim_head(b"IM", 5, 2, True) + by

        def cc_head(tag, np_, nrow, ncol, form, swp):
            it = (lambda v: v.to_bytes(4, "big" if swp else "little"))
            sh = (lambda v: v.to_bytes(2, "little" if swp else "big"))
            return tag + sh(0x4956) + it(np_) + it(nrow) + it(ncol) + it(1) + it(form) + it(0)
        rim_we = cc_head(b"WE", 3, 2, 4, 0x8001, False) + rng.integers(0, 256, 24, dtype=np.uint8).tobytes()
        rim_vi = cc_head(b"VI", 2, 3, 2, 0xc004, True) + (rng.standard_normal(12) * 3).astype("<f4").tobytes()
        rat_head = bytearray(124)
        rat_head[0:4] = (4).to_bytes(4, "little")
        for off, v in ((8, 1), (12, 3), (16, 2), (20, 6)):   # d, width, height, variant
            rat_head[off:off + 4] = v.to_bytes(4, "little")
        rat = bytes(rat_head) + (rng.standard_normal(3 * 2 * 2) * 2).astype("<f4").tobytes()

        # FITS: 80-byte header lines, padded to 36-line blocks, big-endian samples
        def fits(cards, data):
            lines = [c.ljust(80).encode() for c in ["SIMPLE  =                    T"] + cards + ["END"]]
            head = b"".join(lines)
            head += b" " * 80 * (-len(lines) % 36)   # standard: the header fills 36-line blocks
            return head + data
        fit_f32 = fits(["BITPIX  =                  -32 / float", "NAXIS   =                    2",
                        "NAXIS1  =                    5", "NAXIS2  =                    3"],
                       (rng.standard_normal(15) * 3).astype(">f4").tobytes())
        fit_i16 = fits(["BITPIX  =                   16", "NAXIS   =                    3",
                        "NAXIS1  =                    4", "NAXIS2  =                    2",
                        "NAXIS3  =                    3"], rng.integers(-900, 900, 24, dtype=np.int16).astype(">i2").tobytes())
        fit_f64 = fits(["BITPIX  =                  -64", "NAXIS   =                    2",
                        "NAXIS1  =                    3", "NAXIS2  =                    2"]
                       + [f"COMMENT card {i}" for i in range(40)],
                       (rng.standard_normal(6) * 2).astype(">f8").tobytes())

        # PDS: a label of KEY = VALUE lines, the samples at record ^IMAGE - 1
        def pds(lines, record, nrec, data):
            label = ("PDS_VERSION_ID = PDS3\n" + "".join(l + "\n" for l in lines) + "END\n").encode()
            assert len(label) <= record * nrec
            return label.ljust(record * nrec, b" ") + data
        pds_f32 = pds(["RECORD_TYPE = FIXED_LENGTH", "RECORD_BYTES = 256", "^IMAGE = 3", "OBJECT = IMAGE",
                       "LINES = 3", "LINE_SAMPLES = 4", "SAMPLE_BITS = 32", "SAMPLE_TYPE = PC_REAL",
                       "BANDS = 1", "END_OBJECT = IMAGE"], 256, 2,
                      (rng.standard_normal(12) * 5).astype("<f4").tobytes())
        pds_u16 = pds(["RECORD_TYPE = FIXED_LENGTH", "RECORD_BYTES = 512", "^IMAGE = 2", "OBJECT = IMAGE",
                       "LINES = 3", "LINE_SAMPLES = 4", "SAMPLE_BITS = 16", "SAMPLE_TYPE = LSB_UNSIGNED_INTEGER",
                       "SAMPLE_DISPLAY_DIRECTION = RIGHT", "LINE_DISPLAY_DIRECTION = DOWN",
                       "LINE_PREFIX_BYTES = 1", "BANDS = 1", "END_OBJECT = IMAGE"], 512, 1,
                      rng.integers(0, 65536, 15, dtype=np.uint16).astype("<u2").tobytes())
        # VICAR: "LBLSIZE=" and a 9-character size, KEY=VALUE tokens, then the records
        def vic(n, tokens, records):
            label = ("LBLSIZE=" + f"{n:<9d}" + " " + " ".join(tokens)).ljust(n)
            assert len(label) == n
            return label.encode() + records
        vic_real = vic(256, ["FORMAT='REAL'", "TYPE='IMAGE'", "ORG='BSQ'", "NL=3", "NS=4", "NB=1", "NBB=0",
                             "NLB=0", "RECSIZE=16", "INTFMT='LOW'"],
                       (rng.standard_normal(12) * 4).astype("<f4").tobytes())
        half = rng.integers(-3000, 3000, (3, 5), dtype=np.int16)
        vic_half = vic(300, ["FORMAT='HALF'", "TYPE='IMAGE'", "ORG='BSQ'", "NL=3", "NS=5", "NB=1", "NBB=2",
                             "NLB=1", "RECSIZE=12", "INTFMT='HIGH'"],
                       bytes(12) + b"".join(b"\xaa\xbb" + row.astype(">i2").tobytes() for row in half))
        vic_byte = vic(200, ["FORMAT='BYTE'", "TYPE='IMAGE'", "ORG='BSQ'", "NL=2", "NS=3", "NB=2", "NBB=0",
                             "NLB=0", "RECSIZE=3"], rng.integers(0, 256, 12, dtype=np.uint8).tobytes())
        ccsd_label = ("CCSD3ZF0000100000001NJPL3IF0PDS200000001 = SFDU_LABEL\nRECORD_TYPE = FIXED_LENGTH\n"
                      "RECORD_BYTES = 256\n^IMAGE = 2\nOBJECT = IMAGE\nLINES = 2\nLINE_SAMPLES = 3\n"
                      "SAMPLE_BITS = 32\nSAMPLE_TYPE = PC_REAL\nEND_OBJECT = IMAGE\nEND\n").encode()
        assert len(ccsd_label) <= 256
        ccsd = ccsd_label.ljust(256, b" ") + (rng.standard_normal(6) * 2).astype("<f4").tobytes()
        pds_und = pds(["RECORD_TYPE = UNDEFINED", "^IMAGE = 301", "OBJECT = IMAGE", "LINES = 2",
                       "LINE_SAMPLES = 5", "SAMPLE_BITS = 8", "SAMPLE_TYPE = UNSIGNED_INTEGER", "BANDS = 1",
                       "END_OBJECT = IMAGE"], 300, 1, rng.integers(0, 256, 10, dtype=np.uint8).tobytes())
        for key, data in (("ffd", ffd), ("pcm", pcm), ("p7", p7), ("p9", p9), ("p9_16", p9_16), ("p2_float", p2f),
                          ("lum", lum), ("lum12", lum12), ("rim_ir", rim_ir), ("rat", rat),
                          ("fit_f32", fit_f32), ("fit_i16_3ch", fit_i16), ("fit_f64_long", fit_f64),
                          ("pds_f32", pds_f32), ("pds_u16_flips_prefix", pds_u16), ("pds_undefined", pds_und),
                          ("vic_real", vic_real), ("vic_half_high_nbb_nlb", vic_half), ("vic_byte_2bands", vic_byte),
                          ("ccsd", ccsd),
                          ("rim_mi", rim_mi), ("rim_im", rim_im), ("rim_we", rim_we), ("rim_vi", rim_vi)):
            # (the reference aborts on "RI" files: it tells them only after 4 header bytes and its
            # reader asserts 2; rim_ri is read here and checked against rim_ir in tests/test_cli.py)
            src = os.path.join(td, "in." + key)
            open(src, "wb").write(data)
            o = os.path.join(td, "back.npy")
            subprocess.run([O.REF_BIN, "-i", src, "-n", "0", "-o", o], check=True, capture_output=True)
            a = np.load(o)
            res["read"][key] = {"shape": list(a.shape), "out": a.ravel().tolist(), "bytes": list(data)}
        # GDAL VRT: three tiles pasted into an 8x5 raster, read from the VRT's directory
        tiles = {"a.npy": (rng.standard_normal((3, 4)) * 3).astype(np.float32),
                 "b.npy": (rng.random((3, 4, 3)) * 100).astype(np.float32),
                 "c.npy": rng.integers(0, 256, (2, 8), dtype=np.uint8)}
        vrt_text = ('<VRTDataset rasterXSize="8" rasterYSize="5">\n'
                    '  <VRTRasterBand dataType="Float32" band="1">\n')
        for fname, (x0, y0, w, h) in (("a.npy", (0, 0, 4, 3)), ("b.npy", (4, 0, 4, 3)), ("c.npy", (0, 3, 8, 2))):
            vrt_text += ('    <SimpleSource>\n'
                         f'      <SourceFilename relativeToVRT="1">{fname}</SourceFilename>\n'
                         f'      <SrcRect xOff="0" yOff="0" xSize="{w}" ySize="{h}"/>\n'
                         f'      <DstRect xOff="{x0}" yOff="{y0}" xSize="{w}" ySize="{h}"/>\n'
                         '    </SimpleSource>\n')
        vrt_text += "  </VRTRasterBand>\n</VRTDataset>\n"
        vd = os.path.join(td, "vrt")
        os.makedirs(vd)
        tile_bytes = {}
        for fname, a in tiles.items():
            np.save(os.path.join(vd, fname), a)
            tile_bytes[fname] = list(open(os.path.join(vd, fname), "rb").read())
        open(os.path.join(vd, "m.vrt"), "w").write(vrt_text)
        o = os.path.join(td, "back.npy")
        subprocess.run([O.REF_BIN, "-i", os.path.join(vd, "m.vrt"), "-n", "0", "-o", o], check=True,
                       capture_output=True)
        a = np.load(o)
        res["vrt"] = {"text": vrt_text, "tiles": tile_bytes, "shape": list(a.shape), "out": a.ravel().tolist()}
    with open(os.path.join(OUT, "io_more.json"), "w") as fh:
        json.dump(res, fh)
    return len(res["write"]) + len(res["read"]) + 1


def mini_cases(rng):
    """The GS-only copy of the ftr viewers (ftr/minisimpois.c) from its own main."""
    k = 0
    for (pd, h, w) in [(1, 13, 17), (2, 20, 9), (1, 1, 25), (1, 24, 24)]:
        for a in (["-t", "0.25"], ["-t", "0.45", "-n", "25", "-s", "3"], ["-t", "0.2", "-n", "4", "-s", "1"]):
            g = noisy(rng, pd, h, w, 0.35)
            f = (rng.standard_normal(g.shape) * 0.05).astype(np.float32) if k % 2 else None
            out = O.run_reference(g, f, args=a, binary=O.MINI_BIN)
            save(f"mini_{k:03d}", g, f, args=a, out=out)
            k += 1
    return k


def amle_cases(rng):
    """The reference amle command: `amle in.npy [mask.npy] out.npy` with its
    environment (AMLE_NN, AMLE_NITER, AMLE_INIT)."""
    import tempfile
    k = 0
    shapes = [(20, 30), (33, 17), (1, 9), (12, 1), (48, 40), (7, 7)]
    for si, (h, w) in enumerate(shapes):
        for nn, niter in [(4, 1), (4, 30), (6, 5), (8, 12), (16, 5), (32, 3)]:
            x = (rng.standard_normal((h, w)) * 0.5).astype(np.float32)
            x += synth.gaussian_field(rng, h, w, 3)
            x[rng.random((h, w)) < 0.4] = np.nan
            env = {"AMLE_NN": nn, "AMLE_NITER": niter}
            mask = None
            if k % 5 == 3:
                mask = (rng.random((h, w)) < 0.2).astype(np.float32)
            out = O.run_reference_amle(x, mask=mask, env=env)
            save(f"amle_{k:03d}", x[None], mask=mask, env=env, out=out[None])
            k += 1
    # AMLE_INIT: a start image for the upper iterate at the unknowns
    with tempfile.TemporaryDirectory() as td:
        for (h, w) in [(16, 21), (30, 30)]:
            x = synth.gaussian_field(rng, h, w, 3)
            x[rng.random((h, w)) < 0.5] = np.nan
            ini = (rng.standard_normal((h, w))).astype(np.float32)
            pi = os.path.join(td, "init.npy")
            np.save(pi, ini)
            env = {"AMLE_NN": 8, "AMLE_NITER": 9, "AMLE_INIT": pi}
            out = O.run_reference_amle(x, env=env)
            env["AMLE_INIT"] = "init"
            save(f"amle_{k:03d}", x[None], env=env, out=out[None], init=ini[None])
            k += 1
    # all known, all unknown, one unknown pixel
    for x in [synth.gaussian_field(rng, 9, 11, 2), np.full((6, 5), np.nan, np.float32),
              np.full((1, 1), np.nan, np.float32)]:
        env = {"AMLE_NN": 4, "AMLE_NITER": 3}
        out = O.run_reference_amle(x, env=env)
        save(f"amle_{k:03d}", x[None].astype(np.float32), env=env, out=out[None])
        k += 1
    return k


def amle_cli_cases():
    """The reference amle command's texts, usage error and exit codes, and
    the bytes of a file it writes (tests/golden/amle_cli.json)."""
    import subprocess
    import tempfile
    res = {}
    for a in ["-h", "--help", "--version", "-?"]:
        r = subprocess.run([O.AMLE_BIN, a], capture_output=True, text=True)
        res[a] = {"stdout": r.stdout, "stderr": r.stderr, "rc": r.returncode}
    r = subprocess.run([O.AMLE_BIN, "a", "b", "c", "d"], capture_output=True, text=True)
    res["extra_args"] = {"stderr": r.stderr.replace(O.AMLE_BIN, "ARGV0"), "rc": r.returncode}
    with tempfile.TemporaryDirectory() as td:
        a, b = os.path.join(td, "a.npy"), os.path.join(td, "b.npy")
        np.save(a, np.zeros((4, 5, 1), np.float32))
        np.save(b, np.zeros((4, 6, 1), np.float32))
        r = subprocess.run([O.AMLE_BIN, a, b, os.path.join(td, "o.npy")], capture_output=True, text=True)
        res["mask_mismatch"] = {"rc": r.returncode, "tail": r.stderr.strip().split(": ", 1)[-1]}
        # a one-iteration fill: raster and colour order agree on a 1-pixel hole
        x = np.arange(20, dtype=np.float32).reshape(4, 5) / 7
        x[2, 2] = np.nan
        np.save(a, x)
        o = os.path.join(td, "o.npy")
        e = dict(os.environ, AMLE_NITER="1")
        subprocess.run([O.AMLE_BIN, a, "", o], check=True, env=e, capture_output=True)
        res["file"] = {"in": x.ravel().tolist(), "out_bytes": list(open(o, "rb").read())}
    with open(os.path.join(OUT, "amle_cli.json"), "w") as fh:
        json.dump(res, fh)
    return len(res)


def main():
    if not O.have_reference():
        O.build(reference=True)
    if sys.argv[1:] == ["io_more"]:
        print(f"wrote {io_more_cases()} writer/reader cases into {OUT}")
        return
    if sys.argv[1:] == ["raw"]:
        print(f"wrote {raw_cases()} raw-image cases into {OUT}")
        return
    if sys.argv[1:] == ["text"]:
        print(f"wrote {text_cases()} text-format cases into {OUT}")
        return
    if sys.argv[1:] == ["trans"]:
        print(f"wrote {trans_cases()} transformation cases into {OUT}")
        return
    if sys.argv[1:] == ["amle"]:
        n = amle_cases(np.random.default_rng(5150))
        print(f"wrote {n} AMLE cases and {amle_cli_cases()} AMLE command cases into {OUT}")
        return
    rng = np.random.default_rng(20261203)
    n1 = pin_cases(rng)
    n2 = conv_cases(rng)
    n3 = cli_cases()
    n4 = io_cases()
    n5 = mini_cases(np.random.default_rng(4242))
    n6 = amle_cases(np.random.default_rng(5150)) + amle_cli_cases()
    n7 = trans_cases() + text_cases() + raw_cases() + io_more_cases()
    print(f"wrote {n1} pin cases, {n2} converged cases, {n3} CLI cases, {n4} I/O cases, "
          f"{n5} minisimpois cases, {n6} AMLE cases and {n7} transformation cases into {OUT}")


if __name__ == "__main__":
    main()
