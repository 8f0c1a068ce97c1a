"""Loading of the golden fixtures in tests/golden/ (shared by CPU and GPU tests)."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def parse_args(args, env):
    """simpois option values as main_simpois reads them (simpois.c:357-360):
    atof, then truncation to int where the solver takes an int."""
    opt = {"t": "0.25", "n": "10", "s": "99", "c": "0"}
    k = 0
    while k < len(args):
        a = args[k]
        if a.startswith("-") and a[1:] in opt:
            opt[a[1:]] = args[k + 1]
            k += 2
        else:
            k += 1
    kw = dict(tstep=float(np.float32(float(opt["t"]))), niter=int(float(opt["n"])),
              scale=int(float(opt["s"])), cgrad=float(opt["c"]))
    kw["pmsfac"] = float(env.get("PMSFAC", 3))
    kw["ponlit"] = float(env.get("PONLIT", 0))
    kw["cg_eps"] = float(env.get("CG_EPS", -1))
    return kw


def load(path):
    z = np.load(path)
    d = {k: z[k] for k in z.files}
    d["args"] = json.loads(str(d["args"]))
    d["env"] = json.loads(str(d["env"]))
    d["extra"] = json.loads(str(d["extra"])) if "extra" in d else {}
    d["f"] = d.get("f")
    d["mask"] = d.get("mask")
    d["init"] = d.get("init")
    d["name"] = os.path.splitext(os.path.basename(path))[0]
    return d


def cases(prefix):
    return sorted(glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def amle_inputs(d):
    """(x, nn, niter, init) of an amle_* fixture as the reference ran it:
    mask > 0 becomes NaN (src/amle.c:357-360), AMLE_NN / AMLE_NITER truncated
    to int, AMLE_INIT the stored start image."""
    x = d["g"].copy()
    if d["mask"] is not None:
        x[:, d["mask"] > 0] = np.nan
    nn = int(float(d["env"].get("AMLE_NN", 4)))
    niter = int(float(d["env"].get("AMLE_NITER", 100)))
    return x, nn, niter, d["init"]


def same_bits_or_nan(a, b):
    """Bit-equal where finite or infinite; NaN where the other is NaN (the
    NaN of 0/0 has another sign bit on x86-64 than on aarch64 or the GPU)."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32)))
