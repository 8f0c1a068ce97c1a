"""The batch entry points' Python marshalling: the numpy views of
simpois_image and simpois_report match the ctypes structures field by field."""
import ctypes

import numpy as np

from imscript_gb300 import lib


def test_image_array_matches_the_ctypes_structure():
    rows = [(0x1000, 0, 0x2000, 640, 480, 3, 0.25, 1e-6), (0x3000, 0x4000, 0x5000, 7, 9, 1, -0.08, 0.0)]
    keep, arr = lib.image_array(rows)
    for k, r in enumerate(rows):
        im = arr[k]
        assert (im.inp, im.dat or 0, im.out, im.w, im.h, im.pd) == r[:6]
        assert im.tstep == np.float32(r[6]) and im.rtol == r[7]
    assert keep.dtype.itemsize == ctypes.sizeof(lib.Image)


def test_report_dicts_match_as_dict():
    reps = (lib.Report * 5)()
    for k in range(5):
        reps[k].status, reps[k].unknowns, reps[k].iterations = k, 10 * k, 3 + k
        reps[k].refinements, reps[k].rel_residual, reps[k].rel_residual_out = 1, 1e-7 * k, -1.0
    assert lib.report_dicts(reps) == [r.as_dict() for r in reps]
    assert lib.report_dicts(reps, 3) == [r.as_dict() for r in reps][:3]
