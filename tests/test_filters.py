"""Film filters (src/filter.rs:44-124) beyond the box: the product's host
filter table against the oracle's restatement, for every kind."""
import ctypes as C

import numpy as np
import pytest

from pbrt_rust_gb300 import abi
from pbrt_rust_gb300.scene import Camera, Film, Filter
from pbrt_rust_gb300.transform import Transform

FILTERS = [Filter.mean(0.5, 0.5), Filter.triangle(2.0, 1.5), Filter.gaussian(2.0, 2.0, 2.0),
           Filter.mitchell(2.0, 2.0, 1.0 / 3.0, 1.0 / 3.0), Filter.lanczos(3.0, 2.5, 3.0)]


def camera(filt):
    return Camera.perspective(Transform(), (-1, 1, -1, 1), 0.0, 1.0, 0.0, 1e30, 60.0, Film.image(32, 24, filt))


@pytest.mark.parametrize("filt", FILTERS, ids=lambda f: f.kind)
def test_filter_table_matches_oracle(lib, oracle, filt):
    cam = camera(filt).to_abi()
    got = (C.c_float * 256)()
    assert lib.pbrtgpu_filter_table(C.byref(cam), got) == 0
    ev = oracle.load().oracle_filter_eval
    kind = abi.FILTERS[filt.kind]
    want = np.zeros(256, np.float32)
    for y in range(16):
        fy = np.float32((np.float32(y) + np.float32(0.5)) * np.float32(filt.y_width) / np.float32(16.0))
        for x in range(16):
            fx = np.float32((np.float32(x) + np.float32(0.5)) * np.float32(filt.x_width) / np.float32(16.0))
            want[y * 16 + x] = ev(kind, filt.x_width, filt.y_width, filt.p0, filt.p1, fx, fy)
    assert np.array_equal(np.frombuffer(got, np.float32).view(np.uint32), want.view(np.uint32))
    if filt.kind != "box":
        assert len(set(want.tolist())) > 4  # a real, varying table


def test_unknown_filter_kind_is_refused(lib):
    cam = camera(Filter.mean(0.5, 0.5)).to_abi()
    cam.filter_kind = 9
    got = (C.c_float * 256)()
    assert lib.pbrtgpu_filter_table(C.byref(cam), got) == 1
