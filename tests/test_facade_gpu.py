"""The C++ facade (opencamlib_gb300/include/ocl/ocl.hpp), compiled into
tests/facade/facade_test.cpp the way client code of the reference library
uses it, reproduces the reference's golden results on the GPU."""
import math
import os
import subprocess

import numpy as np
import pytest

from tests.helpers import golden

pytestmark = pytest.mark.gpu

ARGS = {"ball": ["ball", "6", "20"], "bull": ["bull", "6", "1", "20"], "cyl": ["cyl", "6", "20"],
        "cone": ["cone", "6", repr(math.pi / 4), "20"], "ballcone": ["ballcone", "2", "6", repr(math.pi / 4)]}


@pytest.fixture(scope="module")
def exe():
    from opencamlib_gb300 import _build
    _build.build_library()
    p = _build.build_facade_test()
    assert p and os.path.exists(p)
    return p


def _run(exe, tmp_path, mode, tris, data, extra):
    t = tmp_path / "t.bin"
    d = tmp_path / "d.bin"
    o = tmp_path / "o.bin"
    np.ascontiguousarray(tris, dtype=np.float64).tofile(t)
    np.ascontiguousarray(data, dtype=np.float64).tofile(d)
    r = subprocess.run([exe, mode, str(t), str(d), str(o)] + extra, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return np.fromfile(o, dtype=np.float64)


@pytest.mark.parametrize("cname", sorted(ARGS))
def test_facade_batch_drop(exe, tmp_path, cname):
    g = golden("drop_heightfield")
    out = _run(exe, tmp_path, "drop", g["tris"], g["cl"], ARGS[cname]).reshape(-1, 7)
    assert np.max(np.abs(out[:, 2] - g[f"{cname}_z"])) <= 1e-5
    np.testing.assert_array_equal(out[:, 6].astype(np.int32), g[f"{cname}_type"])


@pytest.mark.parametrize("cname", ["ball", "bull"])
def test_facade_push(exe, tmp_path, cname):
    g = golden("push_heightfield")
    out = _run(exe, tmp_path, "push", g["tris"], g["fib_x"], ["0"] + ARGS[cname])
    counts = g[f"{cname}_0_counts"]
    k = 0
    ival = g[f"{cname}_0_ival"]
    j = 0
    for n in counts:
        assert int(out[k]) == n
        k += 1
        for _ in range(int(n)):
            assert abs(out[k] - ival[j, 0]) < 1e-9 and abs(out[k + 1] - ival[j, 1]) < 1e-9
            k += 10
            j += 1


def test_facade_path(exe, tmp_path):
    g = golden("path_heightfield")
    out = _run(exe, tmp_path, "path", g["tris"], g["spans"], ["0.37", "-5.0"] + ARGS["ball"]).reshape(-1, 7)
    assert np.max(np.abs(out[:, :3] - g["ball_pdc_xyz"])) <= 1e-7
