"""The reference-side binding (opencamlib_gb300/integration/reference_binding.cpp),
compiled against the reference's own headers: every cutter object the
reference's drop-cutter accepts maps to a descriptor from which the oracle
derives exactly the object's own fields (diameter, radius, length,
center_height, normal lengths; for composites the radius/height/zoffset
vectors), ConeCutter's folded length included
(src/cutters/conecutter.cpp:39-49: length = radius / tan(angle) + l).
Only built where the reference tree is present."""
import math

import numpy as np
import pytest

from opencamlib_gb300 import _abi

checker = pytest.importorskip("oracle.checker")

pytestmark = pytest.mark.skipif(not checker.available("binding"),
                                reason="reference-side binding not built (reference tree absent)")

BASIC = [(1, (6.0, 20.0)), (1, (0.3, 1.7)), (2, (3.0, 20.0)), (2, (7.1, 4.3)), (3, (8.0, 1.5, 20.0)),
         (3, (2.0, 0.999, 5.0)), (4, (6.0, math.pi / 4, 20.0)), (4, (6.0, math.pi / 3, 7.3)),
         (4, (10.0, 0.3, 50.0)), (4, (1.0, 1.2, 0.1)), (4, (3.3, 0.7853981, 1e-3)), (4, (12.7, 1.3, 33.0))]
PRESETS = [(11, (6.0, 20.0)), (12, (6.0, 20.0)), (13, (2.0, 6.0, math.pi / 4)), (14, (2.0, 6.0, math.pi / 4)),
           (15, (4.0, 1.0, 8.0, math.pi / 4)), (16, (2.0, math.pi / 3, 6.0, math.pi / 5))]


@pytest.mark.parametrize("kind,args", BASIC + PRESETS)
def test_descriptor_reproduces_reference_fields(kind, args):
    st, desc, ref = checker.binding_cutter(kind, args)
    assert st == _abi.OK
    np.testing.assert_array_equal(checker.cutter_fields(desc), ref)


def test_cone_length_argument_round_trips():
    """The descriptor's l gives back the reference object's length bit for
    bit, even where length - radius / tan(angle) is not that l."""
    rng = np.random.default_rng(5)
    for _ in range(200):
        d, a, l = 0.5 + 20 * rng.random(), 0.05 + 1.45 * rng.random(), 1e-3 + 50 * rng.random()
        st, desc, ref = checker.binding_cutter(4, (d, a, l))
        assert st == _abi.OK and desc.kind == _abi.CUTTER_CONE
        r = desc.base.diameter / 2
        assert r / math.tan(desc.base.angle) + desc.base.length == ref[6]


def test_drop_through_binding_without_device():
    """mesh_create/batch_drop reach the library: NO_DEVICE on a host without
    a GPU, the lifted z on one with a GPU."""
    st, z = checker.binding_drop()
    if st == _abi.OK:
        assert z > -5.0
    else:
        assert st == _abi.NO_DEVICE
