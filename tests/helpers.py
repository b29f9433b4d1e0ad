"""Shared test helpers."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def push_records_equal(res, g, prefix, exact=True, sort=False, tol=0.0, cc_tol=1e-6):
    """Compare per-fiber interval records with a golden set.  With sort=True
    both sides are ordered by lower t (the GPU returns sorted intervals, the
    reference keeps insertion order).  exact=False: endpoints within tol (in
    fiber parameter t), CC points within cc_tol mm, CC types identical."""
    counts = g[prefix + "_counts"]
    ival = g[prefix + "_ival"]
    cc = g[prefix + "_cc"]
    ty = g[prefix + "_type"]
    assert len(res) == len(counts)
    k = 0
    for f, r in enumerate(res):
        n = int(counts[f])
        assert len(r) == n, (f, len(r), n)
        ref = [(ival[k + j, 0], ival[k + j, 1], cc[k + j, :3], cc[k + j, 3:], ty[k + j, 0], ty[k + j, 1])
               for j in range(n)]
        k += n
        got = list(r)
        if sort:
            ref.sort(key=lambda x: x[0])
            got.sort(key=lambda x: x[0])
        for a, b in zip(got, ref):
            if exact:
                assert a[0] == b[0] and a[1] == b[1], (f, a[:2], b[:2])
                np.testing.assert_array_equal(a[2], b[2])
                np.testing.assert_array_equal(a[3], b[3])
                assert a[4] == b[4] and a[5] == b[5]
            else:
                assert abs(a[0] - b[0]) <= tol and abs(a[1] - b[1]) <= tol, (f, a[:2], b[:2])
                assert a[4] == b[4] and a[5] == b[5], (f, a[4:], b[4:])
                assert np.max(np.abs(a[2] - b[2])) <= cc_tol and np.max(np.abs(a[3] - b[3])) <= cc_tol, (f, a, b)
