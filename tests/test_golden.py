"""The oracle reproduces the committed golden fixture bit for bit (pins the
oracle across compilers and machines; see tests/golden/make_golden.py)."""
import os

import numpy as np

from tests.golden.make_golden import CASE, run

HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_reproduces_golden_fixture():
    ref = np.load(os.path.join(HERE, "golden", "weibel2d_small.npz"))
    p, out = run()
    for k in ref.files:
        a, b = out[k], ref[k]
        assert a.shape == b.shape, k
        if a.dtype.kind == "f":
            np.testing.assert_array_equal(a.view(np.int64), b.view(np.int64), err_msg=k)
        else:
            np.testing.assert_array_equal(a, b, err_msg=k)
    assert CASE["nx"] == p.nx
