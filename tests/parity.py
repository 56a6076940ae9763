"""Parity assertions: integers bit-exact, FP64 within a relative tolerance of the oracle."""
import math

import numpy as np

# FP64 aggregates: the GPU folds partial sums in a different (fixed) order than the serial
# loop; the difference is bounded by the rounding of the two orders, well inside 1e-12 relative.
RTOL_F64 = 1e-12


def assert_same(got, ref, rtol=RTOL_F64, path="out"):
    if isinstance(ref, (tuple, list)):
        assert isinstance(got, (tuple, list)) and len(got) == len(ref), "%s: shape %r vs %r" % (path, got, ref)
        for i, (g, r) in enumerate(zip(got, ref)):
            assert_same(g, r, rtol, "%s[%d]" % (path, i))
        return
    if isinstance(ref, float):
        if math.isnan(ref):
            assert math.isnan(got), "%s: %r vs NaN" % (path, got)
            return
        if math.isinf(ref):
            assert got == ref, "%s: %r vs %r" % (path, got, ref)
            return
        tol = rtol * max(abs(ref), 1e-300)
        assert abs(got - ref) <= tol, "%s: %r vs %r (rel %.3g)" % (path, got, ref,
                                                                   abs(got - ref) / max(abs(ref), 1e-300))
        return
    assert got == ref, "%s: %r vs %r" % (path, got, ref)


def assert_table_same(got, ref, rtol=RTOL_F64):
    """`got`: DeviceTable.export() dict; `ref`: oracle Op result dict."""
    assert got["len"] == ref["len"], (got["len"], ref["len"])
    for c, (g, r) in enumerate(zip(got["cols"], ref["cols"])):
        if np.issubdtype(r.dtype, np.floating):
            np.testing.assert_allclose(g, r, rtol=rtol, atol=0, err_msg="column %d" % c)
        else:
            np.testing.assert_array_equal(g, r, err_msg="column %d" % c)
