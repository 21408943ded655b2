"""The setup-time autotuner of mixed-precision handles (transform form and Vort2Flux order).

It times candidate forms on the GPU and keeps the fastest; every handle of one shape in a process
takes the same choice (so an ensemble member and the same problem stepped alone stay bitwise
equal); IBGB300_AUTOTUNE=0 keeps the fixed size rules; FP64 handles are never tuned.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solver(ib, wl, precision="mixed"):
    prob = wl.problem()
    st = ib.initstate(prob)
    st._gamma[:] = wl.initial_gamma()
    s = ib.initsolver(prob, st, precision=precision)
    s.vort2flux(st)
    return st, s


def test_choice_is_the_fastest_measured_and_in_effect(ib, lib):
    from ibgb300 import _lib as L
    wl = ib.workloads.scaled(ib.workloads.two_body_large(), 256, 256, nlevels=3)
    st, s = _solver(ib, wl)
    tune = s.autotune()
    assert tune["chosen"] is not None
    ms = tune["ms"]
    # the warp passes in both orders and both y-pass occupancies, the Stockham passes and the
    # tensor-core GEMMs were timed
    assert {"warp/levels", "warp/sequential", "warp/levels/y8", "warp/sequential/y8", "stockham/sequential",
            "tensor/sequential"} <= set(ms)
    # the fastest, or the size rule's choice when it is within 1% of the fastest
    assert ms[tune["chosen"]] <= 1.01 * min(ms.values())
    info = L.IbInfo()
    assert lib.ib_get_info(s.handle, ctypes.byref(info)) == 0
    form, order = tune["chosen"].split("/")[:2]
    assert info.transform_form == {"stockham": L.IB_FORM_STOCKHAM, "warp": L.IB_FORM_WARP,
                                   "tensor": L.IB_FORM_TENSOR}[form]
    assert info.vort2flux_order == (L.IB_V2F_LEVELS if order == "levels" else L.IB_V2F_SEQUENTIAL)
    # a second handle of the same shape reuses the decision and steps to the same bits
    st2, s2 = _solver(ib, wl)
    assert s2.autotune() == tune
    for i in range(3):
        ib.advance_(st, s, i * wl.dt)
        ib.advance_(st2, s2, i * wl.dt)
    np.testing.assert_array_equal(st.qty.gamma, st2.qty.gamma)
    s.close()
    s2.close()


def test_switched_off_and_fp64_untuned(ib):
    wl = ib.workloads.scaled(ib.workloads.two_body_large(), 128, 128, nlevels=2)
    os.environ["IBGB300_AUTOTUNE"] = "0"
    try:
        _, s = _solver(ib, wl)
        assert s.autotune()["chosen"] is None
        s.close()
    finally:
        os.environ.pop("IBGB300_AUTOTUNE", None)
    _, s = _solver(ib, wl, precision="fp64")
    assert s.autotune()["chosen"] is None
    s.close()
