"""A blown-up state is reported, not turned into plausible numbers: FP64 totals beyond
the FP32 range, infinities and NaN reach the FP32 primitives as infinities / NaN, and
the step sets PHD_STATUS_NONFINITE ("Non-finite primitive state after flux update").
The bad values are planted in the totals on the host side of the test; nothing here
can fault the device."""
import ctypes

import numpy as np
import pytest
import torch

import phd_code_gb300 as pkg
import phd_code_gb300._lib as L
from _util import lattice_mesh, smooth_state

pytestmark = pytest.mark.gpu


def _stepper():
    m = lattice_mesh(10, "periodic", seed=2)
    st = pkg.FluxStepper(m, smooth_state(m), gamma=1.4, cfl=0.5, solver="hllc", moving=True, precision="fp32")
    st.step(1)
    st.check_status()
    return st, m


def _status(st):
    return st.clock.read().status


@pytest.mark.parametrize("field,value", [(1, 1e300), (2, -1e300), (1, float("inf")), (3, float("nan")),
                                         (1, float("nan"))])
def test_update_reports_nonfinite_totals(field, value):
    st, m = _stepper()
    k = 7                                              # a real cell
    st.cons[field, k] = value
    st.step(1)
    torch.cuda.synchronize()
    assert _status(st) & L.STATUS_NONFINITE
    assert not np.isfinite(st.prim4[k].cpu().numpy()).any()
    with pytest.raises(RuntimeError, match="Non-finite primitive state"):
        st.check_status()


@pytest.mark.parametrize("value,expect", [(1e39, np.inf), (-1e39, -np.inf), (1e300, np.inf),
                                          (float("nan"), np.nan)])
def test_primitive_recovery_saturates(value, expect):
    """phd_prim_f32 narrows the FP64 totals with round-to-nearest into FP32: a mass just
    above the FP32 range (1e39 > 3.4e38) becomes an infinite density, not a wrapped
    exponent, and NaN stays NaN; the status bit is set."""
    st, m = _stepper()
    k = 3
    st.cons[0, k] = value
    rc = L.lib().phd_prim_f32(st.dmesh.ref, ctypes.byref(st.params), L.ptr(st.cons), L.ptr(st.prim4),
                              st.clock.ptr, L.stream_handle())
    L.check(rc, "phd_prim_f32")
    torch.cuda.synchronize()
    rho = float(st.prim4[k, 0].item())
    if np.isnan(expect):
        assert np.isnan(rho)
    else:
        assert rho == expect
    assert _status(st) & L.STATUS_NONFINITE
    # the other cells are untouched by the bad one
    others = np.delete(st.prim4.cpu().numpy(), k, axis=0)
    assert np.isfinite(others).all()


def test_finite_totals_keep_status_clear():
    st, m = _stepper()
    st.step(3)
    torch.cuda.synchronize()
    assert _status(st) == 0
