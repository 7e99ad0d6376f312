"""Bounded waits of the slab forward projector.  Failure is made on purpose without
faulting or hanging anything: with the wait limit at 0 every copy wait that is not
already satisfied gives up at once, the CTA samples from global memory instead, the
result still meets the parity bound, and the host reads the flag from the device
error word.  With the default limit no wait gives up."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("geom", [0, 2])
def test_waits_that_give_up_fall_back_and_are_reported(cuda, orc, geom):
    import mexct
    from mexct import ops, phantoms

    W, H, nP = 64, 48, 24
    vol = phantoms.ellipsoids(W, count=5, seed=11, nz=H)
    ang = phantoms.angles_full(nP)
    ref = orc.fp(vol, 1000.0, ang, nP, geom)
    try:
        ops.set_wait_limit(0)
        ops.device_errors(clear=True)
        got = mexct.CUDAmex_FP(vol, 1000.0, ang, nP, geom)
        flags = ops.device_errors(clear=True)
    finally:
        ops.set_wait_limit(-1)
    assert rel_l2(got, ref) <= 1e-5
    assert flags & 1, "no wait gave up with a zero limit"
    again = mexct.CUDAmex_FP(vol, 1000.0, ang, nP, geom)
    assert ops.device_errors() == 0
    assert rel_l2(again, ref) <= 1e-5
