"""parker_weight.m on the host (mexct_parker_weight; CPU only) against the FP64
oracle's window: the window rounded to single and multiplied into the single
sinogram, as the reference does (fbp_reconstruction/parker_weight.m:72-73), so
the result is bit for bit sino * float32(window) broadcast along u."""
import numpy as np
import pytest

F = np.float32
GEOMS = {0: "par3d", 1: "fan3d", 2: "cone3d"}


def _scan(extent, nP, decreasing=False):
    a = np.linspace(0.0, extent, nP).astype(F)
    return a[::-1].copy() if decreasing else a


@pytest.mark.parametrize("geom", [0, 1, 2])
@pytest.mark.parametrize("extent,q,decreasing", [
    (np.pi + 0.6, 1.0, False),    # a short scan with some overscan: original Parker
    (np.pi + 0.6, 0.1, False),    # modified weights (Wesarg et al.)
    (np.pi + 0.6, 1.0, True),     # decreasing angles: the fan angle flips sign
    (2 * np.pi, 1.0, False),      # a full turn
    (np.pi, 0.5, False),          # less than pi + fan angle: no redundant data
])
def test_parker_weight_matches_oracle_window(lib, orc, geom, extent, q, decreasing):
    import mexct

    W, nP, sad = 48, 37, 120.0
    rng = np.random.default_rng(geom * 10 + int(q * 10))
    sino = np.asfortranarray(rng.uniform(0.5, 2.0, (W, W, nP)).astype(F))
    ang = _scan(extent, nP, decreasing)
    got = mexct.parker_weight(sino, ang, {"type": GEOMS[geom], "SAD": sad}, q)
    win = orc.parker_window(W, ang, geom, q, sad).astype(F)  # [nP, W]
    want = sino * win.T[:, None, :]
    assert got.dtype == F and got.shape == sino.shape
    assert np.array_equal(got, want)
    if geom != 0 and extent < 2 * np.pi:
        assert np.any(win < 0.999)  # the window is not trivially 1


def test_parker_weight_checks_its_arguments(lib):
    from mexct import _lib
    import mexct

    ang = np.linspace(0, 4, 9).astype(F)
    with pytest.raises(_lib.MexctError) as ei:
        mexct.parker_weight(np.ones((8, 6, 9), F), ang, {"type": "cone3d", "SAD": 100.0})
    assert ei.value.status == _lib.ERR_UNSUPPORTED  # the reference needs W == H
    with pytest.raises(ValueError):
        mexct.parker_weight(np.ones((8, 8, 9), F), ang, {"type": "helix", "SAD": 100.0})
    with pytest.raises(_lib.MexctError) as ei:
        mexct.parker_weight(np.ones((8, 8, 9), F), ang, {"type": "fan3d", "SAD": 0.0})
    assert ei.value.status == _lib.ERR_ARG
