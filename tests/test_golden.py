"""Committed golden vectors (tests/golden/golden.npz, made by make_golden.py).

CPU: the oracle reproduces the fixture (pins the oracle against regressions).
GPU: the CUDA path matches the fixture within the FP32 tolerance.
"""
import numpy as np
import pytest

from conftest import rel_l2


@pytest.fixture(scope="module")
def golden():
    from golden import make_golden

    return make_golden.load()


def test_oracle_reproduces_golden(orc, golden):
    from golden import make_golden

    x, y = golden
    got = make_golden.outputs(x)
    assert sorted(got) == sorted(y)
    for k in y:
        np.testing.assert_allclose(got[k], y[k], rtol=1e-12, atol=1e-12, err_msg=k)


TOL = 1e-5  # FP32 vs FP64 golden, relative L2


@pytest.mark.gpu
def test_cuda_path_matches_golden(cuda, golden):
    import mexct

    x, y = golden
    for g in (0, 1, 2):
        fp = mexct.CUDAmex_FP(x["vol"], 1000.0, x["ang"], x["nP"], g)
        assert rel_l2(fp, y["fp%d" % g]) <= TOL, "fp%d" % g
        bp = mexct.CUDAmex_BP(x["sino"], 1000.0, x["ang"], g)
        assert rel_l2(bp, y["bp%d" % g]) <= TOL, "bp%d" % g
        mu = np.array(x["mu0"], dtype=np.float32, order="F", copy=True)
        mexct.CUDAmex_oscIter(mu, x["pre"], x["post"], 5, y["order5_1"].astype(np.int32),
                              x["ang"], 1000.0, g)
        assert rel_l2(mu, y["osc%d" % g]) <= TOL, "osc%d" % g
        pf = mexct.preFilterSinogram(x["sq"], {"type": ["par3d", "fan3d", "cone3d"][g], "SAD": 1000.0},
                                     x["sqa"], "hamming", 1.0, 1.0)
        assert rel_l2(pf, y["pf%d" % g]) <= TOL, "pf%d" % g
    g3 = mexct.CUDAmex_general3D_FP(x["vol"], x["hang"], x["pts"], 6)
    assert rel_l2(g3, y["g3dfp"]) <= TOL
    gb = mexct.CUDAmex_general3D_BP(x["hsino"], x["hang"], x["pts"], x["W"], x["H"])
    assert rel_l2(gb, y["g3dbp"]) <= TOL
    tv = mexct.CUDAmex_TVmin_3D(x["tvin"], 0.02)
    assert rel_l2(tv, y["tv"]) <= TOL
