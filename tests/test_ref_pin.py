"""Parity pinned to the reference's own outputs (tests/golden/ref_golden.npz).

The fixture holds outputs of the reference's CUDA kernels, compiled unmodified from
its .cu files and run on a GB300 (tests/golden/make_ref_golden.py).

CPU: the FP64 oracle, with the texture unit's weight rule (TEX_HW) and the
reference's binary32 stepping, reproduces every reference output to a few 1e-6
(what is left is the reference's FP32 summation); its default exact mode differs
from the reference by the stated texture-filter and stepping difference.
GPU: the CUDA library against the same outputs: the texture FP variant bit for
bit, the default exact-weight path within the stated texture difference.
"""
import numpy as np
import pytest

from conftest import rel_l2

SAD = 1000.0

# Oracle (TEX_HW + binary32 stepping) vs reference, relative L2.  Measured on the
# committed fixture: FP 1.2e-7 .. 3.6e-7, BP 5e-8 .. 1.5e-6, OSC 1.9e-7,
# general3D FP 1.8e-7 / 4.6e-7, general3D BP 3e-8 / 4e-8 (float atomics),
# TV 1.4e-7 / 2.7e-6 (FP32 against FP64 descent steps).
PIN_TOL = 3e-6
# Exact-weight oracle (the library's arithmetic) vs reference: the texture unit's
# 8-bit weights and the reference's binary32 stepping.  Measured: FP <= 2.1e-4,
# BP <= 8.5e-4, OSC <= 3.7e-4, general3D FP <= 1.5e-4.
TEXTURE_DIFF = {"fp": 3e-4, "bp": 1e-3, "osc": 5e-4, "g3dfp": 2e-4, "g3dbp": 5e-6, "tv": 5e-6}


@pytest.fixture(scope="module")
def refgold():
    from golden import make_ref_golden

    return make_ref_golden.load()


def _oracle_outputs(orc, x):
    s, m, g = x["s"], x["m"], x["g"]
    out = {}
    for geom in (0, 1, 2):
        for tag, d in (("s", s), ("m", m)):
            out["%s_fp%d" % (tag, geom)] = orc.fp(d["vol"], SAD, d["ang"], len(d["ang"]), geom)
            out["%s_bp%d" % (tag, geom)] = orc.bp(d["sino"], SAD, d["ang"], geom)
        out["s_osc%d" % geom] = orc.osc_iter(s["mu0"], s["pre"], s["post"], 5, s["order5_1"], s["ang"], SAD, geom)
    for tag, d in (("s", s), ("g", g)):
        S, Z = d["vol"].shape[0], d["vol"].shape[2]
        out["%s_g3dfp" % tag] = orc.g3d_fp(d["vol"], d["hang"], d["pts"], len(d["hang"]))
        out["%s_g3dbp" % tag] = orc.g3d_bp(d["hsino"], d["hang"], d["pts"], S, Z)
    out["s_tv"] = orc.tvmin3d(s["tvin"], 0.02, 20)
    out["g_tv"] = orc.tvmin3d(g["tvin"], 0.05, 20)
    return out


def _kind(key):
    k = key.split("_", 1)[1].rstrip("0123456789")
    return k


def test_fixture_is_from_the_reference_on_a_gb300(refgold):
    _, y, meta = refgold
    assert "GB300" in meta["gpu"]
    assert "unmodified" in meta["kernels"]
    assert len([k for k in y if not k.startswith("s_oscp")]) == 21


def test_oracle_reproduces_reference_outputs(orc, refgold):
    """With the texture unit's weights and the reference's binary32 stepping the
    oracle lands on the reference's own outputs (pins the oracle)."""
    x, y, _ = refgold
    with orc.tex_weights(orc.TEX_HW), orc.ref_steps(1):
        got = _oracle_outputs(orc, x)
    errs = {k: rel_l2(got[k], y[k]) for k in got}
    bad = {k: v for k, v in errs.items() if v > PIN_TOL}
    assert not bad, bad


def test_exact_oracle_difference_from_reference_is_stated(orc, refgold):
    """The library's arithmetic (exact FP32 weights, exact sample positions)
    differs from the reference by no more than the stated texture difference,
    and by more than the pin (the difference is real, and attributed)."""
    x, y, _ = refgold
    got = _oracle_outputs(orc, x)
    for k in got:
        e = rel_l2(got[k], y[k])
        assert e <= TEXTURE_DIFF[_kind(k)], (k, e)
    assert rel_l2(got["m_fp2"], y["m_fp2"]) > 10 * PIN_TOL


def test_stepping_difference_is_small_at_fixture_sizes(orc, refgold):
    """Binary32 stepping alone moves the oracle by well under 1e-5 at these
    sizes (1.25e-5 for FP at 512^3, stated in the design notes)."""
    x, _, _ = refgold
    m = x["m"]
    a = orc.fp(m["vol"], SAD, m["ang"], len(m["ang"]), 2)
    with orc.ref_steps(1):
        b = orc.fp(m["vol"], SAD, m["ang"], len(m["ang"]), 2)
    assert 0 < rel_l2(b, a) < 1e-5


@pytest.mark.gpu
def test_texture_variant_is_the_reference_bit_for_bit(cuda, refgold):
    """MEXCT_FP_TEXTURE: the reference's sampling arithmetic on the same texture
    hardware reproduces its FP output exactly."""
    import torch
    from mexct import _lib, ops

    x, y, _ = refgold
    for tag in ("s", "m"):
        d = x[tag]
        dvol = torch.from_numpy(np.ascontiguousarray(d["vol"].transpose(2, 1, 0))).cuda()
        for geom in (0, 1, 2):
            out = ops.fp_dev(dvol, SAD, d["ang"], geom, variant=_lib.FP_TEXTURE)
            got = out.cpu().numpy().transpose(2, 1, 0)
            ref = y["%s_fp%d" % (tag, geom)]
            assert np.array_equal(got, ref), (tag, geom, rel_l2(got, ref))


@pytest.mark.gpu
def test_cuda_path_vs_reference_outputs(cuda, refgold):
    """The default (exact-weight) CUDA path differs from the reference's outputs
    by no more than the stated texture difference."""
    import mexct

    x, y, _ = refgold
    s, m, g = x["s"], x["m"], x["g"]
    for geom in (0, 1, 2):
        for tag, d in (("s", s), ("m", m)):
            fp = mexct.CUDAmex_FP(d["vol"], SAD, d["ang"], len(d["ang"]), geom)
            assert rel_l2(fp, y["%s_fp%d" % (tag, geom)]) <= TEXTURE_DIFF["fp"]
            bp = mexct.CUDAmex_BP(d["sino"], SAD, d["ang"], geom)
            assert rel_l2(bp, y["%s_bp%d" % (tag, geom)]) <= TEXTURE_DIFF["bp"]
        mu = np.array(s["mu0"], dtype=np.float32, order="F", copy=True)
        mexct.CUDAmex_oscIter(mu, s["pre"], s["post"], 5, s["order5_1"], s["ang"], SAD, geom)
        assert rel_l2(mu, y["s_osc%d" % geom]) <= TEXTURE_DIFF["osc"]
    for tag, d in (("s", s), ("g", g)):
        S, Z = d["vol"].shape[0], d["vol"].shape[2]
        g3 = mexct.CUDAmex_general3D_FP(d["vol"], d["hang"], d["pts"], len(d["hang"]))
        assert rel_l2(g3, y["%s_g3dfp" % tag]) <= TEXTURE_DIFF["g3dfp"]
        gb = mexct.CUDAmex_general3D_BP(d["hsino"], d["hang"], d["pts"], S, Z)
        assert rel_l2(gb, y["%s_g3dbp" % tag]) <= TEXTURE_DIFF["g3dbp"]
    assert rel_l2(mexct.CUDAmex_TVmin_3D(s["tvin"], 0.02), y["s_tv"]) <= TEXTURE_DIFF["tv"]
    assert rel_l2(mexct.CUDAmex_TVmin_3D(g["tvin"], 0.05), y["g_tv"]) <= TEXTURE_DIFF["tv"]
