"""Single shading functions of the oracle pinned against known answers restated independently in
numpy (tests/golden/gen_golden.py): the Wächter-Binder offset bit for bit in float32, GGX visible-normal
sampling in float64 with the shader RNG's draws; and the Disney evaluation's FP32 and FP64 modes
against each other."""
import numpy as np

import kat_cases


def test_offset_matches_golden(O):
    rec, want = kat_cases.offset_cases()
    got = O.kat(O.KAT_OFFSET, rec, 32)[:, :3].astype(np.float32).view(np.uint32)
    assert np.array_equal(got, want)


def test_ggx_vndf_matches_golden(O):
    rec, h, state = kat_cases.ggx_cases()
    got = O.kat(O.KAT_GGX_VNDF, rec, 64)
    assert np.allclose(got[:, :3], h, rtol=1e-12, atol=1e-12)
    assert np.array_equal(got[:, 3].astype(np.uint64), state)
    g32 = O.kat(O.KAT_GGX_VNDF, rec, 32)
    assert np.allclose(g32[:, :3], h, rtol=2e-5, atol=2e-5)


def test_disney_fp32_agrees_with_fp64(O):
    rec = kat_cases.disney_cases()
    a = O.kat(O.KAT_EVAL_DISNEY, rec, 32)
    b = O.kat(O.KAT_EVAL_DISNEY, rec, 64)
    fin = np.isfinite(b).all(axis=1)
    assert fin.mean() > 0.9
    ok = np.abs(a[fin] - b[fin]) <= 1e-4 * np.abs(b[fin]) + 1e-5
    assert ok.all(axis=1).mean() >= 0.98
