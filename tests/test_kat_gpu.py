"""The device's own shading functions (reina_device_kat: the code the integrators run) against the known
answers: the Wächter-Binder offset bit for bit (it moves float bit patterns, so it must be exact), GGX
visible-normal sampling against the float64 fixture and the oracle's FP32 evaluation (same RNG state
after the draws), and the Disney evaluation against the oracle's FP32 evaluation."""
import numpy as np
import pytest

import kat_cases

pytestmark = pytest.mark.gpu


def test_device_offset_is_bit_exact(R, gpu_ctx):
    rec, want = kat_cases.offset_cases()
    got = R.device_kat(gpu_ctx, R.KAT_OFFSET, rec)[:, :3].view(np.uint32)
    assert np.array_equal(got, want)


def test_device_ggx_vndf(R, O, gpu_ctx):
    rec, h, state = kat_cases.ggx_cases()
    got = R.device_kat(gpu_ctx, R.KAT_GGX_VNDF, rec)
    assert np.array_equal(got[:, 3].view(np.uint32).astype(np.uint64), state)
    assert np.allclose(got[:, :3], h, rtol=2e-5, atol=2e-5)
    o32 = O.kat(O.KAT_GGX_VNDF, rec, 32)
    assert np.allclose(got[:, :3], o32[:, :3], rtol=1e-5, atol=1e-6)


def test_device_eval_disney(R, O, gpu_ctx):
    rec = kat_cases.disney_cases()
    got = R.device_kat(gpu_ctx, R.KAT_EVAL_DISNEY, rec).astype(np.float64)
    ref = O.kat(O.KAT_EVAL_DISNEY, rec, 32)
    ok = (np.abs(got - ref) <= 1e-4 * np.abs(ref) + 1e-5) | (np.isnan(got) & np.isnan(ref))
    assert ok.all(axis=1).mean() >= 0.99
