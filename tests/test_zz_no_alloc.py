"""The allocation-free render entry point (reina_render_device_noalloc) against the regular device entry
point (reina_render_device), through the C ABI.

The allocation-free entry point is for callers that cannot call cudaMalloc while they run (a host whose
allocator owns all device memory, a process whose memory budget is already handed out, a frame loop
that cannot take a cudaMalloc's synchronization); it keeps the render's path state in a fixed array
inside the library.  Two calls in a row must each reproduce the regular render, so the second call also
shows that the shared array is cleared where it must be.  This file sorts last so that a run stopping at
its first failure has already run every other test.
"""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode,W,H", [(1, 256, 256), (0, 160, 96)])
def test_noalloc_render_matches_regular_render_twice(R, gpu_ctx, mode, W, H):
    torch = pytest.importorskip("torch")
    d = scenes.material_zoo(R)
    scene = d.to_product(R, gpu_ctx)
    iv, ip = scenes.cornell_camera(R, W, H)
    spp = 4
    pc = R.push_consts(iv, ip, total_emissive_weight=scene.emissive_weight, spp=spp, max_bounces=8, focus_dist=3.4)
    opts = R.render_options(W, H, mode, 1)
    stream = torch.cuda.current_stream().cuda_stream

    acc_ref = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    smp_ref = torch.zeros((W * H, spp, 3), dtype=torch.float32, device="cuda")
    R.render_device(gpu_ctx, scene, pc, opts, acc_ref.data_ptr(), smp_ref.data_ptr(), stream)
    torch.cuda.synchronize()
    ref_acc, ref_smp = acc_ref.cpu().numpy(), smp_ref.cpu().numpy()
    assert np.isfinite(ref_acc).all() and ref_acc[..., :3].mean() > 0.01

    outs = [(torch.full((H, W, 4), -7.0, dtype=torch.float32, device="cuda"),
             torch.full((W * H, spp, 3), -7.0, dtype=torch.float32, device="cuda")) for _ in range(2)]
    # A first call loads the library's module on the device if nothing has yet (CUDA's lazy module loading),
    # which reserves the fixed array; free memory is compared over the calls after it.
    warm = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    R.render_device_noalloc(gpu_ctx, scene, pc, opts, warm.data_ptr(), 0, stream)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for acc, smp in outs:
        R.render_device_noalloc(gpu_ctx, scene, pc, opts, acc.data_ptr(), smp.data_ptr(), stream)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before, "the allocation-free render changed free device memory"
    # The pass-by-pass wavefront and the wave engine give bit-identical images, so equality is exact.
    for call, (acc, smp) in enumerate(outs):
        a, s = acc.cpu().numpy(), smp.cpu().numpy()
        assert np.array_equal(s, ref_smp, equal_nan=True), call
        assert np.array_equal(a, ref_acc, equal_nan=True), call


def test_noalloc_render_rejects_images_above_its_limit(R, gpu_ctx):
    torch = pytest.importorskip("torch")
    d = scenes.cornell(R)
    scene = d.to_product(R, gpu_ctx)
    W, H = 257, 256
    assert W * H > R.NOALLOC_MAX_PIXELS
    iv, ip = scenes.cornell_camera(R, W, H)
    pc = R.push_consts(iv, ip, total_emissive_weight=scene.emissive_weight, spp=1, max_bounces=2)
    acc = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(R.ReinaError) as e:
        R.render_device_noalloc(gpu_ctx, scene, pc, R.render_options(W, H, 1, 1), acc.data_ptr(), 0,
                                torch.cuda.current_stream().cuda_stream)
    assert e.value.code == R.REINA_ERR_INVALID
    assert str(R.NOALLOC_MAX_PIXELS) in str(e.value)
