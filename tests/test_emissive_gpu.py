"""The emissive CDF build on the GPU (reina_scene_set_emissive_build(REINA_EMISSIVE_DEVICE)) against the
host build (Instance::computeCDF, src/scene/Instance.cpp:15-53, and the duplicate search of
Instances::computeSamplingDataEmissives, Instances.cpp:52-114): the packed sampling data — instance
records, triangle CDFs, instance CDF, weights and areas — bit for bit, on scenes with several emissive
instances of shared and distinct models, rotated and scaled transforms, duplicates that the search
folds together, and a large emissive mesh; and the renders of both builds are identical."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


def build_pair(R, ctx, make):
    out = []
    for where in (R.EMISSIVE_HOST, R.EMISSIVE_DEVICE):
        s = make(R, ctx)
        s.set_emissive_build(where)
        s.build()
        out.append(s)
    return out


def emissive_field(R, ctx):
    """Six emissive instances: three copies of one sphere (two identical transforms: duplicates), two of a
    second sphere, and a quad; plus a non-emissive floor."""
    s = R.Scene(ctx)
    v1, i1, _ = R.icosphere(3, 0.1, 5)
    v2, i2, _ = R.icosphere(2, 0.2, 9)
    a = s.define_object(v1, i1)
    b = s.define_object(v2, i2)
    lv, li = scenes.quad((-0.3, 0.99, -0.3), (0.6, 0, 0), (0, 0, 0.6))
    m = lambda e: R.Material(material_idx=0, albedo=(0.7, 0.7, 0.7), emission=e)
    # (model, emission, pose): instances 0 and 1 share model and pose, so their CDFs are the same
    for obj, e, k in [(a, (3.0, 2.0, 1.0), 0), (a, (3.0, 2.0, 1.0), 0), (a, (0.5, 4.0, 0.2), 1),
                      (b, (1.0, 1.0, 1.0), 2), (b, (2.0, 0.5, 0.5), 3)]:
        t = np.eye(4, dtype=np.float32)
        ang = 0.37 * k
        c, sn = np.cos(ang), np.sin(ang)
        t[:3, :3] = (0.2 + 0.05 * (k % 3)) * np.array([[c, 0, sn], [0, 1, 0], [-sn, 0, c]], np.float32)
        t[:3, 3] = (-0.6 + 0.3 * (k % 3), -0.2, -0.4)
        s.add_instance(obj, t, m(e))
    s.add_object(lv, li, material=m((10.0, 9.0, 8.0)))
    fv, fi = scenes.quad((-1, -1, -1), (2, 0, 0), (0, 0, 2))
    s.add_object(fv, fi, material=m((0.0, 0.0, 0.0)))
    return s


def emissive_big(R, ctx):
    """One emissive 1.3M-triangle displaced sphere (level-8 icosphere) and a floor."""
    s = R.Scene(ctx)
    v, i, _ = R.icosphere(8, 0.1, 1)
    s.add_object(v, i, material=R.Material(material_idx=0, albedo=(0.5, 0.5, 0.5), emission=(1.0, 0.8, 0.6)))
    fv, fi = scenes.quad((-2, -1.2, -2), (4, 0, 0), (0, 0, 4))
    s.add_object(fv, fi, material=R.Material(material_idx=0, albedo=(0.5, 0.5, 0.5)))
    return s


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("make", [emissive_field, emissive_big])
def test_device_cdf_build_equals_host(R, gpu_ctx, make):
    host, dev = build_pair(R, gpu_ctx, make)
    (ih, th, ch), (idv, tdv, cdv) = host.export_emissive(), dev.export_emissive()
    assert ih.size >= 1 and th.size > 0
    assert same_bits(ih, idv)
    assert same_bits(th, tdv)
    assert same_bits(ch, cdv)
    assert host.emissive_weight == dev.emissive_weight
    if make is emissive_field:   # the two identical instances share one CDF range
        assert len({(int(r["cdfRangeStart"]), int(r["cdfRangeEnd"])) for r in ih}) == ih.size - 1
    host.close()
    dev.close()


def test_device_cdf_build_renders_identically(R, gpu_ctx):
    host, dev = build_pair(R, gpu_ctx, emissive_field)
    iv, ip = scenes.cornell_camera(R, 48, 40)
    imgs = []
    for s in (host, dev):
        pc = R.push_consts(iv, ip, total_emissive_weight=s.emissive_weight, spp=4, max_bounces=5, focus_dist=3.4)
        acc, _, _ = R.render(gpu_ctx, s, pc, R.render_options(48, 40, R.MODE_NEE_MIS, 3))
        imgs.append(acc)
    assert np.array_equal(imgs[0], imgs[1])
    assert imgs[0][..., :3].mean() > 0
    host.close()
    dev.close()
