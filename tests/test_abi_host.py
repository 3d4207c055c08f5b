"""CPU tests of the C ABI and the host logic: exported symbols, struct layouts, scene assembly (emissive
CDFs, offsets, errors) and the structure of the quantized BVH8 — all without a GPU (host-only context)."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include" / "reina").glob("*.h"))


def declared_functions() -> list[str]:
    names = []
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(reina_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(R):
    lib = R.load_library()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_headers_compile_as_c_and_layouts(tmp_path):
    src = tmp_path / "t.c"
    src.write_text(
        '#include "reina/reina_c.h"\n'
        "#include <stddef.h>\n"
        "_Static_assert(sizeof(InstanceProperties) == 120, \"props\");\n"
        "_Static_assert(offsetof(InstanceProperties, interpNormals) == 44, \"interp\");\n"
        "_Static_assert(offsetof(InstanceProperties, sheen) == 116, \"sheen\");\n"
        "_Static_assert(sizeof(RtPushConsts) == 160, \"push\");\n"
        "_Static_assert(offsetof(RtPushConsts, maxBounces) == 156, \"maxb\");\n"
        "_Static_assert(sizeof(EmissiveInstanceData) == 112, \"emissive\");\n"
        "_Static_assert(offsetof(EmissiveInstanceData, cullBackface) == 100, \"cull\");\n"
        "_Static_assert(sizeof(reina_ray) == 32, \"ray\");\n"
        "_Static_assert(sizeof(reina_hit) == 16, \"hit\");\n"
        "int main(void) { return 0; }\n")
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", f"-I{ROOT / 'include'}", "-c", str(src), "-o",
                        str(tmp_path / "t.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_version_and_errors(R, host_ctx):
    assert "sm_103a" in R.version()
    s = R.Scene(host_ctx)
    with pytest.raises(R.ReinaError) as e:
        s.add_instance(3)
    assert e.value.code == R.REINA_ERR_INVALID and "out of range" in str(e.value)
    with pytest.raises(R.ReinaError) as e:
        s.define_object(np.zeros((3, 4), np.float32), np.array([0, 1, 7], np.uint32))
    assert e.value.code == R.REINA_ERR_INVALID
    with pytest.raises(R.ReinaError) as e:
        s.stats()
    assert e.value.code == R.REINA_ERR_STATE


def _quad(y=0.0, s=1.0, flip=False):
    v = np.array([[-s, y, -s, 1], [s, y, -s, 1], [s, y, s, 1], [-s, y, s, 1]], np.float32)
    i = np.array([0, 2, 1, 0, 3, 2] if not flip else [0, 1, 2, 0, 2, 3], np.uint32)
    return v, i


def test_no_emissive_scene_is_rejected_when_required(R, host_ctx):
    s = R.Scene(host_ctx)
    s.add_object(*_quad())
    with pytest.raises(R.ReinaError) as e:
        s.build(require_emissive=True)
    assert e.value.code == R.REINA_ERR_NO_EMISSIVE
    assert "at least one emissive" in str(e.value)
    s2 = R.Scene(host_ctx)
    s2.add_object(*_quad())
    s2.build(require_emissive=False)
    assert s2.emissive_weight == 0.0
    with pytest.raises(R.ReinaError) as e:
        s2.build()
    assert e.value.code == R.REINA_ERR_STATE
    with pytest.raises(R.ReinaError) as e:
        s2.add_object(*_quad())
    assert e.value.code == R.REINA_ERR_STATE


def test_emissive_weight_matches_instance_cdf_formula(R, host_ctx):
    """Scene::getEmissiveWeight = Σ over emissive instances of Σ tri_area * luminance(emission)
    (src/scene/Instance.cpp:15-53, Instances.cpp:178-190), with the area taken after vec4(v,1) * transform."""
    s = R.Scene(host_ctx)
    v, i = _quad(2.0, 0.5)
    e1 = (17.0, 12.0, 4.0)
    e2 = (1.0, 2.0, 3.0)
    T = np.eye(4, dtype=np.float32)
    T[0, 3] = 0.25      # translation (row 0, column 3); the transposed product ignores it
    T[0, 1] = 0.5       # M v shears x by y (area kept); v M tilts the quad (area grows by sqrt(1.25))
    s.add_object(v, i, material=R.Material(emission=e1))
    s.add_object(v, i, transform=T, material=R.Material(emission=e2))
    s.add_object(*_quad(), material=R.Material())
    s.build(require_emissive=True)

    def lum(e):
        return np.float32(0.2126 * e[0] + 0.7152 * e[1] + 0.0722 * e[2])

    def area(vv, M):
        p = (vv.astype(np.float32) @ M.astype(np.float32))[:, :3]   # row vector times matrix
        tri = p[i.reshape(-1, 3)]
        return 0.5 * np.linalg.norm(np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]), axis=1)

    w1 = float((area(v, np.eye(4)) * lum(e1)).sum())
    w2 = float((area(v, T) * lum(e2)).sum())
    assert s.emissive_weight == pytest.approx(w1 + w2, rel=1e-6)


def _decode_nodes(nodes: np.ndarray):
    p = nodes[:, 0:12].copy().view(np.float32)
    e = nodes[:, 12:15].astype(np.int32)
    imask = nodes[:, 15]
    base = nodes[:, 16:24].copy().view(np.uint32)
    meta = nodes[:, 24:32]
    q = nodes[:, 32:80].reshape(-1, 6, 8).astype(np.float64)
    return p, e, imask, base, meta, q


@pytest.mark.parametrize("level", [0, 2, 5])
def test_bvh8_structure_is_complete_and_conservative(R, host_ctx, level):
    v, i, _ = R.icosphere(level, 0.1, 1)
    s = R.Scene(host_ctx)
    s.add_object(v, i)
    s.build()
    st = s.stats()
    ntri = i.size // 3
    assert st["triangle_count"] == ntri
    nodes, tris = s.export_bvh()
    assert 1 <= st["max_depth"] <= 64
    tri_v = tris.copy().view(np.float32).reshape(-1, 12)
    prims = tris.copy().view(np.uint32).reshape(-1, 12)[:, 3]
    assert np.array_equal(np.sort(prims), np.arange(ntri, dtype=np.uint32))
    world = v[i.reshape(-1, 3)][:, :, :3].astype(np.float32)
    rec = np.stack([tri_v[:, 0:3], tri_v[:, 4:7], tri_v[:, 8:11]], axis=1)
    assert np.array_equal(rec, world[prims])

    p, e, imask, base, meta, q = _decode_nodes(nodes)
    seen_nodes = np.zeros(len(nodes), bool)
    seen_tris = np.zeros(ntri, bool)

    def subtree(n, depth):
        assert depth <= 64
        assert not seen_nodes[n]
        seen_nodes[n] = True
        scale = np.ldexp(1.0, e[n] - 127)
        lo_all = np.full(3, np.inf)
        hi_all = np.full(3, -np.inf)
        inner_rank = 0
        for slot in range(8):
            m = int(meta[n, slot])
            if m == 0:
                assert not (imask[n] >> slot) & 1
                continue
            qlo = q[n, 0:3, slot]
            qhi = q[n, 3:6, slot]
            blo = p[n].astype(np.float64) + qlo * scale
            bhi = p[n].astype(np.float64) + qhi * scale
            if (imask[n] >> slot) & 1:
                assert m == 0x20 | (24 + slot)
                child = int(base[n, 0]) + inner_rank
                inner_rank += 1
                clo, chi = subtree(child, depth + 1)
            else:
                cnt = {1: 1, 3: 2, 7: 3}[m >> 5]
                off = m & 31
                assert off + cnt <= 24
                t0 = int(base[n, 1]) + off
                pts = rec[t0:t0 + cnt].reshape(-1, 3).astype(np.float64)
                for k in range(cnt):
                    assert not seen_tris[prims[t0 + k]]
                    seen_tris[prims[t0 + k]] = True
                clo, chi = pts.min(axis=0), pts.max(axis=0)
            assert (blo < clo).all() and (bhi > chi).all(), "quantized box must strictly contain its content"
            # the traversal's plane offsets may round up to 2^-9 quanta inward: the builder keeps at
            # least 2^-8 quanta of margin around the content
            assert (clo - blo >= scale / 256).all() and (bhi - chi >= scale / 256).all()
            lo_all = np.minimum(lo_all, clo)
            hi_all = np.maximum(hi_all, chi)
        assert inner_rank == bin(int(imask[n])).count("1")
        return lo_all, hi_all

    subtree(0, 1)
    assert seen_nodes.all() and seen_tris.all()


def test_scene_outliving_its_context(R):
    """Destroying a context detaches its scenes: later calls on them fail with REINA_ERR_STATE and
    destroying them is safe."""
    ctx = R.Context(-1)
    s = R.Scene(ctx)
    v, i = _quad()
    s.add_object(v, i, material=R.Material(emission=(1.0, 1.0, 1.0)))
    s.build()
    ctx.close()
    iv, ip = R.camera_matrices((0, 0, 3), (0, 0, -1))
    pc = R.push_consts(iv, ip, spp=1)
    with pytest.raises(R.ReinaError) as e:
        R.render(ctx2 := R.Context(-1), s, pc, R.render_options(4, 4))
    assert e.value.code == R.REINA_ERR_STATE and "destroyed" in str(e.value)
    ctx2.close()
    s.close()


def test_batch_validation_on_host(R, host_ctx):
    """Batched-render arguments are checked before any GPU work: the plain-form flag is refused."""
    s = R.Scene(host_ctx)
    v, i = _quad()
    s.add_object(v, i, material=R.Material(emission=(1.0, 1.0, 1.0)))
    s.build()
    iv, ip = R.camera_matrices((0, 0, 3), (0, 0, -1))
    pc = R.push_consts(iv, ip, spp=1, total_emissive_weight=s.emissive_weight)
    for bad in (R.render_options(4, 4, megakernel=True), R.render_options(4, 4, pass_by_pass=True)):
        with pytest.raises(R.ReinaError) as e:
            R.render_batch(host_ctx, [R.RenderJob(s, pc, bad)])
        assert e.value.code == R.REINA_ERR_INVALID
    with pytest.raises(R.ReinaError) as e:   # the two plain forms exclude each other
        R.render(host_ctx, s, pc, R.render_options(4, 4, megakernel=True, pass_by_pass=True))
    assert e.value.code == R.REINA_ERR_INVALID
    with pytest.raises(R.ReinaError) as e:
        R.render_batch(host_ctx, [R.RenderJob(s, pc, R.render_options(4, 4))])
    assert e.value.code == R.REINA_ERR_STATE   # host-only context
    other = R.Context(-1)
    try:
        with pytest.raises(R.ReinaError) as e:
            R.render_batch(other, [R.RenderJob(s, pc, R.render_options(4, 4))])
        assert e.value.code == R.REINA_ERR_INVALID   # scene of another context
    finally:
        other.close()
    s.close()


@pytest.mark.parametrize("n", [1, 2, 5, 12])
def test_geodesic_sphere_is_closed_and_outward(R, n):
    """Frequency-n geodesic sphere: 10n^2+2 vertices, 20n^2 triangles, every edge shared by exactly two
    oppositely wound triangles (no cracks between icosahedron faces), all faces wound outward."""
    v, i, nrm = R.geodesic(n, 0.0, 1)
    assert v.shape == (10 * n * n + 2, 4) and i.size == 60 * n * n
    t = i.reshape(-1, 3)
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]]).tolist()
    fwd = set(map(tuple, e))
    assert len(fwd) == len(e) and fwd == {(b, a) for a, b in fwd}
    p = v[t][:, :, :3].astype(np.float64)
    cr = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    assert ((cr * p.mean(1)).sum(1) > 0).all()
    assert np.allclose(np.linalg.norm(v[:, :3], axis=1), 1.0, atol=1e-6)
    assert np.unique(i).size == v.shape[0]
    vd, _, _ = R.geodesic(n, 0.1, 3)
    r = np.linalg.norm(vd[:, :3], axis=1)
    assert (np.abs(r - 1.0) <= 0.1 + 1e-6).all()


def test_server_needs_a_gpu_context(R, host_ctx):
    with pytest.raises(R.ReinaError) as e:
        R.Server(host_ctx)
    assert e.value.code == R.REINA_ERR_STATE


@pytest.mark.parametrize("kw", [dict(fifo=True, shortest=True), dict(fifo=True, fair=True),
                                dict(shortest=True, fair=True), dict(aging=float("nan")), dict(wave_lanes=17)])
def test_server_policy_flags_exclude_each_other(R, host_ctx, kw):
    with pytest.raises(R.ReinaError) as e:
        R.Server(host_ctx, **kw)
    assert e.value.code == R.REINA_ERR_INVALID



def test_emissive_export_and_device_build_on_host(R, host_ctx):
    """The packed emissive data of a host build: each instance's triangle CDF ends at 1, the instance CDF
    ends at 1, weights sum to the scene's emissive weight; the device build needs a GPU context."""
    def make():
        s = R.Scene(host_ctx)
        v, i, _ = R.icosphere(2, 0.1, 4)
        o = s.define_object(v, i)
        for k, e in enumerate([(1.0, 1.0, 1.0), (2.0, 0.0, 0.5), (1.0, 1.0, 1.0)]):
            t = np.eye(4, dtype=np.float32)
            t[0, 3] = 0.5 * k
            s.add_instance(o, t, R.Material(emission=e))
        return s
    s = make()
    with pytest.raises(R.ReinaError) as e:
        s.set_emissive_build(2)
    assert e.value.code == R.REINA_ERR_INVALID
    s.build()
    inst, tris, cdf_i = s.export_emissive()
    assert inst.size == 3 and cdf_i.size == 3 and cdf_i[-1] == 1.0
    for r in inst:
        assert tris[r["cdfRangeEnd"]] == 1.0 and r["cdfRangeEnd"] - r["cdfRangeStart"] + 1 == 320
    assert abs(float(inst["weight"].sum()) - s.emissive_weight) <= 1e-5 * s.emissive_weight
    # instances 0 and 2 have the same CDF (a translation does not change areas): one shared range
    assert (inst[0]["cdfRangeStart"], inst[0]["cdfRangeEnd"]) == (inst[2]["cdfRangeStart"], inst[2]["cdfRangeEnd"])
    d = make()
    d.set_emissive_build(R.EMISSIVE_DEVICE)
    with pytest.raises(R.ReinaError) as e:
        d.build()
    assert e.value.code == R.REINA_ERR_STATE


@pytest.mark.parametrize("pos,front,up,fovy,aspect", [((0, 0, 3.4), (0, 0, -1), (0, 1, 0), 40.0, 1.0),
                                                      ((0.0, 0.4, 3.6), (0.0, -0.12, -1.0), (0, 1, 0), 40.0, 16 / 9),
                                                      ((2, -1, 0.5), (-1, 0.3, 0.2), (0, 1, 0), 25.0, 0.8)])
def test_camera_matrices_invert_lookat_and_perspective(R, pos, front, up, fovy, aspect):
    """Camera::getInvViewMatrix / getInvProjMatrix (src/graphics/Camera.cpp:10-11): the inverses of
    lookAt(pos, pos + front, up) and perspective(fovy, aspect, 0.1, 100) (right-handed, clip depth -1..1),
    restated here in float64 and checked by multiplying out."""
    iv, ip = R.camera_matrices(pos, front, up, np.radians(fovy), aspect)
    IV = np.asarray(iv, np.float64).reshape(4, 4).T   # column-major storage
    IP = np.asarray(ip, np.float64).reshape(4, 4).T
    p, f, u = np.asarray(pos, float), np.asarray(front, float), np.asarray(up, float)
    f = f / np.linalg.norm(f)
    s = np.cross(f, u)
    s /= np.linalg.norm(s)
    uu = np.cross(s, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = s, uu, -f
    view[:3, 3] = [-s @ p, -uu @ p, f @ p]
    t = np.tan(np.radians(fovy) / 2)
    n, fa = 0.1, 100.0
    proj = np.zeros((4, 4))
    proj[0, 0], proj[1, 1] = 1 / (aspect * t), 1 / t
    proj[2, 2], proj[2, 3], proj[3, 2] = -(fa + n) / (fa - n), -2 * fa * n / (fa - n), -1.0
    assert np.allclose(IV @ view, np.eye(4), atol=1e-5)
    assert np.allclose(IP @ proj, np.eye(4), atol=1e-5)
