"""CPU tests of the boundary's file formats: Wavefront OBJ models, glTF 2.0 scenes (.gltf with a base64
buffer and .glb), the run configuration (config.toml), the SaveManager schedule and the PNG writer.
All inputs are written by the tests themselves."""
import base64
import json
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest
from conftest import reference_dir

CUBE_OBJ = """# unit cube, quads, normals per face, uvs
v -0.5 -0.5 -0.5
v 0.5 -0.5 -0.5
v 0.5 0.5 -0.5
v -0.5 0.5 -0.5
v -0.5 -0.5 0.5
v 0.5 -0.5 0.5
v 0.5 0.5 0.5
v -0.5 0.5 0.5
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 -1
vn 0 0 1
vn -1 0 0
vn 1 0 0
vn 0 -1 0
vn 0 1 0
f 1/1/1 4/4/1 3/3/1 2/2/1
f 5/1/2 6/2/2 7/3/2 8/4/2
f 1/1/3 5/2/3 8/3/3 4/4/3
f 2/1/4 3/4/4 7/3/4 6/2/4
f 1/1/5 2/2/5 6/3/5 5/4/5
f 4/1/6 8/4/6 7/3/6 3/2/6
"""


def test_obj_quads_uvs_normals(R, host_ctx, tmp_path):
    p = tmp_path / "cube.obj"
    p.write_text(CUBE_OBJ)
    s = R.Scene(host_ctx)
    oid = s.define_object_obj(p)
    m = s.export_object(oid)
    assert m["indices"].size == 36                 # 6 quads -> 12 triangles
    assert m["vertices"].shape == (24, 4)          # one vertex per distinct (v, vt, vn)
    assert np.all(m["vertices"][:, 3] == 1.0)
    assert m["tex_coords"].shape == (24, 2)
    # UVs flipped: every corner's v is 1 - the file's v
    assert set(np.round(m["tex_coords"][:, 1], 6)) <= {0.0, 1.0}
    t = m["tbns"].reshape(-1, 3, 3)                # columns T, B, N
    T, B, N = t[:, 0], t[:, 1], t[:, 2]
    assert np.allclose(np.linalg.norm(N, axis=1), 1.0) and np.allclose(np.linalg.norm(T, axis=1), 1.0, atol=1e-5)
    assert np.allclose((T * N).sum(1), 0.0, atol=1e-5) and np.allclose((B * N).sum(1), 0.0, atol=1e-5)
    # face normals are the file's (axis aligned); triangle winding agrees with them
    v = m["vertices"][:, :3][m["indices"].reshape(-1, 3)]
    fn = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    n0 = N[m["indices"].reshape(-1, 3)[:, 0]]
    assert ((fn * n0).sum(1) > 0).all()


def test_obj_without_normals_gets_smooth_normals(R, host_ctx, tmp_path):
    v, i, _ = R.icosphere(2, 0.0, 1)
    lines = [f"v {x} {y} {z}" for x, y, z in v[:, :3]]
    lines += [f"f {a + 1} {b + 1} {c + 1}" for a, b, c in i.reshape(-1, 3)]
    # negative (relative) indices for the last face
    n = v.shape[0]
    a, b, c = (int(x) for x in i.reshape(-1, 3)[-1])
    lines[-1] = f"f {a - n} {b - n} {c - n}"
    p = tmp_path / "sphere.obj"
    p.write_text("\n".join(lines) + "\n")
    s = R.Scene(host_ctx)
    m = s.export_object(s.define_object_obj(p))
    assert np.array_equal(m["indices"].reshape(-1, 3).shape, i.reshape(-1, 3).shape)
    assert m["vertices"].shape[0] == n and m["tex_coords"].shape[0] == 0
    N = m["tbns"].reshape(-1, 3, 3)[:, 2]
    # smooth normals of a unit icosphere point (nearly) radially
    assert (np.sum(N * m["vertices"][:, :3], axis=1) > 0.99).all()
    T = m["tbns"].reshape(-1, 3, 3)[:, 0]
    assert np.all(T == 0.0)   # no UVs: zero tangent frame, as the reference leaves it


@pytest.mark.parametrize("text,msg", [("v 0 0 0\nv 1 0 0\nf 1 2 3\n", "out of range"),
                                      ("v 0 0 0\nf 1 1\n", "fewer than 3"),
                                      ("v 0 0\n", "malformed vertex"),
                                      ("# nothing\n", "no faces")])
def test_obj_errors(R, host_ctx, tmp_path, text, msg):
    p = tmp_path / "bad.obj"
    p.write_text(text)
    s = R.Scene(host_ctx)
    with pytest.raises(R.ReinaError) as e:
        s.define_object_obj(p)
    assert e.value.code == R.REINA_ERR_IO and msg in str(e.value)
    with pytest.raises(R.ReinaError) as e:
        s.define_object_obj(tmp_path / "missing.obj")
    assert e.value.code == R.REINA_ERR_IO


def make_gltf(glb: bool, normals=True, scenes_list=True):
    """Two nodes: a parent with TRS (translate x+2, rotate 90 deg about y, scale 2) holding mesh 0 and a
    child with a matrix (translate y+1) holding mesh 0 again; mesh 0 has two primitives (triangle with
    TANGENT vec4 and material 0; quad with indices and material 1)."""
    pos0 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    nrm0 = np.array([[0, 0, 1]] * 3, np.float32)
    tan0 = np.array([[1, 0, 0, -1]] * 3, np.float32)
    pos1 = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    nrm1 = np.array([[0, 0, 1]] * 4, np.float32)
    uv1 = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    idx1 = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    blobs = [pos0, nrm0, tan0, pos1, nrm1, uv1, idx1]
    data = b""
    views = []
    for bl in blobs:
        while len(data) % 4:
            data += b"\0"
        views.append({"buffer": 0, "byteOffset": len(data), "byteLength": bl.nbytes})
        data += bl.tobytes()
    acc = [{"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"},
           {"bufferView": 1, "componentType": 5126, "count": 3, "type": "VEC3"},
           {"bufferView": 2, "componentType": 5126, "count": 3, "type": "VEC4"},
           {"bufferView": 3, "componentType": 5126, "count": 4, "type": "VEC3"},
           {"bufferView": 4, "componentType": 5126, "count": 4, "type": "VEC3"},
           {"bufferView": 5, "componentType": 5126, "count": 4, "type": "VEC2"},
           {"bufferView": 6, "componentType": 5123, "count": 6, "type": "SCALAR"}]
    attr0 = {"POSITION": 0, "TANGENT": 2}
    if normals:
        attr0["NORMAL"] = 1
    s = 2 ** -0.5
    doc = {
        "asset": {"version": "2.0"},
        "scene": 0,
        "scenes": [{"nodes": [0]}] if scenes_list else [],
        "nodes": [{"mesh": 0, "translation": [2, 0, 0], "rotation": [0, s, 0, s], "scale": [2, 2, 2], "children": [1]},
                  {"mesh": 0, "matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 1, 0, 1]}],
        "meshes": [{"primitives": [{"attributes": attr0, "material": 0},
                                   {"attributes": {"POSITION": 3, "NORMAL": 4, "TEXCOORD_0": 5}, "indices": 6,
                                    "material": 1}]}],
        "materials": [{"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.4, 0.6, 1], "metallicFactor": 0.3,
                                                "roughnessFactor": 0.05},
                       "emissiveFactor": [1, 0.5, 0],
                       "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 4}}},
                      {"doubleSided": True, "extensions": {"KHR_materials_transmission": {"transmissionFactor": 0.8},
                                                           "KHR_materials_ior": {"ior": 1.33}}}],
        "accessors": acc,
        "bufferViews": views,
        "buffers": [{"byteLength": len(data)}],
    }
    if not glb:
        doc["buffers"][0]["uri"] = "data:application/octet-stream;base64," + base64.b64encode(data).decode()
        return json.dumps(doc).encode()
    js = json.dumps(doc).encode()
    while len(js) % 4:
        js += b" "
    while len(data) % 4:
        data += b"\0"
    body = struct.pack("<I", len(js)) + b"JSON" + js + struct.pack("<I", len(data)) + b"BIN\0" + data
    return b"glTF" + struct.pack("<II", 2, 12 + len(body)) + body


@pytest.mark.parametrize("glb", [False, True])
def test_gltf_scene(R, host_ctx, tmp_path, glb):
    p = tmp_path / ("s.glb" if glb else "s.gltf")
    p.write_bytes(make_gltf(glb))
    s = R.Scene(host_ctx)
    s.set_accel(R.ACCEL_FLAT)   # the checks below read world-space triangle records
    st = s.add_gltf(p)
    assert st == {"meshes": 1, "primitives": 2, "instances": 4, "skipped_primitives": 0, "ignored_textures": 0}
    assert s.object_count() == 2
    tri = s.export_object(0)
    tb = tri["tbns"].reshape(-1, 3, 3)
    assert np.allclose(tb[:, 0], [1, 0, 0]) and np.allclose(tb[:, 2], [0, 0, 1])
    assert np.allclose(tb[:, 1], [0, -1, 0])           # B = cross(N, T) * w with w = -1
    quad = s.export_object(1)
    assert np.array_equal(quad["indices"], [0, 1, 2, 0, 2, 3]) and quad["tex_coords"].shape == (4, 2)
    s.build()
    st2 = s.stats()
    assert st2["triangle_count"] == 2 * (1 + 2) and st2["instance_count"] == 4
    nodes, tris = s.export_bvh()
    t = tris.copy().view(np.float32).reshape(-1, 12)
    prims = tris.copy().view(np.uint32).reshape(-1, 12)[:, 3]
    world = np.stack([t[:, 0:3], t[:, 4:7], t[:, 8:11]], 1)[np.argsort(prims)]
    # instance 0: parent (T * R_y(90) * S(2)) applied to the triangle (0,0,0),(1,0,0),(0,1,0)
    assert np.allclose(world[0], [[2, 0, 0], [2, 0, -2], [2, 2, 0]], atol=1e-5)
    # instance 2: child = parent * translate(0,1,0): origin maps to parent(0,1,0) = (2, 2, 0)
    assert np.allclose(world[3][0], [2, 2, 0], atol=1e-5)
    assert s.emissive_weight > 0    # material 0 is emissive (factor x strength)


def test_gltf_errors(R, host_ctx, tmp_path):
    p = tmp_path / "n.gltf"
    p.write_bytes(make_gltf(False, normals=False))
    with pytest.raises(R.ReinaError) as e:
        R.Scene(host_ctx).add_gltf(p)
    assert e.value.code == R.REINA_ERR_IO and "normals" in str(e.value)
    p.write_bytes(make_gltf(False, scenes_list=False))
    with pytest.raises(R.ReinaError) as e:
        R.Scene(host_ctx).add_gltf(p)
    assert "No scenes" in str(e.value)
    p.write_bytes(b"{ not json")
    with pytest.raises(R.ReinaError) as e:
        R.Scene(host_ctx).add_gltf(p)
    assert e.value.code == R.REINA_ERR_IO


CONFIG = """# run settings
[camera]
[camera.dof]
focus_dist = 3.5
defocus_multiplier = 2  # percent

[sampling]
samples_per_pixel = 4
max_bounces = 9
direct_clamp = 50
indirect_clamp = 5.5

[saving]
save_on_samples = [300, 100, 200]
save_on_times = [30.5, 10]

[postprocessing]
[postprocessing.bloom]
radius = 4.0
threshold = 0.9
intensity = 0.02

[postprocessing.tonemap]
exposure = -1
"""


def test_config_and_schedule(R, tmp_path):
    p = tmp_path / "config.toml"
    p.write_text(CONFIG)
    c = R.load_config(p)
    assert c.focus_dist == pytest.approx(3.5) and c.defocus_multiplier == pytest.approx(0.02)
    assert (c.samples_per_pixel, c.max_bounces) == (4, 9)
    assert c.direct_clamp == 50 and c.indirect_clamp == pytest.approx(5.5)
    assert (c.bloom.radius, c.bloom.threshold, c.bloom.intensity) == pytest.approx((4.0, 0.9, 0.02))
    assert c.tonemap.exposure == -1
    assert list(c.save_on_samples[:c.save_on_samples_count]) == [300, 100, 200]
    sch = R.SaveSchedule(c)
    assert sch.next(100, 0.0) == ""                       # a point is passed only when exceeded
    assert sch.next(101, 0.0) == "output_100spp.png"
    assert sch.next(1000, 100.0) == "output_200spp.png"   # one save per call, samples first
    assert sch.next(1000, 100.0) == "output_300spp.png"
    assert sch.next(1000, 100.0) == "output_10sec.png"
    assert sch.next(1000, 100.0) == "output_30sec.png"
    assert sch.next(10 ** 9, 1e9) == ""


def test_config_optional_keys(R, tmp_path):
    """Absent: the reference's hard-coded values (src/Reina.cpp:54-55,91,138-140); present: read."""
    p = tmp_path / "config.toml"
    p.write_text(CONFIG)
    c = R.load_config(p)
    assert (c.width, c.height, c.seed, c.mode) == (1080, 1350, 1, R.MODE_REINA)
    assert c.scene_path == b"" and c.fov_degrees == 25.0
    assert list(c.camera_pos) == pytest.approx([-1.6899, 0.317017, 1.6386]) and list(c.look_at) == pytest.approx([0, 0.962, 0])
    p.write_text(CONFIG + '\n[render]\nwidth = 320\nheight = 200\nseed = 9\nmode = "nee"\n[scene]\npath = "scenes/a b.glb"\n'
                 '[camera]\npos = [1, 2.5, -3]\nlook_at = [0, 0, 0]\nfov = 40.5\n')
    c = R.load_config(p)
    assert (c.width, c.height, c.seed, c.mode) == (320, 200, 9, R.MODE_NEE_MIS)
    assert c.scene_path == b"scenes/a b.glb" and c.fov_degrees == pytest.approx(40.5)
    assert list(c.camera_pos) == [1.0, 2.5, -3.0] and list(c.look_at) == [0.0, 0.0, 0.0]
    for bad in ('[render]\nmode = "fast"\n', '[camera]\npos = [1, 2]\n', '[render]\nwidth = 0\n'):
        p.write_text(CONFIG + "\n" + bad)
        with pytest.raises(R.ReinaError) as e:
            R.load_config(p)
        assert e.value.code == R.REINA_ERR_IO


@pytest.mark.parametrize("drop", ["max_bounces", "exposure", "save_on_times"])
def test_config_missing_key(R, tmp_path, drop):
    p = tmp_path / "config.toml"
    p.write_text("\n".join(l for l in CONFIG.splitlines() if not l.startswith(drop)))
    with pytest.raises(R.ReinaError) as e:
        R.load_config(p)
    assert e.value.code == R.REINA_ERR_IO and drop in str(e.value)


def read_png(data: bytes):
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    off, chunks = 8, {}
    while off < len(data):
        n = struct.unpack(">I", data[off:off + 4])[0]
        typ = data[off + 4:off + 8]
        body = data[off + 8:off + 8 + n]
        crc = struct.unpack(">I", data[off + 8 + n:off + 12 + n])[0]
        assert crc == zlib.crc32(typ + body)
        chunks.setdefault(typ, b"")
        chunks[typ] += body
        off += 12 + n
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    raw = zlib.decompress(chunks[b"IDAT"])
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 4 * w)
    assert (rows[:, 0] == 0).all() and depth == 8 and ctype == 6
    return rows[:, 1:].reshape(h, w, 4)


@pytest.mark.parametrize("w,h", [(1, 1), (37, 5), (300, 300)])
def test_png_round_trip(R, tmp_path, w, h):
    img = (np.arange(w * h * 4) * 7919 % 256).astype(np.uint8).reshape(h, w, 4)
    p = tmp_path / "o.png"
    R.write_png(p, img)
    assert np.array_equal(read_png(p.read_bytes()), img)


def png_bytes(rgba: np.ndarray) -> bytes:
    """A minimal RGBA8 PNG (filter 0 rows, zlib) written by the test."""
    h, w = rgba.shape[:2]

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    raw = b"".join(b"\0" + rgba[y].astype(np.uint8).tobytes() for y in range(h))
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))


def test_gltf_textures(R, host_ctx, tmp_path):
    """Images from a data URI, a buffer view and a percent-encoded relative file become scene textures in
    image order (not flipped); a JPEG image is left out and its material reference counted as ignored."""
    rng = np.random.default_rng(5)
    imgs = [rng.integers(0, 256, (3 + k, 4 + k, 4)).astype(np.uint8) for k in range(3)]
    pngs = [png_bytes(a) for a in imgs]
    (tmp_path / "tex dir").mkdir()
    (tmp_path / "tex dir" / "c.png").write_bytes(pngs[2])
    pos = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    nrm = np.array([[0, 0, 1]] * 4, np.float32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    data = b""
    views = []
    for bl in [pos.tobytes(), nrm.tobytes(), uv.tobytes(), idx.tobytes(), pngs[1]]:
        while len(data) % 4:
            data += b"\0"
        views.append({"buffer": 0, "byteOffset": len(data), "byteLength": len(bl)})
        data += bl
    prim = {"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2}, "indices": 3}
    doc = {
        "asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0]}], "nodes": [{"mesh": 0}],
        "meshes": [{"primitives": [dict(prim, material=0), dict(prim, material=1), dict(prim, material=2)]}],
        "materials": [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}}, "normalTexture": {"index": 1}},
                      {"pbrMetallicRoughness": {"baseColorTexture": {"index": 2}}, "normalTexture": {"index": 3}},
                      {}],
        "textures": [{"source": 0}, {"source": 1}, {"source": 2}, {"source": 3}],
        "images": [{"uri": "data:image/png;base64," + base64.b64encode(pngs[0]).decode()},
                   {"bufferView": 4, "mimeType": "image/png"},
                   {"uri": "tex%20dir/c.png"},
                   {"uri": "data:image/jpeg;base64," + base64.b64encode(b"\xff\xd8\xff\xe0 jpeg").decode()}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": 4, "type": "VEC3"},
                      {"bufferView": 1, "componentType": 5126, "count": 4, "type": "VEC3"},
                      {"bufferView": 2, "componentType": 5126, "count": 4, "type": "VEC2"},
                      {"bufferView": 3, "componentType": 5123, "count": 6, "type": "SCALAR"}],
        "bufferViews": views,
        "buffers": [{"byteLength": len(data), "uri": "data:application/octet-stream;base64," +
                     base64.b64encode(data).decode()}],
    }
    p = tmp_path / "t.gltf"
    p.write_text(json.dumps(doc))
    s = R.Scene(host_ctx)
    st = s.add_gltf(p)
    assert st["ignored_textures"] == 1 and st["instances"] == 3
    assert s.texture_count() == 3
    props = s.instance_properties()
    assert list(props["textureID"]) == [0, 2, -1]
    assert list(props["normalMapTexID"]) == [1, -1, -1]
    assert list(props["bumpMapTexID"]) == [-1, -1, -1]
    s.build()
    for k in range(3):   # texels as written: no vertical flip for glTF images
        assert np.array_equal(s.export_texture(k), imgs[k])


REF_MODELS = reference_dir("models")


@pytest.mark.skipif(REF_MODELS is None, reason="REINA_REFERENCE_DIR unset or without models/")
def test_reference_obj_models(R, host_ctx):
    """Every OBJ the reference ships loads as one model: polygons fanned into triangles, one TBN and UV per
    vertex when the file has UVs (Assimp's JoinIdenticalVertices / CalcTangentSpace / FlipUVs flags,
    src/scene/Models.cpp:120), unit-length normals."""
    for f in sorted(REF_MODELS.glob("*.obj")):
        text = f.read_text()
        faces = [l.split()[1:] for l in text.splitlines() if l.startswith("f ")]
        want_tris = sum(len(fc) - 2 for fc in faces)
        s = R.Scene(host_ctx)
        oid = s.define_object_obj(f)
        m = s.export_object(oid)
        assert m["indices"].size == 3 * want_tris, f.name
        n = m["tbns"].reshape(-1, 3, 3)[:, 2]
        assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-4), f.name
        has_vt = any(l.startswith("vt ") for l in text.splitlines())
        assert (m["tex_coords"].shape[0] > 0) == has_vt, f.name
