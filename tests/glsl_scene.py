"""Loads a test scene (scenes.SceneDesc) into the reference's own shaders run on the host
(oracle/glsl/ref_glsl.py): the storage buffers packed as the reference packs them, and the traversal
triangles of the product's built scene.

Buffers (bindings of shaderCommon.h.glsl and closestHitCommon.h.glsl), packed like
Models::addModel (src/scene/Models.cpp:24-92) and Scene::addInstance (src/scene/Scene.cpp:27-54):
  2 vertices (vec4), 3 indices offset by the model's first vertex, 5 TBNs (mat3, column-major),
  6 TBN indices offset by the model's first TBN, 10 texture coordinates (vec2), 11 texture-coordinate
  indices offset by the model's first coordinate (0xFFFFFFFF kept), 4 InstanceProperties, one per
  instance in order (gl_InstanceCustomIndexEXT = the instance's index, src/tools/vktools.cpp:480-481);
  the SBT record offset of an instance is its material index (vktools.cpp:483).
The emissive-sampling buffers (7, 8, 9) are read only by directLight, which the reference never calls
(skipNEE = true, raytrace.rgen.glsl:146), so they stay empty.
"""
from __future__ import annotations

import numpy as np


def pack_models(desc):
    """The reference's global model buffers and each model's ModelRange offsets."""
    verts, idx, tbns, tbn_idx, uvs, uv_idx = [], [], [], [], [], []
    ranges = []
    nv = nt = nu = ni = nti = nui = 0
    for v4, i, t9, ti, uv, ui in desc.objects:
        i = np.asarray(i, np.uint32).reshape(-1)
        has_uv = uv is not None and len(uv) > 0
        ranges.append({"indexOffset": ni, "tbnsIndexOffset": nti, "texIndexOffset": nui if has_uv else 0xFFFFFFFF})
        verts.append(np.asarray(v4, np.float32).reshape(-1, 4))
        idx.append(i + np.uint32(nv))
        ni += i.size
        if t9 is not None:
            t9 = np.asarray(t9, np.float32).reshape(-1, 9)
            tbns.append(t9)
            tidx = np.asarray(ti, np.uint32).reshape(-1)
            tbn_idx.append(tidx + np.uint32(nt))
            nti += tidx.size
            nt += t9.shape[0]
        if has_uv:
            uv = np.asarray(uv, np.float32).reshape(-1, 2)
            uvs.append(uv)
            u = np.asarray(ui, np.uint32).reshape(-1)
            uv_idx.append(np.where(u == 0xFFFFFFFF, u, u + np.uint32(nu)).astype(np.uint32))
            nui += u.size
            nu += uv.shape[0]
        nv += verts[-1].shape[0]

    def cat(parts, shape, dtype):
        return np.concatenate(parts).astype(dtype) if parts else np.zeros(shape, dtype)

    return {
        2: cat(verts, (0, 4), np.float32), 3: cat(idx, (0,), np.uint32), 5: cat(tbns, (0, 9), np.float32),
        6: cat(tbn_idx, (0,), np.uint32), 10: cat(uvs, (0, 2), np.float32), 11: cat(uv_idx, (0,), np.uint32),
    }, ranges


def instance_properties(R, desc, ranges):
    """One InstanceProperties record per instance (Scene::addInstance's field order)."""
    props = np.zeros(len(desc.instances), R.INSTANCE_PROPERTIES_DTYPE)
    for k, (obj, _, mats, fm) in enumerate(desc.instances):
        if fm is not None or len(mats) != 1:
            raise ValueError("per-face materials have no counterpart in the reference")
        m, rg = mats[0], ranges[obj]
        p = props[k]
        p["indicesOffset"], p["tbnsIndicesOffset"], p["texIndicesOffset"] = rg["indexOffset"], rg["tbnsIndexOffset"], rg["texIndexOffset"]
        p["albedo"], p["emission"] = m.albedo, m.emission
        p["roughness"], p["ior"], p["interpNormals"], p["absorption"] = m.roughness, m.ior, int(m.interp_normals), m.absorption
        p["textureID"], p["normalMapTexID"], p["bumpMapTexID"] = m.texture_id, m.normal_map_id, m.bump_map_id
        p["cullBackface"] = int(m.cull_backface)
        p["anisotropic"], p["subsurface"], p["clearcoatGloss"] = m.anisotropic, m.subsurface, m.clearcoat_gloss
        p["sheenTint"], p["specularTint"] = m.sheen_tint, m.specular_tint
        p["metallic"], p["clearcoat"], p["specularTransmission"], p["sheen"] = m.metallic, m.clearcoat, m.specular_transmission, m.sheen
    return props


def load(G, R, desc, product_scene):
    """Hands the scene to the reference shaders' host runtime; returns the InstanceProperties packed here."""
    bufs, ranges = pack_models(desc)
    props = instance_properties(R, desc, ranges)
    for b, a in bufs.items():
        G.set_buffer(b, a)
    G.set_buffer(4, props)
    for b in (7, 8, 9):
        G.set_buffer(b, np.zeros(0, np.uint8))
    if product_scene.stats().get("two_level"):
        raise ValueError("build the product scene flat (ACCEL_FLAT): its traversal triangles are the world-space ones")
    nodes, trec = product_scene.export_bvh()
    rec = trec.view(np.float32).reshape(-1, 12)
    tris9 = np.ascontiguousarray(rec[:, [0, 1, 2, 4, 5, 6, 8, 9, 10]])
    ids = rec[:, 3].copy().view(np.uint32)
    info = np.array([product_scene.prim_info(int(p)) for p in ids], np.uint32).reshape(-1, 2)
    o2w = np.stack([np.asarray(T, np.float32)[:3, :].T.reshape(12) for _, T, _, _ in desc.instances])
    sbt = np.array([mats[0].material_idx for _, _, mats, _ in desc.instances], np.uint32)
    G.set_scene(tris9, info[:, 0], info[:, 1], ids, o2w, np.arange(len(desc.instances), dtype=np.uint32), sbt)
    G.set_textures(list(desc.textures))
    return props


def push_bytes(pc) -> np.ndarray:
    """RtPushConsts (a ctypes structure) as its 160 bytes."""
    import ctypes

    return np.frombuffer(ctypes.string_at(ctypes.addressof(pc), ctypes.sizeof(pc)), np.uint8).copy()
