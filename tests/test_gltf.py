"""glTF 2.0 ingestion (f184gi_gltf_load), standing in for Foreground/SceneGraph/glTFSceneImporter.cpp.

Files are written here with numpy: a .gltf with a .bin beside it, the same with a data URI, and a .glb; node
trees with matrix and T*R*S transforms, triangle lists/strips/fans, u8/u16/u32 and missing indices, materials.
The node transform and the sun direction are checked against the reference's own Math library.
"""
import base64
import json
import struct

import numpy as np
import pytest

QUAT = [0.18257419, 0.36514837, 0.54772256, 0.73029674]  # x, y, z, w (unit)


def _scene_doc(bin_uri):
    """Buffer: positions of a quad (4 x vec3 f32) + u16 indices [0,1,2, 0,2,3] + a strip of 4 + u8 fan indices."""
    pos = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    idx16 = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    idx8 = np.array([0, 1, 2, 3], np.uint8)
    blob = pos.tobytes() + idx16.tobytes() + idx8.tobytes()
    blob += b"\0" * ((-len(blob)) % 4)
    doc = {
        "asset": {"version": "2.0"},
        "scene": 0,
        "scenes": [{"nodes": [0, 3]}],
        "nodes": [
            {"translation": [10, 0, 0], "children": [1, 2]},
            {"mesh": 0, "rotation": QUAT, "scale": [2, 3, 4]},
            {"mesh": 1, "matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 5, 0, 1]},
            {"mesh": 2},
        ],
        "meshes": [
            {"primitives": [{"attributes": {"POSITION": 0}, "indices": 1, "material": 0}]},
            {"primitives": [{"attributes": {"POSITION": 0}, "mode": 5, "material": 1}]},
            {"primitives": [{"attributes": {"POSITION": 0}, "indices": 2, "mode": 6},
                            {"attributes": {"POSITION": 0}, "mode": 1}]},
        ],
        "materials": [{"pbrMetallicRoughness": {"baseColorFactor": [1.0, 0.5, 0.0, 1.0], "roughnessFactor": 0.25}},
                      {"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.4, 0.6, 1.0]}}],
        "buffers": [{"byteLength": len(blob)}],
        "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 48},
                        {"buffer": 0, "byteOffset": 48, "byteLength": 12},
                        {"buffer": 0, "byteOffset": 60, "byteLength": 4}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": 4, "type": "VEC3"},
                      {"bufferView": 1, "componentType": 5123, "count": 6, "type": "SCALAR"},
                      {"bufferView": 2, "componentType": 5121, "count": 4, "type": "SCALAR"}],
    }
    if bin_uri is not None:
        doc["buffers"][0]["uri"] = bin_uri
    return doc, blob, pos


def _quat_matrix(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _expected(pos):
    """World triangles, albedo, roughness in the loader's order (depth-first node walk)."""
    tris, alb, rough = [], [], []
    M1 = _quat_matrix(QUAT) * np.array([2.0, 3.0, 4.0])
    w1 = pos.astype(np.float64) @ M1.T + np.array([10.0, 0, 0])
    for t in ([0, 1, 2], [0, 2, 3]):
        tris.append(w1[t]), alb.append(0xFF0080FF), rough.append(0.25)
    w2 = pos.astype(np.float64) + np.array([10.0, 5.0, 0])
    for t in ([0, 1, 2], [2, 1, 3]):  # strip: the second triangle reversed
        tris.append(w2[t]), alb.append(int(round(0.2 * 255)) | int(round(0.4 * 255)) << 8 | int(round(0.6 * 255)) << 16
                                       | 255 << 24), rough.append(1.0)
    w3 = pos.astype(np.float64)
    for t in ([0, 1, 2], [0, 2, 3]):  # fan
        tris.append(w3[t]), alb.append(0xFFFFFFFF), rough.append(1.0)
    return np.array(tris, np.float32).reshape(-1, 9), np.array(alb, np.uint32), np.array(rough, np.float32)


def _check(sc, pos):
    tri, alb, rough = _expected(pos)
    assert sc.ntris == 6 and sc.nobjects == 3
    assert np.allclose(sc.tri_xyz.reshape(-1, 9), tri, atol=1e-5)
    assert np.array_equal(sc.albedo, alb)
    assert np.allclose(sc.roughness, rough)
    assert list(sc.object_count) == [2, 2, 2]


def test_gltf_with_bin_file(lib, tmp_path):
    import final184_gb300 as g

    doc, blob, pos = _scene_doc("scene.bin")
    (tmp_path / "scene.bin").write_bytes(blob)
    (tmp_path / "scene.gltf").write_text(json.dumps(doc))
    _check(g.SyntheticScene.from_gltf(tmp_path / "scene.gltf"), pos)


def test_gltf_with_data_uri_and_glb(lib, tmp_path):
    import final184_gb300 as g

    _, blob, _ = _scene_doc(None)
    doc, blob, pos = _scene_doc("data:application/octet-stream;base64," + base64.b64encode(blob).decode())
    (tmp_path / "inline.gltf").write_text(json.dumps(doc))
    _check(g.SyntheticScene.from_gltf(tmp_path / "inline.gltf"), pos)
    doc, blob, pos = _scene_doc(None)
    js = json.dumps(doc).encode()
    js += b" " * ((-len(js)) % 4)
    glb = struct.pack("<III", 0x46546C67, 2, 12 + 8 + len(js) + 8 + len(blob))
    glb += struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(blob), 0x004E4942) + blob
    (tmp_path / "scene.glb").write_bytes(glb)
    _check(g.SyntheticScene.from_gltf(tmp_path / "scene.glb"), pos)


def test_gltf_errors(lib, tmp_path):
    import final184_gb300 as g

    with pytest.raises(g.F184Error) as e:
        g.SyntheticScene.from_gltf(tmp_path / "missing.gltf")
    assert e.value.code == g._abi.ERR_NOTFOUND
    (tmp_path / "bad.gltf").write_text('{"asset": {"version": "2.0"}, "nodes": [')
    with pytest.raises(g.F184Error) as e:
        g.SyntheticScene.from_gltf(tmp_path / "bad.gltf")
    assert e.value.code == g._abi.ERR_INVALID and "JSON" in str(e.value)
    doc, blob, _ = _scene_doc("scene.bin")
    (tmp_path / "scene.bin").write_bytes(blob)
    doc["accessors"][1]["count"] = 600  # past the end of its buffer view
    (tmp_path / "over.gltf").write_text(json.dumps(doc))
    with pytest.raises(g.F184Error) as e:
        g.SyntheticScene.from_gltf(tmp_path / "over.gltf")
    assert "out of range" in str(e.value)
    doc, _, _ = _scene_doc("scene.bin")
    doc["accessors"][0]["sparse"] = {"count": 1}
    (tmp_path / "sparse.gltf").write_text(json.dumps(doc))
    with pytest.raises(g.F184Error) as e:
        g.SyntheticScene.from_gltf(tmp_path / "sparse.gltf")
    assert "sparse" in str(e.value)


def test_node_transform_and_sun_match_the_reference_math(lib, orc):
    import ctypes as C

    import final184_gb300 as g

    ref = orc.ref_lib()
    if ref is None:
        pytest.skip("the reference sources are not here")
    got = (C.c_float * 3)()
    g.load().f184gi_reference_sun_direction(got)
    want = np.zeros(3, np.float32)
    v = np.array([0, 0, -1], np.float32)  # arrays held by name: their buffers must outlive the calls
    ref.ref_quat_euler_rotate(-75.0, -30.0, 50.0, v.ctypes.data, want.ctypes.data)
    assert np.allclose(np.array(got), want, atol=2e-6)
    m = np.zeros(12, np.float32)
    t = np.array([10, 0, 0], np.float32)
    q = np.array([QUAT[3], QUAT[0], QUAT[1], QUAT[2]], np.float32)
    sc = np.array([2, 3, 4], np.float32)
    ref.ref_matrix_trs(t.ctypes.data, q.ctypes.data, sc.ctypes.data, m.ctypes.data)
    M = m.reshape(3, 4)
    mine = np.c_[_quat_matrix(QUAT) * np.array([2.0, 3.0, 4.0]), [10.0, 0, 0]]
    assert np.allclose(M, mine, atol=1e-5)


@pytest.mark.gpu
def test_gltf_scene_voxelizes_like_the_oracle(lib, orc, tmp_path):
    import torch

    import final184_gb300 as g

    doc, blob, _ = _scene_doc("scene.bin")
    (tmp_path / "scene.bin").write_bytes(blob)
    (tmp_path / "scene.gltf").write_text(json.dumps(doc))
    sc = g.SyntheticScene.from_gltf(tmp_path / "scene.gltf")
    dim, res = 32, 256
    gi = g.VoxelGI(0)
    grid = gi.create_grid(dim, 3, g.FMT_F32, 0, res, g.GRID_KEEP_COUNTS)
    dev = torch.device("cuda:0")
    td = torch.from_numpy(sc.tri_xyz).to(dev)
    ad = torch.from_numpy(sc.albedo.view(np.int32)).to(dev)
    gi.voxelize(grid, td.data_ptr(), ad.data_ptr(), sc.ntris, sc.light, bounds=sc.bounds)
    gi.sync()
    counts = gi.read_counts(grid)
    b = sc.bounds
    fo = orc.grid_frame(orc.make_bounds((b.min.x, b.min.y, b.min.z), (b.max.x, b.max.y, b.max.z)), dim,
                        np.array(sc.light.direction, np.float32))
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), res, res, sc.tri_xyz))
    _, cnt = orc.voxelize(fo, dim, res, sc.tri_xyz, sc.albedo,
                          orc.make_light(list(sc.light.luminance), list(sc.light.direction)), sd)
    assert np.array_equal(counts, cnt) and int(cnt.sum()) > 0
    gi.close()
