"""The C ABI without a GPU: the library loads, exports every declared symbol, struct layouts agree with C,
host-side helpers match the reference's own Math/CCamera compiled from source, and argument checks fail loudly."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "f184gi.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(f184gi_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 28
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "final184_gb300", "libf184gi.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_ctypes_mirror_covers_header(lib):
    from final184_gb300 import _abi

    assert set(declared_functions()) == set(_abi.PROTOTYPES)


def test_struct_layouts_match_c():
    from final184_gb300 import _abi

    structs = {"f184gi_vec3": _abi.Vec3, "f184gi_bounds": _abi.Bounds, "f184gi_light": _abi.Light,
               "f184gi_grid_desc": _abi.GridDesc, "f184gi_grid_frame": _abi.GridFrame, "f184gi_view": _abi.View,
               "f184gi_cone_params": _abi.ConeParams, "f184gi_config": _abi.Config, "f184gi_scene": _abi.Scene,
               "f184gi_move": _abi.Move, "f184gi_march_params": _abi.MarchParams,
               "f184gi_server_config": _abi.ServerConfig, "f184gi_request": _abi.Request,
               "f184gi_request_result": _abi.RequestResult, "f184gi_server_stats": _abi.ServerStats}
    src = '#include <stddef.h>\n#include <stdio.h>\n#include "f184gi.h"\nint main(void){\n'
    for name in structs:
        src += '  printf("%%zu\\n", sizeof(%s));\n' % name
    for name, cls in structs.items():  # then every field's offset, in the mirror's order
        for field, _ in cls._fields_:
            src += '  printf("%%zu\\n", offsetof(%s, %s));\n' % (name, field)
    src += "  return 0;\n}\n"
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "s")
        # plain C99 with strict warnings: the header is what a C (or cgo / ctypes) caller includes
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                        c, "-o", exe], check=True)
        sizes = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    for (name, cls), sz in zip(structs.items(), sizes):
        assert C.sizeof(cls) == sz, name
    offsets = iter(sizes[len(structs):])
    for name, cls in structs.items():
        for field, _ in cls._fields_:
            assert getattr(cls, field).offset == next(offsets), (name, field)
    assert C.sizeof(_abi.Vec3) == 12 and C.sizeof(_abi.Bounds) == 32


def test_boundary_types_match_reference_layout(orc):
    ref = orc.ref_lib()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    from final184_gb300 import _abi

    assert ref.ref_sizeof(0) == C.sizeof(_abi.Vec3) == 12  # tc::Vector3
    assert ref.ref_sizeof(1) == C.sizeof(_abi.Bounds) == 32  # tc::BoundingBox with padding
    assert ref.ref_sizeof(3) == 64  # tc::Matrix4: the view/proj layout of f184gi_view


@pytest.mark.parametrize("fovy,aspect,near,far", [(59.0, 16 / 9, 0.1, 100.0), (59.0, 1.0, 0.1, 1000.0),
                                                  (90.0, 4 / 3, 0.5, 20.0), (30.0, 2.0, 1.0, 50.0)])
def test_perspective_matches_reference_ccamera(lib, orc, fovy, aspect, near, far):
    ref = orc.ref_lib()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    import final184_gb300 as g

    want = np.zeros(16, np.float32)
    ref.ref_calc_perspective(fovy, aspect, near, far, want.ctypes.data_as(C.c_void_p))
    got = g.perspective(fovy, aspect, near, far).ravel()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("mx,my,near,far", [(20.0, 20.0, 1.0, 20.0), (16.0, 16.0, 1.0, 20.0), (3.0, 5.0, 0.1, 9.0)])
def test_ortho_matches_reference_ccamera(lib, orc, mx, my, near, far):
    ref = orc.ref_lib()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    import final184_gb300 as g

    want = np.zeros(16, np.float32)
    ref.ref_calc_ortho(mx, my, near, far, want.ctypes.data_as(C.c_void_p))
    assert np.array_equal(g.ortho(mx, my, near, far).ravel().view(np.uint32), want.view(np.uint32))


def test_inverse_matches_reference(lib, orc):
    ref = orc.ref_lib()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    import final184_gb300 as g

    rng = np.random.default_rng(3)
    for _ in range(20):
        eye = rng.uniform(-8, 8, 3)
        tgt = eye + rng.normal(size=3)
        m = (g.perspective(59.0, 1.7, 0.1, 100.0).astype(np.float64) @ g.look_at(eye, tgt)).astype(np.float32)
        want = np.zeros(16, np.float32)
        mm = np.ascontiguousarray(m.ravel())  # held by name: its buffer must outlive the call
        ref.ref_matrix4_inverse(mm.ctypes.data_as(C.c_void_p), want.ctypes.data_as(C.c_void_p))
        got = g.mat4_inverse(m).ravel()
        assert np.allclose(got, want, rtol=1e-4, atol=1e-5)


def test_look_at_is_rigid_inverse(lib):
    import final184_gb300 as g

    v = g.look_at([1.0, 2.0, 3.0], [4.0, 2.5, -1.0]).astype(np.float64)
    r = v[:3, :3]
    assert np.allclose(r @ r.T, np.eye(3), atol=1e-6)
    eye_h = np.array([1.0, 2.0, 3.0, 1.0])
    assert np.allclose(v @ eye_h, [0, 0, 0, 1], atol=1e-5)
    fwd = np.array([3.0, 0.5, -4.0])
    fwd /= np.linalg.norm(fwd)
    assert np.allclose(r @ fwd, [0, 0, -1], atol=1e-6)  # the camera looks down its -Z


def test_frame_from_bounds_matches_oracle(lib, orc):
    import final184_gb300 as g

    rng = np.random.default_rng(11)
    for dim in (16, 64, 256, 512):
        mn = rng.uniform(-20, 0, 3).astype(np.float32)
        mx = (mn + rng.uniform(0.5, 30, 3)).astype(np.float32)
        ld = rng.normal(size=3).astype(np.float32)
        f1 = g.frame_from_bounds(g.make_bounds(mn, mx), dim, ld)
        f2 = orc.grid_frame(orc.make_bounds(mn, mx), dim, ld)
        assert bytes(f1) == bytes(f2)


def test_grid_bytes_and_errors(lib):
    import final184_gb300 as g
    from final184_gb300 import _abi

    d = _abi.GridDesc(256, 8, g.FMT_F32, 0, 2048, 0)
    n = C.c_uint64()
    assert lib.f184gi_grid_bytes(C.byref(d), C.byref(n)) == 0
    levels = 256 ** 3 + sum(((256 >> l) + 2) ** 3 for l in range(1, 8))  # levels >= 1 carry a ring of zeros
    # the frame is followed on the device by its voxel map as FP32 pairs (8 floats)
    assert n.value == levels * 16 + 2048 * 2048 * 8 + C.sizeof(_abi.GridFrame) + 32
    bad = _abi.GridDesc(100, 3, 0, 0, 1024, 0)
    assert lib.f184gi_grid_bytes(C.byref(bad), C.byref(n)) == _abi.ERR_INVALID
    assert b"power of two" in lib.f184gi_last_error()
    bad = _abi.GridDesc(64, 9, 0, 0, 1024, 0)
    assert lib.f184gi_grid_bytes(C.byref(bad), C.byref(n)) == _abi.ERR_INVALID
    assert lib.f184gi_voxelize(None, 1, None, None, 0, None, None, None, 0, None) == _abi.ERR_INVALID
    assert lib.f184gi_trace(None, 1, None, 0, None, None) == _abi.ERR_INVALID
    assert lib.f184gi_abi_version() == 1


def test_scene_generator_deterministic_and_sized(lib):
    import final184_gb300 as g

    a = g.SyntheticScene(184, 20000, 200)
    b = g.SyntheticScene(184, 20000, 200)
    assert a.ntris == b.ntris and 18000 <= a.ntris <= 22000
    assert np.array_equal(a.tri_xyz, b.tri_xyz) and np.array_equal(a.albedo, b.albedo)
    assert np.all(np.abs(a.tri_xyz) <= 10.0)
    assert a.nobjects == 201 and int(a.object_count.sum()) == a.ntris
    assert np.all((a.roughness >= 0.1) & (a.roughness <= 0.9))
    c = g.SyntheticScene(185, 20000, 200)
    assert not np.array_equal(a.tri_xyz, c.tri_xyz)
    big = g.SyntheticScene(1184, 500000, 2000)
    assert 450000 <= big.ntris <= 550000
    ld = np.array(a.light.direction)
    assert abs(np.linalg.norm(ld) - 1) < 1e-5 and ld[1] < 0  # the sun shines downwards


def test_move_objects_is_seeded_and_rigid(lib):
    import final184_gb300 as g

    a = g.SyntheticScene(184, 20000, 200)
    before = a.tri_xyz.copy()
    moved = a.move_objects(5, 0.05, 1.0)
    assert len(moved) == 10 and 0 not in moved
    b = g.SyntheticScene(184, 20000, 200)
    assert np.array_equal(b.move_objects(5, 0.05, 1.0), moved)
    assert np.array_equal(a.tri_xyz, b.tri_xyz)
    changed = np.any(before.reshape(-1, 9) != a.tri_xyz.reshape(-1, 9), axis=1)
    for o in range(a.nobjects):
        f, n = a.object_first[o], a.object_count[o]
        if o not in moved:
            assert not changed[f:f + n].any()
        else:  # rigid translation: every vertex moved by the same offset
            d = (a.tri_xyz.reshape(-1, 3)[f * 3:(f + n) * 3] - before.reshape(-1, 3)[f * 3:(f + n) * 3])
            assert np.allclose(d, d[0], atol=1e-5)
