"""Build recipes for the test-only checker libraries (TEST INFRASTRUCTURE ONLY).

  oracle/_build/liboracle.so  -- the CPU restatement in oracle.cpp (FP64 oracle + FP32 CPU baseline)
  oracle/_ref/libf184ref.so   -- the reference's own Math library and CCamera (Foreground/SceneGraph/Camera.cpp),
                                 compiled from the reference sources where they lie, plus ref_shim.cpp; only
                                 built when that tree is present (it is not on GPU machines).
  oracle/_ref/libf184glsl.so  -- the reference's shader functions compiled as C++ (glsl_pin.py), same condition.

The reference tree is taken from the F184_REFERENCE environment variable (default /root/reference).
"""
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("F184_REFERENCE", "/root/reference")
LIB = os.path.join(HERE, "_build", "liboracle.so")
SCENE_LIB = os.path.join(HERE, "_build", "libscenehost.so")
PRODUCT_CSRC = os.path.join(HERE, "..", "final184_gb300", "csrc")
REF_LIB = os.path.join(HERE, "_ref", "libf184ref.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle(force=False):
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    src = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "oracle.h"),
           os.path.join(HERE, "..", "include", "f184gi.h")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in src):
        # -ffp-contract=off: every FP64 operation rounds on its own, as on the device
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
              src[0], "-o", LIB])
    return LIB


def build_scene_host(force=False):
    """The product's seeded scene generator and camera helpers (csrc/scene.cpp, host C++) as a library of their own,
    for the CPU arms of the benchmark, which must not load the CUDA library."""
    os.makedirs(os.path.dirname(SCENE_LIB), exist_ok=True)
    src = [os.path.join(PRODUCT_CSRC, "scene.cpp"), os.path.join(HERE, "scene_host_shim.cpp")]
    deps = src + [os.path.join(PRODUCT_CSRC, "gi_internal.h"), os.path.join(HERE, "..", "include", "f184gi.h")]
    if force or not os.path.exists(SCENE_LIB) or any(os.path.getmtime(s) > os.path.getmtime(SCENE_LIB) for s in deps):
        cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", cuda_inc, *src, "-o",
              SCENE_LIB])
    return SCENE_LIB


def build_ref(force=False):
    """Compile the reference Math library + CCamera into oracle/_ref (x86 or Arm, no SSE path)."""
    if not os.path.isdir(REF_ROOT):
        return None
    os.makedirs(os.path.dirname(REF_LIB), exist_ok=True)
    shim = os.path.join(HERE, "ref_shim.cpp")
    if os.path.exists(REF_LIB) and not force and os.path.getmtime(shim) <= os.path.getmtime(REF_LIB):
        return REF_LIB
    math_src = sorted(glob.glob(os.path.join(REF_ROOT, "Math", "*.cpp")))
    cam_src = os.path.join(REF_ROOT, "Foreground", "SceneGraph", "Camera.cpp")
    stub_dir = os.path.join(HERE, "ref_stub")  # MathAPI.h: the export macro CMake would generate
    # -ffp-contract=off: the scalar Math code rounds every operation, on Arm (which has FMA) as on x86
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-I", stub_dir, "-I", os.path.join(REF_ROOT, "Math"),
          "-I", os.path.join(REF_ROOT, "Foreground", "SceneGraph"), *math_src, cam_src, shim, "-o", REF_LIB])
    return REF_LIB


def build(force=False):
    build_oracle(force)
    build_scene_host(force)
    try:
        build_ref(force)
    except RuntimeError as e:  # the reference pin is optional; the oracle is not
        print("warning: reference Math/Camera build failed:", str(e).splitlines()[0])
    try:
        from . import glsl_pin
    except ImportError:  # run as a script
        import glsl_pin
    try:
        glsl_pin.build(force)
    except RuntimeError as e:
        print("warning: reference shader pin build failed:", str(e).splitlines()[0])


if __name__ == "__main__":
    build(force=True)
    print(LIB, REF_LIB if os.path.exists(REF_LIB) else "(no reference build)")
