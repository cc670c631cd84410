"""The C++ host adapter (include/f184gi_foreground.hpp): it compiles against the C ABI without a GPU, and on a
GPU its RenderList / BuildMips / TraceViews frame gives byte-identical output to the plain C ABI calls, and a
RenderList of the primitives CullList keeps inside the camera frustum gives the same L0 bytes as the C ABI
voxelizing those primitives' triangles."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_adapter(tmp):
    exe = os.path.join(tmp, "adapter_main")
    libdir = os.path.join(ROOT, "final184_gb300")
    # the header is included by the renderer's own sources: it must build warning-free under strict flags
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           os.path.join(ROOT, "tests", "cpp", "adapter_main.cpp"), "-o", exe, "-L", libdir, "-lf184gi",
           "-Wl,-rpath," + libdir, "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64")]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_adapter_compiles(lib, tmp_path):
    assert os.path.exists(build_adapter(str(tmp_path)))


@pytest.mark.gpu
def test_adapter_matches_c_abi(lib, tmp_path):
    exe = build_adapter(str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("matches") == 2
