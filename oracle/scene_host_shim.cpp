// scene_host_shim.cpp -- the two library helpers the seeded scene generator (final184_gb300/csrc/scene.cpp) calls,
// so that it links into a host-only library without the CUDA library.  TEST / BASELINE INFRASTRUCTURE ONLY: the CPU
// arms of bench.py build the benchmark's scenes and cameras with it (the same generator, so the same triangles)
// without loading the product's libf184gi.so.
#include <string>

namespace f184 {
int fail(int code, const std::string&) { return code; }
// f184gi_mat4_inverse is not used by the CPU arms; it reports a singular matrix rather than guess.
bool invert4(const double*, double*) { return false; }
}  // namespace f184
