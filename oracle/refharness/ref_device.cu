// ref_device.cu — compiles the reference's own CUDA sources, unmodified, into
// one device image (cubin) for the reference-kernel harness.
//
// TEST INFRASTRUCTURE ONLY (a checker, never part of the product). The files
// are included from the reference tree where they lie; build_ref.py passes
// its src/ directory as the include path. Nothing here is copied.
//
// One adjustment is made with the preprocessor, not by editing a file: the
// reference's io/gpu_model.cu:187 calls std::memset with the MSVC-only size
// argument `sizeof PTXBlockStatistic` and relies on <cstring> arriving
// transitively. The macro below replaces the size argument of that single
// memset call by the size of its destination object, which is the same value,
// so the unmodified file compiles with GCC-based toolchains.
#include <cstring>

#include "solver/device_context.cu"
#include "solver/density_kernels.cu"
#include "solver/force_kernels.cu"
#include "solver/integration_kernels.cu"
#include "grid/sph_arrangement.cu"

#define memset(dst, value, bytes) memset(dst, value, sizeof(*(dst)))
#include "io/gpu_model.cu"
#undef memset
