// Link-time wrappers that let the reference's unmodified objects run as an
// oracle.  TEST INFRASTRUCTURE ONLY: every artefact oracle/build_ref.sh makes
// links with -Wl,--wrap=cudaMemcpy -Wl,--wrap=_Z9setup_rngyy, so the
// reference's calls to those two functions land here.
//
// cudaMemcpy: the host list filters (sop.cu:1351-1448, 1707-1823) stage the
//   coordinates and lists through the device arrays.  With host copies on
//   (ref_host_copies(1)), the harness points those arrays at host buffers and
//   every copy is a host memmove, so the filters run on a machine without a
//   GPU.  Off (the default), the CUDA runtime's own copy runs.
// setup_rng (GPUvars.cu:430-453): underdamped_ctrl seeds cuRAND with the
//   constant 1234 (sop.cu:139), so every run of the reference draws the same
//   noise.  When SOP_REF_CURAND_SEED is set, its value replaces the seed
//   passed in; independent trajectories for the statistical comparison need
//   it.  Unset, the seed passes through unchanged.
#include <cuda_runtime_api.h>

#include <cstdlib>
#include <cstring>

extern "C" {

cudaError_t __real_cudaMemcpy(void* dst, const void* src, size_t count, enum cudaMemcpyKind kind);
void __real__Z9setup_rngyy(unsigned long long seed, unsigned long long offset);

static int g_host_copies = 0;

void ref_host_copies(int on) { g_host_copies = on; }

cudaError_t __wrap_cudaMemcpy(void* dst, const void* src, size_t count, enum cudaMemcpyKind kind) {
  if (g_host_copies) {
    if (count) std::memmove(dst, src, count);
    return cudaSuccess;
  }
  return __real_cudaMemcpy(dst, src, count, kind);
}

void __wrap__Z9setup_rngyy(unsigned long long seed, unsigned long long offset) {
  const char* s = std::getenv("SOP_REF_CURAND_SEED");
  if (s && *s) seed = std::strtoull(s, nullptr, 10);
  __real__Z9setup_rngyy(seed, offset);
}

}  // extern "C"
