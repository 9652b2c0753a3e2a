// Stand-in for the three CUDPP 1.x calls the reference makes: the plans of
// alloc_cudpp (GPUvars.cu:237-288) and the sorts and scans of the GPU list
// drivers (sop.cu:1000-1254, 1513-1616).
//
// TEST INFRASTRUCTURE ONLY (linked into oracle/_ref by oracle/build_ref.sh).
// CUDPP is not part of this toolchain, and the reference does not pin a
// version (Makefile:16-18 points at a local install of the 1.x series).  The
// published semantics of the calls it uses:
//
//   cudppSort(plan, keys, values, keyBits, n)
//     LSD radix sort of n (uint key, 4-byte value) pairs on the low keyBits
//     bits of the key, in place.  LSD radix sort is stable, so with the 0/1
//     flags of the list drivers (0 = keep) it is a stable partition: the kept
//     records first, in their original order.
//   cudppScan(plan, out, in, n)
//     inclusive prefix sum of n uints (the reference's plan asks for
//     CUDPP_OPTION_FORWARD | CUDPP_OPTION_INCLUSIVE, GPUvars.cu:245-249).
//
// Both are provided with CUB, which ships with the CUDA toolkit:
// DeviceRadixSort::SortPairs on bits [0, keyBits) and DeviceScan::InclusiveSum,
// on the legacy default stream the reference itself uses.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "cudpp.h"

namespace {

// Grow-only device scratch, kept for the life of the process.
struct Scratch {
  void* p = nullptr;
  size_t bytes = 0;
  bool reserve(size_t want) {
    if (want <= bytes) return true;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    if (cudaMalloc(&p, want) != cudaSuccess) return false;
    bytes = want;
    return true;
  }
};

Scratch g_tmp, g_keys_alt, g_vals_alt;

}  // namespace

CUDPPResult cudppPlan(CUDPPHandle* plan, CUDPPConfiguration config, size_t, size_t, size_t) {
  if (!plan) return CUDPP_ERROR_UNKNOWN;
  if (config.algorithm != CUDPP_SORT_RADIX && config.algorithm != CUDPP_SCAN)
    return CUDPP_ERROR_UNKNOWN;
  *plan = static_cast<CUDPPHandle>(config.algorithm) + 1;
  return CUDPP_SUCCESS;
}

CUDPPResult cudppSort(CUDPPHandle plan, void* keys, void* values, int keyBits, size_t n) {
  if (plan != static_cast<CUDPPHandle>(CUDPP_SORT_RADIX) + 1 || keyBits < 1 || keyBits > 32)
    return CUDPP_ERROR_UNKNOWN;
  if (n == 0) return CUDPP_SUCCESS;
  const size_t vb = n * sizeof(unsigned int);
  if (!g_keys_alt.reserve(vb) || !g_vals_alt.reserve(vb)) return CUDPP_ERROR_UNKNOWN;
  unsigned int* k = static_cast<unsigned int*>(keys);
  unsigned int* v = static_cast<unsigned int*>(values);
  cub::DoubleBuffer<unsigned int> kb(k, static_cast<unsigned int*>(g_keys_alt.p));
  cub::DoubleBuffer<unsigned int> vbuf(v, static_cast<unsigned int*>(g_vals_alt.p));
  size_t tb = 0;
  if (cub::DeviceRadixSort::SortPairs(nullptr, tb, kb, vbuf, static_cast<int>(n), 0, keyBits) !=
      cudaSuccess)
    return CUDPP_ERROR_UNKNOWN;
  if (!g_tmp.reserve(tb > 0 ? tb : 1)) return CUDPP_ERROR_UNKNOWN;
  if (cub::DeviceRadixSort::SortPairs(g_tmp.p, tb, kb, vbuf, static_cast<int>(n), 0, keyBits) !=
      cudaSuccess)
    return CUDPP_ERROR_UNKNOWN;
  if (kb.Current() != k &&
      cudaMemcpy(k, kb.Current(), vb, cudaMemcpyDeviceToDevice) != cudaSuccess)
    return CUDPP_ERROR_UNKNOWN;
  if (vbuf.Current() != v &&
      cudaMemcpy(v, vbuf.Current(), vb, cudaMemcpyDeviceToDevice) != cudaSuccess)
    return CUDPP_ERROR_UNKNOWN;
  return CUDPP_SUCCESS;
}

CUDPPResult cudppScan(CUDPPHandle plan, void* out, const void* in, size_t n) {
  if (plan != static_cast<CUDPPHandle>(CUDPP_SCAN) + 1) return CUDPP_ERROR_UNKNOWN;
  if (n == 0) return CUDPP_SUCCESS;
  const unsigned int* src = static_cast<const unsigned int*>(in);
  unsigned int* dst = static_cast<unsigned int*>(out);
  size_t tb = 0;
  if (cub::DeviceScan::InclusiveSum(nullptr, tb, src, dst, static_cast<int>(n)) != cudaSuccess)
    return CUDPP_ERROR_UNKNOWN;
  if (!g_tmp.reserve(tb > 0 ? tb : 1)) return CUDPP_ERROR_UNKNOWN;
  if (cub::DeviceScan::InclusiveSum(g_tmp.p, tb, src, dst, static_cast<int>(n)) != cudaSuccess)
    return CUDPP_ERROR_UNKNOWN;
  return CUDPP_SUCCESS;
}
