/* Stand-in for the CUDA SDK 3.x cutil_inline.h that the reference includes
 * (global.h:6, GPUvars.h:11).  Only the two macros the reference uses and the
 * since-removed cudaThreadSynchronize are provided.  Used only to compile the
 * reference's own sources into oracle/_ref for host-side parity checks. */
#ifndef SOP_ORACLE_CUTIL_STUB_H
#define SOP_ORACLE_CUTIL_STUB_H
#include <cuda_runtime.h>
#include <sys/types.h>
#include <cstdio>
#include <cstdlib>
#define cutilSafeCall(call)                                              \
  do {                                                                   \
    cudaError_t cutil_err_ = (call);                                     \
    if (cutil_err_ != cudaSuccess) {                                     \
      std::fprintf(stderr, "cuda error %d at %s:%d\n", (int)cutil_err_, \
                   __FILE__, __LINE__);                                  \
      std::exit(-1);                                                     \
    }                                                                    \
  } while (0)
#define cutilCheckMsg(msg) cutilSafeCall(cudaGetLastError())
#define cudaThreadSynchronize cudaDeviceSynchronize
#endif
