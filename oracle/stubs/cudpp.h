/* Declarations of the CUDPP 1.x names the reference uses (GPUvars.cu:237-288,
 * sop.cu:1000-2600): the plan, sort and scan entry points and their enums.
 * The definitions in oracle/ref_cudpp_stub.cpp return an error; the host
 * routines exercised through oracle/_ref never reach them. */
#ifndef SOP_ORACLE_CUDPP_STUB_H
#define SOP_ORACLE_CUDPP_STUB_H
#include <cstddef>
typedef size_t CUDPPHandle;
enum CUDPPResult { CUDPP_SUCCESS = 0, CUDPP_ERROR_UNKNOWN = 9999 };
enum CUDPPOption { CUDPP_OPTION_FORWARD = 0x1, CUDPP_OPTION_INCLUSIVE = 0x8 };
enum CUDPPDatatype { CUDPP_UINT = 3 };
enum CUDPPOperator { CUDPP_ADD = 0 };
enum CUDPPAlgorithm { CUDPP_SCAN = 0, CUDPP_SORT_RADIX = 7 };
struct CUDPPConfiguration {
  CUDPPOperator op;
  CUDPPDatatype datatype;
  CUDPPAlgorithm algorithm;
  unsigned int options;
};
CUDPPResult cudppPlan(CUDPPHandle* plan, CUDPPConfiguration config, size_t n, size_t rows,
                      size_t rowPitch);
CUDPPResult cudppSort(CUDPPHandle plan, void* keys, void* values, int keyBits, size_t n);
CUDPPResult cudppScan(CUDPPHandle plan, void* out, const void* in, size_t n);
#endif
