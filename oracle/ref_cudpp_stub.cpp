// Link-time definitions for the CUDPP names (see stubs/cudpp.h).  They fail
// loudly: the reference's GPU list drivers are not used through oracle/_ref.
#include "cudpp.h"
CUDPPResult cudppPlan(CUDPPHandle* plan, CUDPPConfiguration, size_t, size_t, size_t) {
  if (plan) *plan = 0;
  return CUDPP_ERROR_UNKNOWN;
}
CUDPPResult cudppSort(CUDPPHandle, void*, void*, int, size_t) { return CUDPP_ERROR_UNKNOWN; }
CUDPPResult cudppScan(CUDPPHandle, void*, const void*, size_t) { return CUDPP_ERROR_UNKNOWN; }
