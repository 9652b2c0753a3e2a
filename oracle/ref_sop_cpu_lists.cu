// The reference's sop.cu compiled with its host-only list routines.
//
// TEST INFRASTRUCTURE ONLY (built into oracle/_ref/libsopref.so by
// oracle/build_ref.sh).  GPUvars.h:33 defines USE_GPU_NL_PL, which selects
// the CUDPP-based GPU list drivers of sop.cu (924-1262, 1452-1620).  With the
// define taken back, sop.cu compiles its host filters instead:
// update_neighbor_list (sop.cu:1351-1448) and update_pair_list
// (sop.cu:1707-1823), the routines that pin the oracle's list predicates.
//
// The reference's own header chain is included first (sop.h pulls in
// GPUvars.h behind its include guard), the define is removed, and the
// unmodified sop.cu follows; its own #include "sop.h" is then a no-op.  No
// reference file is copied or edited.
#include "sop.h"
#undef USE_GPU_NL_PL
#include "sop.cu"
