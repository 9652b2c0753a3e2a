// The reference's energy.cu with its host noise generator.
//
// TEST INFRASTRUCTURE ONLY (built into oracle/_ref/sop2ref_hostrng.x by
// oracle/build_ref.sh).  GPUvars.h:26 defines USE_CURAND, which selects the
// cuRAND kernel for the random force (energy.cu:154-167).  With the define
// taken back, energy.cu compiles its host path instead (energy.cu:168-188):
// the forces are copied to the host, each gets var * gasdev() from the
// reference's own generator (random_generator.cpp:83-108, seeded by
// `set run`, param.cpp:274-279) and goes back.  The reference's own headers
// come first (behind their include guards), the define is removed, and the
// unmodified energy.cu follows.
#include "energy.h"
#undef USE_CURAND
#include "energy.cu"
