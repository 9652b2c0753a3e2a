// The reference's sop.cu without its cuRAND set-up (sop.cu:136-139), to go
// with ref_energy_hostrng.cu.  TEST INFRASTRUCTURE ONLY; the reference's own
// headers first, the define taken back, then the unmodified sop.cu.
#include "sop.h"
#undef USE_CURAND
#include "sop.cu"
