// Library identification (host only).
#include "common.cuh"

extern "C" const char *seqm_version(void) { return "pyseqm_gb300 0.1 (sm_103a, FP64 Jacobi/SP2 SCF)"; }
