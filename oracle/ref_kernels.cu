// Translation unit that compiles the reference's device kernels UNCHANGED
// (cuda_aid.cu and the reduce3 template of cuda_aid.cuh, read from the
// reference tree through the include path) into a cubin for sm_103a.  The
// host harness oracle/ref_harness.cpp loads it and replays the reference's
// host code.  Built by oracle/Makefile into oracle/_ref/ (never committed).
#include "cuda_aid.cu"

// cuda_scft.cu:34 instantiates reduce3<double>; do the same here.
template __global__ void reduce3<double>(double *g_idata, double *g_odata, unsigned int n);
