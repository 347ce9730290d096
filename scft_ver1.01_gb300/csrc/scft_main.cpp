// Drop-in driver for the struct API: the same three calls as the reference's
// main (main.cpp:20-41) -- init_scft (flags + ab.txt + phi_<i>.dat), fft_test
// (the timed Free loop, printing F every AverIt iterations and writing
// pha_<i>.dat every 10*AverIt) and finalize_cufft.  Run it in a directory
// holding ab.txt and phi_<i>.dat, e.g.
//     scft_gb300_driver -step=200 [-precision=fp32]
#include "cuda_scft.h"
#include "init.h"
#include "init_cuda.h"
#include "struct.h"

int main(int argc, char **argv) {
  GPU_INFO gpu_info;
  CUFFT_INFO cufft_info;
  init_scft(&cufft_info, &gpu_info, argc, argv);
  if (gpu_info.kernal_type != 1) return 0;
  if (!cufft_info.gb300) return 1;
  fft_test(&gpu_info, &cufft_info);
  finalize_cufft(&gpu_info, &cufft_info);
  return 0;
}
