// Prints the device map that init_scft (init.cpp:8-37) parses from the
// reference's flags: -GPU_N=<n> and -gpu<i>=<device>.  Run with -kernal=CPU so
// that no device is touched (the CPU branch only parses and prints).
#include <stdio.h>

#include "init.h"
#include "struct.h"

int main(int argc, char **argv) {
  GPU_INFO gpu_info;
  CUFFT_INFO cufft_info;
  init_scft(&cufft_info, &gpu_info, argc, argv);
  printf("kernal_type=%d GPU_N=%d map=", gpu_info.kernal_type, gpu_info.GPU_N);
  for (int i = 0; i < gpu_info.GPU_N; ++i) printf("%s%d", i ? "," : "", gpu_info.whichGPUs[i]);
  printf(" MaxIT=%d\n", cufft_info.MaxIT);
  return 0;
}
