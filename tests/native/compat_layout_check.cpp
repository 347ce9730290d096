// Built by tests/test_driver_gpu.py with -DSCFT_COMPAT_FP64_LAYOUT: a driver
// of the struct API that reads qa_cu/qcb_cu after getConc in the reference's
// g[b][r][s] layout and checks them against the library's contour-outer
// slices (scft_get_q).  Prints "layout_maxdiff=<x> reference_layout=<0|1>".
#include <stdio.h>

#include <vector>

#include "cuda_scft.h"
#include "init.h"
#include "init_cuda.h"
#include "struct.h"

int main(int argc, char **argv) {
  GPU_INFO gpu_info;
  CUFFT_INFO c;
  init_scft(&c, &gpu_info, argc, argv);
  if (!c.gb300) return 2;
  getConc(&gpu_info, &c);
  int NsA = 0, dNsB = 0;
  scft_get_ns(c.gb300, &NsA, &dNsB);
  const long M = c.NxNyNz;
  const int B = c.batch;
  double maxdiff = 0.0;
  struct { double *g; int q, ns; } cases[2] = {{c.qa_cu[0], SCFT_Q_A, NsA},
                                                {c.qcb_cu[0], SCFT_Q_CB, dNsB}};
  for (auto &k : cases) {
    std::vector<double> g((size_t)B * M * (k.ns + 1)), sl((size_t)B * M);
    if (cudaMemcpy(g.data(), k.g, sizeof(double) * g.size(), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
      return 3;
    const int ss[4] = {0, 1, k.ns / 2, k.ns};
    for (int s : ss) {
      if (scft_get_q(c.gb300, k.q, s, sl.data()) != SCFT_OK) return 4;
      for (int b = 0; b < B; ++b)
        for (long r = 0; r < M; ++r) {
          const double d = g[((size_t)b * M + r) * (k.ns + 1) + s] - sl[(size_t)b * M + r];
          if (d > maxdiff) maxdiff = d;
          if (-d > maxdiff) maxdiff = -d;
        }
    }
  }
  printf("layout_maxdiff=%g reference_layout=%d\n", maxdiff, c.reference_layout);
  finalize_cufft(&gpu_info, &c);
  return 0;
}
