/* cuda_scft.h -- reference API (cuda_scft.h:1-2) plus the non-header
 * externs of cuda_scft.cu (:14, :61, :140). */
#pragma once
#include "struct.h"

extern void sovDifFft(GPU_INFO *gpu_info, CUFFT_INFO *cufft_info, std::vector<double *> g,
                      std::vector<double *> w, int ns, int sign);
extern void fft_test(GPU_INFO *gpu_info, CUFFT_INFO *cufft_info);
extern void average_value(std::vector<double *> data, GPU_INFO *gpu_info, CUFFT_INFO *cufft_info);
extern void getConc(GPU_INFO *gpu_info, CUFFT_INFO *cufft_info);
extern double Free(GPU_INFO *gpu_info, CUFFT_INFO *cufft_info);
