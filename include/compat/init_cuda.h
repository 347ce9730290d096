/* init_cuda.h -- reference API (init_cuda.h:11-15). */
#pragma once
#include "struct.h"

extern void init_cuda(GPU_INFO *gpu_info, int display);
extern void initialize_cufft(GPU_INFO *gpu_info, CUFFT_INFO *cufft_info);
extern void finalize_cufft(GPU_INFO *gpu_info, CUFFT_INFO *cufft_info);
