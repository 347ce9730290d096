/* init.h -- reference API (init.h:5): flags and ab.txt, then device set-up. */
#pragma once
#include "struct.h"
#include "init_cuda.h"

int init_scft(CUFFT_INFO *cufft_info, GPU_INFO *gpu_info, int argc, char **argv);
