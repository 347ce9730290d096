/* Project-written stand-in for the CUDA-samples header (struct.h:7); empty. */
#pragma once
