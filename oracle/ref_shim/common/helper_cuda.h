/* Stand-in for the CUDA samples' helper_cuda.h (not installed). */
#pragma once
#define checkCudaErrors(x) (x)
