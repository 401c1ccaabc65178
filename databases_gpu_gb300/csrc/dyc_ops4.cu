// Kernels and launchers for 4-byte keys (32-bit key, 32-bit value slots).
#include "dyc_ops.cuh"
template struct dyc::Ops<4>;
