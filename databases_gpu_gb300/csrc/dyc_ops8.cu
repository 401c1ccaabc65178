// Kernels and launchers for 8-byte keys (16-byte {key, value} slots).
#include "dyc_ops.cuh"
template struct dyc::Ops<8>;
