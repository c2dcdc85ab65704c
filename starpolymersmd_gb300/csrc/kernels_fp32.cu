// FP32 fast-path instantiation: float4 state, int64 fixed-point cell sums.
#define SMPC_REAL float
#define SMPC_FAST_F32 1
#define SMPC_COLLIDE_NT 256
#define SMPC_COLLIDE_CT 128
#define SMPC_COLLIDE_CAP 1408
#define SMPC_BIN_NT 256
#define SMPC_MD_NT 1024
#define SMPC_MD_MPT 1
#include "kernels_impl.cuh"
