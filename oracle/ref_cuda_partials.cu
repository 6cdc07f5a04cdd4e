// ref_cuda_partials.cu -- TEST INFRASTRUCTURE ONLY: builds the reference's
// own FP64 CUDA pruning kernel so that the tests can run it and pin the
// oracle to the reference's arithmetic.
//
// The reference compiles crates/b3/src/calculator/cuda_partials/typedefs.h
// followed by kernels.cu with NVRTC at run time, the sizes and scaling
// constants passed as -D definitions (cuda_partials/mod.rs:20-21,240-256).
// Here the same two files are included unchanged from the reference tree
// (oracle/build.py names the directory; nothing of them is copied into this
// repository), with the definitions turned into __constant__ variables so
// that one cubin serves every test case; the tests set them through the
// driver API before each launch.  BLOCK_SIZE keeps the reference's default
// of 32 threads (calculator/mod.rs: CUDAPartials block_size).

__constant__ unsigned ref_num_patterns;
__constant__ unsigned ref_num_leaves;
__constant__ unsigned ref_scale_ln;
__constant__ double ref_scale_threshold;
__constant__ double ref_scale_mult;

#define NUM_PATTERNS ref_num_patterns
#define NUM_LEAVES ref_num_leaves
#define SCALE_LN ref_scale_ln
#define SCALE_THRESHOLD ref_scale_threshold
#define SCALE_MULT ref_scale_mult
#define BLOCK_SIZE 32

#include "typedefs.h"
#include "kernels.cu"
