// ref_cuda_propagations.cu -- TEST INFRASTRUCTURE ONLY: builds the
// reference's CUDA "propagations" calculator kernels (update_leaves,
// propose, update_likelihoods), its default GPU calculator, so that the
// tests can run them beside the oracle and time them on the same GPU.
//
// The reference compiles crates/b3/src/calculator/cuda_propagations/
// typedefs.h followed by kernels.cu with NVRTC at run time, the sizes,
// scaling constants and block sizes passed as -D definitions
// (cuda_propagations/mod.rs:330-350).  The two files are included unchanged
// from the reference tree (oracle/build.py names the directory); the sizes
// and constants become __constant__ variables set before each launch, the
// block sizes keep the reference's defaults (propagation blocks of 64
// threads, leaf blocks of 256: calculator/mod.rs CUDAPropagations).

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
#define PROP_BLOCK_SIZE 64
#define LEAF_BLOCK_SIZE 256

#include "typedefs.h"
#include "kernels.cu"
