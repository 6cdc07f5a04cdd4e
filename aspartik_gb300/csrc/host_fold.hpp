// host_fold.hpp -- the block-sum fold of the FP32 four-state walks, on the
// host.  The walks' blocks write their sums to mapped host memory and the
// host adds them in the order the device's one-warp fold (block_fold in
// runs4.cuh) uses, so a result does not depend on which side folds: lane l
// adds sums l, l + 32, l + 64, ... in order, then a shuffle-down tree of
// offsets 16, 8, 4, 2, 1 leaves the total in lane 0.
#pragma once

#include <cstdint>

namespace b3g {

inline double fold_block_sums(const double *sums, uint32_t count)
{
	double lane[32];
	for (uint32_t l = 0; l < 32; ++l) {
		double sum = 0.0;
		for (uint32_t k = l; k < count; k += 32)
			sum += sums[k];
		lane[l] = sum;
	}
	// lane l takes lane l + off's value of the previous level: updating in
	// increasing l reads each partner before it changes
	for (uint32_t off = 16; off > 0; off >>= 1)
		for (uint32_t l = 0; l + off < 32; ++l)
			lane[l] += lane[l + off];
	return lane[0];
}

} // namespace b3g
