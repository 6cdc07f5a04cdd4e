// index_width.hpp -- when a pruning walk may form its element indices in
// 32 bits.
//
// A walk addresses partials and scale counts as slot * C * ldp + column (in
// partial vectors); 32-bit indices are used when every such index stays
// below 2^31.  Host-only and free of CUDA types, so that the decision can be
// compiled and checked on its own.
#pragma once

#include <cstdint>

namespace b3g {

// The caller's slot count is not known (the allocation-free entry point
// takes caller-owned buffers of any size): indices must be 64-bit.
constexpr uint64_t kUnknownSlots = ~0ull;

constexpr uint64_t kNarrowIndexLimit = 1ull << 31;

// True when slot * C * ldp + column < 2^31 for every slot < `slots`.
constexpr bool narrow_index(uint64_t slots, uint64_t C, uint64_t ldp)
{
	return slots != kUnknownSlots && C > 0 && ldp > 0 &&
	       slots <= kNarrowIndexLimit / (C * ldp) &&
	       slots * C * ldp < kNarrowIndexLimit;
}

// The allocation-free entry point trusts slot ids up to 2^32 - 1 in
// buffers it did not allocate, so it always walks with 64-bit indices.
constexpr bool noalloc_narrow_index(uint64_t C, uint64_t ldp)
{
	return narrow_index(kUnknownSlots, C, ldp);
}

} // namespace b3g
