// verbatim.hpp -- the byte layout of the reference's state files
// (crates/verbatim/src/lib.rs: VerbatimWriter / VerbatimReader).
//
// Little-endian primitives, each preceded by zero bytes up to a multiple of
// its own size counted from the start of the stream (lib.rs:14-27, 102-119);
// a tag is its raw bytes (lib.rs:67-74); a slice is its u32 length, then,
// when it is not empty, zero bytes up to a multiple of the element's
// alignment, then the elements (lib.rs:76-93, 229-258).  Bytes are written
// one by one, so the host's byte order does not matter.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace b3g {
namespace verbatim {

class Writer {
      public:
	const std::vector<uint8_t> &bytes() const { return out_; }

	void tag(const uint8_t *t, size_t n) { out_.insert(out_.end(), t, t + n); }
	void u32(uint32_t v) { uint_le(v, 4); }
	void u64(uint64_t v) { uint_le(v, 8); }
	void i64(int64_t v) { uint_le((uint64_t)v, 8); }
	void f64(double v)
	{
		uint64_t b;
		std::memcpy(&b, &v, 8);
		uint_le(b, 8);
	}
	// a u128 given as its low and high 64-bit halves
	void u128(uint64_t lo, uint64_t hi)
	{
		pad(16);
		put_le(lo, 8);
		put_le(hi, 8);
	}
	void slice_u32(const uint32_t *v, size_t n)
	{
		u32((uint32_t)n);
		if (n)
			pad(4);
		for (size_t i = 0; i < n; ++i)
			put_le(v[i], 4);
	}
	void slice_f64(const double *v, size_t n)
	{
		u32((uint32_t)n);
		if (n)
			pad(8);
		for (size_t i = 0; i < n; ++i) {
			uint64_t b;
			std::memcpy(&b, &v[i], 8);
			put_le(b, 8);
		}
	}

      private:
	void pad(size_t a)
	{
		while (out_.size() % a)
			out_.push_back(0);
	}
	void put_le(uint64_t v, size_t n)
	{
		for (size_t k = 0; k < n; ++k)
			out_.push_back((uint8_t)(v >> (8 * k)));
	}
	void uint_le(uint64_t v, size_t n)
	{
		pad(n);
		put_le(v, n);
	}
	std::vector<uint8_t> out_;
};

// Reads what Writer writes; a short stream or a wrong tag throws
// std::runtime_error (padding bytes are skipped unread, as the reference
// does).
class Reader {
      public:
	Reader(const uint8_t *p, size_t n) : p_(p), n_(n) {}
	size_t offset() const { return at_; }
	size_t left() const { return n_ - at_; }

	// true when the next n bytes are the tag (consumed), false otherwise
	bool tag(const uint8_t *t, size_t n)
	{
		need(n);
		if (std::memcmp(p_ + at_, t, n) != 0)
			return false;
		at_ += n;
		return true;
	}
	uint32_t u32() { return (uint32_t)uint_le(4); }
	uint64_t u64() { return uint_le(8); }
	int64_t i64() { return (int64_t)uint_le(8); }
	double f64()
	{
		const uint64_t b = uint_le(8);
		double v;
		std::memcpy(&v, &b, 8);
		return v;
	}
	void u128(uint64_t &lo, uint64_t &hi)
	{
		skip_pad(16);
		lo = get_le(8);
		hi = get_le(8);
	}
	std::vector<uint32_t> slice_u32()
	{
		const uint32_t n = u32();
		if (n)
			skip_pad(4);
		need((size_t)n * 4);
		std::vector<uint32_t> v(n);
		for (uint32_t i = 0; i < n; ++i)
			v[i] = (uint32_t)get_le(4);
		return v;
	}
	std::vector<double> slice_f64()
	{
		const uint32_t n = u32();
		if (n)
			skip_pad(8);
		need((size_t)n * 8);
		std::vector<double> v(n);
		for (uint32_t i = 0; i < n; ++i) {
			const uint64_t b = get_le(8);
			std::memcpy(&v[i], &b, 8);
		}
		return v;
	}

      private:
	void need(size_t n)
	{
		if (n > n_ - at_)
			throw std::runtime_error("state ends early (offset " +
						 std::to_string(at_) + ")");
	}
	void skip_pad(size_t a)
	{
		const size_t r = at_ % a;
		if (r) {
			need(a - r);
			at_ += a - r;
		}
	}
	uint64_t get_le(size_t n)
	{
		need(n);
		uint64_t v = 0;
		for (size_t k = 0; k < n; ++k)
			v |= (uint64_t)p_[at_ + k] << (8 * k);
		at_ += n;
		return v;
	}
	uint64_t uint_le(size_t n)
	{
		skip_pad(n);
		return get_le(n);
	}
	const uint8_t *p_;
	size_t n_;
	size_t at_ = 0;
};

} // namespace verbatim
} // namespace b3g
