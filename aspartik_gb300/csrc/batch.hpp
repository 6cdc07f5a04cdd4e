// batch.hpp -- many calculators evaluated by one graph-replayed launch
// (batch.cu).
#pragma once

#include "calculator.hpp"

#include <vector>

namespace b3g {

class Batch {
      public:
	Batch(Calculator *const *members, uint32_t count);
	~Batch();
	Batch(const Batch &) = delete;
	Batch &operator=(const Batch &) = delete;
	// replays the step for every member that staged a proposal
	void run();
	// waits; out[i] = member i's log-likelihood, NaN if it had nothing
	void log_likelihoods(double *out);
	float last_ms();

      private:
	void release();
	std::vector<Calculator *> members_;
	std::vector<uint32_t> order_; // members by cost, descending
	int device_ = -1;
	cudaStream_t stream_ = nullptr;
	cudaStream_t stream2_ = nullptr; // the graph's short-list branch
	cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
	cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
	MemberDesc *d_desc_ = nullptr;
	MemberStep *d_steps_ = nullptr, *h_steps_ = nullptr;
	double *d_lnl_ = nullptr, *h_lnl_ = nullptr;
	unsigned *d_work_ = nullptr;
	double *d_tile_sums_ = nullptr;
	unsigned *d_tickets_ = nullptr;
	cudaGraph_t graph_ = nullptr;
	cudaGraphExec_t exec_ = nullptr;
	BatchParams bp_{};
	uint32_t max_entries_ = 0, ctas_ = 0;
	// one contiguous staging block for every member (copied by one graph
	// node); each member's h_stage_ / d_stage_ point into it while it is
	// in the batch
	unsigned char *h_block_ = nullptr, *d_block_ = nullptr;
	size_t block_bytes_ = 0;
	bool direct_c_[5] = {}; // members with 1, 2 or 4 categories present
	bool ran_ = false;
	std::vector<uint8_t> evaluated_;
};

} // namespace b3g
