// hetero.hpp -- per-pattern class mixture over several calculators
// (hetero.cu).
//
// Restates HeteroLikelihood (crates/b3/src/likelihood/hetero.rs:97-168): K
// classes, each a calculator over all patterns with its own substitution
// model and clock; pattern p belongs to class c(p) and the likelihood is
// sum_p w_p lnL_{c(p)}(p).  When only the assignment changes the sum is
// taken again over the classes' accepted per-pattern values, with no
// pruning (hetero.rs:117-120, 150-160).
//
// Here the accepted per-pattern values of every class stay on the device
// (one copy per class, refreshed on accept from the class calculator's
// per-pattern output), the assignment is double-buffered on the device, and
// the sum is one deterministic kernel on the mixture's own stream, ordered
// after the members' streams by events (no host synchronisation).
#pragma once

#include "calculator.hpp"

#include <vector>

namespace b3g {

constexpr uint32_t kHeteroMaxClasses = 16;

struct HeteroParams {
	const double *site[kHeteroMaxClasses]; // per class: [ldp] lnL per pattern
	const uint32_t *classes;               // [ldp] class of each pattern
	const uint32_t *weights;               // [ldp]
	double *block_sums;
	unsigned *ticket;
	double *lnl_out;
	uint32_t num_patterns;
	uint32_t num_classes;
};

cudaError_t launch_hetero_sum(const HeteroParams &p, cudaStream_t s);

class Hetero {
      public:
	Hetero(Calculator *const *members, uint32_t count);
	~Hetero();
	Hetero(const Hetero &) = delete;
	Hetero &operator=(const Hetero &) = delete;

	// propose a class for every pattern (values < count)
	void set_classes(const uint32_t *classes);
	// members evaluated since their last accept/reject contribute their
	// new per-pattern values, the others their accepted ones
	double log_likelihood();
	void accept();
	void reject();

      private:
	void release();
	std::vector<Calculator *> members_;
	uint32_t P_ = 0, ldp_ = 0;
	int device_ = -1;
	cudaStream_t stream_ = nullptr;
	cudaEvent_t ev_member_ = nullptr;
	double *d_accepted_ = nullptr; // [K][ldp]
	uint32_t *d_classes_ = nullptr; // [2][ldp]: accepted, proposed
	uint32_t *h_classes_ = nullptr; // pinned staging [ldp]
	double *d_block_sums_ = nullptr;
	unsigned *d_ticket_ = nullptr;
	double *d_lnl_ = nullptr, *h_lnl_ = nullptr;
	bool classes_proposed_ = false;
};

} // namespace b3g
