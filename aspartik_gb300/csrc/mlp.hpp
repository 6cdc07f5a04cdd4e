// mlp.hpp -- the delayed-acceptance surrogate: a small fully connected
// network (input -> H -> H -> H -> 1, GELU) trained and evaluated on the
// GPU by the kernels of mlp.cu.
//
// It models the log-likelihood as a function of the neighbourhood a tree
// move touches; stage one of delayed-acceptance Metropolis-Hastings uses the
// difference f(x_new) - f(x_old).  Training minimises
//     mean_n (f(x_new,n) - f(x_old,n) - dlnL_n)^2
// over pairs the chain itself produced, with Adam.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace b3g {

class Mlp {
      public:
	static constexpr uint32_t kLayers = 4; // 3 hidden + output

	Mlp(uint32_t in_dim, uint32_t hidden, uint64_t seed, int device);
	~Mlp();
	Mlp(const Mlp &) = delete;
	Mlp &operator=(const Mlp &) = delete;

	uint32_t num_params() const { return n_params_; }
	uint32_t in_dim() const { return in_; }
	void get_params(float *out);
	void set_params(const float *in);

	// f(x) for n rows of host inputs [n][in]
	void forward(const float *x, uint32_t n, float *out);
	// loss and gradient (flat, parameter order) of the pair objective
	float loss_grad(const float *x_new, const float *x_old,
			const float *delta, uint32_t n, float *grad);
	// Adam over `epochs` passes of shuffled minibatches; returns the last
	// epoch's mean loss
	float train(const float *x_new, const float *x_old, const float *delta,
		    uint32_t n, uint32_t epochs, uint32_t batch, float lr,
		    uint64_t seed);
	// pairs evaluated by one launch at most
	static constexpr uint32_t kDeltaMax = 256;
	// f(x_new) - f(x_old) for one pair (one fused cluster launch)
	float delta(const float *x_new, const float *x_old);
	// the same for `count` pairs, x_new and x_old [count][in], in one
	// launch (a cluster per pair)
	void deltas(const float *x_new, const float *x_old, uint32_t count, float *out);
	// Inference contexts: context 0 is the network's own stream and mapped
	// staging; contexts 1..n-1 have their own highest-priority stream and
	// staging, so that host threads screen concurrently (their launches go
	// ahead of queued evaluation blocks).
	void ensure_contexts(uint32_t n);
	void deltas(uint32_t ctx, const float *x_new, const float *x_old, uint32_t count,
		    float *out);

      private:
	void ensure_batch(uint32_t rows);
	void forward_device(uint32_t rows);   // d_x_ rows -> d_y_
	void backward_device(uint32_t rows);  // d_dy_ -> d_grad_
	uint32_t in_, hidden_;
	uint32_t dims_[kLayers + 1];
	uint32_t w_off_[kLayers], b_off_[kLayers];
	uint32_t n_params_ = 0;
	int device_ = -1;
	cudaStream_t stream_ = nullptr;
	float *d_params_ = nullptr, *d_grad_ = nullptr, *d_m_ = nullptr,
	      *d_v_ = nullptr;
	uint32_t adam_t_ = 0;
	// activations for up to cap_ rows: z (pre) and a (post) per layer
	uint32_t cap_ = 0;
	float *d_x_ = nullptr;
	float *d_z_[kLayers] = {};
	float *d_a_[kLayers] = {};
	float *d_da_[kLayers] = {};
	float *d_y_ = nullptr, *d_dy_ = nullptr, *d_delta_ = nullptr,
	      *d_loss_ = nullptr;
	float *d_pair_ = nullptr, *h_pair_ = nullptr; // inference staging
	struct InferCtx {
		cudaStream_t stream;
		float *h, *d;
	};
	std::vector<InferCtx> extra_; // contexts 1.. (context 0: the above)
};

} // namespace b3g
