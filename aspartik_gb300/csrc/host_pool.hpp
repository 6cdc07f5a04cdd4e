// host_pool.hpp -- a fixed set of host threads that run one job per call,
// the calling thread taking part.  The MCMC driver spreads a step's chains
// over them: every thread proposes and launches its own chains' evaluations,
// then reads their results, so the host work of several chains overlaps
// instead of queueing behind one thread.
#pragma once

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace b3g {

class HostPool {
      public:
	// threads - 1 workers (threads >= 1); each runs `init` once before the
	// constructor returns (an exception from it ends the pool and is
	// rethrown here)
	HostPool(uint32_t threads, const std::function<void()> &init)
	    : size_(threads < 1 ? 1 : threads), errors_(size_)
	{
		pending_.store(size_ - 1, std::memory_order_relaxed);
		for (uint32_t w = 1; w < size_; ++w)
			threads_.emplace_back([this, w, init] {
				if (init) {
					try {
						init();
					} catch (...) {
						errors_[w] = std::current_exception();
					}
				}
				pending_.fetch_sub(1, std::memory_order_acq_rel);
				work(w);
			});
		while (pending_.load(std::memory_order_acquire) != 0)
			std::this_thread::yield();
		for (auto &e : errors_)
			if (e) {
				shutdown();
				std::rethrow_exception(e);
			}
	}
	~HostPool() { shutdown(); }
	HostPool(const HostPool &) = delete;
	HostPool &operator=(const HostPool &) = delete;

	uint32_t size() const { return size_; }

	// job(w) for every w in [0, size()), w = 0 on the calling thread;
	// returns when every thread is done and rethrows the exception of the
	// lowest w that threw
	void run(const std::function<void(uint32_t)> &job)
	{
		for (auto &e : errors_)
			e = nullptr;
		if (size_ > 1) {
			job_ = &job;
			pending_.store(size_ - 1, std::memory_order_relaxed);
			{
				std::lock_guard<std::mutex> l(m_);
				gen_.fetch_add(1, std::memory_order_release);
			}
			cv_.notify_all();
		}
		try {
			job(0);
		} catch (...) {
			errors_[0] = std::current_exception();
		}
		// the workers end within the step: wait by spinning
		while (size_ > 1 && pending_.load(std::memory_order_acquire) != 0) {
		}
		for (auto &e : errors_)
			if (e)
				std::rethrow_exception(e);
	}

      private:
	void shutdown()
	{
		{
			std::lock_guard<std::mutex> l(m_);
			stop_.store(true, std::memory_order_release);
		}
		cv_.notify_all();
		for (auto &t : threads_)
			if (t.joinable())
				t.join();
	}

	// A worker spins on the job counter for up to a millisecond after each
	// job (the next step follows within tens of microseconds, and a wake-up
	// from sleep costs about as much as a step), then sleeps.
	void work(uint32_t w)
	{
		using clock = std::chrono::steady_clock;
		constexpr auto kSpin = std::chrono::microseconds(1000);
		uint64_t seen = 0;
		for (;;) {
			uint64_t g = gen_.load(std::memory_order_acquire);
			const auto t0 = clock::now();
			for (uint32_t k = 1; g == seen; ++k) {
				if (stop_.load(std::memory_order_acquire))
					return;
				if ((k & 1023u) == 0 && clock::now() - t0 > kSpin)
					break;
				g = gen_.load(std::memory_order_acquire);
			}
			if (g == seen) {
				std::unique_lock<std::mutex> l(m_);
				cv_.wait(l, [&] {
					return stop_.load(std::memory_order_acquire) ||
					       gen_.load(std::memory_order_acquire) != seen;
				});
				if (stop_.load(std::memory_order_acquire))
					return;
				g = gen_.load(std::memory_order_acquire);
			}
			seen = g;
			try {
				(*job_)(w);
			} catch (...) {
				errors_[w] = std::current_exception();
			}
			pending_.fetch_sub(1, std::memory_order_acq_rel);
		}
	}

	uint32_t size_;
	std::vector<std::thread> threads_;
	const std::function<void(uint32_t)> *job_ = nullptr;
	std::atomic<uint64_t> gen_{0};
	std::atomic<uint32_t> pending_{0};
	std::atomic<bool> stop_{false};
	std::mutex m_;
	std::condition_variable cv_;
	std::vector<std::exception_ptr> errors_;
};

} // namespace b3g
