// mcmc_abi.cpp -- C ABI of the native MCMC driver (include/b3g.h).
#include "host_math.hpp"
#include <cmath>
#include "mcmc.hpp"

#include <algorithm>
#include <cstring>
#include <new>

namespace b3g {
void set_last_error(const char *message);
}

namespace {

template <typename F> b3g_status guarded(F &&f)
{
	try {
		f();
		b3g::set_last_error("");
		return B3G_OK;
	} catch (const b3g::Error &e) {
		b3g::set_last_error(e.what());
		return e.status;
	} catch (const std::bad_alloc &) {
		b3g::set_last_error("host allocation failed");
		return B3G_ERR_OUT_OF_MEMORY;
	} catch (const std::exception &e) {
		b3g::set_last_error(e.what());
		return B3G_ERR_STATE;
	} catch (...) {
		b3g::set_last_error("unknown error");
		return B3G_ERR_STATE;
	}
}

b3g::Mcmc *mcmc_of(b3g_mcmc *m)
{
	if (!m)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null mcmc");
	return reinterpret_cast<b3g::Mcmc *>(m);
}

} // namespace

extern "C" {

namespace {

b3g::McmcConfig config_of(const b3g_mcmc_config *config)
{
	b3g::McmcConfig c{};
	c.num_chains = config->num_chains;
	c.num_categories = config->num_categories;
	c.precision = config->precision;
	c.model = config->model;
	c.seed = config->seed;
	c.heat = config->heat;
	c.swap_every = config->swap_every;
	c.sample_every = config->sample_every;
	c.tune_every = config->tune_every;
	c.device = config->device;
	std::memcpy(c.weights, config->op_weights, sizeof(c.weights));
	if (config->da_reserved != 0)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "da_reserved must be 0");
	if (config->da_pilot_steps &&
	    (config->da_hidden < 32 || config->da_hidden % 32 ||
	     config->da_hidden > 1024 || config->da_epochs < 1))
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT,
				 "delayed acceptance needs da_hidden a multiple "
				 "of 32 in 32..1024 and da_epochs >= 1");
	c.da_pilot_steps = config->da_pilot_steps;
	c.da_epochs = config->da_epochs;
	c.da_hidden = config->da_hidden;
	c.da_drift_limit = config->da_drift_limit;
	if (config->clock_categories > 64)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT,
				 "at most 64 relaxed-clock categories");
	c.clock_categories = config->clock_categories;
	if (config->launch > B3G_MCMC_LAUNCH_INDEPENDENT)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "unknown launch mode");
	c.launch = config->launch;
	if (config->host_threads > 256)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "at most 256 host threads");
	c.host_threads = config->host_threads;
	return c;
}

} // namespace

B3G_API b3g_status b3g_mcmc_create(const b3g_mcmc_config *config,
				   uint32_t num_leaves, uint32_t num_patterns,
				   const uint8_t *samples,
				   const uint32_t *weights,
				   const uint32_t *parents,
				   const double *heights, b3g_mcmc **out)
{
	return guarded([&] {
		if (!config || !samples || !weights || !parents || !heights || !out)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null argument");
		*out = nullptr;
		auto *m = new b3g::Mcmc(config_of(config), num_leaves, num_patterns,
					samples, weights, parents, heights);
		*out = reinterpret_cast<b3g_mcmc *>(m);
	});
}

B3G_API b3g_status b3g_mcmc_create_multi(const b3g_mcmc_config *config,
					 uint32_t num_problems,
					 const b3g_mcmc_problem *problems,
					 b3g_mcmc **out)
{
	return guarded([&] {
		if (!config || !problems || !out || num_problems < 1)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null argument");
		*out = nullptr;
		std::vector<b3g::Problem> ps(num_problems);
		for (uint32_t k = 0; k < num_problems; ++k)
			ps[k] = b3g::Problem{problems[k].num_leaves, problems[k].num_patterns,
					     problems[k].samples, problems[k].weights,
					     problems[k].parents, problems[k].heights};
		auto *m = new b3g::Mcmc(config_of(config), ps);
		*out = reinterpret_cast<b3g_mcmc *>(m);
	});
}

B3G_API b3g_status b3g_mcmc_launch_stats(b3g_mcmc *mcmc, uint32_t *batched,
					 double *device_ms, uint64_t *launches)
{
	return guarded([&] {
		if (!batched || !device_ms || !launches)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		const b3g::Mcmc *m = mcmc_of(mcmc);
		*batched = m->batched() ? 1u : 0u;
		*device_ms = m->batch_device_ms();
		*launches = m->batch_launches();
	});
}

B3G_API void b3g_mcmc_destroy(b3g_mcmc *mcmc)
{
	delete reinterpret_cast<b3g::Mcmc *>(mcmc);
}

B3G_API b3g_status b3g_mcmc_set_parameters(b3g_mcmc *mcmc, double kappa,
					   const double *rates,
					   const double *frequencies,
					   double alpha, double birth_rate)
{
	return guarded([&] {
		mcmc_of(mcmc)->set_parameters(kappa, rates, frequencies, alpha,
					      birth_rate);
	});
}

B3G_API b3g_status b3g_mcmc_set_clock(b3g_mcmc *mcmc, double sd,
				      const uint32_t *categories)
{
	return guarded([&] { mcmc_of(mcmc)->set_clock(sd, categories); });
}

B3G_API b3g_status b3g_lognormal_categories(double sd, uint32_t k, double *rates)
{
	return guarded([&] {
		if (!rates || k < 1 || !(sd > 0.0) || !std::isfinite(sd))
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT,
					 "need sd > 0, k >= 1 and an output");
		b3g::lognormal_categories(sd, (int)k, rates);
	});
}

B3G_API b3g_status b3g_mcmc_run(b3g_mcmc *mcmc, uint64_t steps)
{
	return guarded([&] { mcmc_of(mcmc)->run(steps); });
}

B3G_API b3g_status b3g_mcmc_samples(b3g_mcmc *mcmc, uint64_t *steps,
				    uint32_t *parents, double *heights,
				    double *parameters, uint64_t capacity,
				    uint64_t *count)
{
	return guarded([&] {
		if (!count)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null count");
		const b3g::Mcmc &m = *mcmc_of(mcmc);
		const uint64_t n = m.num_samples();
		*count = n;
		const uint64_t k = std::min(capacity, n);
		const uint64_t nodes = n ? m.sample_parents().size() / n : 0;
		if (steps)
			std::copy(m.sample_steps().begin(), m.sample_steps().begin() + k, steps);
		if (parents)
			std::copy(m.sample_parents().begin(),
				  m.sample_parents().begin() + k * nodes, parents);
		if (heights)
			std::copy(m.sample_heights().begin(),
				  m.sample_heights().begin() + k * nodes, heights);
		if (parameters)
			std::copy(m.sample_params().begin(),
				  m.sample_params().begin() + k * b3g::kSampleParams,
				  parameters);
	});
}

B3G_API b3g_status b3g_mcmc_trace(b3g_mcmc *mcmc, uint32_t field,
				  double *out, uint64_t capacity,
				  uint64_t *count)
{
	return guarded([&] {
		if (field > 7 || !count)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "bad trace field");
		const auto &t = mcmc_of(mcmc)->trace(field);
		*count = t.size();
		if (out)
			std::copy(t.begin(),
				  t.begin() + std::min<uint64_t>(capacity, t.size()),
				  out);
	});
}

B3G_API b3g_status b3g_mcmc_chain_trace(b3g_mcmc *mcmc, uint32_t chain,
					uint32_t field, double *out, uint64_t capacity,
					uint64_t *count)
{
	return guarded([&] {
		if (field > 7 || !count)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "bad trace field");
		const b3g::Mcmc &m = *mcmc_of(mcmc);
		if (chain >= m.num_chains())
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "no such chain");
		*count = 0;
		if ((size_t)chain * 8 + field >= m.chain_trace_size())
			return; // nothing recorded yet
		const auto &t = m.chain_trace(chain, field);
		*count = t.size();
		if (out)
			std::copy(t.begin(),
				  t.begin() + std::min<uint64_t>(capacity, t.size()),
				  out);
	});
}

B3G_API b3g_status b3g_mcmc_operator_stats(b3g_mcmc *mcmc, uint32_t op,
					   uint64_t *counts, double *tuning)
{
	return guarded([&] {
		if (op >= b3g::kOpCount || !counts || !tuning)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "bad operator");
		mcmc_of(mcmc)->op_stats(op, counts, tuning);
	});
}

B3G_API b3g_status b3g_mcmc_set_tuning(b3g_mcmc *mcmc, uint32_t op,
				       double tuning)
{
	return guarded([&] { mcmc_of(mcmc)->set_tuning(op, tuning); });
}

B3G_API b3g_status b3g_mcmc_swaps(b3g_mcmc *mcmc, uint64_t *tried,
				  uint64_t *accepted)
{
	return guarded([&] {
		if (!tried || !accepted)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*tried = mcmc_of(mcmc)->swaps_tried();
		*accepted = mcmc_of(mcmc)->swaps_accepted();
	});
}

B3G_API b3g_status b3g_mcmc_da_stats(b3g_mcmc *mcmc, uint64_t *counts,
				     double *values)
{
	return guarded([&] {
		if (!counts || !values)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		const b3g::DaStats &d = mcmc_of(mcmc)->da_stats();
		counts[0] = d.pilot_pairs;
		counts[1] = d.stage1_rejects;
		counts[2] = d.stage2_accepts;
		counts[3] = d.stage2_rejects;
		counts[4] = d.exact_evaluations;
		counts[5] = d.fallback;
		values[0] = d.train_loss;
		values[1] = d.drift_rms;
	});
}

B3G_API b3g_status b3g_mcmc_dump(b3g_mcmc *mcmc, uint8_t *out,
				 uint64_t capacity, uint64_t *size)
{
	return guarded([&] {
		if (!size)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null size");
		const std::vector<uint8_t> state = mcmc_of(mcmc)->dump();
		*size = state.size();
		if (!out)
			return;
		if (capacity < state.size())
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT,
					 "buffer smaller than the checkpoint");
		std::memcpy(out, state.data(), state.size());
	});
}

B3G_API b3g_status b3g_mcmc_load(b3g_mcmc *mcmc, const uint8_t *state,
				 uint64_t size)
{
	return guarded([&] { mcmc_of(mcmc)->load(state, (size_t)size); });
}

static_assert(sizeof(b3g_state_operator) == sizeof(b3g::VerbatimOp),
	      "b3g_state_operator mirrors VerbatimOp");
static_assert(B3G_STATE_TREE == b3g::kVpTree &&
		      B3G_STATE_BIRTH_RATE == b3g::kVpBirthRate &&
		      B3G_STATE_KAPPA == b3g::kVpKappa &&
		      B3G_STATE_ALPHA == b3g::kVpAlpha &&
		      B3G_STATE_RATES == b3g::kVpRates &&
		      B3G_STATE_FREQUENCIES == b3g::kVpFreqs &&
		      B3G_STATE_CLOCK_SD == b3g::kVpClockSd &&
		      B3G_STATE_CLOCK_CATEGORIES == b3g::kVpClockCategories,
	      "state parameter ids");

B3G_API b3g_status b3g_mcmc_dump_verbatim(b3g_mcmc *mcmc, uint32_t chain,
					  const uint32_t *params,
					  uint32_t num_params,
					  const b3g_state_operator *ops,
					  uint32_t num_ops, uint8_t *out,
					  uint64_t capacity, uint64_t *size)
{
	return guarded([&] {
		if (!size)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null size");
		const std::vector<uint8_t> state = mcmc_of(mcmc)->dump_verbatim(
			chain, params, num_params,
			reinterpret_cast<const b3g::VerbatimOp *>(ops), num_ops);
		*size = state.size();
		if (!out)
			return;
		if (capacity < state.size())
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT,
					 "buffer smaller than the state");
		std::memcpy(out, state.data(), state.size());
	});
}

B3G_API b3g_status b3g_mcmc_load_verbatim(b3g_mcmc *mcmc, uint32_t chain,
					  const uint32_t *params,
					  uint32_t num_params,
					  const b3g_state_operator *ops,
					  uint32_t num_ops, const uint8_t *state,
					  uint64_t size)
{
	return guarded([&] {
		mcmc_of(mcmc)->load_verbatim(
			chain, params, num_params,
			reinterpret_cast<const b3g::VerbatimOp *>(ops), num_ops, state,
			(size_t)size);
	});
}

B3G_API b3g_status b3g_mcmc_check(b3g_mcmc *mcmc, double *max_rel_diff)
{
	return guarded([&] {
		if (!max_rel_diff)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*max_rel_diff = mcmc_of(mcmc)->check_full_recompute();
	});
}

B3G_API b3g_status b3g_mcmc_chain_state(b3g_mcmc *mcmc, uint32_t chain,
					uint32_t *parents, double *heights,
					double *lnl, double *beta)
{
	return guarded([&] {
		b3g::Mcmc *m = mcmc_of(mcmc);
		if (chain >= m->num_chains() || !parents || !heights || !lnl || !beta)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "bad chain or output");
		m->chain_state(chain, parents, heights, lnl, beta);
	});
}

} // extern "C"
