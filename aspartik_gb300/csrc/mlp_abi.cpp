// mlp_abi.cpp -- C ABI of the delayed-acceptance surrogate (include/b3g.h).
#include "calculator.hpp"
#include "mlp.hpp"

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
	}
}

b3g::Mlp *mlp_of(b3g_surrogate *s)
{
	if (!s)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null surrogate");
	return reinterpret_cast<b3g::Mlp *>(s);
}

void need(const void *p)
{
	if (!p)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null argument");
}

} // namespace

extern "C" {

B3G_API b3g_status b3g_surrogate_create(uint32_t inputs, uint32_t hidden,
					uint64_t seed, int32_t device,
					b3g_surrogate **out)
{
	return guarded([&] {
		need(out);
		*out = nullptr;
		if (inputs > hidden)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT,
					 "surrogate inputs must not exceed hidden");
		auto *m = new b3g::Mlp(inputs, hidden, seed, device);
		*out = reinterpret_cast<b3g_surrogate *>(m);
	});
}

B3G_API void b3g_surrogate_destroy(b3g_surrogate *s)
{
	delete reinterpret_cast<b3g::Mlp *>(s);
}

B3G_API uint32_t b3g_surrogate_num_params(const b3g_surrogate *s)
{
	return s ? reinterpret_cast<const b3g::Mlp *>(s)->num_params() : 0u;
}

B3G_API b3g_status b3g_surrogate_get_params(b3g_surrogate *s, float *out)
{
	return guarded([&] {
		need(out);
		mlp_of(s)->get_params(out);
	});
}

B3G_API b3g_status b3g_surrogate_set_params(b3g_surrogate *s, const float *in)
{
	return guarded([&] {
		need(in);
		mlp_of(s)->set_params(in);
	});
}

B3G_API b3g_status b3g_surrogate_forward(b3g_surrogate *s, const float *x,
					 uint32_t n, float *out)
{
	return guarded([&] {
		need(x);
		need(out);
		if (n < 1)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "n must be >= 1");
		mlp_of(s)->forward(x, n, out);
	});
}

B3G_API b3g_status b3g_surrogate_loss_grad(b3g_surrogate *s,
					   const float *x_new,
					   const float *x_old,
					   const float *delta, uint32_t n,
					   float *loss, float *grad)
{
	return guarded([&] {
		need(x_new);
		need(x_old);
		need(delta);
		need(loss);
		if (n < 1)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "n must be >= 1");
		*loss = mlp_of(s)->loss_grad(x_new, x_old, delta, n, grad);
	});
}

B3G_API b3g_status b3g_surrogate_train(b3g_surrogate *s, const float *x_new,
				       const float *x_old, const float *delta,
				       uint32_t n, uint32_t epochs,
				       uint32_t batch, float lr, uint64_t seed,
				       float *final_loss)
{
	return guarded([&] {
		need(x_new);
		need(x_old);
		need(delta);
		const float l = mlp_of(s)->train(x_new, x_old, delta, n, epochs,
						 batch, lr, seed);
		if (final_loss)
			*final_loss = l;
	});
}

B3G_API b3g_status b3g_surrogate_delta(b3g_surrogate *s, const float *x_new,
				       const float *x_old, float *out)
{
	return guarded([&] {
		need(x_new);
		need(x_old);
		need(out);
		*out = mlp_of(s)->delta(x_new, x_old);
	});
}

B3G_API b3g_status b3g_surrogate_deltas(b3g_surrogate *s, const float *x_new,
					const float *x_old, uint32_t n,
					float *out)
{
	return guarded([&] {
		need(x_new);
		need(x_old);
		need(out);
		if (n < 1 || n > b3g::Mlp::kDeltaMax)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT,
					 "1..256 pairs per call");
		mlp_of(s)->deltas(x_new, x_old, n, out);
	});
}

} // extern "C"
