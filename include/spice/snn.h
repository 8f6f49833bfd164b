// spice/snn.h -- the reference's C++20 user API (spice/include/spice/snn.h:16-75) on the GB300
// engine.  A program written against spice2's snn for the sample models compiles against this
// header unchanged in its calls: snn(dt, max_delay, {seed}), add_population<Model>(size, model),
// connect<Synapse>(from, to, fixed_probability(p) | adj_list, delay, {params}), step(), and the
// population handle's spikes(age) / get_neurons().  Everything runs on the GPU through the C ABI of
// spice_gb300.h; violated preconditions throw std::logic_error with the reference's message
// (spice/src/util/assert.cpp:8-15).
//
// The models of the reference's samples are built into the engine: poisson (samples/brunel.cpp:
// 23-31), lif (brunel.cpp:39-62), lif_cond (samples/vogels.cpp:10-46), external_input
// (samples/external_input.cpp:17-30); synapses fixed_weight (brunel.cpp:67-70), excitatory /
// inhibitory (vogels.cpp:48-60).  Any other model type is a user model (the reference's Neuron
// concepts, concepts.h:10-58): compiled with nvcc, this header instantiates GPU kernels over it --
// a stateful model's `SPICE_HD bool update(neuron&, float dt, auto& rng) const` (no random stream:
// draws return 0), a stateless model's `SPICE_HD bool update(float dt, auto& rng) const` drawing once
// per neuron and step from the reference's stream -- and the engine launches them each window.
// Synapses into a user neuron add their `weight` to the float member named by their
// `static constexpr auto field`.
#pragma once

#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "spice_gb300.h"

#if defined(__CUDACC__)
#include <cuda_runtime.h>
// Marks a user model's update() / deliver() for the GPU.
#define SPICE_HD __host__ __device__
#else
#define SPICE_HD
#endif

namespace spice {

namespace detail {
inline void check(int rc) {
	if (rc == SPICE_OK) return;
	std::string const msg = spice_last_error();
	if (rc == SPICE_EINVAL) throw std::logic_error(msg);
	throw std::runtime_error(msg);
}
}  // namespace detail

namespace util {
// util::seed_seq{seeds...} (spice/include/spice/util/random.h:149-152): the list of 32-bit seeds.
struct seed_seq {
	std::vector<uint32_t> seeds;
	seed_seq(std::initializer_list<uint32_t> il) : seeds(il) {}
};

// generate_canonical<Real, LeftOpen>(rng) (random.h:236-247) for user models: float from the top
// 24 bits, double from the top 53 bits (left-open: ((u >> 11) + 1) / 2^53).
template <class Real, bool LeftOpen = false, class Rng>
SPICE_HD Real generate_canonical(Rng& rng) {
	uint64_t const u = rng();
	if constexpr (std::is_same_v<Real, float>)
		return (float)(u >> 40) * (1.0f / 16777216.0f);
	else
		return LeftOpen ? (double)((u >> 11) + 1) * (1.0 / 9007199254740992.0)
		                : (double)(u >> 11) * (1.0 / 9007199254740992.0);
}
}  // namespace util

// ---- models ----
struct poisson {
	float rate = 20;  // Hz
	static constexpr int model = SPICE_NEURON_POISSON;
	std::vector<float> params() const { return {rate}; }
};
struct lif {
	struct neuron {
		float V    = 0;
		int32_t Twait = 0;
	};
	float Vthres = 0.02f, TmemInv = 50.f;
	int32_t Tref = 20;
	static constexpr int model = SPICE_NEURON_LIF;
	std::vector<float> params() const { return {Vthres, float(Tref), TmemInv}; }
};
struct lif_cond {
	struct neuron {
		float V = -0.06f, Gex = 0, Gin = 0;
		int32_t Twait = 0;
	};
	static constexpr int model = SPICE_NEURON_LIF_COND;
	std::vector<float> params() const { return {}; }
};
struct external_input {
	std::vector<std::vector<int32_t>> trains;
	static constexpr int model = SPICE_NEURON_EXTERNAL;
	std::vector<float> params() const { return {}; }
};
struct fixed_weight {
	float weight;
	std::vector<float> params() const { return {weight, float(SPICE_FIELD_V)}; }
};
struct excitatory {
	float weight;
	std::vector<float> params() const { return {weight, float(SPICE_FIELD_GEX)}; }
};
struct inhibitory {
	float weight;
	std::vector<float> params() const { return {weight, float(SPICE_FIELD_GIN)}; }
};

// ---- topologies (spice/include/spice/topology.h:37-58) ----
class fixed_probability {
public:
	explicit fixed_probability(double p) : _p(p) {}
	double p() const { return _p; }

private:
	double _p;
};

class adj_list {
public:
	void connect(int64_t src, int64_t dst) {
		_pairs.push_back((int32_t)src);
		_pairs.push_back((int32_t)dst);
	}
	int64_t size() const { return (int64_t)_pairs.size() / 2; }
	std::vector<int32_t> const& pairs() const { return _pairs; }

private:
	std::vector<int32_t> _pairs;
};

namespace detail {
template <class T>
inline constexpr bool is_builtin_model = std::is_same_v<T, poisson> || std::is_same_v<T, lif> ||
                                         std::is_same_v<T, lif_cond> || std::is_same_v<T, external_input>;
template <class T, class = void>
struct has_neuron : std::false_type {};
template <class T>
struct has_neuron<T, std::void_t<typename T::neuron>> : std::true_type {};
template <class T, class = void>
struct has_field : std::false_type {};
template <class T>
struct has_field<T, std::void_t<decltype(T::field)>> : std::true_type {};
template <class>
inline constexpr bool always_false = false;

#if defined(__CUDACC__)
// xoroshiro128+ (random.h:222-234) positioned in the step's stream.
struct device_rng {
	uint64_t s0, s1;
	__device__ uint64_t operator()() {
		uint64_t const r = s0 + s1;
		uint64_t const t = s0 ^ s1;
		s0 = ((s0 << 24) | (s0 >> 40)) ^ t ^ (t << 16);
		s1 = (t << 37) | (t >> 27);
		return r;
	}
};
// Stateful user models get no random stream (the reference's sequential stream has no parallel
// position for a model that draws a data-dependent number of times); draws return 0.
struct no_rng {
	__device__ uint64_t operator()() const { return 0; }
};

// One window of a stateful user population: per neuron, per step, the inputs of the step's slot
// (the engine's per-group counts replayed as sequential float adds into the group's field, or the
// atomic-mode field sums), then the user's update(); spikes to the bitmap and the step's list.
template <class Neur>
__global__ void __launch_bounds__(256) user_update_kernel(const spice_user_window w, const Neur neur) {
	using N            = typename Neur::neuron;
	int64_t const i    = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	bool const valid   = i < w.size;
	int const lane     = threadIdx.x & 31;
	N* const st        = static_cast<N*>(w.state);
	N n{};
	if (valid) n = st[i];
	auto field = [&](int f) -> float& {
		return *reinterpret_cast<float*>(reinterpret_cast<char*>(&n) + w.field_offset[f]);
	};
	auto apply = [&](int64_t slot) {
		if (w.mode == SPICE_MODE_DETERMINISTIC) {
			uint32_t* const wp = w.cnt + (slot * w.size + i) * w.W;
			uint32_t x[4] = {0, 0, 0, 0};
			for (int j = 0; j < w.W && j < 4; j++) x[j] = wp[j];
			for (int g = 0; g < w.ngroups; g++) {
				uint32_t const word = x[w.group_word[g]];
				uint32_t c          = w.group_bits[g] == 32 ? word : (word >> w.group_shift[g]) & 0xffffu;
				float& f            = field(w.group_field[g]);
				float v             = f;
				for (; c; c--) v = __fadd_rn(v, w.group_weight[g]);
				f = v;
			}
			if (w.zero_inputs)
				for (int j = 0; j < w.W && j < 4; j++)
					if (x[j]) wp[j] = 0;
		} else {
			float* const ap = w.acc + (slot * w.size + i) * w.F;
			for (int f = 0; f < 3; f++) {
				int const sl = w.field_slot[f];
				if (sl < 0) continue;
				float const x = ap[sl];
				if (x != 0.0f) {
					field(f) = __fadd_rn(field(f), x);
					if (w.zero_inputs) ap[sl] = 0.0f;
				}
			}
		}
	};
	if (w.apply_only) {
		if (valid) {
			apply(w.slot0);
			st[i] = n;
		}
		return;
	}
	int slot = w.slot0, hslot = w.hslot0;
	no_rng rng;
	for (int k = 0; k < w.K; k++) {
		bool spike = false;
		if (valid) {
			apply(slot);
			spike = neur.update(n, w.dts[k], rng);
		}
		unsigned const mask = __ballot_sync(0xffffffffu, spike);
		int64_t const word  = i >> 5;
		if (lane == 0 && word < w.nwords) w.bits[(int64_t)hslot * w.nwords + word] = mask;
		if (mask) {
			int base = 0;
			if (lane == 0) base = atomicAdd(w.counts + k * w.npop + w.pop, __popc(mask));
			base = __shfl_sync(0xffffffffu, base, 0);
			if (spike)
				w.list[(int64_t)(w.list_k0 + k) * w.size + base + __popc(mask & ((1u << lane) - 1u))] = (int32_t)i;
		}
		slot  = slot + 1 == (int)w.D ? 0 : slot + 1;
		hslot = hslot + 1 == w.Hb ? 0 : hslot + 1;
	}
	if (valid) st[i] = n;
}

// One step (blockIdx.y) of a stateless user population: thread c owns neurons [32c, 32c + 32),
// jumps to stream position draw_offset + 32c with the step's jump table (XOR of 16 table entries
// picked by the bytes of x^(draw_offset + 32c) mod P), and calls update(dt, rng) per neuron.
template <class Neur>
__global__ void __launch_bounds__(256) user_source_kernel(const spice_user_window w, const Neur neur) {
	int const k       = blockIdx.y;
	int64_t const c   = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	int const lane    = threadIdx.x & 31;
	int const hslot   = (w.hslot0 + k) % w.Hb;
	unsigned mask     = 0;
	if (c < w.nwords) {
		const uint64_t* tab  = static_cast<const uint64_t*>(w.tables) + (int64_t)k * 16 * 256 * 2;
		const uint64_t* poly = static_cast<const uint64_t*>(w.chunk_poly) + 2 * c;
		uint64_t const plo = poly[0], phi = poly[1];
		device_rng rng{0, 0};
		for (int g = 0; g < 16; g++) {
			uint64_t const byte = ((g < 8 ? plo : phi) >> (8 * (g & 7))) & 255;
			rng.s0 ^= tab[2 * (g * 256 + byte)];
			rng.s1 ^= tab[2 * (g * 256 + byte) + 1];
		}
		int const nn = (int)(w.size - 32 * c < 32 ? w.size - 32 * c : 32);
		float const dt = w.dts[k];
		for (int r = 0; r < nn; r++) mask |= (unsigned)(neur.update(dt, rng) ? 1 : 0) << r;
		w.bits[(int64_t)hslot * w.nwords + c] = mask;
	}
	// unordered list: one reservation per warp
	int const cnt = __popc(mask);
	int incl      = cnt;
	for (int d = 1; d < 32; d <<= 1) {
		int const o = __shfl_up_sync(0xffffffffu, incl, d);
		if (lane >= d) incl += o;
	}
	int const total = __shfl_sync(0xffffffffu, incl, 31);
	int base        = 0;
	if (lane == 31 && total) base = atomicAdd(w.counts + k * w.npop + w.pop, total);
	base         = __shfl_sync(0xffffffffu, base, 31);
	int32_t* out = w.list + (int64_t)(w.list_k0 + k) * w.size + base + (incl - cnt);
	for (unsigned m = mask; m; m &= m - 1) *out++ = (int32_t)(32 * c + (__ffs(m) - 1));
}

template <class Neur>
int user_launch(const spice_user_window* w, void* stream, void* ctx) {
	Neur const& neur  = *static_cast<const Neur*>(ctx);
	cudaStream_t const st = static_cast<cudaStream_t>(stream);
	if constexpr (has_neuron<Neur>::value) {
		unsigned const blocks = (unsigned)((w->size + 255) / 256);
		user_update_kernel<Neur><<<blocks, 256, 0, st>>>(*w, neur);
	} else {
		dim3 const grid((unsigned)((w->nwords + 255) / 256), (unsigned)w->K);
		if (w->K > 0) user_source_kernel<Neur><<<grid, 256, 0, st>>>(*w, neur);
	}
	return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
#endif
}  // namespace detail

class snn;

// The handle add_population returns (the neuron_population<Neur>* of snn.h:21-27).
template <class Neur>
class neuron_population {
public:
	int64_t size() const {
		int64_t n = 0;
		detail::check(spice_pop_size(_net, _id, &n));
		return n;
	}
	// NeuronPopulation::spikes(age) (neuron_population.h:147-153): ascending indices.
	std::vector<int32_t> spikes(int64_t age) const {
		int64_t n = 0;
		detail::check(spice_spike_count(_net, _id, age, &n));
		std::vector<int32_t> out((size_t)n);
		detail::check(spice_spikes(_net, _id, age, out.data(), n, &n));
		return out;
	}
	// neuron_population::get_neurons() (neuron_population.h:139-145), copied from the device.
	// Only for models with per-neuron state (lif, lif_cond).
	template <class M = Neur>
	std::vector<typename M::neuron> get_neurons() const {
		std::vector<typename M::neuron> out((size_t)size());
		if constexpr (!detail::is_builtin_model<M>) {
			detail::check(spice_get_user_state(_net, _id, out.data()));
		} else {
			int64_t const n = (int64_t)out.size();
			std::vector<float> V(n), Gex(n), Gin(n);
			std::vector<int32_t> T(n);
			detail::check(spice_get_state(_net, _id, SPICE_FIELD_V, V.data()));
			detail::check(spice_get_state(_net, _id, SPICE_FIELD_TREF, T.data()));
			if constexpr (M::model == SPICE_NEURON_LIF_COND) {
				detail::check(spice_get_state(_net, _id, SPICE_FIELD_GEX, Gex.data()));
				detail::check(spice_get_state(_net, _id, SPICE_FIELD_GIN, Gin.data()));
				for (int64_t i = 0; i < n; i++) out[i] = {V[i], Gex[i], Gin[i], T[i]};
			} else {
				for (int64_t i = 0; i < n; i++) out[i] = {V[i], T[i]};
			}
		}
		return out;
	}
	int id() const { return _id; }

private:
	friend class snn;
	neuron_population(spice_net* net, int id) : _net(net), _id(id) {}
	spice_net* _net;
	int _id;
};

// snn (spice/include/spice/snn.h:16-75).
class snn {
public:
	snn(float dt, float max_delay, util::seed_seq seed) {
		detail::check(spice_net_create(dt, max_delay, seed.seeds.data(), (int)seed.seeds.size(), &_net));
	}
	~snn() { spice_net_destroy(_net); }
	snn(snn const&)            = delete;
	snn& operator=(snn const&) = delete;

	template <class Neur>
	neuron_population<Neur>* add_population(int64_t size, Neur neur = {}) {
		if constexpr (!detail::is_builtin_model<Neur>) {
#if defined(__CUDACC__)
			static_assert(std::is_trivially_copyable_v<Neur>, "a user model must be trivially copyable");
			auto model = std::make_shared<Neur>(neur);
			int id     = -1;
			if constexpr (detail::has_neuron<Neur>::value) {
				using N = typename Neur::neuron;
				static_assert(std::is_trivially_copyable_v<N> && sizeof(N) % 4 == 0,
				              "a user neuron must be a trivially copyable struct of 4-byte members");
				N const init{};
				detail::check(spice_add_user_population(_net, size, 1, (int)sizeof(N), &init, &detail::user_launch<Neur>,
				                                        model.get(), &id));
			} else {
				detail::check(spice_add_user_population(_net, size, 0, 0, nullptr, &detail::user_launch<Neur>, model.get(), &id));
			}
			_models.push_back(model);
			_pops.emplace_back(new neuron_population<Neur>(_net, id));
			return static_cast<neuron_population<Neur>*>(_pops.back().get());
#else
			static_assert(detail::always_false<Neur>,
			              "user-defined models run as GPU kernels: compile this translation unit with nvcc");
			return nullptr;
#endif
		} else {
			auto const prm = neur.params();
			int id         = -1;
			detail::check(spice_add_population(_net, Neur::model, size, prm.data(), (int)prm.size(), &id));
			if constexpr (Neur::model == SPICE_NEURON_EXTERNAL) {
				std::vector<int32_t> counts, idx;
				for (auto const& t : neur.trains) {
					counts.push_back((int32_t)t.size());
					idx.insert(idx.end(), t.begin(), t.end());
				}
				detail::check(spice_set_external_input(_net, id, (int)counts.size(), counts.data(), idx.data()));
			}
			_pops.emplace_back(new neuron_population<Neur>(_net, id));
			return static_cast<neuron_population<Neur>*>(_pops.back().get());
		}
	}

	template <class Syn, class SrcNeur, class DstNeur>
	void connect(neuron_population<SrcNeur>* source, neuron_population<DstNeur>* target,
	             fixed_probability const& c, float delay, Syn syn = {}) {
		auto const prm = params_of(syn, target);
		int id         = -1;
		detail::check(spice_connect_fixed_probability(_net, source->id(), target->id(), c.p(), delay,
		                                              SPICE_SYNAPSE_FIXED_WEIGHT, prm.data(), (int)prm.size(), &id));
	}

	template <class Syn, class SrcNeur, class DstNeur>
	void connect(neuron_population<SrcNeur>* source, neuron_population<DstNeur>* target, adj_list const& c,
	             float delay, Syn syn = {}) {
		auto const prm = params_of(syn, target);
		int id         = -1;
		detail::check(spice_connect_adj_list(_net, source->id(), target->id(), c.pairs().data(), c.size(), delay,
		                                     SPICE_SYNAPSE_FIXED_WEIGHT, prm.data(), (int)prm.size(), &id));
	}

	void step() { detail::check(spice_step(_net)); }  // snn.cpp:7-28
	void run(int64_t steps) { detail::check(spice_run(_net, steps)); }
	void set_mode(int mode) { detail::check(spice_set_mode(_net, mode)); }
	spice_net* handle() { return _net; }

private:
	// Synapse parameters {weight, field}.  Into a user neuron, a synapse adds its `weight` to the
	// float member it names with `static constexpr auto field = &Model::neuron::member;` (the
	// member its deliver() adds to); the member is registered as a target field of the population.
	template <class Syn, class DstNeur>
	std::vector<float> params_of(Syn const& syn, neuron_population<DstNeur>* target) {
		if constexpr (detail::is_builtin_model<DstNeur>) {
			return syn.params();
		} else {
			static_assert(detail::has_field<Syn>::value,
			              "a synapse into a user neuron declares `static constexpr auto field = &Model::neuron::member;`");
			typename DstNeur::neuron probe{};
			int const off = (int)(reinterpret_cast<char const*>(&(probe.*Syn::field)) - reinterpret_cast<char const*>(&probe));
			int fi        = -1;
			detail::check(spice_user_field(_net, target->id(), off, &fi));
			return {syn.weight, float(fi)};
		}
	}

	spice_net* _net = nullptr;
	std::vector<std::shared_ptr<void>> _pops;    // owns the population handles (snn.h:72-74)
	std::vector<std::shared_ptr<void>> _models;  // user models, read by their update kernels' launches
};

}  // namespace spice
