// spice/snn.h -- the reference's C++20 user API (spice/include/spice/snn.h:16-75) on the GB300
// engine.  A program written against spice2's snn compiles against this header unchanged in its
// calls: snn(dt, max_delay, {seed}), add_population<Model>(size, model), connect<Synapse>(from, to,
// fixed_probability(p) | adj_list, delay, {params}), step(), and the population handle's
// spikes(age) / get_neurons().  Everything runs on the GPU through the C ABI of spice_gb300.h;
// violated preconditions throw std::logic_error with the reference's message
// (spice/src/util/assert.cpp:8-15).
//
// Models.  The reference ships no models: its samples define them.  spice::models holds the
// samples' models built into the engine -- poisson (samples/brunel.cpp:23-31), lif (brunel.cpp:
// 39-62), lif_cond (samples/vogels.cpp:10-46), external_input (samples/external_input.cpp:17-30);
// synapses fixed_weight (brunel.cpp:67-70), excitatory / inhibitory (vogels.cpp:48-60) and weighted
// (a per-synapse weight drawn at construction) -- computed the way the reference's -ffast-math
// build computes them, so their results are bit-exact.  Any other type is a user model (the
// reference's concepts, concepts.h:10-104), compiled with nvcc into GPU kernels by this header:
//   neurons  stateless `SPICE_HD bool update(float dt, auto& rng) const` (one draw per neuron and
//            step from the step's stream, the reference's order); stateful `SPICE_HD bool
//            update(neuron&, float dt, auto& rng) const` with a nested trivially copyable `neuron`
//            struct (the members synapses add to are 4-byte floats).  A stateful model that
//            declares `static constexpr int draws_per_update = n`
//            draws n numbers per neuron and step from the step's stream in the reference's order
//            (populations in add order, neurons ascending); without it its draws come from an
//            independent stream per (population, neuron, step) (statistically uniform, not the
//            reference's sequence).  init(neuron&, Int id, rng) / init(span<neuron>, rng) run on
//            the host at add_population with the population's own stream (neuron_population.h:
//            56-67), exactly as the reference runs them.
//   synapses stateless `SPICE_HD void deliver(Dst::neuron&) const` or stateful (a nested `synapse`
//            struct) `SPICE_HD void deliver(synapse const&, Dst::neuron&) const` that add a
//            constant, or a float member of the synapse, to one float member of the target neuron
//            -- found by calling deliver() on probe values at connect time (a synapse may also name
//            the member with `static constexpr auto field = &Dst::neuron::member` and carry it in
//            `weight`).  A stateful synapse with init(synapse&, Int src, Int dst, rng) runs it on
//            the host over the CSR in order with the connection's PerSynapseInit stream
//            (synapse_population.h:30-41); its weights are then delivered by the engine's pull path
//            (bit-exact order).  A plastic synapse (update(synapse&, dt, pre, post) and
//            skip(synapse&, dt, Int n), concepts.h:86-92) runs the reference's lazy catch-up
//            (synapse_population.h:88-139) in kernels instantiated here over its type; its deliver()
//            adds one float member of the synapse to the target (connecting one switches the net to
//            atomic mode: per-step sums of per-synapse weights depend on the order).  Any other
//            deliver() -- setting a flag, taking a minimum, or reading the source neuron
//            (DeliverFromTo, concepts.h:70-79) -- runs as user code into a user-defined target at the
//            end of each step (windows of one step), connection by connection in connect order, each
//            target's synapses in ascending source order; a deliver() that reads neurons of its own
//            target population runs in the reference's exact source-by-source order on one thread.
// Arithmetic: user models compile under nvcc (-fmad=false recommended), not under the reference's
// GCC -ffast-math, so a user model reproduces the reference bit for bit only where both compilers
// evaluate its expressions the same way; the built-in models always do.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <span>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "spice_gb300.h"

// The reference's checks (spice/include/spice/util/assert.h): a failed condition throws
// std::logic_error("Assertion failed (file:line): cond") (spice/src/util/assert.cpp:8-15).
#define SPICE_ASSERT(cond) ((cond) ? (void)0 : ::spice::detail::assert_failed(__FILE__, __LINE__, #cond))
#define SPICE_PRE(cond) SPICE_ASSERT(cond)
#define SPICE_INV(cond) SPICE_ASSERT(cond)

#if defined(__CUDACC__)
#include <cuda_runtime.h>
// Marks a user model's update() / deliver() / skip() for the GPU (init() runs on the host).
#define SPICE_HD __host__ __device__
#else
#define SPICE_HD
#endif

// The reference's integer names (spice/include/spice/util/stdint.h:5-12), which its models use.
using Int8   = std::int8_t;
using Int16  = std::int16_t;
using Int32  = std::int32_t;
using Int    = std::int64_t;
using UInt8  = std::uint8_t;
using UInt16 = std::uint16_t;
using UInt32 = std::uint32_t;
using UInt   = std::uint64_t;

namespace spice {

namespace detail {
[[noreturn]] inline void assert_failed(char const* file, int line, char const* cond) {
	throw std::logic_error(std::string("Assertion failed (") + file + ":" + std::to_string(line) + "): " + cond);
}
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

// xoroshiro64_128p (random.h:222-234): the engine's streams, on the host (init()) and the GPU.
struct xoroshiro64_128p {
	uint64_t s0 = 0, s1 = 0;
	SPICE_HD uint64_t operator()() {
		uint64_t const r = s0 + s1;
		uint64_t const t = s0 ^ s1;
		s0 = ((s0 << 24) | (s0 >> 40)) ^ t ^ (t << 16);
		s1 = (t << 37) | (t >> 27);
		return r;
	}
};

// range(n) / range(first, last): the integers of [first, last) to iterate over (util/range.h).
struct int_range {
	struct iterator {
		Int i;
		constexpr Int operator*() const { return i; }
		constexpr iterator& operator++() {
			++i;
			return *this;
		}
		constexpr bool operator!=(iterator const& o) const { return i != o.i; }
	};
	Int first, last;
	constexpr iterator begin() const { return {first}; }
	constexpr iterator end() const { return {last}; }
	constexpr Int size() const { return last - first; }
};
constexpr int_range range(Int first, Int last) { return {first, last > first ? last : first}; }
constexpr int_range range(Int n) { return range(0, n); }

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

// ---- the samples' models, built into the engine ----
namespace models {
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
	static constexpr int kind = SPICE_SYNAPSE_FIXED_WEIGHT;
	std::vector<float> params() const { return {weight, float(SPICE_FIELD_V)}; }
};
struct excitatory {
	float weight;
	static constexpr int kind = SPICE_SYNAPSE_FIXED_WEIGHT;
	std::vector<float> params() const { return {weight, float(SPICE_FIELD_GEX)}; }
};
struct inhibitory {
	float weight;
	static constexpr int kind = SPICE_SYNAPSE_FIXED_WEIGHT;
	std::vector<float> params() const { return {weight, float(SPICE_FIELD_GIN)}; }
};
// A per-synapse weight wmax * canonical<float> drawn at construction (PerSynapseInit), delivered
// into `field` by the pull path.
struct weighted {
	float wmax;
	int field = SPICE_FIELD_V;
	static constexpr int kind = SPICE_SYNAPSE_WEIGHTED;
	std::vector<float> params() const { return {wmax, float(field)}; }
};
}  // namespace models

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
inline constexpr bool is_builtin_model =
    std::is_same_v<T, models::poisson> || std::is_same_v<T, models::lif> || std::is_same_v<T, models::lif_cond> ||
    std::is_same_v<T, models::external_input>;
template <class T>
inline constexpr bool is_builtin_synapse = std::is_same_v<T, models::fixed_weight> ||
                                           std::is_same_v<T, models::excitatory> ||
                                           std::is_same_v<T, models::inhibitory> || std::is_same_v<T, models::weighted>;
template <class T>
concept has_neuron = requires { typename T::neuron; };
template <class T>
concept has_synapse = requires { typename T::synapse; };
template <class T>
concept has_field = requires { T::field; };
template <class T>
concept declares_draws = requires { T::draws_per_update; };
// the reference's concepts (concepts.h:22-30, 86-104), with this header's stream type
template <class T>
concept per_neuron_init = has_neuron<T> && requires(T const t, typename T::neuron& n, Int id, util::xoroshiro64_128p& rng) {
	t.init(n, id, rng);
};
template <class T>
concept per_population_init = has_neuron<T> && requires(T t, std::span<typename T::neuron> s, util::xoroshiro64_128p& rng) {
	t.init(s, rng);
};
template <class S>
concept per_synapse_init = has_synapse<S> && requires(S const t, typename S::synapse& syn, Int a, Int b,
                                                      util::xoroshiro64_128p& rng) { t.init(syn, a, b, rng); };
template <class S>
concept plastic_synapse = has_synapse<S> && requires(S const t, typename S::synapse& syn, float dt, bool pre, bool post, Int n) {
	t.update(syn, dt, pre, post);
	t.skip(syn, dt, n);
};
template <class S, class N>
concept deliver_to_stateless = requires(S const t, N& n) { t.deliver(n); };
template <class S, class N>
concept deliver_to_stateful = has_synapse<S> && requires(S const t, typename S::synapse const& syn, N& n) { t.deliver(syn, n); };
// DeliverFromTo (concepts.h:70-79): deliver() also reads the source neuron
template <class S, class SrcN, class N>
concept deliver_from_to = requires(S const t, SrcN const& s, N& n) { t.deliver(s, n); } ||
                          (has_synapse<S> && requires(S const t, typename S::synapse const& syn, SrcN const& s, N& n) {
	                          t.deliver(syn, s, n);
                          });
template <class>
inline constexpr bool always_false = false;

// The neuron struct of a target model (built-in or user).
template <class M>
using neuron_t = typename M::neuron;
// The neuron struct of a source model, or a placeholder for a stateless source.
template <class M, bool = has_neuron<M>>
struct source_neuron {
	using type = char;
};
template <class M>
struct source_neuron<M, true> {
	using type = typename M::neuron;
};
template <class M>
using source_neuron_t = typename source_neuron<M>::type;
// deliver() reads the source neuron: both models stateful, the DeliverFromTo form exists and the
// DeliverTo form, which the reference prefers (synapse_population.h:118-132), does not
template <class S, class SrcM, class DstM>
concept delivers_from = has_neuron<SrcM> && has_neuron<DstM> &&
                        deliver_from_to<S, typename SrcM::neuron, typename DstM::neuron> &&
                        !deliver_to_stateless<S, typename DstM::neuron> && !deliver_to_stateful<S, typename DstM::neuron>;

// A built-in target's field index for a byte offset into its neuron struct (lif: V; lif_cond: V, Gex,
// Gin), or -1.
template <class M>
int builtin_field(int offset) {
	if constexpr (std::is_same_v<M, models::lif>) return offset == 0 ? SPICE_FIELD_V : -1;
	else if constexpr (std::is_same_v<M, models::lif_cond>)
		return offset == 0 ? SPICE_FIELD_V : offset == 4 ? SPICE_FIELD_GEX : offset == 8 ? SPICE_FIELD_GIN : -1;
	else return -1;
}

// What deliver() does to a target neuron, found by calling it on probe values: it must add a constant
// (stateless) or one float member of the synapse (stateful; member index `syn_word`) to one float
// member of the neuron (byte offset `dst_offset`).  Returns false otherwise.
struct deliver_probe {
	int dst_offset = -1;
	int syn_word   = -1;
	float constant = 0;
};
template <class N>
SPICE_HD float word_of(N const& n, int w) {
	float f;
	memcpy(&f, reinterpret_cast<char const*>(&n) + 4 * w, 4);
	return f;
}
template <class N>
void set_word(N& n, int w, float f) {
	std::memcpy(reinterpret_cast<char*>(&n) + 4 * w, &f, 4);
}
template <class S, class N, class Deliver>
bool probe_additive(Deliver&& deliver, deliver_probe& out, float syn_value_of_word, bool stateful) {
	(void)syn_value_of_word;
	(void)stateful;
	constexpr int words = (int)(sizeof(N) / 4);
	if constexpr (words == 0) {
		return false;  // no float member to add to
	} else {
		auto same_tail = [](N const& a, N const& b) {  // the bytes after the last whole word
			return std::memcmp(reinterpret_cast<char const*>(&a) + 4 * words, reinterpret_cast<char const*>(&b) + 4 * words,
			                   sizeof(N) - 4 * words) == 0;
		};
		N zero{};
		std::memset(static_cast<void*>(&zero), 0, sizeof zero);
		N n = zero;
		deliver(n);
		if (!same_tail(n, zero)) return false;
		int changed = -1;
		for (int w = 0; w < words; w++)
			if (word_of(n, w) != 0.0f) {
				if (changed >= 0) return false;
				changed = w;
			}
		if (changed < 0) return false;
		float const c     = word_of(n, changed);
		float const xs[4] = {0.5f, -1.25f, 3.0e-3f, 1000.0f};
		for (float x : xs) {  // the same member, now from x: x + c, one IEEE addition
			N m = zero;
			set_word(m, changed, x);
			deliver(m);
			volatile float expect = x;
			expect                = expect + c;
			if (word_of(m, changed) != expect || !same_tail(m, zero)) return false;
			for (int w = 0; w < words; w++)
				if (w != changed && word_of(m, w) != 0.0f) return false;
		}
		out.dst_offset = 4 * changed;
		out.constant   = c;
		return true;
	}
}

#if defined(__CUDACC__)
// xoroshiro128+ positioned in the step's stream.
using device_rng = util::xoroshiro64_128p;

// The counter-based stream of a stateful model without declared draws: xoroshiro128+ seeded by
// SplitMix64-mixing the step's seed with the population and neuron index.
SPICE_HD inline uint64_t splitmix64(uint64_t x) {
	x += 0x9E3779B97F4A7C15ull;
	x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
	x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
	return x ^ (x >> 31);
}
__device__ inline device_rng counter_stream(const uint64_t* step_seed, int pop, int64_t i) {
	uint64_t const a = splitmix64(step_seed[0] ^ splitmix64((uint64_t)i * 2 + 1));
	uint64_t const b = splitmix64(step_seed[1] ^ splitmix64(((uint64_t)pop << 40) ^ (uint64_t)i));
	return device_rng{a, b | 1ull};  // never the all-zero state
}

// The stream position of `draws`-per-neuron model neuron i in step k: the chunk's jump (16 table
// lookups), then (i mod 32) * draws draws.
__device__ inline device_rng jumped_stream(spice_user_window const& w, int k, int64_t i) {
	const uint64_t* tab  = static_cast<const uint64_t*>(w.tables) + (int64_t)k * 16 * 256 * 2;
	const uint64_t* poly = static_cast<const uint64_t*>(w.chunk_poly) + 2 * (i >> 5);
	uint64_t const plo = poly[0], phi = poly[1];
	device_rng rng{0, 0};
	for (int g = 0; g < 16; g++) {
		uint64_t const byte = ((g < 8 ? plo : phi) >> (8 * (g & 7))) & 255;
		rng.s0 ^= tab[2 * (g * 256 + byte)];
		rng.s1 ^= tab[2 * (g * 256 + byte) + 1];
	}
	for (int64_t r = (i & 31) * w.draws; r > 0; r--) rng();
	return rng;
}

// One window of a stateful user population: per neuron, per step, the inputs of the step (the
// engine's per-group counts replayed as sequential float adds, the atomic-mode sums, or the pulled
// per-synapse weights in the reference's order), then the user's update(); spikes to the bitmap
// and the step's list.
template <class Neur>
__global__ void __launch_bounds__(256) user_update_kernel(const spice_user_window w, const Neur neur) {
	using N          = typename Neur::neuron;
	int64_t const i  = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	bool const valid = i < w.size;
	int const lane   = threadIdx.x & 31;
	N* const st      = static_cast<N*>(w.state);
	N n{};
	if (valid) n = st[i];
	auto field = [&](int f) -> float& {
		return *reinterpret_cast<float*>(reinterpret_cast<char*>(&n) + w.field_offset[f]);
	};
	auto apply_pulled = [&](int k) {
		int32_t* const ko  = w.pull_koff + i * (int64_t)(w.pull_nbins + 1);
		int64_t const base = w.pull_base[i];
		if (ko[0] >= 0) {
			for (int f = 0; f < w.pull_F; f++) {
				float& x = field(w.pull_field[f]);
				float v  = x;
				for (int32_t e = ko[k * w.pull_F + f]; e < ko[k * w.pull_F + f + 1]; e++) v = __fadd_rn(v, w.pull_G[base + e]);
				x = v;
			}
			if (w.apply_only)
				for (int f = 0; f < w.pull_F; f++) ko[f] = ko[w.pull_F];
		} else {
			for (int32_t e = 0; e < ko[1]; e++) {
				uint64_t const a  = w.pull_A[base + e];
				uint32_t const mf = (uint32_t)(a >> 32);
				if ((mf >> k) & 1u) {
					float& x = field(w.pull_field[mf >> 16]);
					x        = __fadd_rn(x, __uint_as_float((uint32_t)a));
					if (w.apply_only) w.pull_A[base + e] = a & ~(1ull << 32);
				}
			}
		}
	};
	auto apply = [&](int64_t slot, int k) {
		if (w.direct) {  // inputs arrive in the structs at the end of each step
		} else if (w.pull) {
			apply_pulled(k);
		} else if (w.mode == SPICE_MODE_DETERMINISTIC) {
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
			apply(w.slot0, 0);
			st[i] = n;
		}
		return;
	}
	int slot = w.slot0, hslot = w.hslot0;
	uint64_t h = (valid && w.hist) ? w.hist[i] : 0ull;
	for (int k = 0; k < w.K; k++) {
		bool spike = false;
		if (valid) {
			apply(slot, k);
			const uint64_t* seed = static_cast<const uint64_t*>(w.step_seeds) + 2 * k;
			device_rng rng       = w.draws > 0 ? jumped_stream(w, k, i) : counter_stream(seed, w.pop, i);
			spike                = neur.update(n, w.dts[k], rng);
		}
		h = (h << 1) | (spike ? 1ull : 0ull);  // a plastic synapses' target keeps 64 steps (neuron_population.h:126-132)
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
	if (valid) {
		st[i] = n;
		if (w.hist) w.hist[i] = h;
	}
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

// The catch-up of one plastic synapse to step `time` (synapse_population.h:88-116): the pending pre
// update of its source's last delivery, then every post spike of the target's 64-step history, with
// skip() over the quiet steps.  ~0 >> prefix with prefix up to 64 is computed as x86-64 does
// (shift mod 64).
template <class Syn, class S>
__device__ void user_catch_up(Syn const& syn, S& s, float dt, int64_t time, uint64_t ages, uint64_t hist) {
	int const pre     = (int)(ages >> 63);
	int64_t const age = (int64_t)(ages & ~(1ull << 63));
	if (!(time >= age)) return;
	int64_t const prefix = 63 + pre - time + age;
	uint64_t const mask  = ~0ull >> (prefix & 63);
	if (pre) syn.update(s, dt, true, (hist & (1ull << ((time - age) & 63))) != 0);
	hist &= mask;
	int64_t p = prefix;
	while (hist) {
		int const lz = __clzll((long long)hist);
		syn.skip(s, dt, (Int)(lz - p));
		syn.update(s, dt, false, true);
		hist ^= 1ull << (63 - lz);
		p = lz + 1;
	}
	syn.skip(s, dt, (Int)(64 - p));
}

// Every 64 steps: every synapse catches up, a warp per source, then the source's age is time + 1.
template <class Syn>
__global__ void __launch_bounds__(256) user_plastic_update_all(const spice_user_plastic_call c, const Syn syn) {
	using S = typename Syn::synapse;
	int const lane    = threadIdx.x & 31;
	int64_t const src = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
	if (src >= c.src_size) return;
	S* const st         = static_cast<S*>(c.state);
	uint64_t const ages = c.ages[src];
	for (int64_t e = c.off[src] + lane; e < c.off[src + 1]; e += 32) {
		S x = st[e];
		user_catch_up(syn, x, c.dt, c.time, ages, c.dst_hist[c.nb[e]]);
		st[e] = x;
	}
	__syncwarp();
	if (lane == 0) c.ages[src] = (uint64_t)(c.time + 1);
}

// Delivery of a step's spikes: CTA (w, y) takes 256-synapse chunks y, y + gridDim.y, ... of the row of
// every spiking source of bitmap word w: catch up, add the weight member into the input ring; the
// row's last chunk to finish sets the source's age (time + 1, pending pre update).
template <class Syn>
__global__ void __launch_bounds__(256) user_plastic_deliver(const spice_user_plastic_call c, const Syn syn) {
	using S = typename Syn::synapse;
	S* const st   = static_cast<S*>(c.state);
	int const w   = blockIdx.x;
	uint32_t bits = c.src_bits[(int64_t)c.hslot * c.src_nwords + w];
	unsigned long long ev = 0;
	while (bits) {
		int const r = __ffs(bits) - 1;
		bits &= bits - 1;
		int64_t const src     = 32 * (int64_t)w + r;
		int64_t const e0      = c.off[src], e1 = c.off[src + 1];
		int64_t const nchunks = (e1 - e0 + 255) / 256;
		if (blockIdx.y == 0 && threadIdx.x == 0) ev += (unsigned long long)(e1 - e0);
		for (int64_t ch = blockIdx.y; ch < nchunks; ch += gridDim.y) {
			uint64_t const ages = c.ages[src];
			int64_t const e     = e0 + ch * 256 + threadIdx.x;
			if (e < e1) {
				S x             = st[e];
				int32_t const j = c.nb[e];
				user_catch_up(syn, x, c.dt, c.time, ages, c.dst_hist[j]);
				st[e] = x;
				if (c.deliver)
					atomicAdd(c.dst_acc + (c.slot * c.dst_size + j) * c.F + c.fslot, word_of(x, c.weight_word));
			}
			__syncthreads();  // every thread of this chunk has read the source's age
			if (threadIdx.x == 0) {
				__threadfence();
				if (atomicAdd(c.chunks_done + src, 1u) == (uint32_t)(nchunks - 1)) {
					c.ages[src]        = (uint64_t)(c.time + 1) | (1ull << 63);
					c.chunks_done[src] = 0;
				}
			}
			__syncthreads();
		}
	}
	if (threadIdx.x == 0 && ev) atomicAdd(c.events, ev);
}

template <class Syn>
int user_plastic_launch(const spice_user_plastic_call* c, void* stream, void* ctx) {
	Syn const& syn         = *static_cast<const Syn*>(ctx);
	cudaStream_t const st  = static_cast<cudaStream_t>(stream);
	if (c->what == 0) {
		if (c->src_size > 0) user_plastic_update_all<Syn><<<(unsigned)((c->src_size + 7) / 8), 256, 0, st>>>(*c, syn);
	} else if (c->src_nwords > 0) {
		dim3 const grid((unsigned)c->src_nwords, (unsigned)(c->max_row > 0 ? (c->max_row + 255) / 256 < 65535 ? (c->max_row + 255) / 256 : 65535 : 1));
		user_plastic_deliver<Syn><<<grid, 256, 0, st>>>(*c, syn);
	}
	return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

// One synapse's deliver(), in whichever of the reference's forms the synapse defines, the DeliverTo
// form first (synapse_population.h:118-132).
template <class Syn, class SrcN, class DstN>
__device__ __forceinline__ void deliver_one(Syn const& syn, void* sst, int64_t pos, SrcN const* src, DstN& dst) {
	if constexpr (has_synapse<Syn>) {
		auto const& x = static_cast<typename Syn::synapse const*>(sst)[pos];
		if constexpr (requires { syn.deliver(x, dst); }) syn.deliver(x, dst);
		else syn.deliver(x, *src, dst);
	} else {
		if constexpr (requires { syn.deliver(dst); }) syn.deliver(dst);
		else syn.deliver(*src, dst);
	}
}

// User deliver() code, target-parallel: thread j applies, in ascending source order along its CSC
// column, every synapse whose source spiked in bitmap slot hslot.
template <class Syn, class SrcNeur, class DstNeur>
__global__ void __launch_bounds__(256) user_deliver_targets(const spice_user_deliver_call c, const Syn syn) {
	using SN = source_neuron_t<SrcNeur>;
	using DN = neuron_t<DstNeur>;
	int64_t const j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	unsigned long long ev = 0;
	if (j < c.dst_size) {
		DN d                 = static_cast<DN*>(c.dst_state)[j];
		const uint32_t* bits = c.src_bits + (int64_t)c.hslot * c.src_nwords;
		SN const* src        = static_cast<SN const*>(c.src_state);
		for (int64_t e = c.col_off[j]; e < c.col_off[j + 1]; e++) {
			int32_t const s = c.col_src[e];
			if ((bits[s >> 5] >> (s & 31)) & 1u) {
				deliver_one<Syn>(syn, c.synapse_state, c.col_pos ? c.col_pos[e] : 0, src ? src + s : nullptr, d);
				ev++;
			}
		}
		static_cast<DN*>(c.dst_state)[j] = d;
	}
	for (int o = 16; o > 0; o >>= 1) ev += __shfl_down_sync(0xffffffffu, ev, o);
	if ((threadIdx.x & 31) == 0 && ev) atomicAdd(c.events, ev);
}

// User deliver() code that reads neurons of its own target population: the reference's order
// exactly -- spiking sources ascending, each along its CSR row -- by one thread, so that a later
// source reads what an earlier delivery wrote (synapse_population.h:118-133).
template <class Syn, class SrcNeur, class DstNeur>
__global__ void user_deliver_sequential(const spice_user_deliver_call c, const Syn syn) {
	using SN = source_neuron_t<SrcNeur>;
	using DN = neuron_t<DstNeur>;
	if (blockIdx.x != 0 || threadIdx.x != 0) return;
	const uint32_t* bits = c.src_bits + (int64_t)c.hslot * c.src_nwords;
	SN const* src        = static_cast<SN const*>(c.src_state);
	DN* dst              = static_cast<DN*>(c.dst_state);
	unsigned long long ev = 0;
	for (int w = 0; w < c.src_nwords; w++)
		for (uint32_t x = bits[w]; x; x &= x - 1) {
			int64_t const s = 32 * (int64_t)w + __ffs(x) - 1;
			for (int64_t e = c.off[s]; e < c.off[s + 1]; e++) {
				deliver_one<Syn>(syn, c.synapse_state, e, src + s, dst[c.nb[e]]);
				ev++;
			}
		}
	if (ev) atomicAdd(c.events, ev);
}

template <class Syn, class SrcNeur, class DstNeur>
int user_deliver_launch(const spice_user_deliver_call* c, void* stream, void* ctx) {
	Syn const& syn        = *static_cast<const Syn*>(ctx);
	cudaStream_t const st = static_cast<cudaStream_t>(stream);
	constexpr bool reads  = delivers_from<Syn, SrcNeur, DstNeur>;
	if (reads && c->same_population) user_deliver_sequential<Syn, SrcNeur, DstNeur><<<1, 1, 0, st>>>(*c, syn);
	else if (c->dst_size > 0)
		user_deliver_targets<Syn, SrcNeur, DstNeur><<<(unsigned)((c->dst_size + 255) / 256), 256, 0, st>>>(*c, syn);
	return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

template <class Neur>
int user_launch(const spice_user_window* w, void* stream, void* ctx) {
	Neur const& neur  = *static_cast<const Neur*>(ctx);
	cudaStream_t const st = static_cast<cudaStream_t>(stream);
	if constexpr (has_neuron<Neur>) {
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

// CheckNeuron<T>() / CheckSynapse<T>() (concepts.h:163-228): compile-time checks of a model's
// methods, true when they pass (static_assert with an explanation otherwise).
namespace detail {
struct any_arg {  // converts to any argument type (unevaluated)
	template <class U>
	operator U&() const;
};
template <class T>
concept any_update = requires(T const t, any_arg a) { t.update(a, a); } || requires(T const t, any_arg a) { t.update(a, a, a); };
template <class T>
concept any_deliver = requires(T const t, any_arg a) { t.deliver(a); } || requires(T const t, any_arg a) { t.deliver(a, a); } ||
                      requires(T const t, any_arg a) { t.deliver(a, a, a); };
template <class T>
concept any_syn_update = requires(T const t, any_arg a) { t.update(a, a, a, a); };
template <class T>
concept any_syn_skip = requires(T const t, any_arg a) { t.skip(a, a, a); };
}  // namespace detail

template <class T>
constexpr bool CheckNeuron() {
	static_assert(std::is_default_constructible_v<T>, "a neuron model must be default-constructible");
	static_assert(detail::any_update<T>, "a neuron model defines update(dt, rng) or update(neuron&, dt, rng)");
	return true;
}

template <class T>
constexpr bool CheckSynapse() {
	static_assert(std::is_default_constructible_v<T>, "a synapse model must be default-constructible");
	static_assert(detail::any_deliver<T>, "a synapse model defines deliver()");
	static_assert(detail::any_syn_update<T> == detail::any_syn_skip<T>,
	              "a plastic synapse defines both update(synapse&, dt, pre, post) and skip(synapse&, dt, n)");
	static_assert(!detail::any_syn_update<T> || detail::has_synapse<T>, "a plastic synapse needs a nested `synapse` struct");
	return true;
}

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
	// Only for models with per-neuron state.
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
			if constexpr (detail::has_neuron<Neur>) {
				using N = typename Neur::neuron;
				static_assert(std::is_trivially_copyable_v<N>, "a user neuron must be a trivially copyable struct");
				N const init{};
				detail::check(spice_add_user_population(_net, size, 1, (int)sizeof(N), &init, &detail::user_launch<Neur>,
				                                        model.get(), &id));
				if constexpr (detail::declares_draws<Neur>) detail::check(spice_user_draws(_net, id, (int)Neur::draws_per_update));
				if constexpr (detail::per_neuron_init<Neur> || detail::per_population_init<Neur>) {
					// stateful_neuron_adapter's init with the population's own stream (neuron_population.h:56-67)
					util::xoroshiro64_128p rng;
					detail::check(spice_population_seed(_net, id, &rng.s0, &rng.s1));
					std::vector<N> ns((size_t)size);
					if constexpr (detail::per_neuron_init<Neur>) {
						Int i = 0;
						for (auto& x : ns) neur.init(x, i++, rng);
					} else {
						neur.init(std::span<N>(ns), rng);
					}
					detail::check(spice_set_user_state(_net, id, ns.data()));
				}
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

	// Returns the connection's id (the reference returns nothing; callers may ignore it).
	template <class Syn, class SrcNeur, class DstNeur>
	int connect(neuron_population<SrcNeur>* source, neuron_population<DstNeur>* target,
	            fixed_probability const& c, float delay, Syn syn = {}) {
		plan const pl = plan_of<Syn, SrcNeur, DstNeur>(syn, target);
		int id        = -1;
		detail::check(spice_connect_fixed_probability(_net, source->id(), target->id(), c.p(), delay, pl.kind,
		                                              pl.params.data(), (int)pl.params.size(), &id));
		finish<Syn, SrcNeur, DstNeur>(syn, id, pl);
		return id;
	}

	template <class Syn, class SrcNeur, class DstNeur>
	int connect(neuron_population<SrcNeur>* source, neuron_population<DstNeur>* target, adj_list const& c,
	            float delay, Syn syn = {}) {
		plan const pl = plan_of<Syn, SrcNeur, DstNeur>(syn, target);
		int id        = -1;
		detail::check(spice_connect_adj_list(_net, source->id(), target->id(), c.pairs().data(), c.size(), delay,
		                                     pl.kind, pl.params.data(), (int)pl.params.size(), &id));
		finish<Syn, SrcNeur, DstNeur>(syn, id, pl);
		return id;
	}

	void step() { detail::check(spice_step(_net)); }  // snn.cpp:7-28
	// The per-synapse state of a plastic user connection, CSR order: each synapse as of its last
	// catch-up (its source's last delivery or the last multiple of 64 steps), as the reference's
	// synapse_population holds it.
	template <class Syn>
	std::vector<typename Syn::synapse> get_synapses(int conn) {
		int64_t src = 0, n = 0;
		detail::check(spice_conn_size(_net, conn, &src, &n));
		std::vector<typename Syn::synapse> out((size_t)std::max<int64_t>(n, 1));
		detail::check(spice_get_user_synapse_state(_net, conn, out.data()));
		out.resize((size_t)n);
		return out;
	}
	void run(int64_t steps) { detail::check(spice_run(_net, steps)); }
	void set_mode(int mode) { detail::check(spice_set_mode(_net, mode)); }
	spice_net* handle() { return _net; }

private:
	// How a synapse type reaches the engine: kind + params, and for a stateful synapse with
	// PerSynapseInit the float member of its struct whose per-synapse values are the weights.
	struct plan {
		int kind = SPICE_SYNAPSE_FIXED_WEIGHT;
		std::vector<float> params;
		int weight_word = -1;  // host weights: word of the synapse struct delivered
		bool user_deliver = false;  // deliver() runs as user code (SPICE_SYNAPSE_USER_DELIVER)
	};

	template <class DstNeur>
	int field_index(neuron_population<DstNeur>* target, int offset) {
		if constexpr (detail::is_builtin_model<DstNeur>) {
			int const f = detail::builtin_field<DstNeur>(offset);
			if (f < 0) throw std::logic_error("the synapse's deliver() targets no float state field of the neuron model");
			return f;
		} else {
			int fi = -1;
			detail::check(spice_user_field(_net, target->id(), offset, &fi));
			return fi;
		}
	}

	template <class Syn, class SrcNeur, class DstNeur>
	plan plan_of(Syn const& syn, neuron_population<DstNeur>* target) {
		plan pl;
		if constexpr (detail::is_builtin_synapse<Syn>) {
			pl.kind   = Syn::kind;
			pl.params = syn.params();
			return pl;
		} else {
			using N = detail::neuron_t<DstNeur>;
			// deliver() as user code on the target (and source) neuron structs, in the reference's order
			auto user_code = [&](bool reads_source) {
				if constexpr (detail::is_builtin_model<DstNeur>) {
					throw std::logic_error("a synapse whose deliver() is not an addition of one value to one float member "
					                       "targets user-defined neuron models only");
				} else {
					pl.kind = SPICE_SYNAPSE_USER_DELIVER;
					if constexpr (detail::has_synapse<Syn>)
						pl.params = {float(sizeof(typename Syn::synapse)), reads_source ? 1.0f : 0.0f,
						             detail::per_synapse_init<Syn> ? 1.0f : 0.0f};
					else
						pl.params = {0.0f, reads_source ? 1.0f : 0.0f, 0.0f};
					pl.user_deliver = true;
				}
				return pl;
			};
			if constexpr (!detail::is_builtin_model<SrcNeur> && !detail::is_builtin_model<DstNeur> &&
			              detail::delivers_from<Syn, SrcNeur, DstNeur>) {
				return user_code(true);
			} else if constexpr (detail::has_field<Syn>) {  // the member named by the synapse, its `weight`
				N probe{};
				int const off = (int)(reinterpret_cast<char const*>(&(probe.*Syn::field)) - reinterpret_cast<char const*>(&probe));
				pl.params     = {syn.weight, float(field_index(target, off))};
				return pl;
			} else if constexpr (detail::deliver_to_stateless<Syn, N>) {
				detail::deliver_probe pr;
				if (!detail::probe_additive<Syn, N>([&](N& n) { syn.deliver(n); }, pr, 0.0f, false)) return user_code(false);
				pl.params = {pr.constant, float(field_index(target, pr.dst_offset))};
				return pl;
			} else if constexpr (detail::deliver_to_stateful<Syn, N>) {
				using S = typename Syn::synapse;
				static_assert(std::is_trivially_copyable_v<S> && sizeof(S) % 4 == 0,
				              "a synapse struct must be trivially copyable, of 4-byte members");
				constexpr int words = (int)(sizeof(S) / 4);
				// which member of the synapse struct is delivered: probe each word alone
				int wsel = -1;
				detail::deliver_probe pr;
				for (int wd = 0; wd < words && wsel < 0; wd++) {
					S s{};
					std::memset(static_cast<void*>(&s), 0, sizeof s);
					detail::set_word(s, wd, 0.375f);
					detail::deliver_probe p1;
					if (detail::probe_additive<Syn, N>([&](N& n) { syn.deliver(s, n); }, p1, 0.375f, true) && p1.constant == 0.375f) {
						S s2{};
						std::memset(static_cast<void*>(&s2), 0, sizeof s2);
						detail::set_word(s2, wd, -2.5f);
						detail::deliver_probe p2;
						if (detail::probe_additive<Syn, N>([&](N& n) { syn.deliver(s2, n); }, p2, -2.5f, true) &&
						    p2.constant == -2.5f && p2.dst_offset == p1.dst_offset) {
							wsel = wd;
							pr   = p1;
						}
					}
				}
				if (wsel < 0) {
					if constexpr (detail::plastic_synapse<Syn>)
						throw std::logic_error("a plastic synapse's deliver() must add one float member of the synapse to one "
						                       "float member of the target neuron");
					else
						return user_code(false);
				}
				int const f = field_index(target, pr.dst_offset);
				if constexpr (detail::plastic_synapse<Syn>) {
					pl.kind        = SPICE_SYNAPSE_USER_PLASTIC;
					pl.params      = {float(f), float(sizeof(S)), float(wsel), detail::per_synapse_init<Syn> ? 1.0f : 0.0f};
					pl.weight_word = wsel;
				} else if constexpr (detail::per_synapse_init<Syn>) {
					pl.kind        = SPICE_SYNAPSE_WEIGHTED;
					pl.params      = {0.0f, float(f), 1.0f};  // host weights, the init seed consumed
					pl.weight_word = wsel;
				} else {  // every synapse starts as synapse{}: one weight for the whole connection
					S const s0{};
					pl.params = {detail::word_of(s0, wsel), float(f)};
				}
				return pl;
			} else {
				static_assert(detail::always_false<Syn>,
				              "the synapse's deliver() does not take the target population's neuron struct");
				return pl;
			}
		}
	}

	// A stateful synapse with PerSynapseInit: its init() over the CSR in order, on the host, with the
	// connection's init stream (synapse_population.h:34-41), and the delivered member as the weights.
	template <class Syn, class SrcNeur, class DstNeur>
	void finish(Syn const& syn, int id, plan const& pl) {
		if (pl.user_deliver) {
#if defined(__CUDACC__)
			if constexpr (!detail::is_builtin_model<DstNeur>) {
				static_assert(std::is_trivially_copyable_v<Syn>, "a user synapse model must be trivially copyable");
				auto model = std::make_shared<Syn>(syn);
				_models.push_back(model);
				if constexpr (detail::has_synapse<Syn>) {
					using S = typename Syn::synapse;
					S const init{};
					detail::check(spice_user_deliver(_net, id, &detail::user_deliver_launch<Syn, SrcNeur, DstNeur>, model.get(), &init));
					if constexpr (detail::per_synapse_init<Syn>) host_synapse_init<Syn>(syn, id);
				} else {
					detail::check(spice_user_deliver(_net, id, &detail::user_deliver_launch<Syn, SrcNeur, DstNeur>, model.get(), nullptr));
				}
			}
#else
			throw std::logic_error("synapses with their own deliver() code run as GPU kernels: compile with nvcc");
#endif
			return;
		}
		if constexpr (detail::plastic_synapse<Syn>) {
#if defined(__CUDACC__)
			using S = typename Syn::synapse;
			static_assert(std::is_trivially_copyable_v<Syn>, "a user synapse model must be trivially copyable");
			auto model = std::make_shared<Syn>(syn);
			S const init{};
			detail::check(spice_user_plastic(_net, id, &detail::user_plastic_launch<Syn>, model.get(), &init));
			// per-synapse weights that change over time have no fixed summation order: atomic mode
			detail::check(spice_set_mode(_net, SPICE_MODE_ATOMIC));
			_models.push_back(model);
			if constexpr (detail::per_synapse_init<Syn>) {  // the synapses' init() on the host, CSR order
				int64_t src = 0, nsyn = 0;
				detail::check(spice_conn_size(_net, id, &src, &nsyn));
				std::vector<int64_t> off((size_t)src + 1);
				std::vector<int32_t> nb((size_t)std::max<int64_t>(nsyn, 1));
				detail::check(spice_get_csr(_net, id, off.data(), nb.data()));
				uint64_t seeds[4];
				detail::check(spice_connection_seeds(_net, id, seeds));
				util::xoroshiro64_128p rng{seeds[2], seeds[3]};
				std::vector<S> st((size_t)std::max<int64_t>(nsyn, 1));
				for (int64_t s = 0; s < src; s++)
					for (int64_t e = off[s]; e < off[s + 1]; e++) syn.init(st[e], s, nb[e], rng);
				detail::check(spice_set_user_synapse_state(_net, id, st.data()));
			}
#else
			static_assert(detail::always_false<Syn>, "plastic user synapses run as GPU kernels: compile with nvcc");
#endif
		} else if constexpr (detail::per_synapse_init<Syn>) {
			if (pl.weight_word < 0) return;
			using S = typename Syn::synapse;
			int64_t src = 0, nsyn = 0;
			detail::check(spice_conn_size(_net, id, &src, &nsyn));
			std::vector<int64_t> off((size_t)src + 1);
			std::vector<int32_t> nb((size_t)std::max<int64_t>(nsyn, 1));
			detail::check(spice_get_csr(_net, id, off.data(), nb.data()));
			uint64_t seeds[4];
			detail::check(spice_connection_seeds(_net, id, seeds));
			util::xoroshiro64_128p rng{seeds[2], seeds[3]};
			std::vector<float> w((size_t)std::max<int64_t>(nsyn, 1));
			for (int64_t s = 0; s < src; s++)
				for (int64_t e = off[s]; e < off[s + 1]; e++) {
					S x{};
					syn.init(x, s, nb[e], rng);
					w[e] = detail::word_of(x, pl.weight_word);
				}
			detail::check(spice_set_synapse_weights(_net, id, w.data()));
		} else {
			(void)syn;
			(void)id;
			(void)pl;
		}
	}

	// A synapse type's init(synapse&, src, dst, rng) over the CSR in order with the connection's
	// PerSynapseInit stream (synapse_population.h:34-41): the whole state array, to the engine.
	template <class Syn>
	void host_synapse_init(Syn const& syn, int id) {
		using S = typename Syn::synapse;
		int64_t src = 0, nsyn = 0;
		detail::check(spice_conn_size(_net, id, &src, &nsyn));
		std::vector<int64_t> off((size_t)src + 1);
		std::vector<int32_t> nb((size_t)std::max<int64_t>(nsyn, 1));
		detail::check(spice_get_csr(_net, id, off.data(), nb.data()));
		uint64_t seeds[4];
		detail::check(spice_connection_seeds(_net, id, seeds));
		util::xoroshiro64_128p rng{seeds[2], seeds[3]};
		std::vector<S> st((size_t)std::max<int64_t>(nsyn, 1));
		for (int64_t s = 0; s < src; s++)
			for (int64_t e = off[s]; e < off[s + 1]; e++) syn.init(st[e], s, nb[e], rng);
		detail::check(spice_set_user_synapse_state(_net, id, st.data()));
	}

	spice_net* _net = nullptr;
	std::vector<std::shared_ptr<void>> _pops;    // owns the population handles (snn.h:72-74)
	std::vector<std::shared_ptr<void>> _models;  // user models, read by their update kernels' launches
};

}  // namespace spice
