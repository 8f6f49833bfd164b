// spice/snn.h -- the reference's C++20 user API (spice/include/spice/snn.h:16-75) on the GB300
// engine.  A program written against spice2's snn for the sample models compiles against this
// header unchanged in its calls: snn(dt, max_delay, {seed}), add_population<Model>(size, model),
// connect<Synapse>(from, to, fixed_probability(p) | adj_list, delay, {params}), step(), and the
// population handle's spikes(age) / get_neurons().  Everything runs on the GPU through the C ABI of
// spice_gb300.h; violated preconditions throw std::logic_error with the reference's message
// (spice/src/util/assert.cpp:8-15).
//
// The models are the ones of the reference's samples, built into the engine (the engine's kernels
// are compiled for them): poisson (samples/brunel.cpp:23-31), lif (brunel.cpp:39-62),
// lif_cond (samples/vogels.cpp:10-46), external_input (samples/external_input.cpp:17-30);
// synapses fixed_weight (brunel.cpp:67-70), excitatory / inhibitory (vogels.cpp:48-60).
#pragma once

#include <cstdint>
#include <initializer_list>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "spice_gb300.h"

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
		int64_t const n = size();
		std::vector<float> V(n), Gex(n), Gin(n);
		std::vector<int32_t> T(n);
		detail::check(spice_get_state(_net, _id, SPICE_FIELD_V, V.data()));
		detail::check(spice_get_state(_net, _id, SPICE_FIELD_TREF, T.data()));
		std::vector<typename M::neuron> out((size_t)n);
		if constexpr (M::model == SPICE_NEURON_LIF_COND) {
			detail::check(spice_get_state(_net, _id, SPICE_FIELD_GEX, Gex.data()));
			detail::check(spice_get_state(_net, _id, SPICE_FIELD_GIN, Gin.data()));
			for (int64_t i = 0; i < n; i++) out[i] = {V[i], Gex[i], Gin[i], T[i]};
		} else {
			for (int64_t i = 0; i < n; i++) out[i] = {V[i], T[i]};
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

	template <class Syn, class SrcNeur, class DstNeur>
	void connect(neuron_population<SrcNeur>* source, neuron_population<DstNeur>* target,
	             fixed_probability const& c, float delay, Syn syn = {}) {
		auto const prm = syn.params();
		int id         = -1;
		detail::check(spice_connect_fixed_probability(_net, source->id(), target->id(), c.p(), delay,
		                                              SPICE_SYNAPSE_FIXED_WEIGHT, prm.data(), (int)prm.size(), &id));
	}

	template <class Syn, class SrcNeur, class DstNeur>
	void connect(neuron_population<SrcNeur>* source, neuron_population<DstNeur>* target, adj_list const& c,
	             float delay, Syn syn = {}) {
		auto const prm = syn.params();
		int id         = -1;
		detail::check(spice_connect_adj_list(_net, source->id(), target->id(), c.pairs().data(), c.size(), delay,
		                                     SPICE_SYNAPSE_FIXED_WEIGHT, prm.data(), (int)prm.size(), &id));
	}

	void step() { detail::check(spice_step(_net)); }  // snn.cpp:7-28
	void run(int64_t steps) { detail::check(spice_run(_net, steps)); }
	void set_mode(int mode) { detail::check(spice_set_mode(_net, mode)); }
	spice_net* handle() { return _net; }

private:
	spice_net* _net = nullptr;
	std::vector<std::shared_ptr<void>> _pops;  // owns the population handles (snn.h:72-74)
};

}  // namespace spice
