// The user-model contract of include/spice/snn.h, one case per argument (prints JSON):
//   stream  N steps seed   a stateful model declaring draws_per_update = 1 whose update is the
//                          Poisson test canonical<float>(rng) < 20 dt: the reference's step stream
//                          at the reference's positions, so its raster equals a Poisson
//                          population's that follows a stateful population of size 0
//   init    N seed         init(neuron&, id, rng) and init(span, rng) run with each population's own
//                          stream (neuron_population.h:56-67): the initial states
//   weights N p steps seed a stateful synapse with init(synapse&, src, dst, rng) (PerSynapseInit) and
//                          a stateless synapse whose deliver() adds a constant, no field declared,
//                          on Poisson -> LIF: raster and final V (the engine's weighted and
//                          fixed_weight synapses compute the same)
//   counter N steps seed   a stateful model drawing without declared draws: every neuron's draw of
//                          the last step (statistically uniform, independent streams)
//   nvcc -std=c++20 -gencode arch=compute_103a,code=sm_103a -fmad=false -I include user_contract.cu \
//        -L spice2_gb300 -lspice_gb300 -o user_contract
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <span>
#include <vector>

#include "spice/snn.h"

using namespace spice;

struct stream_poisson {
	struct neuron {
		float last = 0;
	};
	static constexpr int draws_per_update = 1;
	SPICE_HD bool update(neuron& n, float dt, auto& rng) const {
		float const u = util::generate_canonical<float>(rng);
		n.last        = u;
		return u < 20.0f * dt;
	}
};

struct empty_stateful {
	struct neuron {
		float V = 0;
	};
	SPICE_HD bool update(neuron&, float, auto&) const { return false; }
};

struct init_per_neuron {
	struct neuron {
		float V       = 0;
		int32_t Twait = 0;
	};
	void init(neuron& n, Int id, auto& rng) const {
		n.V     = 0.02f * util::generate_canonical<float>(rng);
		n.Twait = (int32_t)(id % 7);
	}
	SPICE_HD bool update(neuron&, float, auto&) const { return false; }
};

struct init_per_population {
	struct neuron {
		float V = 0;
	};
	void init(std::span<neuron> ns, auto& rng) const {
		for (auto& n : ns) n.V = util::generate_canonical<float>(rng);
	}
	SPICE_HD bool update(neuron&, float, auto&) const { return false; }
};

// a per-synapse weight drawn at construction, delivered into the built-in LIF's V
struct drawn_weight {
	float wmax;
	struct synapse {
		float pad = 0;
		float w   = 0;
	};
	void init(synapse& s, Int, Int, auto& rng) const { s.w = wmax * util::generate_canonical<float>(rng); }
	SPICE_HD void deliver(synapse const& s, models::lif::neuron& to) const { to.V += s.w; }
};

// a constant added to V; the member is found by calling deliver() on probe values
struct add_constant {
	float c;
	SPICE_HD void deliver(models::lif::neuron& to) const { to.V += c; }
};

struct counter_draws {
	struct neuron {
		float u = 0;
	};
	SPICE_HD bool update(neuron& n, float, auto& rng) const {
		n.u = util::generate_canonical<float>(rng);
		return false;
	}
};

template <class P>
static void print_raster(std::vector<std::vector<std::vector<int32_t>>> const& r, P const&) {
	printf("\"raster\": [");
	for (size_t t = 0; t < r.size(); t++) {
		printf("%s[", t ? "," : "");
		for (size_t k = 0; k < r[t].size(); k++) {
			printf("%s[", k ? "," : "");
			for (size_t j = 0; j < r[t][k].size(); j++) printf("%s%d", j ? "," : "", r[t][k][j]);
			printf("]");
		}
		printf("]");
	}
	printf("]");
}

int main(int argc, char** argv) {
	if (argc < 2) return 2;
	char const* what = argv[1];
	if (!strcmp(what, "stream")) {
		int const N = atoi(argv[2]), steps = atoi(argv[3]);
		unsigned const seed = (unsigned)atoi(argv[4]);
		snn net(1e-4f, 1e-4f, {seed});
		auto S = net.add_population<stream_poisson>(N);
		std::vector<std::vector<std::vector<int32_t>>> r;
		for (int t = 0; t < steps; t++) {
			net.step();
			r.push_back({S->spikes(0)});
		}
		printf("{");
		print_raster(r, S);
		printf("}\n");
	} else if (!strcmp(what, "init")) {
		int const N = atoi(argv[2]);
		unsigned const seed = (unsigned)atoi(argv[3]);
		snn net(1e-4f, 1e-4f, {seed});
		auto A = net.add_population<init_per_neuron>(N);
		auto B = net.add_population<init_per_population>(N);
		auto a = A->get_neurons();
		auto b = B->get_neurons();
		printf("{\"V\": [");
		for (int i = 0; i < N; i++) printf("%s%.9g", i ? "," : "", a[i].V);
		printf("], \"T\": [");
		for (int i = 0; i < N; i++) printf("%s%d", i ? "," : "", a[i].Twait);
		printf("], \"U\": [");
		for (int i = 0; i < N; i++) printf("%s%.9g", i ? "," : "", b[i].V);
		printf("]}\n");
	} else if (!strcmp(what, "weights")) {
		int const N = atoi(argv[2]);
		double const p = atof(argv[3]);
		int const steps = atoi(argv[4]);
		unsigned const seed = (unsigned)atoi(argv[5]);
		snn net(1e-4f, 3e-4f, {seed});
		auto P = net.add_population<models::poisson>(N, {300.0f});
		auto E = net.add_population<models::lif>(N);
		net.connect<drawn_weight>(P, E, fixed_probability(p), 3e-4f, {0.004f});
		net.connect<add_constant>(E, E, fixed_probability(p), 2e-4f, {-0.001f});
		std::vector<std::vector<std::vector<int32_t>>> r;
		for (int t = 0; t < steps; t++) {
			net.step();
			r.push_back({P->spikes(0), E->spikes(0)});
		}
		auto e = E->get_neurons();
		printf("{");
		print_raster(r, P);
		printf(", \"V\": [");
		for (int i = 0; i < N; i++) printf("%s%.9g", i ? "," : "", e[i].V);
		printf("]}\n");
	} else if (!strcmp(what, "counter")) {
		int const N = atoi(argv[2]), steps = atoi(argv[3]);
		unsigned const seed = (unsigned)atoi(argv[4]);
		snn net(1e-4f, 1e-4f, {seed});
		auto C = net.add_population<counter_draws>(N);
		auto D = net.add_population<counter_draws>(N);
		net.run(steps);
		auto c = C->get_neurons();
		auto d = D->get_neurons();
		printf("{\"u\": [");
		for (int i = 0; i < N; i++) printf("%s%.9g", i ? "," : "", c[i].u);
		printf("], \"v\": [");
		for (int i = 0; i < N; i++) printf("%s%.9g", i ? "," : "", d[i].u);
		printf("]}\n");
	} else {
		return 2;
	}
	return 0;
}
