// Synapses whose deliver() is user code rather than an addition (include/spice/snn.h), one case per
// argument (prints JSON):
//   sssp V E SRC STEPS SEED  shortest paths on a random graph of V vertices and E edges (adj_list,
//                            edge weights 1..9 from init(synapse&, src, dst, rng)): deliver() reads
//                            the firing vertex's distance and lowers the target's (the reference's
//                            samples/sssp.cpp with the predecessor kept as an index).  Source and
//                            target are one population, so the order of deliveries is the reference's
//                            exactly.  Prints the CSR, the weights, the raster and the final vertices.
//   pingpong N STEPS         samples/ping_pong.cpp: two populations of N/2 setting each other's flag
//                            through 1:1 synapses; prints the per-step spike counts.
//   relay NA NB P STEPS SEED a stateful source population firing on a schedule, into a collector
//                            population through two connections: a stateful synapse with a weight
//                            drawn by init(synapse&, src, dst, rng), whose deliver() reads the source
//                            (sum += w * level, a count, the largest source id), and a stateless
//                            deliver(src, dst) taking a maximum, delay 3 steps.  Prints both CSRs,
//                            the weights and the final states of both populations.
//   nvcc -std=c++20 -gencode arch=compute_103a,code=sm_103a -fmad=false -I include deliver_functors.cu \
//        -L spice2_gb300 -lspice_gb300 -o deliver_functors
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "spice/snn.h"

using namespace spice;

static Int edge_weight(Int s, Int d) { return 1 + (s * 7919 + d * 104729) % 9; }

struct vertex {
	Int src;
	struct neuron {
		Int distance = std::numeric_limits<Int>::max();
		Int id       = -1;
		Int previous = -1;
		bool fire    = false;
	};
	void init(neuron& n, Int id, auto&) const {
		n.id = id;
		if (id == src) {
			n.distance = 0;
			n.previous = id;
			n.fire     = true;
		}
	}
	SPICE_HD bool update(neuron& n, float, auto&) const {
		bool const r = n.fire;
		n.fire       = false;
		return r;
	}
};
static_assert(CheckNeuron<vertex>());

struct edge {
	struct synapse {
		Int weight;
	};
	void init(synapse& s, Int src, Int dst, auto&) const { s.weight = edge_weight(src, dst); }
	SPICE_HD void deliver(synapse const& s, vertex::neuron const& from, vertex::neuron& to) const {
		if (from.distance + s.weight < to.distance) {
			to.distance = from.distance + s.weight;
			to.previous = from.id;
			to.fire     = true;
		}
	}
};
static_assert(CheckSynapse<edge>());

struct flag_neuron {
	bool initial;
	struct neuron {
		bool spike_next;
	};
	void init(neuron& n, Int, auto&) const { n.spike_next = initial; }
	SPICE_HD bool update(neuron& n, float, auto&) const {
		bool const r = n.spike_next;
		n.spike_next = false;
		return r;
	}
};

struct set_flag {
	SPICE_HD void deliver(flag_neuron::neuron& n) const { n.spike_next = true; }
};

struct ticker {
	struct neuron {
		float level;
		int32_t id;
		int32_t t;
	};
	void init(neuron& n, Int id, auto& rng) const {
		n.level = util::generate_canonical<float>(rng);
		n.id    = (int32_t)id;
		n.t     = 0;
	}
	SPICE_HD bool update(neuron& n, float, auto&) const {
		n.t++;
		n.level += 0.25f;
		return (n.id + n.t) % 7 == 0;
	}
};

struct collector {
	struct neuron {
		float sum      = 0;
		float peak     = 0;
		int32_t hits   = 0;
		int32_t maxsrc = -1;
	};
	SPICE_HD bool update(neuron&, float, auto&) const { return false; }
};

struct weighted_relay {
	struct synapse {
		float w;
	};
	void init(synapse& s, Int, Int, auto& rng) const { s.w = util::generate_canonical<float>(rng); }
	SPICE_HD void deliver(synapse const& s, ticker::neuron const& from, collector::neuron& to) const {
		to.sum += s.w * from.level;
		to.hits++;
		if (from.id > to.maxsrc) to.maxsrc = from.id;
	}
};

struct peak_relay {
	SPICE_HD void deliver(ticker::neuron const& from, collector::neuron& to) const {
		if (from.level > to.peak) to.peak = from.level;
	}
};

static void print_csr(snn& net, int conn) {
	int64_t src = 0, n = 0;
	spice_conn_size(net.handle(), conn, &src, &n);
	std::vector<int64_t> off((size_t)src + 1);
	std::vector<int32_t> nb((size_t)std::max<int64_t>(n, 1));
	spice_get_csr(net.handle(), conn, off.data(), nb.data());
	printf("{\"off\": [");
	for (int64_t i = 0; i <= src; i++) printf("%s%lld", i ? "," : "", (long long)off[i]);
	printf("], \"nb\": [");
	for (int64_t i = 0; i < n; i++) printf("%s%d", i ? "," : "", nb[i]);
	printf("]}");
}

static uint64_t splitmix(uint64_t& x) {
	uint64_t z = (x += 0x9e3779b97f4a7c15ull);
	z          = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
	z          = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
	return z ^ (z >> 31);
}

int main(int argc, char** argv) {
	if (argc < 2) return 2;
	char const* what = argv[1];
	if (!strcmp(what, "sssp")) {
		Int const V = atoll(argv[2]), E = atoll(argv[3]), src = atoll(argv[4]);
		int const steps = atoi(argv[5]);
		uint64_t x      = (uint64_t)atoll(argv[6]);
		snn net(1, 1, {1337});
		auto vs = net.add_population<vertex>(V, {src});
		adj_list adj;
		for (Int e = 0; e < E; e++) {
			Int const a = (Int)(splitmix(x) % (uint64_t)V), b = (Int)(splitmix(x) % (uint64_t)V);
			if (a != b) adj.connect(a, b);
		}
		int const c = net.connect<edge>(vs, vs, adj, 1);
		printf("{\"csr\": ");
		print_csr(net, c);
		printf(", \"raster\": [");
		for (int t = 0; t < steps; t++) {
			net.step();
			auto const s = vs->spikes(0);
			printf("%s[", t ? "," : "");
			for (size_t j = 0; j < s.size(); j++) printf("%s%d", j ? "," : "", (int)s[j]);
			printf("]");
		}
		auto const w = net.get_synapses<edge>(c);
		printf("], \"w\": [");
		for (size_t i = 0; i < w.size(); i++) printf("%s%lld", i ? "," : "", (long long)w[i].weight);
		auto const n = vs->get_neurons();
		printf("], \"distance\": [");
		for (Int i = 0; i < V; i++)
			printf("%s%lld", i ? "," : "", n[i].distance == std::numeric_limits<Int>::max() ? -1LL : (long long)n[i].distance);
		printf("], \"previous\": [");
		for (Int i = 0; i < V; i++) printf("%s%lld", i ? "," : "", (long long)n[i].previous);
		printf("], \"fire\": [");
		for (Int i = 0; i < V; i++) printf("%s%d", i ? "," : "", (int)n[i].fire);
		printf("]}\n");
	} else if (!strcmp(what, "pingpong")) {
		Int const N = atoll(argv[2]);
		int const steps = atoi(argv[3]);
		snn net(1, 1, {1337});
		auto ping = net.add_population<flag_neuron>(N / 2, {true});
		auto pong = net.add_population<flag_neuron>(N / 2, {false});
		adj_list adj;
		for (Int i = 0; i < N / 2; i++) adj.connect(i, i);
		net.connect<set_flag>(ping, pong, adj, 1);
		net.connect<set_flag>(pong, ping, adj, 1);
		printf("{\"counts\": [");
		for (int t = 0; t < steps; t++) {
			net.step();
			printf("%s[%zu,%zu]", t ? "," : "", ping->spikes(0).size(), pong->spikes(0).size());
		}
		printf("]}\n");
	} else if (!strcmp(what, "relay")) {
		Int const NA = atoll(argv[2]), NB = atoll(argv[3]);
		double const p = atof(argv[4]);
		int const steps = atoi(argv[5]);
		unsigned const seed = (unsigned)atoi(argv[6]);
		snn net(1e-4f, 3e-4f, {seed});
		auto A = net.add_population<ticker>(NA);
		auto B = net.add_population<collector>(NB);
		int const c0 = net.connect<weighted_relay>(A, B, fixed_probability(p), 3e-4f);
		adj_list adj;
		for (Int i = 0; i < NA; i++)
			for (Int j = i % 3; j < NB; j += 5) adj.connect(i, j);
		int const c1 = net.connect<peak_relay>(A, B, adj, 3e-4f);
		auto const a0 = A->get_neurons();
		printf("{\"level0\": [");
		for (Int i = 0; i < NA; i++) printf("%s%.9g", i ? "," : "", a0[i].level);
		net.run(steps);
		printf("], \"csr0\": ");
		print_csr(net, c0);
		printf(", \"csr1\": ");
		print_csr(net, c1);
		auto const w = net.get_synapses<weighted_relay>(c0);
		printf(", \"w\": [");
		for (size_t i = 0; i < w.size(); i++) printf("%s%.9g", i ? "," : "", w[i].w);
		auto const a = A->get_neurons();
		auto const b = B->get_neurons();
		printf("], \"level\": [");
		for (Int i = 0; i < NA; i++) printf("%s%.9g", i ? "," : "", a[i].level);
		printf("], \"sum\": [");
		for (Int i = 0; i < NB; i++) printf("%s%.9g", i ? "," : "", b[i].sum);
		printf("], \"peak\": [");
		for (Int i = 0; i < NB; i++) printf("%s%.9g", i ? "," : "", b[i].peak);
		printf("], \"hits\": [");
		for (Int i = 0; i < NB; i++) printf("%s%d", i ? "," : "", b[i].hits);
		printf("], \"maxsrc\": [");
		for (Int i = 0; i < NB; i++) printf("%s%d", i ? "," : "", b[i].maxsrc);
		printf("]}\n");
	} else {
		return 2;
	}
	return 0;
}
