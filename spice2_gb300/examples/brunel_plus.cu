// The plastic Brunel network of spice2's samples/brunel+.cpp (Brunel with plastic E->E synapses)
// written against include/spice/snn.h with user models: a stateless Poisson source, a stateful LIF,
// a fixed-weight synapse and the sample's STDP synapse (weight W, pre and post traces; update() on
// a pre or post spike, skip() over quiet steps) -- the reference's lazy catch-up runs them on the
// GPU.  Prints per-step spike counts of P, E, I and the E->E weight statistics as JSON.
//   nvcc -std=c++20 --expt-relaxed-constexpr -gencode arch=compute_103a,code=sm_103a -fmad=false \
//        -I include brunel_plus.cu -L spice2_gb300 -lspice_gb300 -o brunel_plus && ./brunel_plus [N steps seed]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "spice/snn.h"

using namespace spice;

struct poisson20 {
	SPICE_HD bool update(float const dt, auto& rng) const { return util::generate_canonical<float>(rng) < 20.0f * dt; }
};

struct lif {
	struct neuron {
		float V   = 0;
		int Twait = 0;
	};
	SPICE_HD bool update(neuron& n, float const dt, auto&) const {
		float const TmemInv = 1.0 / 0.02;
		if (--n.Twait <= 0) {
			if (n.V > 0.02f) {
				n.V     = 0;
				n.Twait = 20;
				return true;
			}
			n.V += (0.0f - n.V) * (dt * TmemInv);
		}
		return false;
	}
};

struct fixed_weight {
	float weight;
	SPICE_HD void deliver(lif::neuron& to) const { to.V += weight; }
};

// STDP with multiplicative depression and soft-bounded potentiation, traces of 20 ms.
struct plastic {
	struct synapse {
		float W     = 1e-4f;
		float Zpre  = 0;
		float Zpost = 0;
	};
	SPICE_HD void deliver(synapse const& syn, lif::neuron& to) const { to.V += syn.W; }
	SPICE_HD void update(synapse& syn, float const dt, bool const pre, bool const post) const {
		float const TstdpInv = 1.0f / 0.02f;
		float const dtInv    = 1.0f / dt;
		syn.W = std::clamp(syn.W - pre * 0.0202f * syn.W * std::exp(-syn.Zpost * dtInv) +
		                       post * 0.01f * (1.0f - syn.W) * std::exp(-syn.Zpre * dtInv),
		                   0.0f, 0.0003f);
		syn.Zpre += pre;
		syn.Zpost += post;
		syn.Zpre -= syn.Zpre * dt * TstdpInv;
		syn.Zpost -= syn.Zpost * dt * TstdpInv;
	}
	SPICE_HD void skip(synapse& syn, float const dt, Int const n) const {
		float const TstdpInv = 1.0f / 0.02f;
		syn.Zpre *= std::pow(1 - dt * TstdpInv, n);
		syn.Zpost *= std::pow(1 - dt * TstdpInv, n);
	}
};

int main(int argc, char** argv) {
	int const N       = argc > 1 ? atoi(argv[1]) : 20000;
	int const steps   = argc > 2 ? atoi(argv[2]) : 300;
	unsigned const sd = argc > 3 ? (unsigned)atoi(argv[3]) : 1337;
	float const dt = 1e-4, delay = 15e-4;
	snn net(dt, delay, {sd});
	auto P = net.add_population<poisson20>(N / 2);
	auto E = net.add_population<lif>(N * 4 / 10);
	auto I = net.add_population<lif>(N / 10);
	net.connect<fixed_weight>(P, E, fixed_probability(0.1), delay, {2.0f / N});
	net.connect<fixed_weight>(P, I, fixed_probability(0.1), delay, {2.0f / N});
	int const ee = net.connect<plastic>(E, E, fixed_probability(0.1), delay);
	net.connect<fixed_weight>(E, I, fixed_probability(0.1), delay, {2.0f / N});
	net.connect<fixed_weight>(I, E, fixed_probability(0.1), delay, {-10.0f / N});
	net.connect<fixed_weight>(I, I, fixed_probability(0.1), delay, {-10.0f / N});
	printf("{\"counts\": [");
	for (int t = 0; t < steps; t++) {
		net.step();
		printf("%s[%zu,%zu,%zu]", t ? "," : "", P->spikes(0).size(), E->spikes(0).size(), I->spikes(0).size());
	}
	auto const syn = net.get_synapses<plastic>(ee);
	double m = 0, m2 = 0, lo = 1e30, hi = -1e30;
	for (auto const& s : syn) {
		m += s.W;
		m2 += (double)s.W * s.W;
		lo = s.W < lo ? s.W : lo;
		hi = s.W > hi ? s.W : hi;
	}
	m /= syn.size();
	printf("], \"W_mean\": %.9g, \"W_std\": %.9g, \"W_min\": %.9g, \"W_max\": %.9g, \"synapses\": %zu}\n", m,
	       std::sqrt(m2 / syn.size() - m * m), lo, hi, syn.size());
	return 0;
}
