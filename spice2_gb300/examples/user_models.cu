// The Brunel network of samples/brunel.cpp written with user-defined models: a stateless Poisson
// source, a stateful LIF and a weight synapse, all plain C++ structs with the reference's
// update()/deliver() signatures, compiled into GPU kernels by include/spice/snn.h.  The LIF
// update is written the way the reference's -ffast-math build executes its leak
// (V * fma(-dt, 1/tau, 1)), so the raster equals the reference's.  Prints the raster as JSON
// (samples/matplot.cpp:96-134).
//   nvcc -std=c++20 -gencode arch=compute_103a,code=sm_103a -fmad=false -I include user_models.cu \
//        -L spice2_gb300 -lspice_gb300 -o user_models && ./user_models [N p steps seed]
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "spice/snn.h"

using namespace spice;

struct my_poisson {
	float rate = 20;
	SPICE_HD bool update(float dt, auto& rng) const { return util::generate_canonical<float>(rng) < rate * dt; }
};

struct my_lif {
	struct neuron {
		float V     = 0;
		int32_t Twait = 0;
	};
	SPICE_HD bool update(neuron& n, float dt, auto&) const {
		if (--n.Twait <= 0) {
			if (n.V > 0.02f) {
				n.V     = 0;
				n.Twait = 20;
				return true;
			}
			n.V = n.V * fmaf(-dt, 50.0f, 1.0f);
		}
		return false;
	}
};

struct my_weight {
	float weight;
	static constexpr auto field = &my_lif::neuron::V;
	SPICE_HD void deliver(my_lif::neuron& to) const { to.V += weight; }
};

int main(int argc, char** argv) {
	int const N       = argc > 1 ? atoi(argv[1]) : 4000;
	double const p    = argc > 2 ? atof(argv[2]) : 0.05;
	int const steps   = argc > 3 ? atoi(argv[3]) : 200;
	unsigned const sd = argc > 4 ? (unsigned)atoi(argv[4]) : 1337;
	float const delay = 15e-4;

	snn net(1e-4f, delay, {sd});
	auto P = net.add_population<my_poisson>(N / 2);
	auto E = net.add_population<my_lif>(N * 4 / 10);
	auto I = net.add_population<my_lif>(N / 10);
	float const we = float(2.0 / N * (0.1 / p)), wi = float(-10.0 / N * (0.1 / p));
	net.connect<my_weight>(P, E, fixed_probability(p), delay, {we});
	net.connect<my_weight>(P, I, fixed_probability(p), delay, {we});
	net.connect<my_weight>(E, E, fixed_probability(p), delay, {we});
	net.connect<my_weight>(E, I, fixed_probability(p), delay, {we});
	net.connect<my_weight>(I, E, fixed_probability(p), delay, {wi});
	net.connect<my_weight>(I, I, fixed_probability(p), delay, {wi});

	std::printf("{\n\t\"name\": \"Brunel (user models)\",\n\t\"spikes\": [\n");
	for (int t = 0; t < steps; t++) {
		net.step();
		std::printf(t == 0 ? "\t\t[" : ",\n\t\t[");
		char const* sep = "";
		long offset     = 0;
		for (auto s : I->spikes(0)) { std::printf("%s%ld", sep, (long)s + offset); sep = ","; }
		offset += I->size();
		for (auto s : E->spikes(0)) { std::printf("%s%ld", sep, (long)s + offset); sep = ","; }
		offset += E->size();
		for (auto s : P->spikes(0)) { std::printf("%s%ld", sep, (long)s + offset); sep = ","; }
		std::printf("]");
	}
	std::printf("\n\t]\n}\n");
	double vsum = 0;
	for (auto const& n : E->get_neurons()) vsum += n.V;
	std::fprintf(stderr, "E mean V %.9g\n", vsum / E->size());
	return 0;
}
