// samples/brunel.cpp of spice2 (lines 75-116) written against include/spice/snn.h: the same calls,
// running on the GPU.  Prints the raster as JSON in the format of samples/matplot.cpp:96-134
// (populations I, E, P, indices offset by the sizes before them).
//   g++ -std=c++20 -I include brunel.cpp -L spice2_gb300 -lspice_gb300 -o brunel && ./brunel [N p steps seed]
#include <cstdio>
#include <cstdlib>

#include "spice/snn.h"

using namespace spice;
using namespace spice::models;  // the samples' models, built into the engine

int main(int argc, char** argv) {
	int const N        = argc > 1 ? atoi(argv[1]) : 20000;
	double const p     = argc > 2 ? atof(argv[2]) : 0.1;
	int const steps    = argc > 3 ? atoi(argv[3]) : 300;
	unsigned const sd  = argc > 4 ? (unsigned)atoi(argv[4]) : 1337;
	float const dt     = 1e-4;
	float const delay  = 15e-4;
	double const scale = 0.1 / p;  // keeps the mean input of the published p = 0.1 network

	snn brunel(dt, delay, {sd});
	auto P = brunel.add_population<poisson>(N / 2);
	auto E = brunel.add_population<lif>(N * 4 / 10);
	auto I = brunel.add_population<lif>(N / 10);

	float const we = float(2.0 / N * scale), wi = float(-10.0 / N * scale);
	brunel.connect<fixed_weight>(P, E, fixed_probability(p), delay, {we});
	brunel.connect<fixed_weight>(P, I, fixed_probability(p), delay, {we});
	brunel.connect<fixed_weight>(E, E, fixed_probability(p), delay, {we});
	brunel.connect<fixed_weight>(E, I, fixed_probability(p), delay, {we});
	brunel.connect<fixed_weight>(I, E, fixed_probability(p), delay, {wi});
	brunel.connect<fixed_weight>(I, I, fixed_probability(p), delay, {wi});

	std::printf("{\n\t\"name\": \"Brunel\",\n\t\"spikes\": [\n");
	for (int t = 0; t < steps; t++) {
		brunel.step();
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
	return 0;
}
