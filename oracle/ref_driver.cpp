// ref_driver.cpp -- runs the spice2 reference itself (TEST INFRASTRUCTURE ONLY).
//
// Compiled by oracle/Makefile against the reference's own headers and its three source files
// (spice/src/{snn,topology,util/assert}.cpp) with the reference's Release flags
// (CMakeLists.txt:42-54, configure.sh:8), into oracle/_ref/ref_driver.  The models below are
// the ones of samples/brunel.cpp:23-70, with the Poisson rate as a member.  Tests use the
// output to pin the CPU restatement (oracle/spice_oracle.c) and the GPU engine to the
// reference; bench.py may time it as the CPU baseline where it was built.
//
// usage:
//   ref_driver net  SPEC OUT     run the network described in SPEC, write results to OUT
//   ref_driver gen  SRC DST P SEED OUT    one fixed_probability CSR (seed_seq{SEED})
//   ref_driver rng  SEED N OUT   seed chain and xoroshiro128+ draws of seed_seq{SEED}
//   ref_driver bcsr N P SEED     checksums of the six Brunel CSRs, seeded as snn seeds them:
//                                seed_seq{SEED}, one seed per stateful population (E, I), then
//                                one per connection (snn.h:21-48, neuron_population.h:56-60)
//   ref_driver brunel_ck N P SEED STEPS BLOCK OUT
//                                runs the Brunel network (samples/brunel.cpp with weights x 0.1/P)
//                                for STEPS steps and writes, per step, the spike count of P, E, I
//                                (int32 x 3) and, per block of BLOCK steps, the raster checksum of
//                                the block and the E and I state checksums at its end (uint64 x 3);
//                                the checksums are oracle.raster_checksum / state_checksum
//   ref_driver plastic_ei N SEED STEPS ETA OUT
//                                the plastic E/I network (conductance LIF, N/5 inhibitory; E->E,
//                                E->I excitatory 0.03, I->I inhibitory 0.3, I->E the iSTDP synapse
//                                below from W 0.3, all fixed_probability(0.02), delay 1 step,
//                                dt 1e-4): per step the spike count of E and I (int32 x 2), then per
//                                population the pooled inter-spike intervals in steps (count, sum,
//                                sum of squares: double x 3), then the build and run seconds
//
// SPEC (text):  dt max_delay seed steps dump_csr
//               pop poisson SIZE RATE | pop lif SIZE | pop lif_cond SIZE
//               conn SRC DST P DELAY WEIGHT        (fixed_probability + fixed_weight into a lif)
//               conn SRC DST P DELAY WEIGHT FIELD  (into a lif_cond: FIELD 1 excitatory (Gex),
//                                                   2 inhibitory (Gin), samples/vogels.cpp:48-60)
//               adj SRC DST DELAY WEIGHT M s0 d0 s1 d1 ...   (adj_list + fixed_weight)
//               wconn SRC DST P DELAY WMAX [FIELD] (fixed_probability + weighted: a per-synapse
//                                                   weight wmax * canonical<float> drawn at
//                                                   construction; FIELD as for conn)
//               stdp POP P DELAY                 (POP -> POP fixed_probability + the STDP synapse of
//                                                 samples/brunel+.cpp:58-99)
//               plastic POP P DELAY SCALE        (POP -> POP fixed_probability + count_syn; the
//                                                 reference keeps the history of a plastic
//                                                 connection's source, snn.h:44-45, so source and
//                                                 target are the same population)
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "spice/snn.h"

using namespace spice;

struct poisson {
	float rate = 20;
	bool update(float dt, auto& rng) const { return util::generate_canonical<float>(rng) < (rate * dt); }
};

struct lif {
	struct neuron {
		float V   = 0;
		int Twait = 0;
	};
	bool update(neuron& n, float dt, auto) const {
		float const TmemInv = 1.0 / 0.02;
		float const Vrest   = 0.0;
		int const Tref      = 20;
		float const Vthres  = 0.02;
		if (--n.Twait <= 0) {
			if (n.V > Vthres) {
				n.V     = Vrest;
				n.Twait = Tref;
				return true;
			}
			n.V += (Vrest - n.V) * (dt * TmemInv);
		}
		return false;
	}
};

// The conductance-based LIF of samples/vogels.cpp:10-46, as written there.
struct lif_cond {
	struct neuron {
		float V     = -0.06;
		float Gex   = 0;
		float Gin   = 0;
		Int32 Twait = 0;
	};

	bool update(neuron& n, float const dt, auto&) const {
		Int32 const Tref    = 50;          // dt
		float const Vrest   = -0.06;       // v
		float const Vthres  = -0.05;       // v
		float const TmemInv = 1.0f / 0.02; // s
		float const Eex     = 0.0;         // v
		float const Ein     = -0.08;       // v
		float const Ibg     = 0.02;        // v

		float const TexInv = 1.0f / 0.005; // s
		float const TinInv = 1.0f / 0.01;  // s

		bool spiked = false;
		if (--n.Twait <= 0) {
			if (n.V > Vthres) {
				n.V     = Vrest;
				n.Twait = Tref;
				spiked  = true;
			} else
				n.V += ((Vrest - n.V) + n.Gex * (Eex - n.V) + n.Gin * (Ein - n.V) + Ibg) *
				       (dt * TmemInv);
		}

		n.Gex -= n.Gex * (dt * TexInv);
		n.Gin -= n.Gin * (dt * TinInv);

		return spiked;
	}
};

struct fixed_weight {
	float weight;
	void deliver(lif::neuron& to) const { to.V += weight; }
};

// samples/vogels.cpp:48-60
struct excitatory {
	float weight;
	void deliver(lif_cond::neuron& to) const { to.Gex += weight; }
};
struct inhibitory {
	float weight;
	void deliver(lif_cond::neuron& to) const { to.Gin += weight; }
};

// A stateful synapse whose weight is drawn per synapse when the connection is built (the
// reference's PerSynapseInit concept, synapse_population.h:34-41: one xoroshiro128+ stream seeded
// after the adjacency's, walked in CSR order): w = wmax * canonical<float>.  A single multiply by a
// value whose scaling is a power of two, so the fast-math build cannot round it differently.
struct weighted {
	float wmax;
	struct synapse {
		float w = 0;
	};
	void init(synapse& s, Int, Int, auto& rng) const { s.w = wmax * util::generate_canonical<float>(rng); }
	void deliver(synapse const& s, lif::neuron& to) const { to.V += s.w; }
};
struct weighted_ex {
	float wmax;
	struct synapse {
		float w = 0;
	};
	void init(synapse& s, Int, Int, auto& rng) const { s.w = wmax * util::generate_canonical<float>(rng); }
	void deliver(synapse const& s, lif_cond::neuron& to) const { to.Gex += s.w; }
};
struct weighted_in {
	float wmax;
	struct synapse {
		float w = 0;
	};
	void init(synapse& s, Int, Int, auto& rng) const { s.w = wmax * util::generate_canonical<float>(rng); }
	void deliver(synapse const& s, lif_cond::neuron& to) const { to.Gin += s.w; }
};

// The counting plastic synapse of test/detail/synapse_population.cpp:84-94 (update adds 1, skip
// adds n), delivering scale * count so the lazy schedule shows in the targets' V.  scale is a power
// of two: the product is exact and the fast-math build cannot round it differently.
struct count_syn {
	float scale;
	struct synapse {
		int count = 0;
	};
	void deliver(synapse const& s, lif::neuron& to) const { to.V += s.count * scale; }
	void update(synapse& s, float, bool, bool) const { s.count++; }
	void skip(synapse& s, float, Int n) const { s.count += n; }
};

// The plastic synapse of samples/brunel+.cpp:58-99 (weight W, pre / post traces Zpre / Zpost).
struct stdp_syn {
	struct synapse {
		float W     = 1e-4;
		float Zpre  = 0;
		float Zpost = 0;
	};
	void deliver(synapse const& syn, lif::neuron& to) const { to.V += syn.W; }
	void update(synapse& syn, float const dt, bool const pre, bool const post) const {
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
	void skip(synapse& syn, float const dt, Int const n) const {
		float const TstdpInv = 1.0f / 0.02f;
		syn.Zpre *= std::pow(1 - dt * TstdpInv, n);
		syn.Zpost *= std::pow(1 - dt * TstdpInv, n);
	}
};

// Inhibitory symmetric STDP (Vogels et al. 2011) against the PlasticSynapse concept: at a pre
// spike W += eta (xpost - 2 rho0 tau), floored at 0; at a post spike W += eta xpre; the traces jump
// by 1 and decay by x -= x dt / tau per step, skip(n) multiplies them by (1 - dt / tau)^n.
struct istdp {
	float eta, alpha, tau_inv;
	struct synapse {
		float W = 0.3f;
		float A = 0;
		float B = 0;
	};
	void deliver(synapse const& s, lif_cond::neuron& to) const { to.Gin += s.W; }
	void update(synapse& s, float const dt, bool const pre, bool const post) const {
		if (pre) s.W = std::max(0.0f, s.W + eta * (s.B - alpha));
		if (post) s.W += eta * s.A;
		s.A += pre;
		s.B += post;
		s.A -= s.A * (dt * tau_inv);
		s.B -= s.B * (dt * tau_inv);
	}
	void skip(synapse& s, float const dt, Int const n) const {
		s.A *= std::pow(1 - dt * tau_inv, n);
		s.B *= std::pow(1 - dt * tau_inv, n);
	}
};

// A plastic synapse that is never built (p = 0): connecting it from a population makes the
// reference keep that population's spike history (snn.h:44-45), which the catch-up of a plastic
// connection INTO the population reads (snn.cpp:17-25 pass c.to->history()).
struct history_only {
	struct synapse {
		float W = 0;
	};
	void deliver(synapse const&, lif_cond::neuron&) const {}
	void update(synapse&, float, bool, bool) const {}
	void skip(synapse&, float, Int) const {}
};

std::vector<float> g_dt;
struct dt_probe {
	bool update(float dt, auto&) const {
		g_dt.push_back(dt);
		return false;
	}
};

template <class T>
static void put(FILE* f, T const& v) { fwrite(&v, sizeof(T), 1, f); }

static int run_gen(int argc, char** argv) {
	if (argc < 7) return 2;
	Int src = atoll(argv[2]), dst = atoll(argv[3]);
	double p = atof(argv[4]);
	unsigned seed = (unsigned)atoll(argv[5]);
	fixed_probability fp(p);
	fp(src, dst);
	std::vector<Int> off(src + 1);
	std::vector<Int32> nb(fp.size());
	fp.generate(off, nb, util::seed_seq{seed});
	FILE* f = fopen(argv[6], "wb");
	Int md = src > 0 ? fp.size() / src : 0;
	put(f, md);
	put(f, off[src]);
	fwrite(off.data(), sizeof(Int), off.size(), f);
	fwrite(nb.data(), sizeof(Int32), off[src], f);
	fclose(f);
	return 0;
}

// Order-sensitive checksum of a CSR with wrapping 64-bit arithmetic (the same function as
// oracle.csr_checksum in oracle/oracle.py).
static UInt csr_checksum(std::vector<Int> const& off, std::vector<Int32> const& nb, Int n) {
	UInt h1 = 0, h2 = 0;
	for (size_t i = 0; i < off.size(); i++)
		h1 += (UInt(off[i]) + 1) * ((UInt(i) * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) | 1);
	for (Int j = 0; j < n; j++)
		h2 += (UInt(UInt32(nb[j])) + 1) * ((UInt(j) * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull) | 1);
	return h1 ^ ((h2 << 1) | (h2 >> 63));
}

static int run_bcsr(int argc, char** argv) {
	if (argc < 5) return 2;
	Int const N = atoll(argv[2]);
	double const p = atof(argv[3]);
	unsigned const seed = (unsigned)atoll(argv[4]);
	util::seed_seq s{seed};
	s++;  // E (stateful)
	s++;  // I (stateful)
	Int const sz[3] = {N / 2, N * 4 / 10, N / 10};
	int const pr[6][2] = {{0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 1}, {2, 2}};
	for (auto& q : pr) {
		fixed_probability fp(p);
		fp(sz[q[0]], sz[q[1]]);
		std::vector<Int> off(sz[q[0]] + 1);
		std::vector<Int32> nb(fp.size());
		fp.generate(off, nb, s++);
		printf("%d %d %lld %llu\n", q[0], q[1], (long long)off.back(),
		       (unsigned long long)csr_checksum(off, nb, off.back()));
	}
	return 0;
}

// Order-sensitive checksums of a raster block and of a LIF population's state (the same functions
// as oracle.raster_checksum / oracle.state_checksum in oracle/oracle.py).
struct raster_ck {
	UInt a = 0, b = 0, j = 0, i = 0;
	void add_count(Int n) { b += (UInt(n) + 7) * ((i++ * 0xD1B54A32D192ED03ull) | 1); }
	void add_spike(Int32 x) { a += (UInt(Int(x)) + 1) * ((j++ * 0x9E3779B97F4A7C15ull) | 1); }
	UInt value() const { return a ^ b; }
};

static UInt state_ck(std::span<lif::neuron const> ns) {
	UInt h1 = 0, h2 = 0, i = 0;
	for (auto const& n : ns) {
		UInt32 v;
		memcpy(&v, &n.V, 4);
		h1 += (UInt(v) + 3) * ((i * 0x9E3779B97F4A7C15ull) | 1);
		h2 += (UInt(UInt32(Int32(n.Twait))) + 5) * ((i * 0xD1B54A32D192ED03ull) | 1);
		i++;
	}
	return h1 ^ h2;
}

static int run_brunel_ck(int argc, char** argv) {
	if (argc < 8) return 2;
	Int const N = atoll(argv[2]);
	double const p = atof(argv[3]);
	unsigned const seed = (unsigned)atoll(argv[4]);
	Int const steps = atoll(argv[5]), block = atoll(argv[6]);
	if (block < 1) return 2;
	float const dt = 1e-4f, delay = 15e-4f;
	snn net(dt, delay, {seed});
	auto* P = net.add_population<poisson>(N / 2, {20.0f});
	auto* E = net.add_population<lif>(N * 4 / 10);
	auto* I = net.add_population<lif>(N / 10);
	float const we = (float)((2.0 / N) * (0.1 / p)), wi = (float)((-10.0 / N) * (0.1 / p));
	net.connect<fixed_weight>(P, E, fixed_probability(p), delay, {we});
	net.connect<fixed_weight>(P, I, fixed_probability(p), delay, {we});
	net.connect<fixed_weight>(E, E, fixed_probability(p), delay, {we});
	net.connect<fixed_weight>(E, I, fixed_probability(p), delay, {we});
	net.connect<fixed_weight>(I, E, fixed_probability(p), delay, {wi});
	net.connect<fixed_weight>(I, I, fixed_probability(p), delay, {wi});
	FILE* f = fopen(argv[7], "wb");
	if (!f) return 2;
	detail::NeuronPopulation* pops[3] = {P, E, I};
	raster_ck ck;
	for (Int t = 0; t < steps; t++) {
		net.step();
		for (auto* q : pops) {
			auto sp = q->spikes(0);
			put(f, (Int32)sp.size());
			ck.add_count((Int)sp.size());
		}
		for (auto* q : pops)
			for (Int32 x : q->spikes(0)) ck.add_spike(x);
		if ((t + 1) % block == 0 || t + 1 == steps) {
			put(f, ck.value());
			put(f, state_ck(E->get_neurons()));
			put(f, state_ck(I->get_neurons()));
			ck = raster_ck{};
		}
	}
	fclose(f);
	return 0;
}

static int run_plastic_ei(int argc, char** argv) {
	if (argc < 7) return 2;
	Int const N = atoll(argv[2]);
	unsigned const seed = (unsigned)atoll(argv[3]);
	Int const steps = atoll(argv[4]);
	float const eta = (float)atof(argv[5]);
	float const dt = 1e-4f;
	auto t0 = std::chrono::steady_clock::now();
	snn net(dt, dt, {seed});
	auto* E = net.add_population<lif_cond>(N * 8 / 10);
	auto* I = net.add_population<lif_cond>(N * 2 / 10);
	net.connect<excitatory>(E, E, fixed_probability(0.02), dt, {0.03f});
	net.connect<excitatory>(E, I, fixed_probability(0.02), dt, {0.03f});
	net.connect<istdp>(I, E, fixed_probability(0.02), dt, {eta, 2.0f * 5.0f * 0.02f, 1.0f / 0.02f});
	net.connect<inhibitory>(I, I, fixed_probability(0.02), dt, {0.3f});
	net.connect<history_only>(E, E, fixed_probability(0.0), dt);
	auto t1 = std::chrono::steady_clock::now();
	FILE* f = fopen(argv[6], "wb");
	if (!f) return 2;
	detail::NeuronPopulation* pops[2] = {E, I};
	std::vector<Int> last[2] = {std::vector<Int>(E->size(), -1), std::vector<Int>(I->size(), -1)};
	double isi[2][3] = {};
	for (Int t = 0; t < steps; t++) {
		net.step();
		for (int k = 0; k < 2; k++) {
			auto sp = pops[k]->spikes(0);
			put(f, (Int32)sp.size());
			for (Int32 x : sp) {
				if (last[k][x] >= 0) {
					double const d = double(t - last[k][x]);
					isi[k][0] += 1;
					isi[k][1] += d;
					isi[k][2] += d * d;
				}
				last[k][x] = t;
			}
		}
	}
	auto t2 = std::chrono::steady_clock::now();
	for (int k = 0; k < 2; k++)
		for (int j = 0; j < 3; j++) put(f, isi[k][j]);
	put(f, std::chrono::duration<double>(t1 - t0).count());
	put(f, std::chrono::duration<double>(t2 - t1).count());
	fclose(f);
	return 0;
}

static int run_rng(int argc, char** argv) {
	if (argc < 5) return 2;
	unsigned seed = (unsigned)atoll(argv[2]);
	Int n = atoll(argv[3]);
	util::seed_seq s{seed};
	FILE* f = fopen(argv[4], "wb");
	for (Int i = 0; i < n; i++) {  // seed chain
		UInt128 v = s++.seed();
		put(f, v.lo);
		put(f, v.hi);
	}
	util::xoroshiro64_128p rng(util::seed_seq{seed});
	for (Int i = 0; i < n; i++) put(f, rng());
	util::xoroshiro64_128p rng2(util::seed_seq{seed});
	util::exponential_distribution<double> ex(499.0);
	for (Int i = 0; i < n; i++) put(f, ex(rng2));
	util::xoroshiro64_128p rng3(util::seed_seq{seed});
	for (Int i = 0; i < n; i++) put(f, util::generate_canonical<float>(rng3));
	util::kahan_sum<float> k;
	for (Int i = 0; i < n; i++) {
		float y = k += 1e-4f;
		if (k >= 1) k.reset();
		put(f, y);
	}
	fclose(f);
	return 0;
}

struct pop_rec {
	int kind;  // 0 poisson, 1 lif, 2 lif_cond
	Int size;
	detail::NeuronPopulation* base;
	detail::neuron_population<lif>* L;
	detail::neuron_population<lif_cond>* C;
	bool is_lif() const { return kind == 1; }
};

// net.connect<Syn>(pops[s], to, topo, delay, {w}) with the source population's own type.
template <class Syn, class To, class Topo>
static void connect_from(snn& net, pop_rec const& s, To* to, Topo&& topo, float delay, float w) {
	if (s.kind == 1) net.connect<Syn>(s.L, to, topo, delay, {w});
	else if (s.kind == 2) net.connect<Syn>(s.C, to, topo, delay, {w});
	else net.connect<Syn>(static_cast<detail::neuron_population<poisson>*>(s.base), to, topo, delay, {w});
}

static int run_net(int argc, char** argv) {
	if (argc < 4) return 2;
	std::ifstream in(argv[2]);
	float dt, max_delay;
	unsigned seed;
	Int steps;
	int dump_csr;
	in >> dt >> max_delay >> seed >> steps >> dump_csr;
	auto t0 = std::chrono::steady_clock::now();
	snn net(dt, max_delay, {seed});
	std::vector<pop_rec> pops;
	std::string kw;
	while (in >> kw) {
		if (kw == "pop") {
			std::string kind;
			Int size;
			in >> kind >> size;
			if (kind == "poisson") {
				float rate;
				in >> rate;
				auto* P = net.add_population<poisson>(size, {rate});
				pops.push_back({0, size, P, nullptr, nullptr});
			} else if (kind == "lif_cond") {
				auto* C = net.add_population<lif_cond>(size);
				pops.push_back({2, size, C, nullptr, C});
			} else {
				auto* L = net.add_population<lif>(size);
				pops.push_back({1, size, L, L, nullptr});
			}
		} else if (kw == "stdp") {
			Int q;
			double p;
			float delay;
			in >> q >> p >> delay;
			net.connect<stdp_syn>(pops[q].L, pops[q].L, fixed_probability(p), delay);
		} else if (kw == "plastic") {
			Int q;
			double p;
			float delay, scale;
			in >> q >> p >> delay >> scale;
			net.connect<count_syn>(pops[q].L, pops[q].L, fixed_probability(p), delay, {scale});
		} else if (kw == "wconn") {
			Int s, d;
			double p;
			float delay, w;
			in >> s >> d >> p >> delay >> w;
			int field = 0;
			if (pops[d].kind == 2) in >> field;
			if (pops[d].kind == 1) connect_from<weighted>(net, pops[s], pops[d].L, fixed_probability(p), delay, w);
			else if (field == 1) connect_from<weighted_ex>(net, pops[s], pops[d].C, fixed_probability(p), delay, w);
			else connect_from<weighted_in>(net, pops[s], pops[d].C, fixed_probability(p), delay, w);
		} else if (kw == "conn" || kw == "adj") {
			Int s, d;
			in >> s >> d;
			double p = 0;
			if (kw == "conn") in >> p;
			float delay, w;
			in >> delay >> w;
			int field = 0;
			if (pops[d].kind == 2) in >> field;
			adj_list adj;
			if (kw == "adj") {
				Int m;
				in >> m;
				for (Int i = 0; i < m; i++) {
					Int a, b;
					in >> a >> b;
					adj.connect(a, b);
				}
			}
			if (pops[d].kind == 1) {
				if (kw == "conn") connect_from<fixed_weight>(net, pops[s], pops[d].L, fixed_probability(p), delay, w);
				else connect_from<fixed_weight>(net, pops[s], pops[d].L, adj, delay, w);
			} else if (field == 1) {
				if (kw == "conn") connect_from<excitatory>(net, pops[s], pops[d].C, fixed_probability(p), delay, w);
				else connect_from<excitatory>(net, pops[s], pops[d].C, adj, delay, w);
			} else {
				if (kw == "conn") connect_from<inhibitory>(net, pops[s], pops[d].C, fixed_probability(p), delay, w);
				else connect_from<inhibitory>(net, pops[s], pops[d].C, adj, delay, w);
			}
		}
	}
	net.add_population<dt_probe>(1);  // stateless: consumes no seed and no draw
	auto t1 = std::chrono::steady_clock::now();
	FILE* f = fopen(argv[3], "wb");
	put(f, (Int)pops.size());
	for (auto& p : pops) put(f, p.size);
	put(f, steps);
	std::vector<std::vector<std::vector<Int32>>> raster(steps);
	for (Int t = 0; t < steps; t++) {
		net.step();
		raster[t].resize(pops.size());
		for (size_t k = 0; k < pops.size(); k++) {
			auto sp = pops[k].base->spikes(0);
			raster[t][k].assign(sp.begin(), sp.end());
		}
	}
	auto t2 = std::chrono::steady_clock::now();
	fwrite(g_dt.data(), sizeof(float), g_dt.size(), f);
	for (Int t = 0; t < steps; t++)
		for (size_t k = 0; k < pops.size(); k++) {
			put(f, (Int)raster[t][k].size());
			fwrite(raster[t][k].data(), sizeof(Int32), raster[t][k].size(), f);
		}
	for (auto& p : pops)
		if (p.kind == 1)
			for (auto& n : p.L->get_neurons()) {
				put(f, n.V);
				put(f, (Int32)n.Twait);
			}
		else if (p.kind == 2)
			for (auto& n : p.C->get_neurons()) {
				put(f, n.V);
				put(f, n.Gex);
				put(f, n.Gin);
				put(f, (Int32)n.Twait);
			}
	put(f, std::chrono::duration<double>(t1 - t0).count());
	put(f, std::chrono::duration<double>(t2 - t1).count());
	fclose(f);
	(void)dump_csr;  // reserved
	return 0;
}

int main(int argc, char** argv) {
	if (argc < 2) return 2;
	try {
		if (!strcmp(argv[1], "net")) return run_net(argc, argv);
		if (!strcmp(argv[1], "gen")) return run_gen(argc, argv);
		if (!strcmp(argv[1], "rng")) return run_rng(argc, argv);
		if (!strcmp(argv[1], "bcsr")) return run_bcsr(argc, argv);
		if (!strcmp(argv[1], "brunel_ck")) return run_brunel_ck(argc, argv);
		if (!strcmp(argv[1], "plastic_ei")) return run_plastic_ei(argc, argv);
	} catch (std::exception const& e) {
		fprintf(stderr, "%s\n", e.what());
		return 3;
	}
	return 2;
}
