/*
 * spice_oracle.c -- CPU restatement of spice2's snn::step path (TEST INFRASTRUCTURE ONLY).
 *
 * Built with -O2 -ffp-contract=off and without -ffast-math so that every float
 * operation below is one IEEE-754 round-to-nearest operation, in the order written.
 * Each function cites the reference file:line (paths inside the spice2 project)
 * whose behaviour it restates.  See spice_oracle.h for the interface.
 */
#include "spice_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static char g_err[512];
const char* spo_last_error(void) { return g_err; }
static int fail(const char* msg) {
	snprintf(g_err, sizeof g_err, "%s", msg);
	return -1;
}

/* ------------------------------------------------------------------------------------------
 * RNG and seeding
 * ---------------------------------------------------------------------------------------- */
static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* random.h:19-26 */
static inline uint64_t fmix64(uint64_t k) {
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdULL;
	k ^= k >> 33;
	k *= 0xc4ceb9fe1a85ec53ULL;
	k ^= k >> 33;
	return k;
}

static const uint64_t MM_C1 = 0x87c37b91114253d5ULL;
static const uint64_t MM_C2 = 0x4cf5ad432745937fULL;
static const spo_u128 MM_H0 = {0x2E4016967F18E81ULL, 0x447567949F9AA86ULL};

/* MurmurHash3_x64_128 with the reference's fixed non-zero seed (random.h:28-107). */
spo_u128 spo_murmur3_bytes(const void* ptr, uint64_t len) {
	const uint8_t* data = (const uint8_t*)ptr;
	spo_u128 h          = MM_H0;
	int64_t nblocks     = (int64_t)(len / 16);
	for (int64_t i = 0; i < nblocks; i++) {
		uint64_t k1, k2;
		memcpy(&k1, data + 16 * i, 8);
		memcpy(&k2, data + 16 * i + 8, 8);
		k1 *= MM_C1; k1 = rotl64(k1, 31); k1 *= MM_C2; h.lo ^= k1;
		h.lo = rotl64(h.lo, 27); h.lo += h.hi; h.lo = h.lo * 5 + 0x52dce729;
		k2 *= MM_C2; k2 = rotl64(k2, 33); k2 *= MM_C1; h.hi ^= k2;
		h.hi = rotl64(h.hi, 31); h.hi += h.lo; h.hi = h.hi * 5 + 0x38495ab5;
	}
	const uint8_t* tail = data + nblocks * 16;
	uint64_t k1 = 0, k2 = 0;
	switch (len & 15) {
		case 15: k2 ^= (uint64_t)tail[14] << 48; /* fall through */
		case 14: k2 ^= (uint64_t)tail[13] << 40; /* fall through */
		case 13: k2 ^= (uint64_t)tail[12] << 32; /* fall through */
		case 12: k2 ^= (uint64_t)tail[11] << 24; /* fall through */
		case 11: k2 ^= (uint64_t)tail[10] << 16; /* fall through */
		case 10: k2 ^= (uint64_t)tail[9] << 8;   /* fall through */
		case 9:
			k2 ^= (uint64_t)tail[8];
			k2 *= MM_C2; k2 = rotl64(k2, 33); k2 *= MM_C1; h.hi ^= k2;
			/* fall through */
		case 8: k1 ^= (uint64_t)tail[7] << 56; /* fall through */
		case 7: k1 ^= (uint64_t)tail[6] << 48; /* fall through */
		case 6: k1 ^= (uint64_t)tail[5] << 40; /* fall through */
		case 5: k1 ^= (uint64_t)tail[4] << 32; /* fall through */
		case 4: k1 ^= (uint64_t)tail[3] << 24; /* fall through */
		case 3: k1 ^= (uint64_t)tail[2] << 16; /* fall through */
		case 2: k1 ^= (uint64_t)tail[1] << 8;  /* fall through */
		case 1:
			k1 ^= (uint64_t)tail[0];
			k1 *= MM_C1; k1 = rotl64(k1, 31); k1 *= MM_C2; h.lo ^= k1;
	}
	h.lo ^= len; h.hi ^= len;
	h.lo += h.hi; h.hi += h.lo;
	h.lo = fmix64(h.lo); h.hi = fmix64(h.hi);
	h.lo += h.hi; h.hi += h.lo;
	return h;
}

/* The one-block murmur3 that advances a seed_seq (random.h:108-139). */
spo_u128 spo_murmur3_u128(spo_u128 k) {
	spo_u128 h = MM_H0;
	k.lo *= MM_C1; k.lo = rotl64(k.lo, 31); k.lo *= MM_C2; h.lo ^= k.lo;
	h.lo = rotl64(h.lo, 27); h.lo += h.hi; h.lo = h.lo * 5 + 0x52dce729;
	k.hi *= MM_C2; k.hi = rotl64(k.hi, 33); k.hi *= MM_C1; h.hi ^= k.hi;
	h.hi = rotl64(h.hi, 31); h.hi += h.lo; h.hi = h.hi * 5 + 0x38495ab5;
	h.lo ^= 16; h.hi ^= 16;
	h.lo += h.hi; h.hi += h.lo;
	h.lo = fmix64(h.lo); h.hi = fmix64(h.hi);
	h.lo += h.hi; h.hi += h.lo;
	return h;
}

/* seed_seq(std::initializer_list<UInt32>) hashes the list's bytes (random.h:149-152). */
spo_u128 spo_seed_from_list(const uint32_t* seeds, int n) {
	return spo_murmur3_bytes(seeds, 4ULL * (uint64_t)n);
}

/* seed_seq::operator++(int): returns the current seed, then advances it (random.h:163-167). */
spo_u128 spo_seed_next(spo_u128* seed) {
	spo_u128 r = *seed;
	*seed      = spo_murmur3_u128(*seed);
	return r;
}

/* xoroshiro64_128p: s0 = seed.lo, s1 = seed.hi (random.h:188-192); xoroshiro128+ step with
 * rotations 24/16/37 (random.h:222-234). */
uint64_t spo_xoroshiro128p_next(uint64_t s[2]) {
	uint64_t r = s[0] + s[1];
	uint64_t t = s[0] ^ s[1];
	s[0]       = rotl64(s[0], 24) ^ t ^ (t << 16);
	s[1]       = rotl64(t, 37);
	return r;
}

/* Computes poly(T) s = sum_i poly_i T^i s: the jump used to skip ahead in a stream. */
void spo_xoroshiro128p_jump(uint64_t s[2], const uint64_t poly[2]) {
	uint64_t a0 = 0, a1 = 0;
	for (int w = 0; w < 2; w++)
		for (int b = 0; b < 64; b++) {
			if ((poly[w] >> b) & 1) { a0 ^= s[0]; a1 ^= s[1]; }
			spo_xoroshiro128p_next(s);
		}
	s[0] = a0;
	s[1] = a1;
}

/* generate_canonical<float, false> on a 64-bit engine: (u >> 40) / 2^24 (random.h:236-247). */
float spo_canonical_f32(uint64_t u) { return (float)(u >> 40) / 16777216.0f; }

/* generate_canonical<double, true>: ((u >> 11) + 1) / 2^53, i.e. (0, 1] (random.h:236-247). */
double spo_canonical_f64_leftopen(uint64_t u) {
	return (double)((u >> 11) + 1) / 9007199254740992.0;
}

/* exponential_distribution<double>::operator(): -scale * log(canonical<double, true>)
 * (random.h:264-276).  log is the C library's double log. */
double spo_exponential(double scale, uint64_t s[2]) {
	return -scale * log(spo_canonical_f64_leftopen(spo_xoroshiro128p_next(s)));
}

/* kahan_sum<float>::operator+= (numeric.h:9-15, built -fno-fast-math) followed by the reset
 * at >= 1 s in snn::step (snn.cpp:8-10).  Returns y, the dt the neurons see. */
float spo_kahan_step(spo_kahan* k, float delta) {
	float y = delta - k->c;
	float t = k->sum + y;
	k->c    = (t - k->sum) - y;
	k->sum  = t;
	if (k->sum >= 1) k->sum = 0;
	return y;
}

/* ------------------------------------------------------------------------------------------
 * fixed_probability (topology.cpp:73-112)
 * ---------------------------------------------------------------------------------------- */

/* fixed_probability::size() / src_count: floor(dst*p + 3*sqrt(dst*p*(1-p))) (topology.cpp:75-78). */
int64_t spo_fp_max_degree(int64_t dst_count, double p) {
	double m = (double)dst_count * p;
	return (int64_t)(m + 3 * sqrt(m * (1 - p)));
}

/* fixed_probability::generate (topology.cpp:78-112): one xoroshiro128+ stream per projection,
 * seeded with the projection's seed; each row accumulates exponential gaps in a double `noise`
 * that restarts at 0, emits dst = index + round(noise) and stops at the first draw with
 * dst >= dst_count or index >= max_degree; that draw is consumed. */
int64_t spo_fp_generate(int64_t src_count, int64_t dst_count, double p, spo_u128 seed,
                        int64_t* offsets, int32_t* neighbors, int64_t* draws) {
	if (draws) *draws = 0;
	if (src_count == 0 || dst_count == 0 || p == 0) {
		for (int64_t i = 0; i <= src_count; i++) offsets[i] = 0;
		return 0;
	}
	uint64_t s[2]      = {seed.lo, seed.hi};
	double scale       = 1 / p - 1;
	int64_t max_degree = spo_fp_max_degree(dst_count, p);
	int64_t count = 0, nd = 0;
	for (int64_t src = 0; src < src_count; src++) {
		offsets[src]  = count;
		int32_t index = 0;
		double noise  = 0;
		for (;;) {
			noise += spo_exponential(scale, s);
			nd++;
			int32_t dst = index + (int32_t)round(noise);
			if ((dst >= dst_count) | (index >= max_degree)) break;
			neighbors[count++] = dst;
			index++;
		}
	}
	offsets[src_count] = count;
	if (draws) *draws = nd;
	return count;
}

/* ------------------------------------------------------------------------------------------
 * Network simulator
 * ---------------------------------------------------------------------------------------- */
typedef struct {
	int kind;
	int64_t size;
	float rate;                   /* POISSON */
	float vthres, tmem_inv;       /* LIF */
	int32_t tref;                 /* LIF */
	float* V; float* Gex; float* Gin; int32_t* T;
	/* spike history: a ring of max_delay steps (neuron_population.h:116-153) */
	int32_t** hist; int64_t* hist_n; int64_t* hist_cap;
	int64_t hist_len, hist_head;  /* hist_head = slot of age 0 */
	/* EXTERNAL */
	int ext_steps, ext_pos; int32_t* ext_counts; int64_t* ext_off; int32_t* ext_idx;
	/* post-spike history of a plastic connection's target: bit k = spiked k steps ago
	 * (neuron_population.h:126-132) */
	uint64_t* post_hist;
} spo_pop;

typedef struct {
	int src, dst, field;
	float weight;
	int64_t delay;
	int64_t* off; int32_t* nb; int64_t nsyn;
	/* plastic synapses (synapse_population.h:27-44, 82-140) */
	int plastic;            /* 0 fixed weight, SPO_SYN_ISTDP, SPO_SYN_COUNT */
	float eta, alpha, cdt;  /* iSTDP: learning rate, 2 rho0 tau, dt / tau */
	double skip_tab[129];   /* pow(1 - dt / tau, n), n = -64 .. 64 */
	float* sW; float* sA; float* sB;  /* per-synapse state in CSR order */
	uint64_t* ages;         /* per source: bit 63 = pending pre update, low bits = step + 1 */
	float* wts;             /* weighted synapses: per-synapse weight in CSR order, else NULL */
} spo_conn;

struct spo_net {
	float dt;
	int64_t max_delay, time, events;
	spo_kahan simtime;
	spo_u128 seed;
	float last_dt;
	int npop, nconn;
	spo_pop pops[16];
	spo_conn conns[64];
};

spo_net* spo_net_create(float dt, float max_delay, const uint32_t* seeds, int nseeds) {
	if (nseeds <= 0) { fail("Assertion failed (random.h:151): il.size() > 0 && \"Please provide at least 1 seed to seed_seq\""); return NULL; }
	spo_net* n = (spo_net*)calloc(1, sizeof(spo_net));
	n->dt        = dt;
	/* snn(dt, max_delay, seed): _max_delay(std::round(max_delay / dt)) (snn.h:18-19) */
	n->max_delay = (int64_t)roundf(max_delay / dt);
	n->seed      = spo_seed_from_list(seeds, nseeds);
	return n;
}

void spo_net_destroy(spo_net* n) {
	if (!n) return;
	for (int i = 0; i < n->npop; i++) {
		spo_pop* p = &n->pops[i];
		free(p->V); free(p->Gex); free(p->Gin); free(p->T);
		for (int64_t k = 0; k < p->hist_len; k++) free(p->hist[k]);
		free(p->hist); free(p->hist_n); free(p->hist_cap);
		free(p->ext_counts); free(p->ext_off); free(p->ext_idx);
	}
	for (int i = 0; i < n->nconn; i++) {
		spo_conn* c = &n->conns[i];
		free(c->off); free(c->nb); free(c->sW); free(c->sA); free(c->sB); free(c->ages); free(c->wts);
	}
	for (int i = 0; i < n->npop; i++) free(n->pops[i].post_hist);
	free(n);
}

int spo_add_population(spo_net* n, int kind, int64_t size, const float* prm, int np) {
	if (n->npop >= 16) return fail("too many populations");
	/* a negative size as the reference's neuron adapters meet it: the stateless and per-population
	 * adapters check it (neuron_population.h:35, :92); a stateful one's vector(size) throws first */
	if (size < 0) {
		if (kind == SPO_POISSON) return fail("Assertion failed (neuron_population.h:35): size >= 0");
		if (kind == SPO_EXTERNAL) return fail("Assertion failed (neuron_population.h:92): size >= 0");
		return fail("cannot create std::vector larger than max_size()");
	}
	if (n->max_delay < 1) return fail("Assertion failed (neuron_population.h:108): max_delay >= 1");
	spo_pop* p = &n->pops[n->npop];
	memset(p, 0, sizeof *p);
	p->kind = kind;
	p->size = size;
	if (kind == SPO_POISSON) {
		p->rate = np > 0 ? prm[0] : 20.0f;
	} else if (kind == SPO_LIF) {
		p->vthres   = np > 0 ? prm[0] : 0.02f;
		p->tref     = np > 1 ? (int32_t)prm[1] : 20;
		p->tmem_inv = np > 2 ? prm[2] : 50.0f;
	} else if (kind != SPO_LIF_COND && kind != SPO_EXTERNAL) {
		return fail("unknown neuron kind");
	}
	if (kind == SPO_LIF || kind == SPO_LIF_COND) {
		/* stateful_neuron_adapter consumes seed++ even without init() (neuron_population.h:56-67) */
		spo_seed_next(&n->seed);
		p->V   = (float*)calloc((size_t)size + 1, sizeof(float));
		p->T   = (int32_t*)calloc((size_t)size + 1, sizeof(int32_t));
		p->Gex = (float*)calloc((size_t)size + 1, sizeof(float));
		p->Gin = (float*)calloc((size_t)size + 1, sizeof(float));
		if (kind == SPO_LIF_COND)
			for (int64_t i = 0; i < size; i++) p->V[i] = -0.06f; /* samples/vogels.cpp:12 */
	}
	p->hist_len = n->max_delay;
	p->hist     = (int32_t**)calloc((size_t)p->hist_len, sizeof(int32_t*));
	p->hist_n   = (int64_t*)calloc((size_t)p->hist_len, sizeof(int64_t));
	p->hist_cap = (int64_t*)calloc((size_t)p->hist_len, sizeof(int64_t));
	p->hist_head = p->hist_len - 1;
	return n->npop++;
}

int spo_set_external(spo_net* n, int pop, int nsteps, const int32_t* counts, const int32_t* idx) {
	if (pop < 0 || pop >= n->npop || n->pops[pop].kind != SPO_EXTERNAL) return fail("not external");
	spo_pop* p = &n->pops[pop];
	free(p->ext_counts); free(p->ext_off); free(p->ext_idx);
	p->ext_steps  = nsteps;
	p->ext_pos    = 0;
	p->ext_counts = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nsteps + 1));
	p->ext_off    = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nsteps + 1));
	int64_t tot   = 0;
	for (int i = 0; i < nsteps; i++) { p->ext_off[i] = tot; p->ext_counts[i] = counts[i]; tot += counts[i]; }
	p->ext_off[nsteps] = tot;
	p->ext_idx = (int32_t*)malloc(sizeof(int32_t) * (size_t)(tot + 1));
	memcpy(p->ext_idx, idx, sizeof(int32_t) * (size_t)tot);
	return 0;
}

static int conn_common(spo_net* n, int src, int dst, float delay, int field) {
	if (src < 0 || src >= n->npop || dst < 0 || dst >= n->npop) return fail("bad population");
	int k = n->pops[dst].kind;
	if (k != SPO_LIF && k != SPO_LIF_COND) return fail("target population must be stateful");
	if (field < 0 || field > 2 || (k == SPO_LIF && field != 0)) return fail("bad target field");
	if (n->nconn >= 64) return fail("too many connections");
	/* snn::connect: d = round(delay/dt), 1 <= d <= max_delay (snn.h:33-38) */
	int64_t d = (int64_t)roundf(delay / n->dt);
	if (!(d >= 1)) return fail("Assertion failed (snn.h:35): d >= 1 && \"The delay must be at least 1dt.\"");
	if (!(d <= n->max_delay))
		return fail("Assertion failed (snn.h:36): d <= _max_delay && \"The delay of a synapse population may not exceed the maximum delay of the network.\"");
	return 0;
}

int spo_connect(spo_net* n, int src, int dst, double p, float delay, int field, float weight) {
	if (conn_common(n, src, dst, delay, field)) return -1;
	if (!(0 <= p && p <= 1)) return fail("Assertion failed (topology.cpp:73): 0 <= p && p <= 1");
	/* the csr of an empty source has no offsets (csr.h:70), which generate refuses (topology.cpp:82) */
	if (n->pops[src].size == 0) return fail("Assertion failed (topology.cpp:82): offsets.size() > src_count");
	spo_conn* c = &n->conns[n->nconn];
	memset(c, 0, sizeof *c);
	c->src = src; c->dst = dst; c->field = field; c->weight = weight;
	c->delay = (int64_t)roundf(delay / n->dt);
	int64_t S = n->pops[src].size, D = n->pops[dst].size;
	int64_t md  = (S > 0) ? spo_fp_max_degree(D, p) : 0;
	c->off = (int64_t*)calloc((size_t)S + 1, sizeof(int64_t));
	c->nb  = (int32_t*)malloc(sizeof(int32_t) * (size_t)(S * (md > 0 ? md : 0) + 1));
	/* synapse_population ctor: _graph(c, seed++) (synapse_population.h:30-31) */
	spo_u128 sd = spo_seed_next(&n->seed);
	c->nsyn = spo_fp_generate(S, D, p, sd, c->off, c->nb, NULL);
	return n->nconn++;
}

/* A fixed_probability connection whose synapses carry their own weight, drawn when the connection
 * is built: the synapse_population ctor seeds the adjacency with seed++ and then, for a
 * PerSynapseInit synapse, walks the CSR in order with one more stream, rng(seed++), calling
 * init(syn, src, dst, rng) per synapse (synapse_population.h:30-41).  The weighted synapse's init
 * draws once: w = wmax * canonical<float>(rng) (random.h:236-247). */
int spo_connect_weighted(spo_net* n, int src, int dst, double p, float delay, int field, float wmax) {
	int const ci = spo_connect(n, src, dst, p, delay, field, 0.0f);
	if (ci < 0) return ci;
	spo_conn* c      = &n->conns[ci];
	spo_u128 const s = spo_seed_next(&n->seed);
	uint64_t rng[2]  = {s.lo, s.hi};
	c->wts = (float*)malloc(sizeof(float) * (size_t)(c->nsyn + 1));
	for (int64_t e = 0; e < c->nsyn; e++) c->wts[e] = wmax * spo_canonical_f32(spo_xoroshiro128p_next(rng));
	return ci;
}

int spo_syn_weights(const spo_net* n, int conn, float* out) {
	if (conn < 0 || conn >= n->nconn || !n->conns[conn].wts) return fail("not a weighted connection");
	memcpy(out, n->conns[conn].wts, sizeof(float) * (size_t)n->conns[conn].nsyn);
	return 0;
}

static int cmp_u64(const void* a, const void* b) {
	uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
	return x < y ? -1 : x > y;
}

int spo_connect_adj(spo_net* n, int src, int dst, int64_t m, const int32_t* pairs, float delay,
                    int field, float weight) {
	if (conn_common(n, src, dst, delay, field)) return -1;
	/* the csr of an empty source has no offsets (csr.h:70), which Topology::generate refuses (topology.cpp:48) */
	if (n->pops[src].size == 0) return fail("Assertion failed (topology.cpp:48): offsets.size() > src_count");
	spo_conn* c = &n->conns[n->nconn];
	memset(c, 0, sizeof *c);
	c->src = src; c->dst = dst; c->field = field; c->weight = weight;
	c->delay = (int64_t)roundf(delay / n->dt);
	int64_t S = n->pops[src].size;
	/* adj_list::connect checks each edge (topology.cpp:56-58); adj_list::generate sorts src<<32|dst
	 * and streams the edges into offsets of S + 1 entries (topology.cpp:15-32, 65-71), with the
	 * stream's checks in its order */
	uint64_t* e = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(m + 1));
	for (int64_t i = 0; i < m; i++) {
		if (pairs[2 * i] < 0) { free(e); return fail("Assertion failed (topology.cpp:57): 0 <= src && src < std::numeric_limits<Int32>::max()"); }
		if (pairs[2 * i + 1] < 0) { free(e); return fail("Assertion failed (topology.cpp:58): 0 <= dst && dst < std::numeric_limits<Int32>::max()"); }
		e[i] = ((uint64_t)(uint32_t)pairs[2 * i] << 32) | (uint32_t)pairs[2 * i + 1];
	}
	qsort(e, (size_t)m, sizeof(uint64_t), cmp_u64);
	{
		int64_t at = 0; /* edge_stream::_src */
		for (int64_t i = 0; i < m; i++) {
			int64_t first = (int64_t)(e[i] >> 32);
			if (!(at < S + 1)) { free(e); return fail("Assertion failed (topology.cpp:16): _src < _offsets.size()"); }
			if (!(first < S + 1)) { free(e); return fail("Assertion failed (topology.cpp:18): edge.first < _offsets.size()"); }
			if (at <= first) at = first + 1;
		}
		if (!(at < S + 1)) { free(e); return fail("Assertion failed (topology.cpp:29): _src < _offsets.size()"); }
		for (int64_t i = 0; i < m; i++) /* a target beyond the population fails the delivery's check */
			if ((int64_t)(e[i] & 0xffffffffu) >= n->pops[dst].size) {
				free(e);
				return fail("Assertion failed (synapse_population.h:119): edge.first < dst_neurons.size()");
			}
	}
	c->off = (int64_t*)calloc((size_t)S + 1, sizeof(int64_t));
	c->nb  = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m + 1));
	int64_t s = 0;
	for (int64_t i = 0; i < m; i++) {
		int64_t es = (int64_t)(e[i] >> 32);
		while (s <= es) c->off[s++] = i;
		c->nb[i] = (int32_t)(e[i] & 0xffffffffu);
	}
	while (s <= S) c->off[s++] = m;
	c->nsyn = m;
	free(e);
	/* the adj_list topology still consumes a seed in the synapse_population ctor */
	spo_seed_next(&n->seed);
	return n->nconn++;
}

static void push_spike(spo_pop* p, int64_t slot, int32_t i) {
	if (p->hist_n[slot] == p->hist_cap[slot]) {
		int64_t nc        = p->hist_cap[slot] ? 2 * p->hist_cap[slot] : 256;
		p->hist[slot]     = (int32_t*)realloc(p->hist[slot], sizeof(int32_t) * (size_t)nc);
		p->hist_cap[slot] = nc;
	}
	p->hist[slot][p->hist_n[slot]++] = i;
}

/* Brunel LIF update (samples/brunel.cpp:45-61, README.md:28-45) as the reference's
 * -ffast-math -march=haswell build executes it: the leak V += (0 - V) * (dt * TmemInv)
 * is compiled to V * fma(-dt, TmemInv, 1).  The threshold test is float V > Vthres
 * (equal to the README's double compare V > 0.02 for every float V). */
static inline int spo_lif_update(float* V, int32_t* T, float dt, float om, float vthres,
                                 int32_t tref) {
	(void)dt;
	if (--(*T) <= 0) {
		if (*V > vthres) {
			*V = 0;
			*T = tref;
			return 1;
		}
		*V = *V * om;
	}
	return 0;
}

/* Conductance LIF (samples/vogels.cpp:10-46) as the reference's -ffast-math -march=haswell build
 * executes it.  GCC 13 folds Vrest + Ibg into one constant (-0.06f + 0.02f = -0.04f), drops
 * Eex = 0, contracts the two products around it into fused multiply-adds and turns the
 * conductance decay G -= G * (dt * Inv) into G * fma(-dt, Inv, 1), like the Brunel leak:
 *   V   = fma(dt * TmemInv, (-0.04f - V) + fma(-Gex, V, Gin * (Ein - V)), V)
 *   Gex = Gex * fma(-dt, TexInv, 1),  Gin = Gin * fma(-dt, TinInv, 1)
 * (the conductances of the V update are the values before their decay, as in the source order).
 * Pinned to the reference binary's states over whole runs (tests/test_oracle.py). */
static inline int spo_lifc_update(float* V, float* Gex, float* Gin, int32_t* T, float dt) {
	const int32_t Tref  = 50;
	const float Vrest   = -0.06f, Vthres = -0.05f, TmemInv = 1.0f / 0.02f;
	const float Ein = -0.08f, VrestIbg = -0.06f + 0.02f;
	const float TexInv = 1.0f / 0.005f, TinInv = 1.0f / 0.01f;
	int spiked = 0;
	float const gex = *Gex, gin = *Gin;
	if (--(*T) <= 0) {
		if (*V > Vthres) {
			*V = Vrest; *T = Tref; spiked = 1;
		} else {
			float const v = *V;
			float const a = gin * (Ein - v);
			float const b = fmaf(-gex, v, a);
			float const c = (VrestIbg - v) + b;
			*V = fmaf(dt * TmemInv, c, v);
		}
	}
	*Gex = gex * fmaf(-dt, TexInv, 1.0f);
	*Gin = gin * fmaf(-dt, TinInv, 1.0f);
	return spiked;
}

/* ---- plastic synapses ----
 * The iSTDP model (inhibitory symmetric STDP, Vogels et al. 2011) written against the reference's
 * PlasticSynapse concept (concepts.h:86-92): update() at a step with a pre and/or post spike,
 * skip(n) over n quiet steps.  Traces decay by x -= x * dt/tau per step, as the sample plastic
 * model of samples/brunel+.cpp:59-99 does; skip(n) multiplies by pow(1 - dt/tau, n) in double and
 * rounds once to float (std::pow(float, Int) promotes to double).  The counting model is the
 * plastic_synapse of test/detail/synapse_population.cpp:84-94: update adds 1, skip adds n. */
static void syn_update(spo_conn* c, int64_t e, int pre, int post) {
	if (c->plastic == SPO_SYN_COUNT) {
		c->sW[e] = c->sW[e] + 1.0f;
		return;
	}
	float W = c->sW[e], xa = c->sA[e], xb = c->sB[e];
	if (pre) {
		float const w = W + c->eta * (xb - c->alpha);
		W             = w > 0.0f ? w : 0.0f;
	}
	if (post) W = W + c->eta * xa;
	xa = xa + (pre ? 1.0f : 0.0f);
	xb = xb + (post ? 1.0f : 0.0f);
	xa = xa - xa * c->cdt;
	xb = xb - xb * c->cdt;
	c->sW[e] = W; c->sA[e] = xa; c->sB[e] = xb;
}

static void syn_skip(spo_conn* c, int64_t e, int64_t n) {
	if (c->plastic == SPO_SYN_COUNT) {
		c->sW[e] = c->sW[e] + (float)n;
		return;
	}
	double const f = c->skip_tab[n + 64];
	c->sA[e] = (float)((double)c->sA[e] * f);
	c->sB[e] = (float)((double)c->sB[e] * f);
}

static int clz64(uint64_t x) { return __builtin_clzll(x); }

/* synapse_population::_update's per-edge catch-up (synapse_population.h:88-116): replays the
 * steps since the synapse was last brought up to date -- the pending pre update of the last
 * delivery, then every post spike in the target's history, with skip() over the quiet steps.
 * The reference computes ~0 >> prefix with prefix up to 64 (pre set and time == age); x86-64
 * shifts by prefix mod 64, and that is what is restated here. */
static void catch_up(spo_conn* c, int64_t e, int64_t time, uint64_t ages, uint64_t hist) {
	int const pre     = (int)(ages >> 63);
	int64_t const age = (int64_t)(ages & ~(1ULL << 63));
	if (!(time >= age)) return;
	int64_t const prefix = 63 + pre - time + age;
	uint64_t const mask  = ~0ULL >> (prefix & 63);
	if (pre) syn_update(c, e, 1, (hist & (1ULL << ((time - age) & 63))) != 0);
	hist &= mask;
	int64_t p = prefix;
	while (hist) {
		int const lz = clz64(hist);
		syn_skip(c, e, lz - p);
		syn_update(c, e, 0, 1);
		hist ^= 1ULL << (63 - lz);
		p = lz + 1;
	}
	syn_skip(c, e, 64 - p);
}

int spo_set_plastic(spo_net* n, int conn, int model, float w0, float eta, float rho0, float tau) {
	if (conn < 0 || conn >= n->nconn) return fail("bad connection");
	if (model != SPO_SYN_ISTDP && model != SPO_SYN_COUNT) return fail("bad plastic model");
	spo_conn* c = &n->conns[conn];
	spo_pop* d  = &n->pops[c->dst];
	int64_t S = n->pops[c->src].size;
	c->plastic = model;
	c->eta     = eta;
	c->alpha   = 2.0f * rho0 * tau;
	c->cdt     = n->dt * (1.0f / tau);
	float const base = 1.0f - c->cdt;
	for (int k = -64; k <= 64; k++) c->skip_tab[k + 64] = pow((double)base, (double)k);
	c->sW   = (float*)malloc(sizeof(float) * (size_t)(c->nsyn + 1));
	c->sA   = (float*)calloc((size_t)(c->nsyn + 1), sizeof(float));
	c->sB   = (float*)calloc((size_t)(c->nsyn + 1), sizeof(float));
	c->ages = (uint64_t*)calloc((size_t)(S + 1), sizeof(uint64_t));
	for (int64_t e = 0; e < c->nsyn; e++) c->sW[e] = model == SPO_SYN_COUNT ? 0.0f : w0;
	if (!d->post_hist) d->post_hist = (uint64_t*)calloc((size_t)(d->size + 1), sizeof(uint64_t));
	return 0;
}

int spo_syn_state(const spo_net* n, int conn, int field, float* out) {
	if (conn < 0 || conn >= n->nconn || !n->conns[conn].plastic) return fail("not a plastic connection");
	const spo_conn* c = &n->conns[conn];
	const float* src  = field == 0 ? c->sW : (field == 1 ? c->sA : c->sB);
	memcpy(out, src, sizeof(float) * (size_t)c->nsyn);
	return 0;
}

void spo_step(spo_net* n) {
	/* snn::step (snn.cpp:7-28) */
	float dt   = spo_kahan_step(&n->simtime, n->dt);
	n->last_dt = dt;
	spo_u128 sd = spo_seed_next(&n->seed);
	uint64_t rng[2] = {sd.lo, sd.hi};
	float om = fmaf(-dt, 50.0f, 1.0f);

	for (int pi = 0; pi < n->npop; pi++) {
		spo_pop* p = &n->pops[pi];
		/* neuron_population::update: the window of max_delay steps slides (neuron_population.h:116-134) */
		p->hist_head = (p->hist_head + 1) % p->hist_len;
		int64_t slot = p->hist_head;
		p->hist_n[slot] = 0;
		switch (p->kind) {
			case SPO_POISSON: {
				float thr = p->rate * dt;
				for (int64_t i = 0; i < p->size; i++)
					if (spo_canonical_f32(spo_xoroshiro128p_next(rng)) < thr) push_spike(p, slot, (int32_t)i);
				break;
			}
			case SPO_LIF: {
				float o = (p->tmem_inv == 50.0f) ? om : fmaf(-dt, p->tmem_inv, 1.0f);
				for (int64_t i = 0; i < p->size; i++)
					if (spo_lif_update(&p->V[i], &p->T[i], dt, o, p->vthres, p->tref)) push_spike(p, slot, (int32_t)i);
				break;
			}
			case SPO_LIF_COND:
				for (int64_t i = 0; i < p->size; i++)
					if (spo_lifc_update(&p->V[i], &p->Gex[i], &p->Gin[i], &p->T[i], dt)) push_spike(p, slot, (int32_t)i);
				break;
			case SPO_EXTERNAL:
				if (p->ext_steps > 0) {
					int k = p->ext_pos;
					for (int64_t j = p->ext_off[k]; j < p->ext_off[k] + p->ext_counts[k]; j++)
						push_spike(p, slot, p->ext_idx[j]);
					p->ext_pos = (k + 1) % p->ext_steps;
				}
				break;
		}
		if (p->post_hist) { /* neuron_population.h:126-132 */
			for (int64_t i = 0; i < p->size; i++) p->post_hist[i] <<= 1;
			for (int64_t k = 0; k < p->hist_n[slot]; k++) p->post_hist[p->hist[slot][k]] |= 1;
		}
	}

	/* every 64 steps all plastic synapses catch up (snn.cpp:17-19, synapse_population.h:70-74) */
	if (n->time % 64 == 0)
		for (int ci = 0; ci < n->nconn; ci++) {
			spo_conn* c = &n->conns[ci];
			if (!c->plastic) continue;
			const uint64_t* h = n->pops[c->dst].post_hist;
			for (int64_t s = 0; s < n->pops[c->src].size; s++) {
				for (int64_t e = c->off[s]; e < c->off[s + 1]; e++) catch_up(c, e, n->time, c->ages[s], h[c->nb[e]]);
				c->ages[s] = (uint64_t)(n->time + 1);
			}
		}

	/* deliveries in connect order, spikes of age d-1 (snn.cpp:21-25, synapse_population.h:82-140) */
	for (int ci = 0; ci < n->nconn; ci++) {
		spo_conn* c = &n->conns[ci];
		if (n->time < c->delay - 1) continue;
		spo_pop* sp = &n->pops[c->src];
		spo_pop* dp = &n->pops[c->dst];
		int64_t slot = ((sp->hist_head - (c->delay - 1)) % sp->hist_len + sp->hist_len) % sp->hist_len;
		float* F = c->field == 0 ? dp->V : (c->field == 1 ? dp->Gex : dp->Gin);
		float w  = c->weight;
		for (int64_t k = 0; k < sp->hist_n[slot]; k++) {
			int32_t s = sp->hist[slot][k];
			if (c->plastic) {
				for (int64_t e = c->off[s]; e < c->off[s + 1]; e++) {
					catch_up(c, e, n->time, c->ages[s], dp->post_hist[c->nb[e]]);
					if (c->plastic == SPO_SYN_ISTDP) F[c->nb[e]] = F[c->nb[e]] + c->sW[e];
					else if (w != 0.0f) F[c->nb[e]] = F[c->nb[e]] + c->sW[e] * w;
				}
				c->ages[s] = (uint64_t)(n->time + 1) | (1ULL << 63);
			} else if (c->wts) {
				for (int64_t e = c->off[s]; e < c->off[s + 1]; e++) F[c->nb[e]] = F[c->nb[e]] + c->wts[e];
			} else {
				for (int64_t e = c->off[s]; e < c->off[s + 1]; e++) F[c->nb[e]] = F[c->nb[e]] + w;
			}
			n->events += c->off[s + 1] - c->off[s];
		}
	}
	n->time++;
}

void spo_run(spo_net* n, int64_t steps) {
	for (int64_t i = 0; i < steps; i++) spo_step(n);
}

int64_t spo_time(const spo_net* n) { return n->time; }
int64_t spo_events(const spo_net* n) { return n->events; }
float spo_last_dt(const spo_net* n) { return n->last_dt; }
int64_t spo_pop_size(const spo_net* n, int pop) {
	return (pop >= 0 && pop < n->npop) ? n->pops[pop].size : -1;
}

/* neuron_population::spikes(age): 0 <= age < number of recorded steps (neuron_population.h:147-153) */
static int64_t age_slot(const spo_net* n, int pop, int age) {
	if (pop < 0 || pop >= n->npop) return -1;
	const spo_pop* p = &n->pops[pop];
	int64_t recorded = n->time < p->hist_len ? n->time : p->hist_len;
	if (!(0 <= age && age < recorded)) return -1;
	return ((p->hist_head - age) % p->hist_len + p->hist_len) % p->hist_len;
}

int64_t spo_spike_count(const spo_net* n, int pop, int age) {
	int64_t s = age_slot(n, pop, age);
	if (s < 0) return fail("Assertion failed (neuron_population.h:148): 0 <= age && age < _spike_counts.size()");
	return n->pops[pop].hist_n[s];
}

int64_t spo_spikes(const spo_net* n, int pop, int age, int32_t* out) {
	int64_t s = age_slot(n, pop, age);
	if (s < 0) return fail("Assertion failed (neuron_population.h:148): 0 <= age && age < _spike_counts.size()");
	const spo_pop* p = &n->pops[pop];
	memcpy(out, p->hist[s], sizeof(int32_t) * (size_t)p->hist_n[s]);
	return p->hist_n[s];
}

static void* field_ptr(const spo_pop* p, int field) {
	switch (field) {
		case 0: return p->V;
		case 1: return p->Gex;
		case 2: return p->Gin;
		case 3: return p->T;
	}
	return NULL;
}

int spo_get_state(const spo_net* n, int pop, int field, void* out) {
	if (pop < 0 || pop >= n->npop) return fail("bad population");
	void* f = field_ptr(&n->pops[pop], field);
	if (!f) return fail("population has no such state field");
	memcpy(out, f, 4 * (size_t)n->pops[pop].size);
	return 0;
}

int spo_set_state(spo_net* n, int pop, int field, const void* in) {
	if (pop < 0 || pop >= n->npop) return fail("bad population");
	void* f = field_ptr(&n->pops[pop], field);
	if (!f) return fail("population has no such state field");
	memcpy(f, in, 4 * (size_t)n->pops[pop].size);
	return 0;
}

int64_t spo_conn_synapses(const spo_net* n, int conn) {
	return (conn >= 0 && conn < n->nconn) ? n->conns[conn].nsyn : -1;
}

int spo_conn_csr(const spo_net* n, int conn, int64_t* offsets, int32_t* neighbors) {
	if (conn < 0 || conn >= n->nconn) return fail("bad connection");
	const spo_conn* c = &n->conns[conn];
	int64_t S         = n->pops[c->src].size;
	memcpy(offsets, c->off, sizeof(int64_t) * (size_t)(S + 1));
	memcpy(neighbors, c->nb, sizeof(int32_t) * (size_t)c->nsyn);
	return 0;
}
