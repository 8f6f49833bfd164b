/*
 * spice_oracle.h -- CPU restatement of spice2's snn::step path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle: tests/, the smoke check
 * in __graft_entry__.py and the cpu_baseline leg of bench.py call it to check or
 * time the GPU engine.  The product (spice2_gb300/, include/) never links,
 * imports or calls anything here.
 *
 * Every function restates one piece of the reference algorithm in plain C and
 * cites the reference file:line it follows (paths inside the spice2 project).
 * Floating point is strict IEEE (built with -O2 -ffp-contract=off, no
 * -ffast-math); where the reference's -ffast-math build rewrites an
 * expression, the rewritten form is spelled out explicitly (see spo_lif_update).
 *
 * Parity pins: the restatement is checked against the reference itself,
 * compiled here from its own sources (oracle/Makefile -> oracle/_ref), and
 * against the raster head the reference publishes in its README.
 */
#ifndef SPICE_ORACLE_H
#define SPICE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { uint64_t lo, hi; } spo_u128;

/* ---- RNG and seeding (spice/include/spice/util/random.h) ---- */
spo_u128 spo_murmur3_bytes(const void* data, uint64_t len);       /* random.h:32-107  */
spo_u128 spo_murmur3_u128(spo_u128 k);                            /* random.h:108-139 */
spo_u128 spo_seed_from_list(const uint32_t* seeds, int n);        /* random.h:149-152 */
spo_u128 spo_seed_next(spo_u128* seed);                           /* random.h:163-167 (post-increment) */
uint64_t spo_xoroshiro128p_next(uint64_t s[2]);                   /* random.h:222-234 */
void spo_xoroshiro128p_jump(uint64_t s[2], const uint64_t poly[2]); /* applies poly(T) to the state */
float spo_canonical_f32(uint64_t u);                              /* random.h:236-247, Real=float */
double spo_canonical_f64_leftopen(uint64_t u);                    /* random.h:236-247, Real=double, LeftOpen */
double spo_exponential(double scale, uint64_t s[2]);              /* random.h:264-276 */

/* ---- Kahan-compensated sim time (spice/include/spice/util/numeric.h:6-24, snn.cpp:8-10) ---- */
typedef struct { float c, sum; } spo_kahan;
float spo_kahan_step(spo_kahan* k, float delta); /* returns the compensated increment y; resets sum at >= 1 */

/* ---- fixed_probability (spice/src/topology.cpp:73-112) ---- */
int64_t spo_fp_max_degree(int64_t dst_count, double p);
/* Writes offsets[src_count+1] and neighbors; neighbors must hold src_count*max_degree
 * entries.  Returns the synapse count, and the number of xoroshiro draws consumed in
 * *draws (if non-NULL). */
int64_t spo_fp_generate(int64_t src_count, int64_t dst_count, double p, spo_u128 seed,
                        int64_t* offsets, int32_t* neighbors, int64_t* draws);

/* ---- the network simulator (spice/src/snn.cpp:7-28 and detail/neuron_population.h, detail/synapse_population.h) ---- */
enum {
	SPO_POISSON  = 0, /* stateless: canonical<float>(rng) < rate*dt   (samples/brunel.cpp:27-30) */
	SPO_LIF      = 1, /* Brunel LIF {V, T}                            (samples/brunel.cpp:39-62)  */
	SPO_LIF_COND = 2, /* conductance LIF {V, Gex, Gin, T}             (samples/vogels.cpp:10-46)  */
	SPO_EXTERNAL = 3, /* per-population update from a cyclic train   (samples/external_input.cpp:17-30) */
};

/* plastic synapse models (spo_set_plastic) */
enum {
	SPO_SYN_ISTDP = 1, /* inhibitory symmetric STDP (Vogels et al. 2011) on pre/post traces */
	SPO_SYN_COUNT = 2  /* counts update() calls and skipped steps (test/detail/synapse_population.cpp:84-94) */
};

typedef struct spo_net spo_net;

spo_net* spo_net_create(float dt, float max_delay, const uint32_t* seeds, int nseeds);
void spo_net_destroy(spo_net* net);
/* params: POISSON {rate}; LIF {Vthres, Tref, TmemInv}; LIF_COND {} (vogels constants);
 * EXTERNAL: none (set the train with spo_set_external).  Returns the population id. */
int spo_add_population(spo_net* net, int kind, int64_t size, const float* params, int nparams);
int spo_set_external(spo_net* net, int pop, int nsteps, const int32_t* counts,
                     const int32_t* indices);
/* fixed_probability(p) projection with a fixed_weight-style synapse adding `weight`
 * to state field `field` of the target (0=V, 1=Gex, 2=Gin).  Returns the connection id,
 * or -1 with a message from spo_last_error(). */
int spo_connect(spo_net* net, int src, int dst, double p, float delay, int field, float weight);
/* fixed_probability with a per-synapse weight wmax * canonical<float>, drawn from the
 * PerSynapseInit stream (one seed after the adjacency's) in CSR order. */
int spo_connect_weighted(spo_net* net, int src, int dst, double p, float delay, int field, float wmax);
int spo_syn_weights(const spo_net* net, int conn, float* out);
/* Makes connection `conn` plastic (the reference's synapse_population with a PlasticSynapse model,
 * synapse_population.h:27-140): per-synapse state, lazy catch-up from the target's post history at
 * each delivery and every 64 steps.  iSTDP: W starts at w0; pre spike W += eta (x_post - 2 rho0 tau)
 * (W >= 0), post spike W += eta x_pre; traces decay with tau.  The iSTDP delivery adds the synapse's
 * W to the connection's target field; the counting model's delivery adds count * (the connection's
 * weight), nothing for weight 0. */
int spo_set_plastic(spo_net* net, int conn, int model, float w0, float eta, float rho0, float tau);
/* Per-synapse state in CSR order: field 0 W (counting model: the count), 1 x_pre, 2 x_post. */
int spo_syn_state(const spo_net* net, int conn, int field, float* out);
/* adj_list projection (spice/src/topology.cpp:56-71): n (src, dst) pairs. */
int spo_connect_adj(spo_net* net, int src, int dst, int64_t n, const int32_t* pairs,
                    float delay, int field, float weight);
void spo_step(spo_net* net);
void spo_run(spo_net* net, int64_t steps);
int64_t spo_time(const spo_net* net);
int64_t spo_events(const spo_net* net); /* synaptic events delivered so far */
int64_t spo_spike_count(const spo_net* net, int pop, int age);
int64_t spo_spikes(const spo_net* net, int pop, int age, int32_t* out);
int64_t spo_pop_size(const spo_net* net, int pop);
/* State fields of a stateful population: field 0=V (float), 1=Gex, 2=Gin (float), 3=T (int32). */
int spo_get_state(const spo_net* net, int pop, int field, void* out);
int spo_set_state(spo_net* net, int pop, int field, const void* in);
/* CSR of a connection (offsets[src+1], neighbors[syn]); returns the synapse count. */
int64_t spo_conn_synapses(const spo_net* net, int conn);
int spo_conn_csr(const spo_net* net, int conn, int64_t* offsets, int32_t* neighbors);
float spo_last_dt(const spo_net* net);
const char* spo_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
