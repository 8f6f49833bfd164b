/*
 * spice_gb300.h -- C ABI of the GB300-native snn::step engine.
 *
 * The reference (denniskb/spice2) has no C ABI: its boundary is the C++20 template API of
 * spice/include/spice/snn.h plus the two virtual interfaces NeuronPopulation
 * (spice/include/spice/detail/neuron_population.h:17-25) and SynapsePopulation
 * (spice/include/spice/detail/synapse_population.h:17-24).  Each entry point below replaces one
 * member of that boundary (cited beside it) with plain pointers and sizes, so a C, Python
 * (ctypes), Go (cgo) or Java (JNI) host can drive the engine.  The C++ front end in
 * include/spice/ re-exposes the reference's own names on top of these calls.
 *
 * Conventions
 *   - Every call returns an int status: SPICE_OK (0) or one of the SPICE_E* codes below.  The
 *     message of the last failure on the calling thread is spice_last_error().  Failed
 *     preconditions carry the reference's wording ("Assertion failed (file:line): cond",
 *     spice/src/util/assert.cpp:8-15).  No C++ exception crosses the ABI.
 *   - A spice_net owns all of its populations and connections (snn.h:72-74).  Population and
 *     connection ids are small integers in add order.
 *   - One CUDA stream per net; a net is not thread-safe.  Host buffers are plain host memory;
 *     calls that return data synchronise the net's stream.
 *   - All device work runs on the current CUDA device at spice_net_create time.
 */
#ifndef SPICE_GB300_H
#define SPICE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPICE_OK 0
#define SPICE_EINVAL 1    /* a precondition failed (SPICE_PRE in the reference)            */
#define SPICE_ECUDA 2     /* a CUDA runtime call failed                                     */
#define SPICE_ENOMEM 3    /* device or host allocation failed                               */
#define SPICE_ESTATE 4    /* the call is not valid in the net's current state              */
#define SPICE_EOVERFLOW 5 /* a caller buffer is too small; the needed size is returned      */

/* Neuron models (the user-model structs of samples/brunel.cpp, samples/vogels.cpp and
 * samples/external_input.cpp, built in so non-C++ hosts can use them). */
enum {
	SPICE_NEURON_POISSON  = 0, /* stateless; params {rate_hz=20}; one draw per neuron and step  */
	SPICE_NEURON_LIF      = 1, /* {V, Tref}; params {Vthres=0.02, Tref=20, TmemInv=50}          */
	SPICE_NEURON_LIF_COND = 2, /* {V, Gex, Gin, Tref}; samples/vogels.cpp constants             */
	SPICE_NEURON_EXTERNAL = 3, /* per-population update replaying a cyclic spike train          */
};

/* Synapse models. */
enum {
	/* fixed_weight (samples/brunel.cpp:67-70): deliver adds params[0] (weight) to state field
	 * params[1] of the target (0 = V, 1 = Gex, 2 = Gin; default 0). */
	SPICE_SYNAPSE_FIXED_WEIGHT = 0,
	/* Plastic synapses (the reference's PlasticSynapse concept, concepts.h:86-92, driven by
	 * synapse_population.h:82-140): per-synapse state brought up to date lazily -- at each
	 * delivery of its source's spike and every 64 steps -- from the target's 64-step post-spike
	 * history.  A net with plastic connections steps in windows of one step.
	 * ISTDP: inhibitory symmetric STDP (Vogels et al. 2011; no model of this kind ships with the
	 * reference).  params {w0, field, eta, rho0 (Hz), tau (s)}: W starts at w0; a pre spike does
	 * W = max(0, W + eta (x_post - 2 rho0 tau)), a post spike W += eta x_pre; traces add 1 per
	 * spike and decay by x -= x dt/tau per step (skip(n): x *= (1 - dt/tau)^n, in double).
	 * Delivery adds W to the target field; the sum over a step's events is order-dependent, so
	 * ISTDP needs SPICE_MODE_ATOMIC.
	 * COUNT: the counting model of the reference's tests (test/detail/synapse_population.cpp:
	 * 84-94): update() adds 1, skip(n) adds n; params {scale, field}: delivery adds scale * count
	 * (scale 0: delivers nothing, allowed in either mode). */
	SPICE_SYNAPSE_ISTDP = 1,
	SPICE_SYNAPSE_COUNT = 2,
	/* WEIGHTED: a stateful synapse whose weight is drawn per synapse when the connection is built
	 * -- the reference's StatefulSynapse + PerSynapseInit concepts (concepts.h:60-104): the
	 * synapse_population ctor seeds the adjacency with seed++, then walks the CSR in order with
	 * one more stream rng(seed++), calling init(syn, src, dst, rng) (synapse_population.h:30-41).
	 * Here init draws once: w = params[0] * canonical<float>(rng); params {wmax, field[, source]}.
	 * source 0 (default): that init; 1: the weights are the host's (spice_set_synapse_weights,
	 * e.g. a user synapse's own init() run on the host with the seed of spice_connection_seeds),
	 * the connection still consumes the init seed; 2: host weights, no init seed (a stateful
	 * synapse without PerSynapseInit).  Delivery adds w to the target field.  Every population
	 * receiving weighted synapses is delivered by the pull path (see SPICE_TUNE_PULL), bit-exact
	 * with the reference in either mode. */
	SPICE_SYNAPSE_WEIGHTED = 3,
	/* USER_PLASTIC: a plastic synapse written as user code (the reference's PlasticSynapse
	 * concept, concepts.h:86-92): per-synapse state is an array of synapse_bytes-byte structs in
	 * CSR order, brought up to date lazily like the built-in plastic synapses; its update()/skip()
	 * run in kernels of the user's translation unit (include/spice/snn.h) that the engine calls
	 * through spice_user_plastic.  params {field, synapse_bytes, weight_word[, init]}: delivery adds
	 * the float at 4-byte word weight_word of a synapse's state to the target field (atomic mode);
	 * init = 1 when the synapse has a PerSynapseInit init() (the connection then consumes that
	 * stream's seed, synapse_population.h:34-41, and the host sets the initial state). */
	SPICE_SYNAPSE_USER_PLASTIC = 4,
	/* USER_DELIVER: a synapse whose deliver() is arbitrary user code on the target neuron (and,
	 * for the reference's DeliverFromTo concept, concepts.h:70-79, the source neuron): setting a
	 * flag, taking a minimum, anything but adding one value to one float member.  Targets of such
	 * synapses (stateful user populations) receive every input at the end of each step directly into
	 * their neuron structs, connection by connection in connect order (snn.cpp:21-25), through the
	 * kernels registered with spice_user_deliver; their other inputs (fixed_weight, weighted) are
	 * added the same way by the engine; nets with them step in windows of one step.  params
	 * {synapse_bytes (0: stateless), reads_source, init}: reads_source = 1 when deliver() takes the
	 * source neuron; init = 1 when the synapse has a PerSynapseInit init() (the connection consumes
	 * that stream's seed, and the host sets the initial state). */
	SPICE_SYNAPSE_USER_DELIVER = 5,
};

/* Delivery modes. */
enum {
	SPICE_MODE_DETERMINISTIC = 0, /* bit-exact with the reference's sequential delivery order */
	SPICE_MODE_ATOMIC        = 1, /* float atomics: fastest, order-dependent rounding          */
};

/* State fields for spice_get_state / spice_set_state. */
enum { SPICE_FIELD_V = 0, SPICE_FIELD_GEX = 1, SPICE_FIELD_GIN = 2, SPICE_FIELD_TREF = 3 };

typedef struct spice_net spice_net;

/* snn::snn(dt, max_delay, seed) -- spice/include/spice/snn.h:18-19.  seeds: the
 * std::initializer_list<UInt32> of util::seed_seq (spice/include/spice/util/random.h:149-152). */
int spice_net_create(float dt, float max_delay, const uint32_t* seeds, int nseeds, spice_net** out);
int spice_net_destroy(spice_net* net);

/* snn::add_population<Neur>(size, neur) -- snn.h:21-27 (neuron_population.h:106-112).  Stateful
 * models consume one seed, as stateful_neuron_adapter does (neuron_population.h:56-60). */
int spice_add_population(spice_net* net, int model, int64_t size, const float* params, int nparams,
                         int* pop_out);

/* snn::connect<Syn>(src, dst, fixed_probability(p), delay, syn) -- snn.h:29-48, with the
 * adjacency of fixed_probability::generate (spice/src/topology.cpp:78-112) generated on the GPU,
 * bit-identical to the reference's for the same seed. */
int spice_connect_fixed_probability(spice_net* net, int src, int dst, double p, float delay,
                                    int synapse, const float* params, int nparams, int* conn_out);

/* snn::connect<Syn>(src, dst, adj_list, delay, syn) -- snn.h:29-48 with adj_list
 * (topology.cpp:56-71); pairs holds npairs (src, dst) int32 pairs. */
int spice_connect_adj_list(spice_net* net, int src, int dst, const int32_t* pairs, int64_t npairs,
                           float delay, int synapse, const float* params, int nparams,
                           int* conn_out);

/* The per-population update of samples/external_input.cpp:17-30: population `pop` (model
 * SPICE_NEURON_EXTERNAL) emits the spikes of train step (i mod nsteps) at its i-th update. */
int spice_set_external_input(spice_net* net, int pop, int nsteps, const int32_t* counts,
                             const int32_t* indices);

int spice_set_mode(spice_net* net, int mode);

/* Launch-shape knobs of the delivery kernel (no counterpart in the reference; may be changed at
 * any time between steps): shared memory per target tile in bytes, and threads per delivery CTA.
 * Results do not depend on them.  Those the caller leaves unset are picked from the network's
 * sizes when it is prepared (its first step): mapping 17 (1 for tiles above 176 KiB), LIF window
 * 9, the largest tile of at most 100 KiB that gives the most delivery CTAs per window (input slots
 * x target tiles) within one wave of one CTA per SM, and 768 / 512 / 256 threads for tiles of at
 * least 64 KiB / 24 KiB / less.  spice2_gb300.autotune measures them on a network instead. */
enum {
	SPICE_TUNE_TILE_BYTES      = 0, /* shared memory per target tile                          */
	SPICE_TUNE_DELIVER_THREADS = 1, /* threads per delivery CTA                               */
	SPICE_TUNE_DELIVER_PARTS   = 2, /* CTAs sharing one (input slot, tile)                    */
	SPICE_TUNE_DELIVER_ALGO    = 3, /* 0: warp-flattened sub-rows, 1: one thread per spike,
	                                   2: one warp per spike, 8 sub-rows in flight,
	                                   3: one thread per spike with 16-byte loads,
	                                   4: one thread per spike, software-pipelined,
	                                   5, 6: 4 or 8 lanes per spike, software-pipelined,
	                                   7: as 5 with <= 32 registers (4 x 512 threads per SM),
	                                   8, 9: 4 lanes per spike, sub-rows staged in shared
	                                   memory, 2 or 4 sub-rows in flight per lane group,
	                                   10 .. 13: staged sub-rows read as aligned 16-byte
	                                   blocks; per lane group and load round trip 2 x 64,
	                                   4 x 32, 1 x 128 or 2 x 96 targets,
	                                   14: as 12 with each sub-row's block pointer and
	                                   target range precomputed while staging, 15 .. 17: as
	                                   14 reading a 16-bit tile-local copy of the targets
	                                   (2 bytes per synapse, rebuilt with the tiles); per lane
	                                   group and round trip 1 x 256, 4 x 64, 2 x 128 targets,
	                                   18, 19: as 15, 17 storing the finished tile by TMA bulk
	                                   copies, 20, 21: as 15, 17 at two 512-thread CTAs per SM
	                                   (<= 64 registers, 1024 staged sub-rows)                */
	SPICE_TUNE_OVERLAP_SOURCES = 4, /* 1: source populations run on a second stream, 0: inline */
	SPICE_TUNE_GRAPH_WINDOWS   = 5, /* batches only: windows per captured CUDA graph, 0: none */
	SPICE_TUNE_LAUNCH          = 7, /* 1 (default): per window, one grid for the neuron update and
	                                   the source populations, then the delivery, each launched
	                                   as the programmatic dependent of the previous kernel;
	                                   0: sources on a second stream joined by events         */
	SPICE_TUNE_SOURCE_STEPS    = 9, /* consecutive steps each Poisson source CTA draws (default 1);
	                                   0: the fewest that keep the window's grid within one wave
	                                   of resident CTAs                                       */
	SPICE_TUNE_PULL            = 8, /* 1: deliver into every stateful built-in population with
	                                   inputs by the pull path, set before the network first
	                                   steps.  The pull path gathers each target's inputs from
	                                   the CSC adjacency of its connections in connect order and
	                                   ascending source order -- the reference's order of
	                                   additions -- and adds them one IEEE addition at a time:
	                                   bit-exact for any per-synapse weights.  It is always used
	                                   for populations with WEIGHTED inputs and, in deterministic
	                                   mode, for populations with more than four distinct input
	                                   weights (the push path replays per-weight event counts).
	                                   Nets with pulled populations step in windows of at most
	                                   16 steps and need max_delay <= 64 steps             */
	SPICE_TUNE_PERSISTENT      = 10, /* 1 (default): a network whose windows are one step long
	                                   (plastic connections, a minimum delay of one step) runs
	                                   each chunk of up to 1024 steps as one cooperative launch,
	                                   the phases of a step (neuron update and sources; the
	                                   periodic plastic catch-up; deliveries and raster)
	                                   separated by grid-wide barriers (2 .. 32: the same with
	                                   that many CTAs per SM, default 4); 0: one launch per phase.
	                                   Taken into account when the network first steps (it sets
	                                   the input ring up for accumulation); after that it can be
	                                   switched off and on.  Not used with user models, pulled
	                                   populations or user deliver() code                      */
	SPICE_TUNE_NEURON_VARIANT  = 6, /* LIF window of the neuron update: 0 unrolled steps, input
	                                   words in registers, 1 rolled steps over words parked in
	                                   shared memory, 2 as 1 with warp-uniform count replay,
	                                   3 as 0 with warp-uniform count replay, 4 as 1 with
	                                   branch-free replay and the spike output (bitmap words,
	                                   list entries) written once per window, 5 as 4 with
	                                   predicated instead of selected adds, 6 as 4 with the
	                                   count bits tested on the packed input word and the
	                                   leak factors computed once per CTA, 7 as 6 with
	                                   predicated adds, a warp-uniform test for counts of 8 or
	                                   more, ballots kept in registers and list entries reserved
	                                   only for the steps with spikes, 8 as 7 with two neurons
	                                   per thread, 9 as 7 with the step's count replay and LIF
	                                   update as predicated PTX (no branch inside a step)     */
};
int spice_set_tuning(spice_net* net, int knob, int64_t value);
/* The knob's current value into *value: the caller's setting, the shape picked from the network's
 * sizes once it is prepared, or (before that, for knobs the caller did not set) the value that
 * stands until then.  SPICE_TUNE_PERSISTENT reads the knob as set (1: on, with the default CTAs
 * per SM).  SPICE_TUNE_GRAPH_WINDOWS belongs to batches (spice_batch_set_tuning). */
int spice_get_tuning(spice_net* net, int knob, int64_t* value);
/* Upper bound on the steps fused into one neuron-update launch (default: the network's
 * minimum connection delay, the largest value that keeps the reference's semantics). */
int spice_set_window(spice_net* net, int max_window);

/* snn::step() -- spice/src/snn.cpp:7-28. */
int spice_step(spice_net* net);
/* `steps` calls of snn::step(), fused into windows of up to min-delay steps. */
int spice_run(spice_net* net, int64_t steps);
/* spice_run that also records every step's spikes (the raster that samples/matplot.cpp:96-134
 * prints): counts_out[steps][npop] and the ascending spike indices, step-major then population
 * order, into spikes_out (capacity entries).  *total_out = number of spikes recorded.  When both
 * buffers are pinned host memory (cudaHostAlloc, cudaHostRegister, a framework's pinned tensors)
 * the GPU writes them directly while it steps; other host memory is filled from an internal
 * pinned buffer when the call returns. */
int spice_run_record(spice_net* net, int64_t steps, int64_t* counts_out, int32_t* spikes_out,
                     int64_t capacity, int64_t* total_out);

/* NeuronPopulation::spikes(age) -- neuron_population.h:147-153: ascending indices of the
 * neurons of `pop` that fired `age` steps ago, 0 <= age < min(steps run, max_delay). */
int spice_spike_count(spice_net* net, int pop, int64_t age, int64_t* n_out);
int spice_spikes(spice_net* net, int pop, int64_t age, int32_t* out, int64_t capacity,
                 int64_t* n_out);

/* neuron_population::get_neurons() -- neuron_population.h:139-145, one SoA field at a time
 * (float fields V/Gex/Gin, int32 field Tref), into or from a host buffer of size() elements. */
int spice_get_state(spice_net* net, int pop, int field, void* host_out);
int spice_set_state(spice_net* net, int pop, int field, const void* host_in);

int spice_pop_size(spice_net* net, int pop, int64_t* size_out);
int spice_time(spice_net* net, int64_t* time_out);
/* Synaptic events delivered so far (sum over delivered spikes of their CSR row lengths). */
int spice_events(spice_net* net, uint64_t* events_out);

/* csr<T> of a connection -- spice/include/spice/detail/csr.h:69-99: offsets (src+1 int64) and
 * neighbors (synapses int32), copied to host buffers. */
int spice_conn_size(spice_net* net, int conn, int64_t* src_out, int64_t* synapses_out);
/* Per-synapse state of a plastic connection, in CSR order, as stored: a synapse holds its state
 * as of its last catch-up (its source's last delivery or the last multiple of 64 steps), exactly
 * like the reference's synapse_population.  field 0 = W (COUNT: the count), 1 = x_pre,
 * 2 = x_post; out holds synapses floats.  For a WEIGHTED connection field 0 is the weight. */
int spice_get_synapse_state(spice_net* net, int conn, int field, float* out);
int spice_get_csr(spice_net* net, int conn, int64_t* offsets_out, int32_t* neighbors_out);
/* The CSC (transposed) adjacency of a connection, as the pull path uses it: col_offsets_out
 * (dst_size + 1 int64) and sources_out (synapses int32, ascending within each target's column;
 * entry j of column d is the j-th synapse into d in the reference's delivery order).  Built on the
 * GPU from the CSR on first use.  No counterpart in the reference (csr.h holds only the CSR). */
int spice_get_csc(spice_net* net, int conn, int64_t* col_offsets_out, int32_t* sources_out);

/* fixed_probability(p) adjacency of one projection (the generator behind
 * spice_connect_fixed_probability) for callers that cannot allocate device memory: real-time loops
 * whose device memory is fixed up front (an allocation may block or fail mid-run), and hosts that
 * own every device buffer themselves (a framework's caching allocator, a cgo or JNI runtime handing
 * out an arena).  No counterpart in the reference.  It allocates nothing: every intermediate buffer
 * lives in one static device array of about 4.3 MiB inside this library, held by every GPU that
 * loads the library until the process exits.  The caller passes device buffers: offsets
 * (src_count + 1 int64) and neighbors (neighbors_capacity int32); the seed is the 128-bit
 * util::seed_seq value (seed_lo, seed_hi) of the projection.  The result equals the adjacency
 * spice_connect_fixed_probability generates for a projection with that seed.
 * Limits: src_count <= 65536 and src_count * (max_degree + 1) <= 262144 draws (max_degree =
 * floor(dst*p + 3 sqrt(dst*p*(1-p)))); larger requests fail with SPICE_EINVAL.  A neighbors buffer
 * that is too small fails with SPICE_EOVERFLOW and *synapses_out = the size needed.
 * The first call on a device (and the first after its context was reset) looks up the scratch
 * array's device address.  Every call uses the
 * same scratch, which keeps the previous call's contents, so calls whose GPU work overlaps (on
 * different streams or threads) race: serialise them.  The call synchronises `stream` (a
 * cudaStream_t, NULL for the default stream) once, to read the synapse count. */
int spice_fixed_probability_noalloc(int64_t src_count, int64_t dst_count, double p, uint64_t seed_lo,
                                    uint64_t seed_hi, int64_t* offsets, int32_t* neighbors,
                                    int64_t neighbors_capacity, int64_t* synapses_out, void* stream);

/* Per-kernel timing with CUDA events recorded on the net's stream around every launch. */
int spice_set_profiling(spice_net* net, int on);
/* kind: 0 = neuron update, 1 = spike delivery, 2 = raster extraction, 3 = source populations
 * (Poisson / external trains).  Returns the number of launches and their summed device time (ms)
 * since profiling was switched on. */
int spice_kernel_stats(spice_net* net, int kind, int64_t* launches_out, double* ms_out);
/* The same launches' device spans, kinds 0 (neuron update, with the sources and raster blocks of
 * its grid) and 1 (spike delivery): per launch, from the first of its CTAs to start to the last to
 * finish on the GPU's global timer, summed (ms), and the number of launches with a span -- the
 * launch's own duration without the fixed cost of the CUDA-event pair around it.  No counterpart
 * in the reference (it has no device).  Other kinds, the persistent steps and user-model launches
 * report no spans. */
int spice_kernel_span(spice_net* net, int kind, int64_t* launches_out, double* ms_out);
/* Number of kernels this library launched on the net's stream so far. */
int spice_launch_count(spice_net* net, int64_t* launches_out);

/* The cudaStream_t the net launches on (for callers that order their own work or time it with
 * CUDA events on the same stream). */
int spice_get_stream(spice_net* net, void** stream_out);
int spice_synchronize(spice_net* net);
const char* spice_last_error(void);

/* ---- User-defined neuron models (the reference's Neuron concepts, concepts.h:10-58) ----
 * The engine keeps the population's state (an array of the user's neuron struct, or nothing for a
 * stateless model), its spike bitmap ring and lists, and delivers synapses into float members of
 * the struct registered as fields; the update is user code: a kernel compiled in the user's nvcc
 * translation unit (include/spice/snn.h instantiates it over the model type) and launched by the
 * callback below on the engine's stream, once per window, with everything it reads and writes
 * described by spice_user_window.
 * Stateful models: per step k of the window, apply the inputs of input-ring slot (slot0 + k) mod D
 * (deterministic: per-group counts replayed as sequential float adds of group_weight into the
 * group's field; atomic: the field sums), clear them when zero_inputs, then update; apply_only = 1
 * (K = 0) asks for the inputs of slot0 to be applied and cleared with no update (state reads).
 * Stateless models draw from the step's random stream: neuron i's stream position is
 * draw_offset + i (one draw per neuron and step, as the reference's sequential loop gives a model
 * that draws once), reached through the step's jump table (tables[k]) and the chunk polynomials
 * chunk_poly[c] = x^(draw_offset + 32 c) mod P (32 neurons per chunk).
 * Spikes: bitmap word (hslot0 + k) mod Hb, bit i; and the unordered list of step k,
 * list[(list_k0 + k) * size ...], reserved with atomicAdd on counts[k * npop + pop].
 * Version 2 adds the per-step seeds, declared draws of stateful models and pulled inputs:
 * a stateful model whose update draws a fixed number of times per neuron (spice_user_draws) takes
 * its draws from the step's stream at position draw_offset + i * draws for neuron i -- the
 * reference's order, populations in add order and neurons ascending (snn.cpp:12-15,
 * neuron_population.h:72-77) -- reached through tables[k], chunk_poly[i / 32] = x^(draw_offset +
 * 32 (i / 32) draws) mod P and (i mod 32) * draws further draws.  A population receiving
 * per-synapse weights is pulled (pull = 1): before step k, for each bin f < pull_F, the weights
 * pull_G[pull_base[i] + e], e in [koff[k * pull_F + f], koff[k * pull_F + f + 1]) with koff =
 * pull_koff + i * (pull_nbins + 1), add in order to field pull_field[f]; when koff[0] < 0 the first
 * koff[1] entries of pull_A (weight bits | (step mask | bin << 16) << 32) with bit k set add instead.
 * apply_only on a pulled population applies the bins of step 0 and empties them (koff[f] =
 * koff[pull_F] for f < pull_F; or clears bit 0 of the masks). */
#define SPICE_USER_ABI_VERSION 2
typedef struct spice_user_window {
	int version;
	int apply_only;
	int64_t t0;
	int K, slot0, hslot0, Hb, list_k0, npop, pop, mode;
	int64_t D;
	const float* dts;          /* [K] */
	const void* tables;        /* [K][16][256] 16-byte jump table entries (stateless) */
	const void* chunk_poly;    /* [nwords] 16-byte polynomials (stateless) */
	int64_t draw_offset;
	void* state;               /* [size] user neuron structs (stateful) */
	int64_t size;
	int neuron_bytes, nwords;
	uint32_t* bits;
	int32_t* list;
	int32_t* counts;
	uint32_t* cnt;             /* deterministic input ring [D][size][W] */
	float* acc;                /* atomic input ring [D][size][F] */
	int W, F, ngroups, zero_inputs;
	int group_word[4], group_shift[4], group_bits[4], group_field[4];
	float group_weight[4];
	int field_offset[3];       /* byte offset of field f in the neuron struct */
	int field_slot[3];         /* atomic mode: index of field f among the F sums (-1: none) */
	/* version >= 2 */
	const void* step_seeds;    /* [K] 16-byte seed_seq values seeding the window's step streams */
	int draws;                 /* stateful: draws per neuron and update (spice_user_draws), else 0 */
	int pull, pull_F, pull_nbins;
	int pull_field[3];
	const int64_t* pull_base;
	uint64_t* pull_A;
	const float* pull_G;
	int32_t* pull_koff;
	uint64_t* hist;            /* target of plastic synapses: per neuron, bit j = spiked j steps ago;
	                              shift in every step's spike bit (neuron_population.h:126-132) */
	int direct;                /* 1: inputs arrive directly in the neuron structs (USER_DELIVER
	                              targets): nothing to apply */
} spice_user_window;
typedef int (*spice_user_update_fn)(const spice_user_window* window, void* stream, void* ctx);
/* stateful: neuron_bytes > 0 (any struct size) and init_neuron = the initial struct (copied to every
 * neuron); the population consumes a seed like every stateful population (neuron_population.h:56-60). */
int spice_add_user_population(spice_net* net, int64_t size, int stateful, int neuron_bytes,
                              const void* init_neuron, spice_user_update_fn fn, void* ctx, int* pop_out);
/* Registers a float member (byte offset) of a stateful user population as a synapse target field;
 * returns its field index (0..2; the same offset gives the same index). */
int spice_user_field(spice_net* net, int pop, int byte_offset, int* field_out);
/* The whole state array of a stateful user population (size * neuron_bytes bytes). */
int spice_get_user_state(spice_net* net, int pop, void* host_out);
int spice_set_user_state(spice_net* net, int pop, const void* host_in);
/* Declares that the update of stateful user population `pop` draws exactly `draws` random numbers
 * per neuron and step from the step's shared stream (the reference hands every stateful neuron
 * that stream, snn.cpp:12-15); the engine then positions each neuron in the reference's order.
 * Without it a stateful user model draws from an independent stream per (population, neuron,
 * step), seeded by mixing the step's seed with the neuron index: statistically uniform and
 * independent, not the reference's sequence.  Before the network first steps.  No counterpart in
 * the reference. */
int spice_user_draws(spice_net* net, int pop, int draws);
/* The seed_seq value a stateful population consumed when it was added: the seed of the stream its
 * init() draws from (stateful_neuron_adapter: rng(seed++), neuron_population.h:56-67). */
int spice_population_seed(spice_net* net, int pop, uint64_t* lo_out, uint64_t* hi_out);
/* The seeds a connection consumed: [0, 1] the adjacency's (_graph(c, seed++)), [2, 3] the
 * PerSynapseInit stream's (rng(seed++), synapse_population.h:30-41) or 0 when it has none. */
int spice_connection_seeds(spice_net* net, int conn, uint64_t* seeds_out);
/* Per-synapse weights of a WEIGHTED connection created with params[2] = 1 or 2 (host weights), in
 * CSR order (spice_get_csr), before the network first steps. */
int spice_set_synapse_weights(spice_net* net, int conn, const float* weights);

/* ---- User plastic synapses (SPICE_SYNAPSE_USER_PLASTIC) ----
 * The engine keeps the per-synapse state, the per-source ages (bit 63: pending pre update, low
 * bits: step + 1) and the target's 64-step spike history, and calls `fn` on its stream:
 *   what = 0 every 64 steps (snn.cpp:17-19): every synapse catches up to `time`, then each
 *            source's age becomes time + 1 (synapse_population.h:68-72);
 *   what = 1 each step (snn.cpp:21-25): the spiking sources of bitmap slot `hslot` catch up their
 *            synapses to `time`, deliver (when `deliver`) the state's word weight_word into
 *            dst_acc[(slot * dst_size + target) * F + fslot], add their row lengths to *events and
 *            set their age to (time + 1) | bit 63.
 * The catch-up of one synapse is synapse_population.h:88-116.  chunks_done (per source, zero) is
 * scratch for kernels that split a row over several CTAs. */
#define SPICE_USER_PLASTIC_ABI_VERSION 1
typedef struct spice_user_plastic_call {
	int version, what;
	int64_t time;
	float dt;
	int hslot;
	int64_t slot;
	int deliver;
	int64_t src_size, dst_size;
	const int64_t* off;
	const int32_t* nb;
	void* state;
	int synapse_bytes, weight_word;
	uint64_t* ages;
	uint32_t* chunks_done;
	int64_t max_row;
	const uint64_t* dst_hist;
	const uint32_t* src_bits;
	int src_nwords;
	float* dst_acc;
	int F, fslot;
	unsigned long long* events;
} spice_user_plastic_call;
typedef int (*spice_user_plastic_fn)(const spice_user_plastic_call* call, void* stream, void* ctx);
/* ---- User deliver() code (SPICE_SYNAPSE_USER_DELIVER) ----
 * Called at the end of every step `time` >= delay - 1 for the spikes of step time - delay + 1
 * (bitmap slot `hslot` of the source): every target whose sources spiked applies deliver() for
 * each such synapse in ascending source order (a target's CSC column, col_pos[e] = the synapse's
 * CSR index, its state's position) -- or, when deliver() reads source neurons of the target's own
 * population, the spiking sources in ascending order each deliver along their CSR row
 * (synapse_population.h:118-133), since a later source may read what an earlier delivery wrote.
 * Adds the delivered synapses to *events. */
#define SPICE_USER_DELIVER_ABI_VERSION 1
typedef struct spice_user_deliver_call {
	int version;
	int64_t time;
	float dt;
	int hslot;
	int64_t src_size, dst_size;
	const int64_t* off;
	const int32_t* nb;
	const int64_t* col_off;
	const int32_t* col_src;
	const int64_t* col_pos;
	const uint32_t* src_bits;
	int src_nwords;
	const void* src_state;     /* source neuron structs (stateful sources) */
	void* dst_state;           /* target neuron structs */
	void* synapse_state;       /* synapse structs, CSR order (stateful synapses), else NULL */
	int same_population;       /* source population == target population */
	unsigned long long* events;
} spice_user_deliver_call;
typedef int (*spice_user_deliver_fn)(const spice_user_deliver_call* call, void* stream, void* ctx);
/* Registers the kernels of USER_DELIVER connection `conn` and its synapses' initial state
 * (synapse_bytes bytes; NULL for stateless synapses), before the network first steps. */
int spice_user_deliver(spice_net* net, int conn, spice_user_deliver_fn fn, void* ctx, const void* init_synapse);

/* Registers the kernels of USER_PLASTIC connection `conn` and the initial state of every synapse
 * (synapse_bytes bytes), before the network first steps. */
int spice_user_plastic(spice_net* net, int conn, spice_user_plastic_fn fn, void* ctx, const void* init_synapse);
/* The whole per-synapse state array of a USER_PLASTIC (or stateful USER_DELIVER) connection, CSR
 * order: set before the network
 * first steps (a PerSynapseInit run on the host), read at any time (each synapse as of its last
 * catch-up, like the reference's synapse_population). */
int spice_set_user_synapse_state(spice_net* net, int conn, const void* host_in);
int spice_get_user_synapse_state(spice_net* net, int conn, void* host_out);

/* ---- Batched networks (no counterpart in the reference) ----
 * Many independent nets stepped together: one launch per kernel kind and window covers the
 * populations and connections of every member, so networks far too small to fill the GPU alone
 * run at the throughput of one large network.  The members are ordinary nets built with the calls
 * above (each with its own populations, connections and seed); they must share dt, max_delay,
 * mode and time, have the same minimum delay and no external_input population.  The batch runs
 * on the members' own device state: between batch runs every per-net call (spikes, state, csr,
 * events, spice_run) works on each member as usual, and a member's results are bit-identical to
 * running it alone.  The window loop is captured in a CUDA graph (SPICE_TUNE_GRAPH_WINDOWS windows
 * per graph launch, default 8); each window's time-dependent values (time, dt, step seeds) are
 * advanced on the device, so the graph is replayed unchanged.  The members must stay alive while
 * the batch exists; tuning knobs 0..4 set on a batch apply to it and to every member. */
typedef struct spice_batch spice_batch;
int spice_batch_create(spice_net* const* nets, int nnets, spice_batch** out);
int spice_batch_destroy(spice_batch* batch);
/* `steps` steps of every member; returns when they are done. */
int spice_batch_run(spice_batch* batch, int64_t steps);
int spice_batch_set_tuning(spice_batch* batch, int knob, int64_t value);
/* Per-kernel timing (CUDA events; windows launched directly, not through the graph).  Kinds as
 * spice_kernel_stats, plus 4 = window prologue (dt, step seeds) and jump tables. */
int spice_batch_set_profiling(spice_batch* batch, int on);
int spice_batch_kernel_stats(spice_batch* batch, int kind, int64_t* launches_out, double* ms_out);
/* Kernels launched for this batch so far (graph replays count their kernels). */
int spice_batch_launch_count(spice_batch* batch, int64_t* launches_out);
int spice_batch_get_stream(spice_batch* batch, void** stream_out);

/* ---- Differentiable recurrent LIF layer (no counterpart in the reference) ----
 * n_in inputs x_t in {0,1} and n_rec LIF neurons, delay 1 step, t = 1..T:
 *   u_t = beta .* v_{t-1} + W_in^T x_{t-1} + W_rec^T s_{t-1},  s_t = H(u_t - theta),
 *   v_t = u_t - theta .* s_t (reset by subtraction),  counts = sum_t s_t.
 * Weights are per synapse in the CSR order of the connectivity (by source); theta and beta are per
 * neuron.  The backward is the adjoint recursion backwards in time with the fast-sigmoid surrogate
 * 1 / (1 + slope |u - theta|)^2 in place of H'.  relaxed = 1 replaces H by the smooth
 * g(x) = (1 + slope x / (1 + slope |x|)) / 2 in the forward and uses its exact derivative (for
 * finite-difference checks).  One CTA per sample keeps the layer in shared memory.
 * All arrays except the CSR of spice_lif_layer_create are device pointers; stream is a
 * cudaStream_t (NULL: default stream).  Layouts: x_bits [batch][steps][ceil(n_in/32)] (bit k of word
 * k/32 = input k), counts and grad_counts [batch][n_rec], spikes [batch][steps][n_rec] (s_t at t-1),
 * v_ckpt [batch][ceil(steps/checkpoint_every) + 1][n_rec].  The forward stores spikes and v every
 * checkpoint_every steps; the backward recomputes each segment from its checkpoint.  Gradients are
 * summed over the batch (a fixed order: bit-reproducible). */
typedef struct spice_lif_layer spice_lif_layer;
int spice_lif_layer_create(int n_in, int n_rec, const int64_t* in_off, const int32_t* in_nb,
                           const int64_t* rec_off, const int32_t* rec_nb, spice_lif_layer** out);
int spice_lif_layer_destroy(spice_lif_layer* layer);
int spice_lif_layer_synapses(spice_lif_layer* layer, int64_t* in_syn_out, int64_t* rec_syn_out);
int spice_lif_forward(spice_lif_layer* layer, int batch, int steps, int checkpoint_every, int relaxed,
                      float slope, const uint32_t* x_bits, const float* w_in, const float* w_rec,
                      const float* theta, const float* beta, float* counts, float* spikes, float* v_ckpt,
                      void* stream);
int spice_lif_backward(spice_lif_layer* layer, int batch, int steps, int checkpoint_every, int relaxed,
                       float slope, const uint32_t* x_bits, const float* w_in, const float* w_rec,
                       const float* theta, const float* beta, const float* spikes, const float* v_ckpt,
                       const float* grad_counts, float* grad_w_in, float* grad_w_rec, float* grad_theta,
                       float* grad_beta, void* stream);

/* Self-test (no reference counterpart): the plastic synapses' trace decay computes
 * (float)((double)x * f) -- the reference's skip() -- in integer arithmetic; this compares it with
 * the GPU's double multiply for `count` random pairs (finite x >= 0 including subnormals, f in
 * [2^-4, 2^5)).  mismatches: pairs whose results differ in any bit; first_a / first_f (either may
 * be NULL): the first such pair. */
int spice_selftest_skip_rounding(int64_t count, uint64_t seed, int64_t* mismatches, uint32_t* first_a,
                                 double* first_f);

#ifdef __cplusplus
}
#endif
#endif
