// internal.h -- engine data structures shared by the host runtime (net.cu) and the kernels.
//
// Device memory layout of one net (all SoA, one CUDA allocation per array):
//   population p:  state fields V/Gex/Gin (f32[N]) and Tref (i32[N]);
//                  spike bitmap ring   bits[Hb][ceil(N/32)]  (ascending order = bit order);
//                  spike list ring     list[K][N] int32 (unordered, consumed by delivery);
//                  input ring          deterministic: cnt[D][N][W] u32 packed per-group counts
//                                      atomic:        acc[D][N][F] f32 per-field sums.
//   connection c:  CSR offsets i64[src+1], neighbors i32[synapses]; weighted synapses also
//                  weights f32[synapses] (CSR order); connections into a pulled population also
//                  the CSC: column starts i64[dst+1], sources i32[synapses] (ascending per
//                  column), weighted ones their weights f32[synapses] in CSC order.
//   pulled population p (inputs gathered per target in the reference's order, pull.cu):
//                  region starts i64[N+1] (prefix of the in-degree over its connections),
//                  active synapses A u64[in-synapses], step-grouped weights G f32[in-synapses],
//                  bin offsets koff i32[N][K*F+1].
//   per run:       dt[t] (Kahan-compensated), per-step xoroshiro state basis T^i(s_t), i < 128.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "rng.h"

namespace spice_gb300 {

constexpr int kMaxPops    = 64;
constexpr int kMaxConns   = 256;
constexpr int kMaxGroups  = 4;   // distinct consecutive (field, weight) runs per target population
constexpr int kMaxWindow  = 64;  // steps fused into one neuron-update launch
constexpr int kBasis      = 128; // states per step basis
constexpr int kJumpTable  = 16 * 256;  // u128 entries of one step's jump table
constexpr int kPoissonChunk = 32; // consecutive Poisson neurons per thread (one jump each)
constexpr int kPullMaxWindow = 16; // steps fused into one window in a net with pulled populations

enum Model { POISSON = 0, LIF = 1, LIF_COND = 2, EXTERNAL = 3, USER = 4 };

struct Group {
	int field;     // 0 V, 1 Gex, 2 Gin
	float weight;  // the fixed_weight of every connection in the group
};

// Device-side view of one population, passed by value to kernels.
struct PopDev {
	int model;
	int nwords;          // ceil(N / 32)
	int64_t size;
	int64_t draw_offset; // first draw of this population in each step's stream
	float* V;
	float* Gex;
	float* Gin;
	int32_t* T;
	float p0, p1, p2;    // model parameters (POISSON: rate; LIF: Vthres, Tref, TmemInv)
	uint32_t* bits;      // [Hb][nwords]
	int32_t* list;       // [K][size]
	// input ring
	uint32_t* cnt;       // deterministic: [D][size][W]
	float* acc;          // atomic:        [D][size][F]
	int W;               // u32 words per neuron and slot (deterministic)
	int F;               // fields per neuron and slot (atomic)
	int ngroups;
	int group_shift[kMaxGroups];  // bit offset of the group's counter in its word (0 or 16)
	int group_word[kMaxGroups];
	int group_bits[kMaxGroups];   // 16 or 32
	int group_field[kMaxGroups];
	float group_weight[kMaxGroups];
	int field_slot[3];   // atomic mode: index of field f in the F per-neuron sums (-1: unused)
	// tiled delivery: targets are accumulated in shared-memory tiles of `tile` neurons
	int tile;            // neurons per tile
	int ntiles;
	int in_begin, in_end;  // this population's incoming connections in the by-target order
	int zero_inputs;     // 1: the input ring is accumulated (mixed delays), consumers clear it;
	                     // 0: each slot is fully overwritten by one delivery, no clearing needed
	const u128* chunk_poly;  // POISSON: x^(draw_offset + 32 c) mod P for chunk c
	int net;             // index of the owning net in a batch (0 outside batches)
	uint64_t* hist;      // targets of plastic connections: post-spike history, bit k = spiked k steps ago
	void* ustate;        // USER: [size] neuron structs of the user's model
	int ubytes;          // USER: bytes per neuron struct (0: stateless)
	// EXTERNAL: cyclic train
	const int32_t* ext_counts;
	const int64_t* ext_off;
	const int32_t* ext_idx;
	int ext_steps;
	// pulled population: every input is gathered per target, in connect order and ascending source
	// order, by the pull kernel over the CSC (pull.cu), instead of the push delivery's input ring
	int pull;                  // 1: pulled
	int pull_F;                // state fields receiving inputs (bins per step)
	int pull_field[3];         // field of bin f
	int pull_nbins;            // K * pull_F: bin (k, f) = k * pull_F + f
	const int64_t* pull_base;  // [size + 1] region of neuron i in pull_A / pull_G
	uint64_t* pull_A;          // active synapses: weight bits | (step mask | f << 16) << 32, CSC order
	float* pull_G;             // the active synapses' weights grouped by bin
	int32_t* pull_koff;        // [size][nbins + 1] bin starts in the region; [i][0] = -1: not grouped,
	                           // [i][1] = number of active synapses (the neuron walks pull_A)
	int32_t* pull_fill;        // [size] entries pushed for the target this window (push-and-sort gather)
	uint4* ps_slot;            // [size][kPushSortSlots] their sort keys (x: low, y: high word) and
	                           // weights (z: bits), one 16-byte store each (push-and-sort gather)
	int direct;                // USER_DELIVER target: inputs applied into the neuron structs at the end of each step
};

struct ConnDev {
	int src, dst;
	int delay;
	int group;
	float weight;
	int field;
	int64_t src_size;
	int64_t dst_size;
	const int64_t* off;
	const int32_t* nb;
	const int32_t* src_list;  // [K][src_size] spike lists of the source population
	uint32_t* dst_cnt;        // deterministic input ring of the target: [D][dst_size][W]
	float* dst_acc;           // atomic input ring of the target: [D][dst_size][F]
	int W, word;              // words per neuron, word of this connection's group
	uint32_t inc;             // 1 << group_shift
	int F, fslot;             // atomic: sums per neuron, index of this connection's field
	const int64_t* bounds;    // [src_size][ntiles of dst + 1]: row positions where each tile starts
	const uint16_t* nb16;     // targets as indices within their tile (nb mod tile), CSR order; built
	                          // for the compact-target delivery mapping only, else null
	// plastic synapses (synapse_population.h:27-140); plastic = 0 for fixed_weight
	int plastic;              // SPICE_SYNAPSE_ISTDP or SPICE_SYNAPSE_COUNT
	float eta, alpha, cdt;    // iSTDP: learning rate, 2 rho0 tau, dt / tau
	float* sW;                // per synapse, CSR order: W (counting model: the count)
	float* sA;                // x_pre
	float* sB;                // x_post
	uint64_t* ages;           // per source: bit 63 = pending pre update, low bits = step + 1
	uint32_t* chunks_done;    // per source: row chunks of the current plastic delivery finished
	int64_t max_row;          // longest row (synapses of one source)
	const uint64_t* dst_hist; // the target population's post-spike history
	const double* skip_tab;   // pow(1 - dt/tau, n) for n = -64 .. 64
	const uint64_t* skip_pk;  // the same factors packed for mul_f32_f64_rn (significand | exponent << 53)
	int src_nwords;           // source bitmap words
	const uint32_t* src_bits; // source spike bitmap ring [Hb][src_nwords]
	// weighted synapses (a per-synapse weight drawn at construction) and pulled targets
	const float* wts;         // weighted: per-synapse weight, CSR order (else null)
	const int64_t* csc_off;   // [dst_size + 1] column starts (pulled targets)
	const int32_t* csc_src;   // [synapses] source of each entry, ascending within a column
	const float* csc_w;       // weighted: weights in CSC order
	const uint32_t* pull_orb; // [src_nwords] bit s: source s spiked in one of the pulled steps
	const uint32_t* pull_wm;  // [src_size] bit k: source s spiked at (first pulled step + k - delay)
	const int32_t* pull_act;  // the window's spiking sources of its (source, delay) set, and their number
	const int* pull_nact;
};

// Window masks of one (source population, delay) pair of pulled connections (pull.cu).
struct PullSet {
	int src, delay, nwords;
	int64_t size;
	const uint32_t* bits;  // the source's bitmap ring [Hb][nwords]
	uint32_t* orb;         // [nwords]
	uint32_t* wm;          // [size]
	int32_t* act;          // [size] the window's spiking sources (any order), push-and-sort gather
	int* nact;             // their number (emptied by k_ps_sort for the next window)
};

// A pulled connection whose spikes' events are counted (row lengths from its CSR).
struct PullEvJob {
	int nwords;
	const uint32_t* bits;
	const int64_t* off;
};

struct Pop {
	PopDev d;
	int64_t ext_pos0 = 0;  // train position at time 0
	std::vector<int32_t> ext_counts_h;
	std::vector<int64_t> ext_off_h;
	bool stateful = false;
	// USER: the update callback and the struct offsets of the fields synapses target
	void* ufn  = nullptr;  // spice_user_update_fn
	void* uctx = nullptr;
	int nfields = 0;
	int field_offset[3] = {0, 0, 0};
	int udraws = 0;        // USER stateful: declared draws per neuron and update (0: counter-based stream)
	u128 seed = {0, 0};    // stateful: the seed its init stream would use (seed_seq value consumed at add)
};

struct Conn {
	ConnDev d;
	int64_t synapses = 0;
	bool weighted    = false;     // per-synapse weights (d.wts)
	float wmax       = 0;
	int wsource      = 0;         // weighted: 0 drawn by the engine, 1 / 2 set by the host (2: no init seed)
	// USER_PLASTIC: the user's per-synapse structs and kernels
	void* ustate     = nullptr;   // [synapses * ubytes], CSR order
	int ubytes       = 0;
	int weight_word  = 0;
	bool init_seed   = false;     // USER_PLASTIC with PerSynapseInit: consumes the init stream's seed
	bool udeliver    = false;     // USER_DELIVER: deliver() is user code (spice_user_deliver)
	bool reads_source = false;    // USER_DELIVER: deliver() takes the source neuron
	int64_t* csc_pos = nullptr;   // CSR index of each CSC entry (USER_DELIVER with synapse state)
	void* ufn        = nullptr;   // spice_user_plastic_fn
	void* uctx       = nullptr;
	std::vector<char> uinit;      // the initial synapse struct
	std::vector<char> uhost;      // whole-array initial state set by the host (PerSynapseInit)
	u128 gseed       = {0, 0};    // the adjacency's seed
	u128 wseed       = {0, 0};    // the PerSynapseInit stream's seed
	uint16_t* nb16    = nullptr;  // owned storage of d.nb16
	int nb16_tile     = 0;        // tile size d.nb16 was built for
	bool adj         = false;
	float w0 = 0, rho0 = 0, tau = 0;  // plastic parameters
};

struct PendingGen {  // a fixed_probability connection whose adjacency is not generated yet
	int conn;
	u128 seed;
	double p;
};

struct KernelStat {
	int64_t launches      = 0;
	double ms             = 0;
	int64_t span_launches = 0;  // launches with a device span (first CTA start to last CTA end)
	double span_ms        = 0;
};

}  // namespace spice_gb300

struct spice_net {
	float dt;
	int64_t max_delay;   // D, in steps
	int64_t time = 0;
	spice_gb300::u128 seed;
	float kahan_c = 0, kahan_sum = 0;
	int mode      = 0;
	int max_window = 0;  // 0 = auto
	bool prepared  = false;
	int device     = 0;
	cudaStream_t stream = nullptr;       // main stream: neuron updates, deliveries, readback
	cudaStream_t stream_src = nullptr;   // source populations (Poisson, external), one window ahead
	cudaEvent_t ev_src[2] = {nullptr, nullptr};   // sources of a parity done
	cudaEvent_t ev_free[2] = {nullptr, nullptr};  // lists/counts of a parity consumed and cleared
	cudaEvent_t ev_tab = nullptr;        // dt and jump tables of the current chunk written
	cudaEvent_t ev_chunk[2] = {nullptr, nullptr};  // the last chunk stepped from buffer b has ended
	int chunk_buf = 0;                   // buffer of the next chunk
	bool has_sources = false;
	bool user_seeds  = false;            // stateful user populations read the step seeds
	std::vector<spice_gb300::Pop> pops;
	std::vector<spice_gb300::Conn> conns;
	int K  = 1;          // window length used by run
	int Hb = 1;          // bitmap ring length
	int64_t total_draws = 0;  // draws per step over all populations
	// device-wide buffers
	unsigned long long* d_events = nullptr;
	int32_t* d_counts  = nullptr;  // [2][K][npop] spikes per window step and population, per parity
	float* d_dt        = nullptr;  // [2][run capacity]
	spice_gb300::u128* d_seeds = nullptr;  // [2][run capacity]
	spice_gb300::u128* d_tables = nullptr;  // [2][run capacity][16][256] jump tables
	int64_t run_cap    = 0;
	spice_gb300::PopDev* d_pops   = nullptr;
	spice_gb300::ConnDev* d_conns = nullptr;
	// host staging
	float* h_dt        = nullptr;
	spice_gb300::u128* h_seeds = nullptr;
	// raster extraction
	// spice_run_record: the raster and the per-step spike counts are written by the GPU straight into
	// mapped pinned host memory (grown on demand), in (step, population) order
	int32_t* h_raster    = nullptr;  // [raster_cap]
	int64_t raster_cap   = 0;
	int64_t* h_rcounts   = nullptr;  // [rcounts_cap]
	int64_t rcounts_cap  = 0;
	int64_t* d_raster_base = nullptr;  // [2] raster position of the current / next window
	// the raster's destination during one spice_run_record call: the staging buffers above, or the
	// caller's own buffers when they are pinned host memory the GPU can write
	int32_t* rec_out   = nullptr;
	int64_t rec_cap    = 0;
	int64_t* rec_counts = nullptr;
	int32_t* d_tmp     = nullptr;  // spikes(age) extraction
	int64_t* d_tmp_n   = nullptr;
	// profiling
	bool profiling = false;
	std::vector<cudaEvent_t> ev_pool;
	std::vector<std::pair<int, int>> ev_pending;  // (kind, event index of the start)
	unsigned long long* d_span = nullptr;         // [event pool size]: per event pair, ~first CTA start and
	                                              // last CTA end of a delivery launch (zeroed after each harvest)
	size_t ev_used = 0;
	spice_gb300::KernelStat stats[5];
	int64_t launches = 0;
	std::vector<void*> allocations;
	std::vector<spice_gb300::PendingGen> gen_pending;
	std::vector<int64_t> ext_t_set;  // per population: step at which its external train was set
	int parity = 0;                  // which half of d_counts the next window writes
	spice_gb300::ConnDev* d_conns_by_dst = nullptr;  // connections grouped by target population
	std::vector<int> by_dst;         // connection ids in that order
	// launch shape (tunable); the values below stand until the network is prepared, which picks
	// the tile, threads, mapping and LIF variant for the network's sizes (default_shape in net.cu)
	// unless the caller set them
	int tile_bytes = 24 * 1024;      // shared memory per delivery tile
	int deliver_threads = 256;       // threads per delivery CTA
	int deliver_parts = 1;           // CTAs per (slot, tile)
	int deliver_algo = 1;            // delivery work mapping
	int overlap_sources = 1;         // source kernels on their own stream
	int neuron_variant  = 0;         // LIF window variant of the neuron update
	bool tile_set = false, threads_set = false, algo_set = false, variant_set = false;  // set by the caller
	int launch_mode     = 1;         // 1: neurons and sources in one grid, programmatic dependent launches
	int src_steps       = 1;         // steps per Poisson CTA (0: the fewest that fit the grid in one wave)
	// persistent steps (step.cu k_persist): windows of one step, one cooperative launch per chunk
	int persist_knob    = 1;         // SPICE_TUNE_PERSISTENT
	bool persist_ok     = false;     // eligible when prepared (the input ring accumulates)
	int persist_grid    = 0;         // resident CTAs over all SMs
	unsigned* d_barrier = nullptr;   // arrival counter of the grid barriers
	int* d_pstatus      = nullptr;   // nonzero: a barrier wait gave up
	int* h_pstatus      = nullptr;   // pinned copy, read after the chunk's event
	std::vector<int64_t> persist_chunks;  // per connection: delivery units per spike
	int sm_count        = 1;
	int dmin = 1, dmax = 1;          // connection delays in steps
	bool plastic = false;            // any plastic connection (windows of one step)
	// pull delivery (pull.cu)
	bool pull_all = false;           // every stateful built-in population with inputs is pulled
	bool any_pull = false;
	bool any_direct = false;         // populations receiving USER_DELIVER synapses (windows of one step)
	std::vector<spice_gb300::PullSet> pull_sets;
	std::vector<spice_gb300::PullEvJob> pull_ev;
	spice_gb300::PullSet* d_pull_sets = nullptr;
	spice_gb300::PullEvJob* d_pull_ev = nullptr;
	std::vector<int> pull_pops;      // pulled populations
	int* d_pull_pops     = nullptr;  // [npull]
	int* d_pull_blk      = nullptr;  // [npull + 1] prefix of their pull CTAs
	int pull_blocks      = 0;
	// push-and-sort gather of the pulled populations (pull.cu k_ps_*): units (pulled connection,
	// source bitmap word); falls back to the CSC scan when a row is too long for the sort key
	bool ps_ok           = false;
	int ps_nconn         = 0;
	int* d_ps_conn       = nullptr;  // [ps_nconn] connection (by-target position) of each pulled connection
	int* d_ps_pop        = nullptr;  // [ps_nconn] its pulled population
	int64_t ps_units     = 0;
};

namespace spice_gb300 {
int set_last_error(int code, std::string const& msg);  // net.cu
int neuron_block_kind(PopDev const& P);                  // net.cu
int net_prepare(spice_net* n);                           // net.cu
}  // namespace spice_gb300
