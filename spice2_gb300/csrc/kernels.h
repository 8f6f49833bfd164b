// kernels.h -- launch wrappers of the engine's CUDA kernels (gen.cu, step.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "internal.h"

namespace spice_gb300 {

// ---- gen.cu ----
struct GenRequest {
	int64_t src, dst;
	double p;
	u128 seed;
	int64_t* offsets;   // out (device), src + 1
	int32_t* neighbors; // out (device)
	int64_t synapses;   // out
};
int64_t fp_max_degree(int64_t dst_count, double p);
// Generates all requested projections (rows of every projection are chained concurrently).
cudaError_t generate_fixed_probability(cudaStream_t stream, std::vector<GenRequest>& reqs);
// Rows whose stop index was recomputed with the exact sequential loop (near-tie sums), process-wide.
extern unsigned long long g_gen_fallbacks;

// Scratch of one projection's generation (generate_fixed_probability_into).
struct GenScratch {
	double* gaps;          // [max_draws]
	uint64_t* fx;          // [max_draws]
	uint64_t* tots;        // [max_draws / 256]
	int32_t* lens;         // [max_src]
	u128* superstates;     // [max_super]
	u128* polys;           // [max_super]
	u128* subpolys;        // [256]
	int64_t* block_sums;   // [max_src / 1024 + 1]
	void* job;             // gen_row_job_bytes()
	unsigned long long* fallbacks;
	int64_t max_draws, max_src, max_super;
};
size_t gen_row_job_bytes();
// w[e] = wmax * canonical<float>(draw e of the stream seeded by `seed`), e < n: the per-synapse
// weights of a weighted connection in CSR order (synapse_population.h:34-41).  Synchronises.
cudaError_t init_synapse_weights(cudaStream_t stream, u128 seed, int64_t n, float wmax, float* w);

// ---- pull.cu ----
// CSC of a CSR (rows sources, ndst targets): col_off[ndst + 1], col_src[synapses] ascending per
// column (CSR order among duplicates), col_w[synapses] = wts in CSC order when wts is not null.
// Allocates and frees its own scratch; synchronises.
// col_pos (when not null): the CSR index of each CSC entry.
cudaError_t build_csc(cudaStream_t stream, const int64_t* off, const int32_t* nb, const float* wts, int64_t rows,
                      int64_t ndst, int64_t synapses, int64_t* col_off, int32_t* col_src, float* col_w,
                      int64_t* col_pos = nullptr);
// A fixed_weight or weighted connection into a USER_DELIVER target: at the end of step `time`, every
// target adds, in ascending source order, the weights of its synapses whose source spiked in bitmap
// slot hslot, to the float at byte offset `field_offset` of its neuron struct.
cudaError_t launch_direct_add(cudaStream_t stream, ConnDev const& c, int hslot, void* dst_state, int neuron_bytes,
                              int field_offset, unsigned long long* events);
// base[i] = sum over nconn column-start arrays (a device array of device pointers) of [i], i <= n.
cudaError_t pull_region_bases(cudaStream_t stream, const int64_t* const* col_offs, int nconn, int64_t n, int64_t* base);

// One window's pull: masks of every (source, delay) set, events of the window that just ended, then
// the active lists and bins of every pulled population.
struct PullArgs {
	int64_t t;               // first pulled step (the next window's first step)
	int K;                   // steps pulled (the net's window length, <= kPullMaxWindow)
	int Hb;                  // bitmap ring length
	int nsets;
	const PullSet* sets;     // [nsets]
	int nev;
	const PullEvJob* ev;     // [nev] one per pulled connection
	int64_t t_emit0;         // the window that just ended (its spikes' events are counted)
	int k_emit;
	unsigned long long* events;
	int npull;
	const int* pull_pops;    // [npull] pulled population ids
	const int* pull_blk;     // [npull + 1] prefix of their k_pull CTAs
	int pull_blocks;
	const PopDev* pops;
	const ConnDev* conns;    // by-target order (PopDev::in_begin / in_end)
	// push-and-sort gather (ps_units > 0): the active synapses of every pulled connection are pushed
	// into their targets' regions, then each target sorts its entries into the scan's order
	int ps_nconn;
	const int* ps_conn;      // [ps_nconn] by-target position of each pulled connection
	const int* ps_pop;       // [ps_nconn] its pulled population
	int64_t ps_units;        // > 0: the push-and-sort gather is used (k_pull_masks lists the spiking sources)
	int ps_grid;             // CTAs of the scatter (resident on every SM; warps stride over the rows)
};
cudaError_t launch_pull(cudaStream_t stream, PullArgs const& a, std::vector<PullSet> const& sets,
                        std::vector<PullEvJob> const& ev);
// the longest source row the push-and-sort gather's sort key can hold (its CSR offset within the row)
constexpr int64_t kPushSortMaxRow = 1ll << 19;
// entries one target can take per window in the push-and-sort gather (more: the scan)
constexpr int kPushSortSlots = 64;
// Largest tile of the compact-target delivery mappings (15 .. 21): their staged sub-rows take
// ~41 KB of static shared memory beside the tile, within the 227 KiB of one CTA.
constexpr int kCompactMaxTileBytes = 176 * 1024;
int pull_blocks_for(int64_t size);  // k_pull CTAs of a population of `size` neurons
// Applies the bins of the first pulled step to the state and empties them (state reads).
cudaError_t launch_pull_apply_first(cudaStream_t stream, PopDev const& P);
cudaError_t generate_fixed_probability_into(cudaStream_t stream, int64_t src, int64_t dst, double p, u128 seed,
                                            GenScratch const& sc, int64_t* offsets, int32_t* neighbors,
                                            int64_t capacity, int64_t* synapses);

// ---- step.cu ----
// Exclusive scan of n int32 row lengths into n + 1 int64 offsets.
cudaError_t scan_row_lengths(cudaStream_t stream, const int32_t* lens, int64_t n, int64_t* offsets);
// The same with caller-provided block sums (n / 1024 + 1 entries).
cudaError_t scan_row_lengths_into(cudaStream_t stream, const int32_t* lens, int64_t n, int64_t* offsets,
                                  int64_t* block_sums);

// Maximum in-degree of target population neurons over the connections of one input group.
cudaError_t max_indegree(cudaStream_t stream, const int32_t* const* nbs, const int64_t* nsyn, int nconn,
                         int64_t dst_size, uint32_t* scratch, uint32_t* max_out);

// Jump tables of steps t < nsteps: tables[t][g][m] = XOR of T^(8g+q)(seed_t) over the bits q of m.
cudaError_t launch_jump_tables(cudaStream_t stream, const u128* seeds, int64_t nsteps, u128* tables);

// Threads per CTA of the neuron update and source populations (one neuron, or one 32-neuron Poisson
// chunk, per thread); smaller CTAs balance the window's grid across the SMs more evenly.
constexpr int kNeuronThreads = 128;
constexpr int kNeuronBlocksPerSM = 2048 / kNeuronThreads;  // resident CTAs of the register-lean kernels
constexpr int kHistKind = 8;  // blk_kind flag of populations with a post-spike history
// Delivery work mappings (SPICE_TUNE_DELIVER_ALGO 0 .. kDeliverAlgos - 1), one kernel per mapping
// and mode.
constexpr int kDeliverAlgos = 22;
// the mappings that read ConnDev::nb16
__host__ __device__ constexpr bool compact_algo(int algo) { return algo >= 15 && algo <= 21; }
constexpr int kDeliverFns   = 2 * kDeliverAlgos;

struct WindowArgs {
	int64_t t0;        // absolute step of the window's first step
	int K;             // steps in this window
	int slot0;         // (t0 - 1) mod D: input slot applied before the update of step t0
	int hslot0;        // t0 mod Hb: bitmap slot of step t0
	int64_t D;         // input ring length (max delay)
	int Hb;            // bitmap ring length
	int npop;
	int mode;
	const PopDev* pops;
	const float* dts;     // dt of steps t0 .. t0+K-1
	const u128* tables;   // jump tables of step t0 (then t0+1, ...)
	const u128* seeds;    // seed_seq values of steps t0 .. t0+K-1 (the step streams' seeds)
	int64_t tab_net_stride;  // 0: one net
	int32_t* counts;      // [K][npop] spikes per step and population (window parity buffer)
	int list_k0;          // first list slot of this window's parity: lists are [2K][size]
	int variant;          // LIF window variant (SPICE_TUNE_NEURON_VARIANT)
	int blk_begin[kMaxPops + 1];
	int blk_kind[kMaxPops];      // 0: per-neuron window CTAs, 1: Poisson step CTAs, 2: external,
	                             // 3: per-neuron CTAs of a LIF whose inputs all add to V (16-bit counts)
	                             // (k_neurons launches kinds 0 and 3, k_sources kinds 1 and 2);
	                             // + kHistKind: the population keeps a post-spike history
	int blk_per_step[kMaxPops];  // Poisson / external: CTAs per step
	int src_steps;               // Poisson: consecutive steps each source CTA draws (>= 1)
	int64_t ext_pos[kMaxPops];   // external: train position of step t0
	unsigned long long* span;    // profiling: [0] ~earliest CTA start, [1] latest CTA end (global ns); else null
};
cudaError_t launch_neurons(cudaStream_t stream, WindowArgs const& a, int nblocks);
struct RasterArgs;
// The neuron blocks of `a`, the source blocks of `s` and (r not null) the raster blocks of `*r` in one
// grid; pdl: launched as the programmatic dependent of the stream's previous kernel.
cudaError_t launch_window(cudaStream_t stream, WindowArgs const& a, int nblocks, WindowArgs const& s, int nsrc_blocks,
                          RasterArgs const* r, bool pdl);
cudaError_t launch_sources(cudaStream_t stream, WindowArgs const& a, int nblocks);

struct DeliverArgs {
	int64_t t0;
	int K;
	int64_t D;
	int nconn;
	int npop;
	int mode;
	const ConnDev* conns;    // grouped by target population (PopDev::in_begin/in_end)
	const PopDev* pops;
	const int32_t* counts;   // [K][npop] of this window
	int32_t* counts_next;    // the other parity buffer, zeroed here
	int counts_next_len;
	unsigned long long* events;
	int64_t slot_lo;         // first input slot the window's spikes reach: t0 + dmin - 1
	int pdl;                 // launched as the programmatic dependent of the stream's previous kernel
	int nslots;              // K + dmax - dmin
	int ntiles_total;
	int tile_begin[kMaxPops + 1];  // prefix over populations of their tile counts
	int smem_bytes;
	int parts;               // CTAs sharing one (slot, tile); > 1 flushes with reductions
	int algo;                // 0: warp-flattened sub-rows, 1: one thread per spike, 2: warp per spike,
	                         // 3: thread per spike with 16-byte loads, 4: thread per spike, pipelined,
	                         // 5 / 6: 4 / 8 lanes per spike, pipelined, 7: 5 at <= 32 registers,
	                         // 8 / 9: 4 lanes per spike with sub-row descriptors staged in shared memory,
	                         // 2 / 4 sub-rows in flight per group
	int list_k0;             // first list slot of this window's parity
	unsigned long long* span;  // profiling: [0] ~earliest CTA start, [1] latest CTA end (global ns); else null
};
// One CTA per (input slot, target tile): shared-memory accumulation, then a coalesced flush.
cudaError_t launch_deliver(cudaStream_t stream, DeliverArgs const& a, int threads);
// bounds[s][t] = position in row s of the first target >= t * tile (t = 0..ntiles).
cudaError_t launch_compact_targets(cudaStream_t stream, const int32_t* nb, int64_t synapses, int tile, uint16_t* nb16);
cudaError_t launch_tile_bounds(cudaStream_t stream, const int64_t* off, const int32_t* nb, int64_t rows, int tile,
                               int ntiles, int64_t* bounds);

// Plastic connections: the periodic catch-up of every synapse (every 64 steps), and the delivery
// of the spikes in bitmap slot hslot into input ring slot `slot` at step `time`.
cudaError_t launch_plastic_update_all(cudaStream_t stream, ConnDev const& c, int64_t time);
cudaError_t launch_selftest_mulround(cudaStream_t stream, int64_t count, uint64_t seed, unsigned long long* mismatches,
                                     unsigned long long* first);
cudaError_t launch_plastic_deliver(cudaStream_t stream, ConnDev const& c, int64_t time, int hslot, int64_t slot,
                                   bool deliver, unsigned long long* events);

// Applies the inputs waiting in ring slot (t - 1) to the state and clears them.
cudaError_t launch_apply_pending(cudaStream_t stream, const PopDev* pops, int npop_dev, const int* stateful,
                                 int nstateful, std::vector<PopDev> const& hpops, int64_t t, int64_t D,
                                 int mode);

// Ascending indices of the set bits of one bitmap step: out[0..n), *n_out.
cudaError_t launch_extract(cudaStream_t stream, const uint32_t* bits, int nwords, int32_t* out, int64_t* n_out);

// Raster of a window: for k < K and population p, the ascending spikes of step t0 + k are
// written at an offset taken from *cursor; tab[(row0 + k) * npop + p] = {offset, count}.
// Raster of one window in (step, population) order: the spikes of step k of population p start at
// the window's base plus the spike counts of the window's earlier (step, population) pairs.
struct RasterArgs {
	int64_t t0;
	int K;
	int Hb;
	int npop;
	const PopDev* pops;
	const int32_t* counts;  // the window's spike counts [K][npop]
	int64_t* base;          // [2]: raster position of this window (base[parity]) and of the next
	int parity;
	int32_t* out;           // raster, capacity entries (mapped host memory)
	int64_t capacity;
	int64_t* step_counts;   // [rows][npop] spike counts (mapped host memory)
	int64_t row0;           // row of the window's first step
	int pdl;                // launched as the programmatic dependent of the stream's previous kernel
};
cudaError_t launch_raster(cudaStream_t stream, RasterArgs const& a);

// Persistent steps (step.cu): every step of a chunk of a network whose windows are one step long
// in one cooperative launch, the phases of a step separated by grid-wide barriers.
constexpr int kPersistThreads = kNeuronThreads;  // the window bodies' CTA size
constexpr int kPersistChunk   = 256;             // synapses of one delivery work unit (a warp's)
constexpr int kPersistPlasticChunk = 64;         // ... of a plastic row (each synapse catches up first)
constexpr int kPersistBlocksPerSM = 4;           // default CTAs per SM (fewer barrier arrivals)
struct PersistArgs {
	int64_t t0;             // first step of the launch
	int nsteps;
	int parity0;            // counts / list half of step t0
	int D, Hb, npop, nconn, mode;
	const PopDev* pops;
	const ConnDev* conns;   // any order (deliveries of one step commute)
	const float* dts;       // dt of steps t0 .. t0 + nsteps - 1
	const u128* tables;     // their jump tables (kJumpTable each; null without Poisson draws)
	int32_t* counts;        // [2][npop] spikes per step, per parity
	unsigned long long* events;
	unsigned* barrier;      // arrival counter, zero at launch
	int* status;            // set nonzero when a barrier wait gave up (results then invalid)
	int any_plastic;
	int nblk;                     // CTA-sized work items of the update phase
	int blk_begin[kMaxPops + 1];  // per population: first work item
	int blk_kind[kMaxPops];       // as WindowArgs::blk_kind
	int blk_per_step[kMaxPops];   // Poisson: items per step
	int64_t ext_pos[kMaxPops];    // external: train position of step t0
	int64_t chunks[kMaxConns];    // per connection: delivery units per spike (ceil(max row / chunk length))
	int start_at_c;               // the first step's update (phase A) ran in the previous launch
	int end_after_a;              // the last step stops after its update (its deliveries follow in the next launch)
	int external_full;            // the periodic catch-up of every plastic synapse runs as its own kernel
	int record;                   // extract the raster of every step (RasterArgs below, K = 1)
	int rec_parity0;              // raster base parity of step t0
	RasterArgs raster;
};
// blocks_per_sm: resident CTAs of the persistent kernel per SM (0: query only).
cudaError_t persist_occupancy(int mode, int* blocks_per_sm);
cudaError_t launch_persist(cudaStream_t stream, PersistArgs const& a, int grid);

// ---- batched networks (step.cu kernels, batch.cu runtime) ----
// The window a batch's kernels step, advanced on the device by k_batch_prologue.
struct BatchClock {
	int64_t t0;          // first step of the current window
	int parity;          // counts / list half of the current window
	int k;               // steps in the current window
	int64_t next_t0;
	int next_parity;
	float kahan_c, kahan_sum;  // the nets' shared dt accumulator (identical dt and time)
};

// Fixed arguments of a batch's kernels.  Populations are numbered net-major; PopDev::net is the
// net, PopDev::in_begin/in_end index `conns` (all nets' connections in by-target order, src
// renumbered to the global population index).
struct BatchArgs {
	const PopDev* pops;
	const ConnDev* conns;
	int npop, nnets;
	const int* nblk_begin;   // [npop + 1] per-neuron CTAs (k_batch_neurons)
	const int* nblk_kind;    // [npop] 0 generic, 3 fast LIF
	int nblk_total;
	const int* sblk_begin;   // [npop + 1] Poisson CTAs per step (k_batch_sources)
	int sblk_total;
	const int* tile_begin;   // [npop + 1] delivery tiles
	int ntiles_total;
	int32_t* counts;         // [2][K][npop]
	float* dts;              // [K] dt of the current window's steps
	u128* step_seeds;        // [nnets][K]
	u128* tables;            // [nnets][K][kJumpTable]
	u128* seed_state;        // [nnets] seed_seq states
	unsigned long long* const* net_events;  // [nnets] each net's event counter
	BatchClock* clock;
	float dt;
	int K, Hb;
	int64_t D;
	int mode, dmin, dmax, parts, algo, smem_bytes, only_fast;
};
cudaError_t launch_batch_prologue(cudaStream_t stream, BatchArgs const& b, int k);
cudaError_t launch_batch_sources(cudaStream_t stream, BatchArgs const& b, int k);
cudaError_t launch_batch_neurons(cudaStream_t stream, BatchArgs const& b);
// Sets the delivery kernel's dynamic shared memory limit for b's mode, mapping and tile size.
cudaError_t configure_batch_deliver(BatchArgs const& b);
cudaError_t launch_batch_deliver(cudaStream_t stream, BatchArgs const& b, int k, int threads);

}  // namespace spice_gb300
