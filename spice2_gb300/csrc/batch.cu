// batch.cu -- batched networks (include/spice_gb300.h, spice_batch_*).
//
// The member nets keep their own device state (populations, input rings, spike bitmaps and lists,
// adjacency); the batch holds concatenated descriptors of all of them (populations numbered
// net-major, connections in by-target order with global population indices), the shared spike
// counters of the window, the per-net step seeds and jump tables, and a device clock.  A window
// of k steps is five launches whatever the number of nets:
//   k_batch_prologue  -- advance the clock, dt of the k steps, every net's step seeds, clear counts
//   k_jump_tables     -- jump tables of every (net, step)            (second stream)
//   k_batch_sources   -- Poisson populations of every net            (second stream)
//   k_batch_neurons   -- per-neuron populations of every net, k steps in registers
//   k_batch_deliver   -- every (input slot, target tile) of every net
// Because nothing time-dependent is passed by the host, a sequence of full windows is captured
// once as a CUDA graph and replayed.
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "spice_gb300.h"
#include "internal.h"
#include "kernels.h"

using namespace spice_gb300;

struct spice_batch {
	std::vector<spice_net*> nets;
	int device          = 0;
	cudaStream_t stream = nullptr, stream_src = nullptr;
	cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
	BatchArgs args{};
	std::vector<void*> allocs;
	bool draws         = false;
	int threads        = 256;
	int overlap        = 1;
	int graph_windows  = 8;
	cudaGraphExec_t graph = nullptr;
	int64_t graph_launches = 0;  // kernels in one replay of the graph
	bool profiling     = false;
	std::vector<cudaEvent_t> ev_pool;
	std::vector<std::pair<int, size_t>> ev_pending;  // (kind, index of the start event)
	size_t ev_used = 0;
	KernelStat stats[5];
	int64_t launches = 0;
};

namespace {

int bfail(int code, std::string const& msg) { return set_last_error(code, msg); }

#define B_CUDA_TRY(x)                                                                                     \
	do {                                                                                                  \
		cudaError_t const e_ = (x);                                                                       \
		if (e_ != cudaSuccess) return bfail(SPICE_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
	} while (0)

#define B_TRY(x)                       \
	do {                               \
		int const r_ = (x);            \
		if (r_ != SPICE_OK) return r_; \
	} while (0)

template <class T>
int balloc(spice_batch* b, T** p, size_t count, bool zero = true) {
	size_t const bytes = sizeof(T) * (count > 0 ? count : 1);
	cudaError_t e      = cudaMalloc((void**)p, bytes);
	if (e != cudaSuccess) {
		*p = nullptr;
		return bfail(e == cudaErrorMemoryAllocation ? SPICE_ENOMEM : SPICE_ECUDA,
		             std::string("cudaMalloc(") + std::to_string(bytes) + " bytes): " + cudaGetErrorString(e));
	}
	b->allocs.push_back(*p);
	if (zero) B_CUDA_TRY(cudaMemsetAsync(*p, 0, bytes, b->stream));
	return SPICE_OK;
}

template <class T>
int upload(spice_batch* b, T** p, std::vector<T> const& h) {
	B_TRY(balloc(b, p, h.size(), false));
	if (!h.empty()) B_CUDA_TRY(cudaMemcpy(*p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
	return SPICE_OK;
}

void drop_graph(spice_batch* b) {
	if (b->graph) cudaGraphExecDestroy(b->graph);
	b->graph = nullptr;
}

int sync_members(spice_batch* b) {
	for (spice_net* n : b->nets) {
		B_CUDA_TRY(cudaStreamSynchronize(n->stream));
		if (n->stream_src) B_CUDA_TRY(cudaStreamSynchronize(n->stream_src));
	}
	return SPICE_OK;
}

// (Re)builds the concatenated descriptors from the members' current layout (tiles, tuning).
int build(spice_batch* b) {
	drop_graph(b);
	B_CUDA_TRY(cudaStreamSynchronize(b->stream));
	for (void* p : b->allocs) cudaFree(p);
	b->allocs.clear();
	int const nn = (int)b->nets.size();
	std::vector<PopDev> hp;
	std::vector<ConnDev> hc;
	std::vector<int> nblk{0}, nkind, sblk{0}, tiles{0};
	int smem = 4, dmin = 1 << 30, dmax = 0;
	bool only_fast = true;
	b->draws = false;
	for (int i = 0; i < nn; i++) {
		spice_net* n      = b->nets[i];
		int const pbase   = (int)hp.size();
		int const cbase   = (int)hc.size();
		for (auto const& pop : n->pops) {
			PopDev d = pop.d;
			d.net    = i;
			d.in_begin += cbase;
			d.in_end += cbase;
			hp.push_back(d);
			int nb = 0, kind = 0, sb = 0;
			if (d.model == POISSON) {
				sb = (d.nwords + kNeuronThreads - 1) / kNeuronThreads;
				b->draws |= d.size > 0;
			} else {
				nb   = (int)((d.size + kNeuronThreads - 1) / kNeuronThreads);
				kind = neuron_block_kind(d);
				if (nb > 0) only_fast &= kind == 3;
			}
			nblk.push_back(nblk.back() + nb);
			nkind.push_back(kind);
			sblk.push_back(sblk.back() + sb);
			tiles.push_back(tiles.back() + d.ntiles);
			if (d.ntiles) smem = std::max(smem, 4 * d.tile * (n->mode == SPICE_MODE_DETERMINISTIC ? d.W : d.F));
		}
		for (int ci : n->by_dst) {
			ConnDev c = n->conns[ci].d;
			c.src += pbase;
			c.dst += pbase;
			hc.push_back(c);
		}
		dmin = std::min(dmin, n->dmin);
		dmax = std::max(dmax, n->dmax);
	}
	spice_net const* n0 = b->nets[0];
	BatchArgs& a        = b->args;
	a.npop              = (int)hp.size();
	a.nnets             = nn;
	a.nblk_total        = nblk.back();
	a.sblk_total        = sblk.back();
	a.ntiles_total      = tiles.back();
	a.dt                = n0->dt;
	a.K                 = n0->K;
	a.Hb                = n0->Hb;
	a.D                 = n0->max_delay;
	a.mode              = n0->mode;
	a.dmin              = dmin;
	a.dmax              = std::max(dmax, dmin);
	a.smem_bytes        = smem;
	a.only_fast         = only_fast ? 1 : 0;
	PopDev* pops = nullptr;
	ConnDev* conns = nullptr;
	int *nb = nullptr, *nk = nullptr, *sb = nullptr, *tb = nullptr;
	B_TRY(upload(b, &pops, hp));
	B_TRY(upload(b, &conns, hc));
	B_TRY(upload(b, &nb, nblk));
	B_TRY(upload(b, &nk, nkind));
	B_TRY(upload(b, &sb, sblk));
	B_TRY(upload(b, &tb, tiles));
	a.pops       = pops;
	a.conns      = conns;
	a.nblk_begin = nb;
	a.nblk_kind  = nk;
	a.sblk_begin = sb;
	a.tile_begin = tb;
	std::vector<unsigned long long*> evp;
	for (spice_net* n : b->nets) evp.push_back(n->d_events);
	unsigned long long** ev = nullptr;
	B_TRY(upload(b, &ev, evp));
	a.net_events = ev;
	B_TRY(balloc(b, &a.counts, (size_t)2 * a.K * std::max(a.npop, 1)));
	B_TRY(balloc(b, &a.dts, (size_t)a.K));
	B_TRY(balloc(b, &a.step_seeds, (size_t)nn * a.K));
	a.tables = nullptr;
	if (b->draws) B_TRY(balloc(b, &a.tables, (size_t)nn * a.K * kJumpTable, false));
	B_TRY(balloc(b, &a.seed_state, (size_t)nn));
	B_TRY(balloc(b, &a.clock, 1));
	B_CUDA_TRY(configure_batch_deliver(a));
	B_CUDA_TRY(cudaStreamSynchronize(b->stream));
	return SPICE_OK;
}

// ---- profiling: CUDA event pairs around launches ----
int prof_begin(spice_batch* b, int kind, cudaStream_t st, size_t* slot) {
	*slot = (size_t)-1;
	if (!b->profiling) return SPICE_OK;
	while (b->ev_used + 2 > b->ev_pool.size()) {
		cudaEvent_t e;
		B_CUDA_TRY(cudaEventCreate(&e));
		b->ev_pool.push_back(e);
	}
	*slot = b->ev_used;
	b->ev_used += 2;
	B_CUDA_TRY(cudaEventRecord(b->ev_pool[*slot], st));
	b->ev_pending.push_back({kind, *slot});
	return SPICE_OK;
}

int prof_end(spice_batch* b, size_t slot, cudaStream_t st) {
	if (slot == (size_t)-1) return SPICE_OK;
	B_CUDA_TRY(cudaEventRecord(b->ev_pool[slot + 1], st));
	return SPICE_OK;
}

int harvest(spice_batch* b) {
	if (b->ev_pending.empty()) return SPICE_OK;
	B_CUDA_TRY(cudaStreamSynchronize(b->stream));
	B_CUDA_TRY(cudaStreamSynchronize(b->stream_src));
	for (auto const& pr : b->ev_pending) {
		float ms = 0;
		B_CUDA_TRY(cudaEventElapsedTime(&ms, b->ev_pool[pr.second], b->ev_pool[pr.second + 1]));
		b->stats[pr.first].launches++;
		b->stats[pr.first].ms += ms;
	}
	b->ev_pending.clear();
	b->ev_used = 0;
	return SPICE_OK;
}

// One window of k steps of every member (the five launches of the file comment).
int enqueue_window(spice_batch* b, int k, int64_t* launched) {
	BatchArgs const& a     = b->args;
	cudaStream_t const src = b->overlap ? b->stream_src : b->stream;
	size_t slot;
	int64_t n = 0;
	B_TRY(prof_begin(b, 4, b->stream, &slot));
	B_CUDA_TRY(launch_batch_prologue(b->stream, a, k));
	n++;
	if (b->overlap) {
		B_CUDA_TRY(cudaEventRecord(b->ev_fork, b->stream));
		B_CUDA_TRY(cudaStreamWaitEvent(b->stream_src, b->ev_fork, 0));
	}
	if (b->draws) {
		B_CUDA_TRY(launch_jump_tables(src, a.step_seeds, (int64_t)a.nnets * a.K, a.tables));
		n++;
	}
	B_TRY(prof_end(b, slot, src));
	if (a.sblk_total > 0) {
		B_TRY(prof_begin(b, 3, src, &slot));
		B_CUDA_TRY(launch_batch_sources(src, a, k));
		B_TRY(prof_end(b, slot, src));
		n++;
	}
	if (b->overlap) B_CUDA_TRY(cudaEventRecord(b->ev_join, b->stream_src));
	if (a.nblk_total > 0) {
		B_TRY(prof_begin(b, 0, b->stream, &slot));
		B_CUDA_TRY(launch_batch_neurons(b->stream, a));
		B_TRY(prof_end(b, slot, b->stream));
		n++;
	}
	if (b->overlap) B_CUDA_TRY(cudaStreamWaitEvent(b->stream, b->ev_join, 0));
	if (a.ntiles_total > 0) {
		B_TRY(prof_begin(b, 1, b->stream, &slot));
		B_CUDA_TRY(launch_batch_deliver(b->stream, a, k, b->threads));
		B_TRY(prof_end(b, slot, b->stream));
		n++;
	}
	*launched += n;
	return SPICE_OK;
}

// Captures graph_windows full windows (k = K) once; replays reuse it until the layout changes.
int ensure_graph(spice_batch* b) {
	if (b->graph) return SPICE_OK;
	cudaGraph_t g = nullptr;
	B_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
	int64_t n = 0;
	int r     = SPICE_OK;
	for (int w = 0; w < b->graph_windows && r == SPICE_OK; w++) r = enqueue_window(b, b->args.K, &n);
	cudaError_t const e = cudaStreamEndCapture(b->stream, &g);
	if (r != SPICE_OK) {
		if (g) cudaGraphDestroy(g);
		return r;
	}
	if (e != cudaSuccess) return bfail(SPICE_ECUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
	cudaError_t const ei = cudaGraphInstantiate(&b->graph, g, 0);
	cudaGraphDestroy(g);
	if (ei != cudaSuccess) {
		b->graph = nullptr;
		return bfail(SPICE_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ei));
	}
	b->graph_launches = n;
	return SPICE_OK;
}

bool same_float(float x, float y) { return memcmp(&x, &y, sizeof(float)) == 0; }

// Members must agree on everything the shared clock and window stand for.
int check_lockstep(spice_batch* b) {
	spice_net const* n0 = b->nets[0];
	for (spice_net const* n : b->nets)
		if (n->time != n0->time || !same_float(n->kahan_c, n0->kahan_c) || !same_float(n->kahan_sum, n0->kahan_sum))
			return bfail(SPICE_ESTATE, "batched nets must be at the same step (a member was stepped on its own)");
	return SPICE_OK;
}

}  // namespace

extern "C" int spice_batch_create(spice_net* const* nets, int nnets, spice_batch** out) {
	if (!out) return bfail(SPICE_EINVAL, "out must not be NULL");
	*out = nullptr;
	if (!nets || nnets <= 0) return bfail(SPICE_EINVAL, "a batch needs at least one net");
	for (int i = 0; i < nnets; i++) {
		if (!nets[i]) return bfail(SPICE_EINVAL, "nets must not be NULL");
		for (int j = 0; j < i; j++)
			if (nets[j] == nets[i]) return bfail(SPICE_EINVAL, "a net appears twice in the batch");
	}
	spice_net* n0 = nets[0];
	for (int i = 0; i < nnets; i++) {
		spice_net* n = nets[i];
		if (n->device != n0->device) return bfail(SPICE_EINVAL, "batched nets must live on the same device");
		if (!same_float(n->dt, n0->dt)) return bfail(SPICE_EINVAL, "batched nets must have the same dt");
		if (n->max_delay != n0->max_delay) return bfail(SPICE_EINVAL, "batched nets must have the same max_delay");
		if (n->mode != n0->mode) return bfail(SPICE_EINVAL, "batched nets must use the same mode");
		for (auto const& p : n->pops)
			if (p.d.model == EXTERNAL || p.d.model == USER)
				return bfail(SPICE_EINVAL, "batched nets cannot have external_input or user-defined populations");
		for (auto const& c : n->conns) {
			if (c.d.plastic) return bfail(SPICE_EINVAL, "batched nets cannot have plastic connections");
			if (c.weighted) return bfail(SPICE_EINVAL, "batched nets cannot have weighted (per-synapse weight) connections");
		}
		if (n->pull_all) return bfail(SPICE_EINVAL, "batched nets cannot use the pull path");
	}
	int dev_prev = 0;
	cudaGetDevice(&dev_prev);
	if (dev_prev != n0->device) B_CUDA_TRY(cudaSetDevice(n0->device));
	for (int i = 0; i < nnets; i++) B_TRY(net_prepare(nets[i]));
	for (int i = 0; i < nnets; i++)
		if (nets[i]->any_pull)
			return bfail(SPICE_EINVAL, "batched nets cannot have pulled populations (more than 4 distinct input weights)");
	for (int i = 0; i < nnets; i++)
		if (nets[i]->K != n0->K || nets[i]->Hb != n0->Hb)
			return bfail(SPICE_EINVAL, "batched nets must have the same minimum delay (window length)");
	auto* b   = new spice_batch();
	b->nets.assign(nets, nets + nnets);
	b->device = n0->device;
	int r     = check_lockstep(b);
	if (r == SPICE_OK) r = sync_members(b);
	cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream_src, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
	if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
	if (e != cudaSuccess) r = bfail(SPICE_ECUDA, std::string("stream/event creation: ") + cudaGetErrorString(e));
	// the first member's launch shape for all (the tile layout lives in each member)
	b->threads    = n0->deliver_threads;
	b->overlap    = n0->overlap_sources;
	b->args.parts = n0->deliver_parts;
	b->args.algo  = n0->deliver_algo;
	for (int i = 1; i < nnets && r == SPICE_OK; i++) {
		r = spice_set_tuning(nets[i], SPICE_TUNE_TILE_BYTES, n0->tile_bytes);
		if (r == SPICE_OK) r = spice_set_tuning(nets[i], SPICE_TUNE_DELIVER_PARTS, n0->deliver_parts);
	}
	if (r == SPICE_OK) r = build(b);
	if (r != SPICE_OK) {
		spice_batch_destroy(b);
		return r;
	}
	*out = b;
	return SPICE_OK;
}

extern "C" int spice_batch_destroy(spice_batch* b) {
	if (!b) return SPICE_OK;
	if (b->stream) cudaStreamSynchronize(b->stream);
	if (b->stream_src) cudaStreamSynchronize(b->stream_src);
	drop_graph(b);
	for (void* p : b->allocs) cudaFree(p);
	for (cudaEvent_t e : b->ev_pool) cudaEventDestroy(e);
	if (b->ev_fork) cudaEventDestroy(b->ev_fork);
	if (b->ev_join) cudaEventDestroy(b->ev_join);
	if (b->stream_src) cudaStreamDestroy(b->stream_src);
	if (b->stream) cudaStreamDestroy(b->stream);
	delete b;
	return SPICE_OK;
}

extern "C" int spice_batch_run(spice_batch* b, int64_t steps) {
	if (!b) return bfail(SPICE_EINVAL, "batch must not be NULL");
	if (steps < 0) return bfail(SPICE_EINVAL, "steps must be >= 0");
	if (steps == 0) return SPICE_OK;
	B_TRY(check_lockstep(b));
	B_TRY(sync_members(b));
	int const nn = (int)b->nets.size();
	BatchArgs const& a  = b->args;
	spice_net const* n0 = b->nets[0];
	std::vector<u128> seeds(nn);
	for (int i = 0; i < nn; i++) seeds[i] = b->nets[i]->seed;
	BatchClock clk{};
	clk.next_t0     = n0->time;
	clk.next_parity = 0;
	clk.kahan_c     = n0->kahan_c;
	clk.kahan_sum   = n0->kahan_sum;
	B_CUDA_TRY(cudaMemcpyAsync(a.seed_state, seeds.data(), sizeof(u128) * nn, cudaMemcpyHostToDevice, b->stream));
	B_CUDA_TRY(cudaMemcpyAsync(a.clock, &clk, sizeof(clk), cudaMemcpyHostToDevice, b->stream));
	int64_t left = steps;
	if (b->graph_windows > 0 && !b->profiling) {
		int64_t const per_graph = (int64_t)b->graph_windows * a.K;
		if (left >= per_graph) B_TRY(ensure_graph(b));
		while (left >= per_graph) {
			B_CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
			b->launches += b->graph_launches;
			left -= per_graph;
		}
	}
	while (left > 0) {
		int const k = (int)std::min<int64_t>(a.K, left);
		B_TRY(enqueue_window(b, k, &b->launches));
		left -= k;
	}
	B_CUDA_TRY(cudaMemcpyAsync(seeds.data(), a.seed_state, sizeof(u128) * nn, cudaMemcpyDeviceToHost, b->stream));
	B_CUDA_TRY(cudaMemcpyAsync(&clk, a.clock, sizeof(clk), cudaMemcpyDeviceToHost, b->stream));
	B_CUDA_TRY(cudaStreamSynchronize(b->stream));
	B_CUDA_TRY(cudaStreamSynchronize(b->stream_src));
	for (int i = 0; i < nn; i++) {
		spice_net* n = b->nets[i];
		n->seed      = seeds[i];
		n->kahan_c   = clk.kahan_c;
		n->kahan_sum = clk.kahan_sum;
		n->time += steps;
	}
	return SPICE_OK;
}

extern "C" int spice_batch_set_tuning(spice_batch* b, int knob, int64_t value) {
	if (!b) return bfail(SPICE_EINVAL, "batch must not be NULL");
	switch (knob) {
		case SPICE_TUNE_TILE_BYTES:
		case SPICE_TUNE_DELIVER_PARTS:
			// the tile layout and the ring convention live in the members
			for (spice_net* n : b->nets) B_TRY(spice_set_tuning(n, knob, value));
			if (knob == SPICE_TUNE_DELIVER_PARTS) b->args.parts = (int)value;
			if (!b->allocs.empty()) B_TRY(build(b));
			return SPICE_OK;
		case SPICE_TUNE_DELIVER_THREADS:
			for (spice_net* n : b->nets) B_TRY(spice_set_tuning(n, knob, value));
			b->threads = (int)value;
			drop_graph(b);
			return SPICE_OK;
		case SPICE_TUNE_DELIVER_ALGO:
			for (spice_net* n : b->nets) B_TRY(spice_set_tuning(n, knob, value));
			b->args.algo = (int)value;
			drop_graph(b);
			if (!b->allocs.empty() && compact_algo((int)value)) B_TRY(build(b));  // members' compact targets
			if (!b->allocs.empty()) B_CUDA_TRY(configure_batch_deliver(b->args));
			return SPICE_OK;
		case SPICE_TUNE_OVERLAP_SOURCES:
			for (spice_net* n : b->nets) B_TRY(spice_set_tuning(n, knob, value));
			B_CUDA_TRY(cudaStreamSynchronize(b->stream));
			B_CUDA_TRY(cudaStreamSynchronize(b->stream_src));
			b->overlap = (int)value;
			drop_graph(b);
			return SPICE_OK;
		case SPICE_TUNE_GRAPH_WINDOWS:
			if (value < 0 || value > 1024) return bfail(SPICE_EINVAL, "graph windows must be in [0, 1024]");
			b->graph_windows = (int)value;
			drop_graph(b);
			return SPICE_OK;
	}
	return bfail(SPICE_EINVAL, "unknown tuning knob");
}

extern "C" int spice_batch_set_profiling(spice_batch* b, int on) {
	if (!b) return bfail(SPICE_EINVAL, "batch must not be NULL");
	B_TRY(harvest(b));
	b->profiling = on != 0;
	for (auto& s : b->stats) s = KernelStat{};
	return SPICE_OK;
}

extern "C" int spice_batch_kernel_stats(spice_batch* b, int kind, int64_t* launches, double* ms) {
	if (!b) return bfail(SPICE_EINVAL, "batch must not be NULL");
	if (kind < 0 || kind > 4) return bfail(SPICE_EINVAL, "unknown kernel kind");
	B_TRY(harvest(b));
	if (launches) *launches = b->stats[kind].launches;
	if (ms) *ms = b->stats[kind].ms;
	return SPICE_OK;
}

extern "C" int spice_batch_launch_count(spice_batch* b, int64_t* out) {
	if (!b || !out) return bfail(SPICE_EINVAL, "NULL argument");
	*out = b->launches;
	return SPICE_OK;
}

extern "C" int spice_batch_get_stream(spice_batch* b, void** out) {
	if (!b || !out) return bfail(SPICE_EINVAL, "NULL argument");
	*out = (void*)b->stream;
	return SPICE_OK;
}
