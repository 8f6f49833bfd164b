// pull.cu -- deterministic delivery of per-synapse weights: the pull path over CSC adjacency.
//
// The reference delivers a step's spikes connection by connection in connect order, and within a
// connection source by source in ascending order, each synapse adding its weight to its target
// (synapse_population.h:118-133, snn.cpp:21-25).  For fixed_weight synapses the engine replays
// per-target event counts (step.cu); a synapse that carries its own weight (the reference's
// StatefulSynapse / PerSynapseInit concepts, concepts.h:60-104, synapse_population.h:34-41) needs
// the weights themselves, in that order.  A population with such inputs is "pulled": per window,
// every target gathers its own inputs from the columns of the CSC adjacency of its incoming
// connections -- connect order, then ascending source, which is exactly the reference's order of
// additions into that target -- and the neuron update adds them one IEEE addition at a time.
//
// Per window [t, t + K) (K <= min delay, so every input comes from spikes older than t):
//   k_pull_masks -- for each (source population, delay d) of a pulled connection, from the
//                   source's spike bitmap ring: orb (one bit per source: spiked at a step
//                   t + k - d, k < K) and wm (per such source, bit k set when it spiked at
//                   t + k - d).  The same launch counts the synaptic events of the window that
//                   just ended for the pulled connections (row lengths of their spikes).
//   k_pull       -- one warp per target neuron: scans the target's CSC column of each incoming
//                   connection (coalesced source indices), keeps the synapses whose source bit is
//                   set in orb (a few percent at biological rates) as an ordered active list
//                   (weight, step mask, field), then groups the list by bin (step k, field f) with
//                   a stable counting sort into the target's region of G, and writes the bin
//                   starts koff.  A region holds as many entries as the target has synapses, so
//                   grouping always fits unless one synapse reaches the target at several steps
//                   of the window and the bins overflow; then koff[i][0] = -1 and the neuron
//                   update walks the active list step by step instead.  Both orders are exact.
// The neuron update of the window (window_neurons, step.cu) then adds, before step t + k, the
// weights of bins (k, f) to field f in G order.
//
// CSC construction (build_csc): source rows are cut into nblk consecutive blocks; cnt[b][d] counts
// block b's entries with target d; an exclusive prefix over b per target gives each block's start
// within each column; then each block writes its rows in order (a barrier between rows), so the
// entries of every column are in ascending source order without a sort.  Duplicate (source,
// target) pairs of an adj_list row keep their CSR order.
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "internal.h"
#include "kernels.h"

namespace spice_gb300 {

namespace {

constexpr int kPullThreads = 256;
constexpr int kPullWarps   = kPullThreads / 32;
constexpr int kMaxBins     = kPullMaxWindow * 3;
constexpr int kPullUnroll  = 8;  // chunks of 32 column entries loaded together by a warp

__device__ __forceinline__ unsigned lanemask_lt_pull() {
	unsigned m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

// ---- CSC construction ----

__global__ void k_csc_count(const int64_t* __restrict__ off, const int32_t* __restrict__ nb, int64_t rows,
                            int64_t rows_per_blk, int64_t ndst, uint32_t* __restrict__ cnt) {
	int64_t const b  = blockIdx.y;
	int64_t const r0 = b * rows_per_blk, r1 = min(rows, r0 + rows_per_blk);
	if (r0 >= r1) return;
	int64_t const e0 = off[r0], e1 = off[r1];
	uint32_t* c      = cnt + b * ndst;
	for (int64_t e = e0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < e1; e += (int64_t)gridDim.x * blockDim.x)
		atomicAdd(c + nb[e], 1u);
}

// Per target d: cnt[b][d] becomes the exclusive prefix over blocks, indeg[d] the column length.
__global__ void k_csc_colscan(uint32_t* __restrict__ cnt, int64_t nblk, int64_t ndst, int32_t* __restrict__ indeg) {
	for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < ndst; d += (int64_t)gridDim.x * blockDim.x) {
		uint32_t run = 0;
		for (int64_t b = 0; b < nblk; b++) {
			uint32_t const c = cnt[b * ndst + d];
			cnt[b * ndst + d] = run;
			run += c;
		}
		indeg[d] = (int32_t)run;
	}
}

// Block b writes its rows in order; the entries of one row are written in parallel.
__global__ void k_csc_fill(const int64_t* __restrict__ off, const int32_t* __restrict__ nb, const float* __restrict__ w,
                           int64_t rows, int64_t rows_per_blk, int64_t ndst, uint32_t* __restrict__ cnt,
                           const int64_t* __restrict__ col_off, int32_t* __restrict__ col_src,
                           float* __restrict__ col_w, int64_t* __restrict__ col_pos) {
	int64_t const b  = blockIdx.x;
	int64_t const r0 = b * rows_per_blk, r1 = min(rows, r0 + rows_per_blk);
	uint32_t* c      = cnt + b * ndst;
	for (int64_t r = r0; r < r1; r++) {
		int64_t const e0 = off[r], e1 = off[r + 1];
		for (int64_t base = e0; base < e1; base += blockDim.x) {
			int64_t const e = base + threadIdx.x;
			bool last       = false;
			int32_t d       = 0;
			uint32_t rank   = 0;
			if (e < e1) {
				d = nb[e];
				while (e - (int64_t)rank - 1 >= e0 && nb[e - rank - 1] == d) rank++;  // earlier duplicates
				int64_t const pos = col_off[d] + c[d] + rank;
				col_src[pos]      = (int32_t)r;
				if (w) col_w[pos] = w[e];
				if (col_pos) col_pos[pos] = e;
				last = e + 1 == e1 || nb[e + 1] != d;
			}
			__syncthreads();
			if (last) c[d] += rank + 1;
			__syncthreads();
		}
	}
}

// base[i] = sum over the pulled connections of their column starts: the prefix of the total
// in-degree, i <= n.
__global__ void k_pull_base(const int64_t* const* __restrict__ col_offs, int nconn, int64_t n, int64_t* __restrict__ base) {
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
		int64_t s = 0;
		for (int c = 0; c < nconn; c++) s += col_offs[c][i];
		base[i] = s;
	}
}

// ---- per window ----

__device__ __forceinline__ int64_t ring_step(int64_t step, int Hb) { return ((step % Hb) + Hb) % Hb; }

// Blocks: first the mask sets (one thread per source bitmap word), then the event jobs.
__global__ void __launch_bounds__(kPullThreads) k_pull_masks(const __grid_constant__ PullArgs a) {
	int b = (int)blockIdx.x;
	for (int s = 0; s < a.nsets; s++) {
		PullSet const S = a.sets[s];
		int const nb    = (S.nwords + kPullThreads - 1) / kPullThreads;
		if (b < nb) {
			int const w      = b * kPullThreads + threadIdx.x;
			bool const valid = w < S.nwords;
			uint32_t x[kPullMaxWindow];
			uint32_t any = 0;
#pragma unroll
			for (int k = 0; k < kPullMaxWindow; k++) {
				int64_t const step = a.t + k - S.delay;
				x[k]               = (valid && k < a.K && step >= 0) ? S.bits[ring_step(step, a.Hb) * S.nwords + w] : 0u;
				any |= x[k];
			}
			if (a.ps_units > 0) {  // the word's spiking sources appended to the set's list (warp-aggregated)
				int const lane = threadIdx.x & 31;
				int const mine = __popc(any);
				int incl       = mine;
#pragma unroll
				for (int d = 1; d < 32; d <<= 1) {
					int const o = __shfl_up_sync(0xffffffffu, incl, d);
					if (lane >= d) incl += o;
				}
				int base = 0;
				if (lane == 31 && incl) base = atomicAdd(S.nact, incl);
				base = __shfl_sync(0xffffffffu, base, 31) + incl - mine;
				for (uint32_t r = any; r; r &= r - 1, base++)  // (a list holds each source at most once)
					if (base < S.size) S.act[base] = 32 * w + __ffs(r) - 1;
			}
			if (!valid) return;
			S.orb[w] = any;
			uint32_t rest = any;
			while (rest) {
				int const bit = __ffs(rest) - 1;
				rest &= rest - 1;
				uint32_t m = 0;
#pragma unroll
				for (int k = 0; k < kPullMaxWindow; k++) m |= ((x[k] >> bit) & 1u) << k;
				S.wm[32 * (int64_t)w + bit] = m;
			}
			return;
		}
		b -= nb;
	}
	// events of the pulled connections' spikes of the window that just ended
	__shared__ unsigned long long ev_sm;
	if (threadIdx.x == 0) ev_sm = 0;
	__syncthreads();
	for (int j = 0; j < a.nev; j++) {
		PullEvJob const J = a.ev[j];
		int const nb      = (J.nwords + kPullThreads - 1) / kPullThreads;
		if (b < nb) {
			int const w = b * kPullThreads + threadIdx.x;
			unsigned long long ev = 0;
			if (w < J.nwords)
				for (int k = 0; k < a.k_emit; k++) {
					uint32_t x = J.bits[ring_step(a.t_emit0 + k, a.Hb) * J.nwords + w];
					while (x) {
						int64_t const s = 32 * (int64_t)w + __ffs(x) - 1;
						x &= x - 1;
						ev += (unsigned long long)(J.off[s + 1] - J.off[s]);
					}
				}
			for (int o = 16; o > 0; o >>= 1) ev += __shfl_down_sync(0xffffffffu, ev, o);
			if ((threadIdx.x & 31) == 0 && ev) atomicAdd(&ev_sm, ev);
			__syncthreads();
			if (threadIdx.x == 0 && ev_sm) atomicAdd(a.events, ev_sm);
			return;
		}
		b -= nb;
	}
}

// One chunk of up to 32 active entries (one per lane; m = step mask, f = field bin) against the
// bins (k, f) = k * F + f.  PLACE = false: adds each bin's entry count to cnt.  PLACE = true:
// writes each entry's weight to G at run[bin] + its rank among the chunk's earlier lanes of that
// bin, then advances run.  Lanes of one bin are handled in lane order within each step k, and steps
// in ascending order, so the entries of every bin keep the active list's order.  With at most one
// step bit per lane (the common case) one pass covers every bin.
template <bool PLACE>
__device__ __forceinline__ void bin_pass(uint32_t m, int f, int F, int nbins, int lane, int* cnt, int* run, float* G,
                                         uint32_t wbits) {
	unsigned const lt = lanemask_lt_pull();
	if (__all_sync(0xffffffffu, __popc(m) <= 1)) {
		int const bn        = m ? (__ffs(m) - 1) * F + f : nbins;  // lanes without a bit: the spare bin
		unsigned const same = __match_any_sync(0xffffffffu, bn);
		if (m) {
			if (PLACE) G[run[bn] + __popc(same & lt)] = __uint_as_float(wbits);
			__syncwarp(same);
			if ((same & lt) == 0) (PLACE ? run : cnt)[bn] += __popc(same);
		}
		__syncwarp();
		return;
	}
	uint32_t all = __reduce_or_sync(0xffffffffu, m);
	while (all) {
		int const k = __ffs(all) - 1;
		all &= all - 1;
		bool const has      = (m >> k) & 1u;
		int const bn        = has ? k * F + f : nbins;
		unsigned const same = __match_any_sync(0xffffffffu, bn);
		if (has) {
			if (PLACE) G[run[bn] + __popc(same & lt)] = __uint_as_float(wbits);
			__syncwarp(same);
			if ((same & lt) == 0) (PLACE ? run : cnt)[bn] += __popc(same);
		}
		__syncwarp();
	}
}

// The pull of one target neuron i of pulled population pi by one warp.  (A variant with the
// window's bitmaps in shared memory and CTAs resident on every SM, looping over the targets, ran
// 2.3x slower: at 16 warps per SM the scan has too few loads in flight.)
__device__ __forceinline__ void pull_target(PullArgs const& a, int pi, int64_t i, int lane, int* bin_cnt_w,
                                            int* bin_run_w) {
	PopDev const& P = a.pops[pi];
	int const F = P.pull_F, nbins = a.K * F;
	int64_t const base = P.pull_base[i];
	int64_t const cap  = P.pull_base[i + 1] - base;
	uint64_t* A        = P.pull_A + base;
	// 1. the active synapses, in connect order and ascending source order
	int64_t nA = 0;
	uint32_t const kmask = a.K >= 32 ? 0xffffffffu : (1u << a.K) - 1u;
	for (int c = P.in_begin; c < P.in_end; c++) {
		ConnDev const& C = a.conns[c];
		int f            = 0;
		while (f + 1 < F && P.pull_field[f] != C.field) f++;
		int64_t const e0    = C.csc_off[i];
		int const len       = (int)(C.csc_off[i + 1] - e0);
		const int32_t* col  = C.csc_src + e0;
		const uint32_t* orb = C.pull_orb;
		const uint32_t* wm  = C.pull_wm;
		const float* cw     = C.csc_w ? C.csc_w + e0 : nullptr;
		uint32_t const fw   = __float_as_uint(C.weight);
		uint32_t const fb   = (uint32_t)f << 16;
		// kPullUnroll coalesced chunks of 32 sources in flight per warp (streamed past L1, which keeps
		// the window's source bits), then their tests and appends in entry order
		for (int eb = 0; eb < len; eb += 32 * kPullUnroll) {
			int32_t src[kPullUnroll];
#pragma unroll
			for (int u = 0; u < kPullUnroll; u++) {
				int const e = eb + 32 * u + lane;
				src[u]      = e < len ? __ldcs(col + e) : -1;
			}
			uint32_t hit[kPullUnroll];
#pragma unroll
			for (int u = 0; u < kPullUnroll; u++) hit[u] = src[u] >= 0 ? (__ldg(orb + (src[u] >> 5)) >> (src[u] & 31)) & 1u : 0u;
#pragma unroll
			for (int u = 0; u < kPullUnroll; u++) {
				if (!__any_sync(0xffffffffu, hit[u] != 0)) continue;  // warp-uniform: no source spiked
				bool act   = hit[u] != 0;
				uint32_t m = 0, wb = 0;
				if (act) {
					m   = __ldg(wm + src[u]) & kmask;
					wb  = cw ? __float_as_uint(__ldg(cw + eb + 32 * u + lane)) : fw;
					act = m != 0;
				}
				unsigned const bal = __ballot_sync(0xffffffffu, act);
				if (act) A[nA + __popc(bal & lanemask_lt_pull())] = (uint64_t)wb | ((uint64_t)(m | fb) << 32);
				nA += __popc(bal);
			}
		}
	}
	__syncwarp();
	int32_t* ko = P.pull_koff + i * (int64_t)(P.pull_nbins + 1);
	// 2. entries per bin (an entry with several step bits lands in several bins)
	for (int bn = lane; bn <= nbins; bn += 32) bin_cnt_w[bn] = 0;
	__syncwarp();
	for (int64_t c0 = 0; c0 < nA; c0 += 32) {
		int64_t const e = c0 + lane;
		uint32_t const mf = e < nA ? (uint32_t)(A[e] >> 32) : 0u;
		bin_pass<false>(mf & 0xffffu, (int)(mf >> 16), F, nbins, lane, bin_cnt_w, bin_run_w, nullptr, 0u);
	}
	__syncwarp();
	// exclusive prefix over the bins
	int64_t total = 0;
	for (int b0 = 0; b0 < nbins; b0 += 32) {
		int const bn = b0 + lane;
		int const v  = bn < nbins ? bin_cnt_w[bn] : 0;
		int incl     = v;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			int const o = __shfl_up_sync(0xffffffffu, incl, d);
			if (lane >= d) incl += o;
		}
		if (bn < nbins) bin_run_w[bn] = (int)total + incl - v;
		total += __shfl_sync(0xffffffffu, incl, 31);
	}
	__syncwarp();
	if (total > cap) {  // several spikes of one source in the window overflow the region: walk A
		if (lane == 0) {
			ko[0] = -1;
			ko[1] = (int32_t)nA;
		}
		return;
	}
	for (int bn = lane; bn < nbins; bn += 32) ko[bn] = bin_run_w[bn];
	if (lane == 0) ko[nbins] = (int32_t)total;
	__syncwarp();
	// 3. stable placement: chunks in order, and within a chunk lanes in order per bin
	float* G = P.pull_G + base;
	for (int64_t c0 = 0; c0 < nA; c0 += 32) {
		int64_t const e = c0 + lane;
		uint64_t const v = e < nA ? A[e] : 0ull;
		uint32_t const mf = (uint32_t)(v >> 32);
		bin_pass<true>(mf & 0xffffu, (int)(mf >> 16), F, nbins, lane, bin_cnt_w, bin_run_w, G, (uint32_t)v);
	}
}

// One warp per target neuron of the pulled populations.
__global__ void __launch_bounds__(kPullThreads) k_pull(const __grid_constant__ PullArgs a) {
	__shared__ int bin_cnt[kPullWarps][kMaxBins + 1];
	__shared__ int bin_run[kPullWarps][kMaxBins + 1];
	int const lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	int const blk  = (int)blockIdx.x;
	int q          = 0;
	while (q + 1 < a.npull && blk >= a.pull_blk[q + 1]) q++;
	int64_t const i = (int64_t)(blk - a.pull_blk[q]) * kPullWarps + wid;
	if (i >= a.pops[a.pull_pops[q]].size) return;
	pull_target(a, a.pull_pops[q], i, lane, bin_cnt[wid], bin_run[wid]);
}

// ---- push-and-sort gather ----
// The scan above reads every synapse of a pulled population once per window.  At biological rates
// a few percent of them carry a spike, so the default gather pushes only those: every synapse of a
// source that spiked in the window adds, per step bit, one entry to its target's slots (64 per
// target, compact, so the scattered writes stay close together) -- the weight and a 64-bit key
// (bin k * F + f, the connection's rank among the target's inputs, the source, the synapse's
// offset in its row) -- and each target then orders its entries by key (each entry's rank is the
// number of smaller keys) into its region.  Key order within a bin is the scan's order (connect order, ascending
// source, CSR order for duplicates), so both gathers give the same bins bit for bit.  A target with
// more entries than its slots or its region takes the scan (pull_target) instead.

// Warps stride over the rows of the window's spiking sources, connection after connection (the
// sources listed by k_pull_masks; a connection's rows start at the warp after the previous
// connection's last, so that the rows spread over all warps).  Latency-bound (the slot
// reservations are atomics with a result): at most 48 registers, so that five CTAs share an SM.
__global__ void __launch_bounds__(kPullThreads, 5) k_ps_scatter(const __grid_constant__ PullArgs a) {
	int const lane  = threadIdx.x & 31;
	int64_t const gw = (int64_t)blockIdx.x * kPullWarps + (threadIdx.x >> 5);
	int64_t const nw = (int64_t)gridDim.x * kPullWarps;
	uint32_t const kmask = a.K >= 32 ? 0xffffffffu : (1u << a.K) - 1u;
	int64_t pre = 0;  // rows of the connections before
	for (int qc = 0; qc < a.ps_nconn; qc++) {
		int const cb     = a.ps_conn[qc];
		ConnDev const& C = a.conns[cb];
		PopDev const& P  = a.pops[a.ps_pop[qc]];
		int64_t const nrows = *C.pull_nact;
		int64_t u = (gw - pre) % nw;
		if (u < 0) u += nw;
		pre += nrows;
		if (u >= nrows) continue;
		int const F = P.pull_F;
		int f       = 0;
		while (f + 1 < F && P.pull_field[f] != C.field) f++;
		uint64_t const crank = (uint64_t)(cb - P.in_begin) << 50;
		for (; u < nrows; u += nw) {
			int64_t const src = C.pull_act[u];
			uint32_t const m  = C.pull_wm[src] & kmask;
			if (!m) continue;
			int64_t const e0 = C.off[src], e1 = C.off[src + 1];
			uint64_t const sk = crank | ((uint64_t)src << 19);
			int const nk = __popc(m);  // entries per synapse: one per step bit, reserved together
			constexpr int U = 4;       // synapses per lane with their reservations in flight together
			for (int64_t eb = e0 + lane; eb < e1; eb += 32 * U) {
				int32_t j[U];
				float w[U];
				int pos[U];
#pragma unroll
				for (int v = 0; v < U; v++)
					if (eb + 32 * v < e1) {
						j[v] = C.nb[eb + 32 * v];
						w[v] = C.wts ? C.wts[eb + 32 * v] : C.weight;
					}
#pragma unroll
				for (int v = 0; v < U; v++)
					if (eb + 32 * v < e1) pos[v] = atomicAdd(P.pull_fill + j[v], nk);
#pragma unroll
				for (int v = 0; v < U; v++) {
					int64_t const e = eb + 32 * v;
					if (e >= e1) break;
					int q = pos[v];
					for (uint32_t mm = m; mm; mm &= mm - 1, q++) {
						if (q >= kPushSortSlots) break;
						uint64_t const key = ((uint64_t)((__ffs(mm) - 1) * F + f) << 58) | sk | (uint64_t)(e - e0);
						P.ps_slot[(int64_t)j[v] * kPushSortSlots + q] =
						    make_uint4((uint32_t)key, (uint32_t)(key >> 32), __float_as_uint(w[v]), 0u);
					}
				}
			}
		}
	}
}

// One warp per target: its pushed entries ordered by key into the bins (weights in G, starts in
// koff).  A counting sort by bin (the key's top bits) gives the bin starts; each entry's place in
// its bin is the number of the bin's entries with a smaller key (keys are distinct), found among
// the bin's few entries parked, grouped by bin, in shared memory.
__global__ void __launch_bounds__(kPullThreads) k_ps_sort(const __grid_constant__ PullArgs a) {
	__shared__ int bin_cnt[kPullWarps][kMaxBins + 1];
	__shared__ int bin_run[kPullWarps][kMaxBins + 1];
	__shared__ uint64_t key_s[kPullWarps][kPushSortSlots];
	int const lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	int const blk  = (int)blockIdx.x;
	if (blk == 0)  // the scatter has read the lists: empty them for the next window
		for (int s2 = threadIdx.x; s2 < a.nsets; s2 += blockDim.x) *a.sets[s2].nact = 0;
	int q          = 0;
	while (q + 1 < a.npull && blk >= a.pull_blk[q + 1]) q++;
	int const pi    = a.pull_pops[q];
	PopDev const& P = a.pops[pi];
	int64_t const i = (int64_t)(blk - a.pull_blk[q]) * kPullWarps + wid;
	if (i >= P.size) return;
	int const nbins    = a.K * P.pull_F;
	int64_t const base = P.pull_base[i];
	int const cap      = (int)(P.pull_base[i + 1] - base);
	int const n        = P.pull_fill[i];
	__syncwarp();
	if (lane == 0) P.pull_fill[i] = 0;  // for the next window
	if (n > cap || n > kPushSortSlots) {  // more entries than the region or the slots: the scan
		pull_target(a, pi, i, lane, bin_cnt[wid], bin_run[wid]);
		return;
	}
	int64_t const sl  = i * kPushSortSlots;
	bool const v0     = lane < n, v1 = lane + 32 < n;
	uint4 const e0    = v0 ? P.ps_slot[sl + lane] : make_uint4(0u, 0u, 0u, 0u);
	uint4 const e1    = v1 ? P.ps_slot[sl + lane + 32] : make_uint4(0u, 0u, 0u, 0u);
	uint64_t const k0 = ((uint64_t)e0.y << 32) | e0.x, k1 = ((uint64_t)e1.y << 32) | e1.x;
	float const w0 = __uint_as_float(e0.z), w1 = __uint_as_float(e1.z);
	int const b0 = (int)(k0 >> 58), b1 = (int)(k1 >> 58);
	int* const cnt = bin_cnt[wid];  // entries per bin
	int* const st  = bin_run[wid];  // bin starts; st[nbins] = n
	for (int b = lane; b <= nbins; b += 32) cnt[b] = 0;
	__syncwarp();
	int p0 = 0, p1 = 0;  // arrival places within the bin (any order: only to park the keys)
	if (v0) p0 = atomicAdd(&cnt[b0], 1);
	if (v1) p1 = atomicAdd(&cnt[b1], 1);
	__syncwarp();
	// exclusive scan over the bins (nbins <= 48): lane l holds bins 2l and 2l + 1
	int const c0 = 2 * lane < nbins ? cnt[2 * lane] : 0;
	int const c1 = 2 * lane + 1 < nbins ? cnt[2 * lane + 1] : 0;
	int incl     = c0 + c1;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		int const o = __shfl_up_sync(0xffffffffu, incl, d);
		if (lane >= d) incl += o;
	}
	int const excl = incl - c0 - c1;
	if (2 * lane <= nbins) st[2 * lane] = excl;
	if (2 * lane + 1 <= nbins) st[2 * lane + 1] = excl + c0;
	__syncwarp();
	uint64_t* const ks = key_s[wid];
	if (v0) ks[st[b0] + p0] = k0;
	if (v1) ks[st[b1] + p1] = k1;
	__syncwarp();
	float* G = P.pull_G + base;
	if (v0) {
		int const s = st[b0], e = s + cnt[b0];
		int r = s;
		for (int j = s; j < e; j++) r += ks[j] < k0;
		G[r] = w0;
	}
	if (v1) {
		int const s = st[b1], e = s + cnt[b1];
		int r = s;
		for (int j = s; j < e; j++) r += ks[j] < k1;
		G[r] = w1;
	}
	// bin starts: koff[b] = the entries in bins below b
	int32_t* ko = P.pull_koff + i * (int64_t)(nbins + 1);
	for (int b = lane; b <= nbins; b += 32) ko[b] = st[b];
}

// The inputs of the first pulled step (bins k = 0), applied now and removed from the bins: state
// reads between steps see the reference's state after step(), which has delivered them already.
__global__ void k_pull_apply_first(PopDev P) {
	int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= P.size) return;
	int32_t* ko        = P.pull_koff + i * (int64_t)(P.pull_nbins + 1);
	int64_t const base = P.pull_base[i];
	float v[3]         = {P.V[i], P.Gex ? P.Gex[i] : 0.0f, P.Gin ? P.Gin[i] : 0.0f};
	if (ko[0] >= 0) {
		for (int f = 0; f < P.pull_F; f++) {
			float x = v[P.pull_field[f]];
			for (int32_t e = ko[f]; e < ko[f + 1]; e++) x = __fadd_rn(x, P.pull_G[base + e]);
			v[P.pull_field[f]] = x;
		}
		for (int f = 0; f < P.pull_F; f++) ko[f] = ko[P.pull_F];  // bins (0, f) are now empty
	} else {
		int32_t const nA = ko[1];
		for (int32_t e = 0; e < nA; e++) {
			uint64_t const a = P.pull_A[base + e];
			uint32_t const mf = (uint32_t)(a >> 32);
			if (mf & 1u) {
				int const fi = P.pull_field[mf >> 16];
				v[fi]        = __fadd_rn(v[fi], __uint_as_float((uint32_t)a));
				P.pull_A[base + e] = a & ~(1ull << 32);
			}
		}
	}
	P.V[i] = v[0];
	if (P.Gex) P.Gex[i] = v[1];
	if (P.Gin) P.Gin[i] = v[2];
}

// A fixed_weight / weighted connection into a USER_DELIVER target, at the end of a step: thread per
// target, ascending source order along its CSC column.
__global__ void k_direct_add(const __grid_constant__ ConnDev C, int hslot, char* __restrict__ dst, int nbytes,
                             int foff, unsigned long long* events) {
	int64_t const j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	unsigned long long ev = 0;
	if (j < C.dst_size) {
		float* const x   = reinterpret_cast<float*>(dst + j * nbytes + foff);
		float v          = *x;
		const uint32_t* bits = C.src_bits + (int64_t)hslot * C.src_nwords;
		for (int64_t e = C.csc_off[j]; e < C.csc_off[j + 1]; e++) {
			int32_t const s = C.csc_src[e];
			if ((bits[s >> 5] >> (s & 31)) & 1u) {
				v = __fadd_rn(v, C.csc_w ? C.csc_w[e] : C.weight);
				ev++;
			}
		}
		*x = v;
	}
	for (int o = 16; o > 0; o >>= 1) ev += __shfl_down_sync(0xffffffffu, ev, o);
	if ((threadIdx.x & 31) == 0 && ev) atomicAdd(events, ev);
}

}  // namespace

cudaError_t launch_direct_add(cudaStream_t stream, ConnDev const& c, int hslot, void* dst_state, int neuron_bytes,
                              int field_offset, unsigned long long* events) {
	if (c.dst_size <= 0) return cudaSuccess;
	k_direct_add<<<(unsigned)((c.dst_size + 255) / 256), 256, 0, stream>>>(c, hslot, static_cast<char*>(dst_state),
	                                                                        neuron_bytes, field_offset, events);
	return cudaGetLastError();
}

cudaError_t build_csc(cudaStream_t stream, const int64_t* off, const int32_t* nb, const float* wts, int64_t rows,
                      int64_t ndst, int64_t synapses, int64_t* col_off, int32_t* col_src, float* col_w,
                      int64_t* col_pos) {
	cudaError_t e = cudaMemsetAsync(col_off, 0, sizeof(int64_t) * (ndst + 1), stream);
	if (e != cudaSuccess || synapses == 0 || rows == 0 || ndst == 0) return e;
	// blocks of rows: at most 1024, and the count array at most 2^25 entries
	int64_t nblk = std::max<int64_t>(1, std::min<int64_t>(1024, (int64_t(1) << 25) / std::max<int64_t>(ndst, 1)));
	nblk         = std::min(nblk, rows);
	int64_t const rows_per_blk = (rows + nblk - 1) / nblk;
	nblk                       = (rows + rows_per_blk - 1) / rows_per_blk;
	uint32_t* cnt  = nullptr;
	int32_t* indeg = nullptr;
	e = cudaMalloc(&cnt, sizeof(uint32_t) * nblk * ndst);
	if (e == cudaSuccess) e = cudaMalloc(&indeg, sizeof(int32_t) * ndst);
	if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * nblk * ndst, stream);
	if (e == cudaSuccess) {
		dim3 const g((unsigned)std::max<int64_t>(1, std::min<int64_t>(256, synapses / nblk / 1024 + 1)), (unsigned)nblk);
		k_csc_count<<<g, 256, 0, stream>>>(off, nb, rows, rows_per_blk, ndst, cnt);
		k_csc_colscan<<<(unsigned)std::min<int64_t>((ndst + 255) / 256, 4096), 256, 0, stream>>>(cnt, nblk, ndst, indeg);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = scan_row_lengths(stream, indeg, ndst, col_off);
	if (e == cudaSuccess) {
		k_csc_fill<<<(unsigned)nblk, 256, 0, stream>>>(off, nb, wts, rows, rows_per_blk, ndst, cnt, col_off, col_src, col_w,
		                                               col_pos);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
	cudaFree(cnt);
	cudaFree(indeg);
	return e;
}

cudaError_t pull_region_bases(cudaStream_t stream, const int64_t* const* col_offs, int nconn, int64_t n, int64_t* base) {
	k_pull_base<<<(unsigned)std::min<int64_t>((n + 256) / 256, 4096), 256, 0, stream>>>(col_offs, nconn, n, base);
	return cudaGetLastError();
}

cudaError_t launch_pull(cudaStream_t stream, PullArgs const& a, std::vector<PullSet> const& sets,
                        std::vector<PullEvJob> const& ev) {
	int64_t nb = 0;
	for (auto const& s : sets) nb += (s.nwords + kPullThreads - 1) / kPullThreads;
	if (a.k_emit > 0)
		for (auto const& j : ev) nb += (j.nwords + kPullThreads - 1) / kPullThreads;
	if (nb > 0) k_pull_masks<<<(unsigned)nb, kPullThreads, 0, stream>>>(a);
	if (a.pull_blocks <= 0) return cudaGetLastError();
	if (a.ps_units > 0) {  // push-and-sort
		k_ps_scatter<<<(unsigned)a.ps_grid, kPullThreads, 0, stream>>>(a);
		k_ps_sort<<<(unsigned)a.pull_blocks, kPullThreads, 0, stream>>>(a);
	} else {
		k_pull<<<(unsigned)a.pull_blocks, kPullThreads, 0, stream>>>(a);
	}
	return cudaGetLastError();
}

int pull_blocks_for(int64_t size) { return (int)((size + kPullWarps - 1) / kPullWarps); }

cudaError_t launch_pull_apply_first(cudaStream_t stream, PopDev const& P) {
	if (P.size <= 0) return cudaSuccess;
	k_pull_apply_first<<<(unsigned)((P.size + 255) / 256), 256, 0, stream>>>(P);
	return cudaGetLastError();
}

}  // namespace spice_gb300
