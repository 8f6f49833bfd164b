// step.cu -- the kernels of snn::step (spice/src/snn.cpp:7-28), fused over min-delay windows.
//
// A spike emitted at step t through a connection of delay d is delivered at the end of step
// t + d - 1 and first seen by the update of step t + d (snn.cpp:21-25).  So with K <= min delay,
// the K updates of a window [t0, t0 + K) only read inputs caused by spikes older than t0, and a
// window is two launches:
//   k_window  -- every neuron runs its K updates with its state in registers.  Before the update
//                of step t it applies the inputs that the reference delivers at the end of step
//                t - 1 (ring slot (t - 1) mod D).  Spikes go to a bitmap (one ballot word per
//                warp: the ascending order of neuron_population::spikes) and to an unordered
//                list per step (warp-aggregated atomics) for delivery.
//   k_deliver -- work-queue delivery, one warp per (spike, connection): the warp streams the CSR
//                row (int32 targets) and adds into ring slot (t + d - 1) mod D.
// Deterministic mode: fixed_weight synapses add one constant per connection, so the reference's
// sequential order (connections in connect order, sources ascending) is reproduced exactly by
// counting events per (target, group of consecutive connections with equal weight) with integer
// atomics and replaying the adds one by one in group order with IEEE round-to-nearest
// (__fadd_rn; the library is built with -fmad=false).  Atomic mode adds float weights with
// atomics (fast, order-dependent rounding).
#include "internal.h"
#include "kernels.h"

namespace spice_gb300 {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ unsigned lanemask_lt() {
	unsigned m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

// Brunel LIF (samples/brunel.cpp:45-61) as the reference's -ffast-math build computes it: the
// leak V += (0 - V) * (dt * TmemInv) becomes V * fma(-dt, TmemInv, 1); V > Vthres in float.
__device__ __forceinline__ bool lif_update(float& V, int32_t& T, float om, float vthres, int32_t tref) {
	T = T - 1;
	if (T <= 0) {
		if (V > vthres) {
			V = 0.0f;
			T = tref;
			return true;
		}
		V = __fmul_rn(V, om);
	}
	return false;
}

// Conductance LIF (samples/vogels.cpp:10-46), strict float arithmetic in source order.
__device__ __forceinline__ bool lifc_update(float& V, float& Gex, float& Gin, int32_t& T, float dt) {
	const int32_t Tref = 50;
	const float Vrest = -0.06f, Vthres = -0.05f, TmemInv = 50.0f;
	const float Eex = 0.0f, Ein = -0.08f, Ibg = 0.02f, TexInv = 200.0f, TinInv = 100.0f;
	bool spiked = false;
	T           = T - 1;
	if (T <= 0) {
		if (V > Vthres) {
			V      = Vrest;
			T      = Tref;
			spiked = true;
		} else {
			float const a = __fsub_rn(Vrest, V);
			float const b = __fmul_rn(Gex, __fsub_rn(Eex, V));
			float const c = __fmul_rn(Gin, __fsub_rn(Ein, V));
			float const s = __fadd_rn(__fadd_rn(__fadd_rn(a, b), c), Ibg);
			V             = __fadd_rn(V, __fmul_rn(s, __fmul_rn(dt, TmemInv)));
		}
	}
	Gex = __fsub_rn(Gex, __fmul_rn(Gex, __fmul_rn(dt, TexInv)));
	Gin = __fsub_rn(Gin, __fmul_rn(Gin, __fmul_rn(dt, TinInv)));
	return spiked;
}

__device__ __forceinline__ float& field_ref(int f, float& V, float& Gex, float& Gin) {
	return f == 0 ? V : (f == 1 ? Gex : Gin);
}

// The inputs delivered at the end of step `slot` to neuron i, applied in the reference's order,
// then cleared.
__device__ __forceinline__ void apply_inputs(PopDev const& P, int mode, int64_t slot, int64_t i, float& V,
                                             float& Gex, float& Gin) {
	if (mode == 0) {
		uint32_t* w = P.cnt + (slot * P.size + i) * P.W;
		uint32_t x[kMaxGroups];
#pragma unroll
		for (int j = 0; j < kMaxGroups; j++)
			if (j < P.W) x[j] = w[j];
		for (int g = 0; g < P.ngroups; g++) {
			uint32_t const word = x[P.group_word[g]];
			uint32_t const n    = P.group_bits[g] == 32 ? word : ((word >> P.group_shift[g]) & 0xffffu);
			if (n) {
				float& f       = field_ref(P.group_field[g], V, Gex, Gin);
				float const wt = P.group_weight[g];
				float v        = f;
				for (uint32_t r = 0; r < n; r++) v = __fadd_rn(v, wt);
				f = v;
			}
		}
#pragma unroll
		for (int j = 0; j < kMaxGroups; j++)
			if (j < P.W && x[j]) w[j] = 0;
	} else {
		float* a = P.acc + (slot * P.size + i) * P.F;
		for (int f = 0; f < 3; f++) {
			int const s = P.field_slot[f];
			if (s < 0) continue;
			float const x = a[s];
			if (x != 0.0f) {
				float& dst = field_ref(f, V, Gex, Gin);
				dst        = __fadd_rn(dst, x);
				a[s]       = 0.0f;
			}
		}
	}
}

// Appends the warp's spikes of one step (mask over lanes) to the step's list.
__device__ __forceinline__ void append_warp(unsigned mask, bool spike, int32_t idx, int32_t* count,
                                            int32_t* list) {
	if (!mask) return;
	int const lane = threadIdx.x & 31;
	int base       = 0;
	if (lane == 0) base = atomicAdd(count, __popc(mask));
	base = __shfl_sync(0xffffffffu, base, 0);
	if (spike) list[base + __popc(mask & lanemask_lt())] = idx;
}

__device__ __forceinline__ void red_add_u32(uint32_t* p, uint32_t v) {
	asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_add_f32(float* p, float v) {
	asm volatile("red.relaxed.gpu.global.add.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}

// Replays the counted inputs of one slot word set (deterministic mode) in group order.
__device__ __forceinline__ void replay_groups(PopDev const& P, const uint32_t* x, float& V, float& Gex, float& Gin) {
	for (int g = 0; g < P.ngroups; g++) {
		uint32_t const word = x[P.group_word[g]];
		uint32_t const n    = P.group_bits[g] == 32 ? word : ((word >> P.group_shift[g]) & 0xffffu);
		if (n) {
			float& f       = field_ref(P.group_field[g], V, Gex, Gin);
			float const wt = P.group_weight[g];
			float v        = f;
			for (uint32_t r = 0; r < n; r++) v = __fadd_rn(v, wt);
			f = v;
		}
	}
}

// Same, when every group lives in one word (no array indexing: keeps the words in registers).
__device__ __forceinline__ void replay_groups1(PopDev const& P, uint32_t word, float& V, float& Gex, float& Gin) {
	for (int g = 0; g < P.ngroups; g++) {
		uint32_t const n = P.group_bits[g] == 32 ? word : ((word >> P.group_shift[g]) & 0xffffu);
		if (n) {
			float& f       = field_ref(P.group_field[g], V, Gex, Gin);
			float const wt = P.group_weight[g];
			float v        = f;
			for (uint32_t r = 0; r < n; r++) v = __fadd_rn(v, wt);
			f = v;
		}
	}
}

template <int MODE>
__device__ void window_neurons(WindowArgs const& a, PopDev const& P, int p, int b) {
	int const N      = (int)P.size;
	int const i      = b * kThreads + threadIdx.x;
	bool const valid = i < N;
	int const lane   = threadIdx.x & 31;
	int const word   = i >> 5;
	float V = 0, Gex = 0, Gin = 0;
	int32_t T = 0;
	if (valid) {
		V = P.V[i];
		T = P.T[i];
		if (P.model == LIF_COND) {
			Gex = P.Gex[i];
			Gin = P.Gin[i];
		}
	}
	float const vthres = P.p0;
	int32_t const tref = (int32_t)P.p1;
	float const tminv  = P.p2;
	int const D = (int)a.D, Hb = a.Hb;
	int slot  = a.slot0;   // (t0 - 1) mod D: inputs applied before the update of step t0
	int hslot = a.hslot0;  // t0 mod Hb
	int32_t* count = a.counts + p;
	int32_t* list  = P.list;
	bool const W1  = MODE == 0 && P.W == 1;
	for (int k0 = 0; k0 < a.K; k0 += 8) {
		// the inputs of the next 8 steps are complete already: issue their loads together
		uint32_t xs[8];
		if (W1) {
			int sl = slot;
#pragma unroll
			for (int u = 0; u < 8; u++) {
				xs[u] = (valid && k0 + u < a.K) ? P.cnt[(int64_t)sl * N + i] : 0u;
				sl    = sl + 1 == D ? 0 : sl + 1;
			}
		}
#pragma unroll
		for (int u = 0; u < 8; u++) {
			int const k = k0 + u;
			if (k >= a.K) break;
			float const dt = a.dts[k];
			bool spike     = false;
			if (valid) {
				if (MODE == 0) {
					if (W1) {
						if (xs[u]) {
							replay_groups1(P, xs[u], V, Gex, Gin);
							P.cnt[(int64_t)slot * N + i] = 0;
						}
					} else {
						uint32_t* w = P.cnt + ((int64_t)slot * N + i) * P.W;
						uint32_t x[kMaxGroups];
						bool any = false;
#pragma unroll
						for (int j = 0; j < kMaxGroups; j++)
							if (j < P.W) {
								x[j] = w[j];
								any |= x[j] != 0;
							}
						if (any) {
							replay_groups(P, x, V, Gex, Gin);
#pragma unroll
							for (int j = 0; j < kMaxGroups; j++)
								if (j < P.W) w[j] = 0;
						}
					}
				} else {
					float* acc = P.acc + ((int64_t)slot * N + i) * P.F;
					for (int f = 0; f < 3; f++) {
						int const sidx = P.field_slot[f];
						if (sidx < 0) continue;
						float const x = acc[sidx];
						if (x != 0.0f) {
							float& dst = field_ref(f, V, Gex, Gin);
							dst        = __fadd_rn(dst, x);
							acc[sidx]  = 0.0f;
						}
					}
				}
				if (P.model == LIF)
					spike = lif_update(V, T, __fmaf_rn(-dt, tminv, 1.0f), vthres, tref);
				else
					spike = lifc_update(V, Gex, Gin, T, dt);
			}
			unsigned const mask = __ballot_sync(0xffffffffu, spike);
			if (lane == 0 && word < P.nwords) P.bits[(int64_t)hslot * P.nwords + word] = mask;
			append_warp(mask, spike, i, count + k * a.npop, list + (int64_t)k * N);
			slot  = slot + 1 == D ? 0 : slot + 1;
			hslot = hslot + 1 == Hb ? 0 : hslot + 1;
		}
	}
	if (valid) {
		P.V[i] = V;
		P.T[i] = T;
		if (P.model == LIF_COND) {
			P.Gex[i] = Gex;
			P.Gin[i] = Gin;
		}
	}
}

// One step of a Poisson population (samples/brunel.cpp:27-30): thread c owns neurons
// [32c, 32c + 32), jumps to draw draw_offset + 32c of the step's stream and draws 32 numbers.
// The jump XORs the basis states T^i(s) selected by the 128 bits of x^(offset) mod P; the CTA
// first tabulates, for each of the 32 nibbles of the polynomial, the XOR of all 16 subsets of its
// 4 basis states, so a jump is 32 table lookups.
__device__ void window_poisson(WindowArgs const& a, PopDev const& P, int p, int b, u128* tab) {
	int const k      = b / a.blk_per_step[p];
	int const cb     = b % a.blk_per_step[p];
	int const hslot  = (a.hslot0 + k) % a.Hb;
	const u128* bas  = a.basis + (int64_t)k * kBasis;
	for (int e = threadIdx.x; e < 32 * 16; e += blockDim.x) {
		int const g = e >> 4, m = e & 15;
		uint64_t lo = 0, hi = 0;
#pragma unroll
		for (int q = 0; q < 4; q++)
			if ((m >> q) & 1) {
				lo ^= bas[4 * g + q].lo;
				hi ^= bas[4 * g + q].hi;
			}
		tab[e] = {lo, hi};
	}
	__syncthreads();
	int64_t const c = (int64_t)cb * kThreads + threadIdx.x;
	float const thr = __fmul_rn(P.p0, a.dts[k]);
	unsigned mask   = 0;
	if (c < P.nwords) {
		u128 const poly = P.chunk_poly[c];
		uint64_t s0 = 0, s1 = 0;
#pragma unroll
		for (int g = 0; g < 16; g++) {
			u128 const v = tab[g * 16 + ((poly.lo >> (4 * g)) & 15)];
			s0 ^= v.lo;
			s1 ^= v.hi;
		}
#pragma unroll
		for (int g = 0; g < 16; g++) {
			u128 const v = tab[(16 + g) * 16 + ((poly.hi >> (4 * g)) & 15)];
			s0 ^= v.lo;
			s1 ^= v.hi;
		}
		int const n = (int)(P.size - 32 * c < 32 ? P.size - 32 * c : 32);
		if (n == 32) {
#pragma unroll 8
			for (int r = 0; r < 32; r++) {
				uint64_t const u = xoro_next(s0, s1);
				mask |= (unsigned)(canonical_f32(u) < thr) << r;
			}
		} else {
			for (int r = 0; r < n; r++) {
				uint64_t const u = xoro_next(s0, s1);
				mask |= (unsigned)(canonical_f32(u) < thr) << r;
			}
		}
		P.bits[(int64_t)hslot * P.nwords + c] = mask;
	}
	// ascending append: warp exclusive scan of the per-thread spike counts
	int const lane = threadIdx.x & 31;
	int const mine = __popc(mask);
	int incl       = mine;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		int const v = __shfl_up_sync(0xffffffffu, incl, d);
		if (lane >= d) incl += v;
	}
	int const total = __shfl_sync(0xffffffffu, incl, 31);
	if (total == 0) return;
	int base = 0;
	if (lane == 31) base = atomicAdd(a.counts + k * a.npop + p, total);
	base = __shfl_sync(0xffffffffu, base, 31);
	int32_t* out = P.list + (int64_t)k * P.size + base + (incl - mine);
	unsigned m   = mask;
	while (m) {
		int const r = __ffs(m) - 1;
		m &= m - 1;
		*out++ = (int32_t)(32 * c + r);
	}
}

// One step of an external population (samples/external_input.cpp:17-30).
__device__ void window_external(WindowArgs const& a, PopDev const& P, int p, int k) {
	uint32_t* bits  = P.bits + (int64_t)((a.hslot0 + k) % a.Hb) * P.nwords;
	for (int j = threadIdx.x; j < P.nwords; j += blockDim.x) bits[j] = 0;
	__syncthreads();
	if (P.ext_steps <= 0) return;
	int64_t const pos = (a.ext_pos[p] + k) % P.ext_steps;
	int32_t const n   = P.ext_counts[pos];
	const int32_t* src = P.ext_idx + P.ext_off[pos];
	for (int j = threadIdx.x; j < n; j += blockDim.x) {
		int32_t const s = src[j];
		atomicOr(bits + (s >> 5), 1u << (s & 31));
		P.list[(int64_t)k * P.size + j] = s;
	}
	if (threadIdx.x == 0) a.counts[k * a.npop + p] = n;
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_window(const __grid_constant__ WindowArgs a) {
	__shared__ PopDev sp;
	__shared__ u128 tab[32 * 16];
	int const b = blockIdx.x;
	int p       = 0;
	while (p + 1 < a.npop && b >= a.blk_begin[p + 1]) p++;
	if (threadIdx.x == 0) sp = a.pops[p];
	__syncthreads();
	int const lb = b - a.blk_begin[p];
	switch (a.blk_kind[p]) {
		case 0: window_neurons<MODE>(a, sp, p, lb); break;
		case 1: window_poisson(a, sp, p, lb, tab); break;
		case 2: window_external(a, sp, p, lb); break;
	}
}

constexpr int kDeliverThreads = 256;

// Work queue: item = (window step k, connection c, j-th spike of c's source at step k); one warp
// per item streams the CSR row with 8 loads in flight per lane and adds with fire-and-forget
// reductions.  The (k, c) prefix of spike counts is built once per CTA (no per-step barriers).
template <int MODE>
__global__ void __launch_bounds__(kDeliverThreads) k_deliver(const __grid_constant__ DeliverArgs a) {
	extern __shared__ int64_t pre[];  // [K * nconn + 1]
	__shared__ unsigned long long ev_block;
	int const C = a.nconn, KC = a.K * C;
	for (int t = threadIdx.x; t < KC; t += blockDim.x) {
		int const k = t / C, c = t - k * C;
		pre[t + 1]  = a.counts[k * a.npop + a.conns[c].src];
	}
	if (threadIdx.x == 0) {
		pre[0]   = 0;
		ev_block = 0;
	}
	if (blockIdx.x == 0)
		for (int j = threadIdx.x; j < a.counts_next_len; j += blockDim.x) a.counts_next[j] = 0;
	__syncthreads();
	int const lane = threadIdx.x & 31;
	if (threadIdx.x < 32) {
		int64_t carry = 0;
		for (int base = 1; base <= KC; base += 32) {
			int64_t v = base + lane <= KC ? pre[base + lane] : 0;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				int64_t const o = __shfl_up_sync(0xffffffffu, v, d);
				if (lane >= d) v += o;
			}
			if (base + lane <= KC) pre[base + lane] = carry + v;
			carry += __shfl_sync(0xffffffffu, v, 31);
		}
	}
	__syncthreads();
	int64_t const total  = pre[KC];
	int64_t const gwarp  = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	int64_t const nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
	unsigned long long my_events = 0;
	for (int64_t item = gwarp; item < total; item += nwarps) {
		int lo = 0, hi = KC;  // largest kc with pre[kc] <= item
		while (hi - lo > 1) {
			int const mid = (lo + hi) >> 1;
			if (pre[mid] <= item) lo = mid;
			else hi = mid;
		}
		int const k = lo / C, c = lo - k * C;
		ConnDev const* Cp = a.conns + c;
		int64_t const ss  = __ldg(&Cp->src_size);
		const int32_t* lst = (const int32_t*)__ldg((const unsigned long long*)&Cp->src_list);
		const int64_t* off = (const int64_t*)__ldg((const unsigned long long*)&Cp->off);
		const int32_t* nb  = (const int32_t*)__ldg((const unsigned long long*)&Cp->nb);
		int const delay    = __ldg(&Cp->delay);
		int const s        = __ldg(lst + (int64_t)k * ss + (item - pre[lo]));
		int64_t const e0   = __ldg(off + s);
		int64_t const e1   = __ldg(off + s + 1);
		int64_t slot       = a.t0 + k + delay - 1;
		slot               = slot % a.D;
		int64_t const dsz  = __ldg(&Cp->dst_size);
		if (MODE == 0) {
			int const W        = __ldg(&Cp->W);
			uint32_t* base     = (uint32_t*)__ldg((const unsigned long long*)&Cp->dst_cnt) + slot * dsz * W + __ldg(&Cp->word);
			uint32_t const inc = __ldg(&Cp->inc);
			for (int64_t e = e0 + lane; e < e1; e += 256) {
				int32_t d[8];
#pragma unroll
				for (int u = 0; u < 8; u++) d[u] = (e + 32 * u < e1) ? __ldg(nb + e + 32 * u) : -1;
#pragma unroll
				for (int u = 0; u < 8; u++)
					if (d[u] >= 0) red_add_u32(base + (int64_t)d[u] * W, inc);
			}
		} else {
			int const F    = __ldg(&Cp->F);
			float* base    = (float*)__ldg((const unsigned long long*)&Cp->dst_acc) + slot * dsz * F + __ldg(&Cp->fslot);
			float const w  = __ldg(&Cp->weight);
			for (int64_t e = e0 + lane; e < e1; e += 256) {
				int32_t d[8];
#pragma unroll
				for (int u = 0; u < 8; u++) d[u] = (e + 32 * u < e1) ? __ldg(nb + e + 32 * u) : -1;
#pragma unroll
				for (int u = 0; u < 8; u++)
					if (d[u] >= 0) red_add_f32(base + (int64_t)d[u] * F, w);
			}
		}
		if (lane == 0) my_events += (unsigned long long)(e1 - e0);
	}
	if (lane == 0 && my_events) atomicAdd(&ev_block, my_events);
	__syncthreads();
	if (threadIdx.x == 0 && ev_block) atomicAdd(a.events, ev_block);
}

__global__ void k_apply_pending(PopDev P, int64_t slot, int mode) {
	int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= P.size) return;
	float V = P.V[i], Gex = 0, Gin = 0;
	if (P.model == LIF_COND) {
		Gex = P.Gex[i];
		Gin = P.Gin[i];
	}
	apply_inputs(P, mode, slot, i, V, Gex, Gin);
	P.V[i] = V;
	if (P.model == LIF_COND) {
		P.Gex[i] = Gex;
		P.Gin[i] = Gin;
	}
}

__global__ void k_basis(const u128* __restrict__ seeds, int64_t nsteps, u128* __restrict__ basis) {
	int64_t const t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (t >= nsteps) return;
	uint64_t s0 = seeds[t].lo, s1 = seeds[t].hi;
	u128* out   = basis + t * kBasis;
	for (int i = 0; i < kBasis; i++) {
		out[i] = {s0, s1};
		xoro_next(s0, s1);
	}
}

// Block-wide exclusive scan of one int per thread; returns the exclusive prefix.  `total` must
// point to shared memory: it receives the block's sum, visible to every thread on return.
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* total) {
	__shared__ int64_t warp_sums[32];
	int const lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	int64_t incl   = v;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		int64_t const o = __shfl_up_sync(0xffffffffu, incl, d);
		if (lane >= d) incl += o;
	}
	if (lane == 31) warp_sums[wid] = incl;
	__syncthreads();
	if (wid == 0) {
		int64_t s  = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
		int64_t si = s;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			int64_t const o = __shfl_up_sync(0xffffffffu, si, d);
			if (lane >= d) si += o;
		}
		warp_sums[lane] = si - s;
		if (lane == (int)(blockDim.x >> 5) - 1) *total = si;
	}
	__syncthreads();
	int64_t const r = warp_sums[wid] + incl - v;
	__syncthreads();
	return r;
}

// Ascending set bits of a bitmap into out[base ...]; one CTA.  Returns the count (thread 0).
__device__ int64_t extract_bits(const uint32_t* bits, int nwords, int32_t* out, int64_t base, int64_t cap) {
	__shared__ int64_t total;
	int64_t running = 0;
	for (int w0 = 0; w0 < nwords; w0 += blockDim.x) {
		int const w       = w0 + threadIdx.x;
		uint32_t const m  = w < nwords ? bits[w] : 0u;
		int64_t const ex  = block_exclusive_scan(__popc(m), &total);
		int64_t pos       = base + running + ex;
		uint32_t mm       = m;
		while (mm) {
			int const r = __ffs(mm) - 1;
			mm &= mm - 1;
			if (pos < cap) out[pos] = 32 * w + r;
			pos++;
		}
		running += total;
		__syncthreads();
	}
	return running;
}

__global__ void k_extract(const uint32_t* bits, int nwords, int32_t* out, int64_t* n_out) {
	int64_t const n = extract_bits(bits, nwords, out, 0, INT64_MAX);
	if (threadIdx.x == 0) *n_out = n;
}

__global__ void k_raster(const __grid_constant__ RasterArgs a) {
	__shared__ int64_t total;
	__shared__ unsigned long long off;
	int const k = blockIdx.x / a.npop, p = blockIdx.x % a.npop;
	PopDev const& P      = a.pops[p];
	const uint32_t* bits = P.bits + ((a.t0 + k) % a.Hb) * P.nwords;
	int64_t c            = 0;
	for (int w = threadIdx.x; w < P.nwords; w += blockDim.x) c += __popc(bits[w]);
	(void)block_exclusive_scan(c, &total);
	if (threadIdx.x == 0) {
		off = atomicAdd(a.cursor, (unsigned long long)total);
		a.tab[((a.row0 + k) * a.npop + p) * 2 + 0] = (int64_t)off;
		a.tab[((a.row0 + k) * a.npop + p) * 2 + 1] = total;
	}
	__syncthreads();
	(void)extract_bits(bits, P.nwords, a.out, (int64_t)off, a.capacity);
}

__global__ void k_count_targets(const int32_t* __restrict__ nb, int64_t n, uint32_t* __restrict__ indeg) {
	for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
		atomicAdd(indeg + nb[e], 1u);
}

__global__ void k_max_u32(const uint32_t* __restrict__ v, int64_t n, uint32_t* __restrict__ out) {
	uint32_t m = 0;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		m = max(m, v[i]);
	for (int d = 16; d; d >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, d));
	if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

constexpr int kScanItems = 1024;

__global__ void k_scan_local(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ out,
                             int64_t* __restrict__ block_sums) {
	int64_t const i = blockIdx.x * (int64_t)kScanItems + threadIdx.x;
	int64_t const v = i < n ? in[i] : 0;
	__shared__ int64_t total;
	int64_t const ex = block_exclusive_scan(v, &total);
	if (i < n) out[i + 1] = ex + v;  // local inclusive
	if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int64_t* sums, int64_t nb) {
	int64_t carry = 0;
	__shared__ int64_t total;
	for (int64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
		int64_t const b = b0 + threadIdx.x;
		int64_t const v = b < nb ? sums[b] : 0;
		int64_t const ex = block_exclusive_scan(v, &total);
		if (b < nb) sums[b] = carry + ex;
		carry += total;
		__syncthreads();
	}
}

__global__ void k_scan_add(int64_t* out, int64_t n, const int64_t* __restrict__ sums) {
	int64_t const i = blockIdx.x * (int64_t)kScanItems + threadIdx.x;
	if (i == 0) out[0] = 0;
	if (i < n) out[i + 1] += sums[blockIdx.x];
}

}  // namespace

cudaError_t scan_row_lengths(cudaStream_t stream, const int32_t* lens, int64_t n, int64_t* offsets) {
	if (n <= 0) return cudaMemsetAsync(offsets, 0, sizeof(int64_t), stream);
	int64_t const nb = (n + kScanItems - 1) / kScanItems;
	int64_t* sums    = nullptr;
	cudaError_t err  = cudaMallocAsync(&sums, sizeof(int64_t) * nb, stream);
	if (err != cudaSuccess) return err;
	k_scan_local<<<(unsigned)nb, kScanItems, 0, stream>>>(lens, n, offsets, sums);
	k_scan_sums<<<1, kScanItems, 0, stream>>>(sums, nb);
	k_scan_add<<<(unsigned)nb, kScanItems, 0, stream>>>(offsets, n, sums);
	err = cudaGetLastError();
	cudaFreeAsync(sums, stream);
	return err;
}

cudaError_t max_indegree(cudaStream_t stream, const int32_t* const* nbs, const int64_t* nsyn, int nconn,
                         int64_t dst_size, uint32_t* scratch, uint32_t* max_out) {
	cudaError_t err = cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * (dst_size > 0 ? dst_size : 1), stream);
	if (err != cudaSuccess) return err;
	err = cudaMemsetAsync(max_out, 0, sizeof(uint32_t), stream);
	if (err != cudaSuccess) return err;
	for (int c = 0; c < nconn; c++)
		if (nsyn[c] > 0) k_count_targets<<<1216, 256, 0, stream>>>(nbs[c], nsyn[c], scratch);
	if (dst_size > 0) k_max_u32<<<304, 256, 0, stream>>>(scratch, dst_size, max_out);
	return cudaGetLastError();
}

cudaError_t launch_basis(cudaStream_t stream, const u128* seeds, int64_t nsteps, u128* basis) {
	if (nsteps <= 0) return cudaSuccess;
	k_basis<<<(unsigned)((nsteps + 127) / 128), 128, 0, stream>>>(seeds, nsteps, basis);
	return cudaGetLastError();
}

cudaError_t launch_window(cudaStream_t stream, WindowArgs const& a, int nblocks) {
	if (nblocks <= 0) return cudaSuccess;
	if (a.mode == 0)
		k_window<0><<<nblocks, kThreads, 0, stream>>>(a);
	else
		k_window<1><<<nblocks, kThreads, 0, stream>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_deliver(cudaStream_t stream, DeliverArgs const& a, int nblocks) {
	if (nblocks <= 0) return cudaSuccess;
	size_t const smem = sizeof(int64_t) * ((size_t)a.K * a.nconn + 1);
	if (a.mode == 0)
		k_deliver<0><<<nblocks, kDeliverThreads, smem, stream>>>(a);
	else
		k_deliver<1><<<nblocks, kDeliverThreads, smem, stream>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_apply_pending(cudaStream_t stream, const PopDev*, int, const int* stateful, int nstateful,
                                 std::vector<PopDev> const& hpops, int64_t t, int64_t D, int mode) {
	int64_t const slot = ((t - 1) % D + D) % D;
	for (int j = 0; j < nstateful; j++) {
		PopDev const& P = hpops[stateful[j]];
		if (P.size <= 0) continue;
		k_apply_pending<<<(unsigned)((P.size + 255) / 256), 256, 0, stream>>>(P, slot, mode);
	}
	return cudaGetLastError();
}

cudaError_t launch_extract(cudaStream_t stream, const uint32_t* bits, int nwords, int32_t* out, int64_t* n_out) {
	k_extract<<<1, 1024, 0, stream>>>(bits, nwords, out, n_out);
	return cudaGetLastError();
}

cudaError_t launch_raster(cudaStream_t stream, RasterArgs const& a) {
	if (a.K <= 0 || a.npop <= 0) return cudaSuccess;
	k_raster<<<a.K * a.npop, 1024, 0, stream>>>(a);
	return cudaGetLastError();
}

}  // namespace spice_gb300
