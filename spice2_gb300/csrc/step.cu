// step.cu -- the kernels of snn::step (spice/src/snn.cpp:7-28), fused over min-delay windows.
//
// A spike emitted at step t through a connection of delay d is delivered at the end of step
// t + d - 1 and first seen by the update of step t + d (snn.cpp:21-25).  So with K <= min delay,
// the K updates of a window [t0, t0 + K) only read inputs caused by spikes older than t0, and a
// window is two launches on one stream, each the programmatic dependent of the previous one:
//   k_window  -- every neuron runs its K updates with its state in registers (window_lif_* and
//                window_neurons).  Before the update of step t it applies the inputs that the
//                reference delivers at the end of step t - 1 (ring slot (t - 1) mod D).  Spikes go
//                to a bitmap (one ballot word per warp: the ascending order of
//                neuron_population::spikes) and to an unordered list per step for delivery.  The
//                same grid runs the source populations (Poisson, external trains) and, when
//                recording, the previous window's raster.
//   delivery  -- one CTA per (input slot, target tile): the spikes of every connection into the
//                tile's population that reach the slot add into a shared-memory tile of
//                counters, which is then stored to the ring slot.  Twenty work mappings
//                (k_deliver*, SPICE_TUNE_DELIVER_ALGO) with identical results.
// Deterministic mode: fixed_weight synapses add one constant per connection, so the reference's
// sequential order (connections in connect order, sources ascending) is reproduced exactly by
// counting events per (target, group of consecutive connections with equal weight) with integer
// atomics and replaying the adds one by one in group order with IEEE round-to-nearest
// (__fadd_rn; the library is built with -fmad=false).  Atomic mode adds float weights with
// atomics (fast, order-dependent rounding).
// Also here: the plastic synapses' catch-up and delivery (k_plastic_*), the batched-network
// kernels (k_batch_*), tile bounds, scans and the raster.
#include "spice_gb300.h"
#include "internal.h"
#include "kernels.h"
#include "mulround.h"

namespace spice_gb300 {

namespace {

constexpr int kThreads = kNeuronThreads;

// Programmatic dependent launch (sm_90+): griddep_wait() returns once the preceding kernel of the
// stream has completed and its writes are visible (at once when there is no programmatic edge);
// griddep_launch() lets the following kernel's CTAs be scheduled while this one still runs.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

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

// Conductance LIF (samples/vogels.cpp:10-46) as the reference's -ffast-math -march=haswell build
// computes it: Vrest + Ibg folded into -0.04f, Eex = 0 dropped, the products contracted into fused
// multiply-adds, and the conductance decay G -= G * (dt * Inv) turned into G * fma(-dt, Inv, 1):
//   V = fma(dt * TmemInv, (-0.04f - V) + fma(-Gex, V, Gin * (Ein - V)), V)
// with the conductances of before their decay.
__device__ __forceinline__ bool lifc_update(float& V, float& Gex, float& Gin, int32_t& T, float dt) {
	const int32_t Tref = 50;
	const float Vrest = -0.06f, Vthres = -0.05f, TmemInv = 50.0f;
	const float Ein = -0.08f, VrestIbg = -0.04f, TexInv = 200.0f, TinInv = 100.0f;
	bool spiked = false;
	T           = T - 1;
	if (T <= 0) {
		if (V > Vthres) {
			V      = Vrest;
			T      = Tref;
			spiked = true;
		} else {
			float const a = __fmul_rn(Gin, __fsub_rn(Ein, V));
			float const b = __fmaf_rn(-Gex, V, a);
			float const c = __fadd_rn(__fsub_rn(VrestIbg, V), b);
			V             = __fmaf_rn(__fmul_rn(dt, TmemInv), c, V);
		}
	}
	Gex = __fmul_rn(Gex, __fmaf_rn(-dt, TexInv, 1.0f));
	Gin = __fmul_rn(Gin, __fmaf_rn(-dt, TinInv, 1.0f));
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

__device__ __forceinline__ void red_add_u32(uint32_t* p, uint32_t v) {
	asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_add_f32(float* p, float v) {
	asm volatile("red.relaxed.gpu.global.add.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}

// The per-window values the population bodies read, for a batch (from its device clock).  The
// bodies are templates over the argument type: plain nets pass their WindowArgs / DeliverArgs
// (kernel parameters, read from the constant bank), batches these register structs.  tables: the
// jump tables of step k of net j are tables + (j * tab_net_stride + k).
struct WinCtx {
	int K, slot0, hslot0, Hb, npop, list_k0;
	int64_t D;
	const float* dts;
	const u128* tables;
	int64_t tab_net_stride;
	int32_t* counts;
};


struct DelCtx {
	int64_t t0, D, slot_lo;
	int K, npop, list_k0, parts;
	const ConnDev* conns;
	const int32_t* counts;
	unsigned long long* events;  // the target population's net's event counter
};


// v += w, n times, one IEEE add at a time (the reference's n sequential deliver() calls), with the
// loop overhead paid once per four adds.
__device__ __forceinline__ float add_n(float v, float w, uint32_t n) {
	for (; n >= 4; n -= 4) v = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(v, w), w), w), w);
	if (n >= 2) {
		v = __fadd_rn(__fadd_rn(v, w), w);
		n -= 2;
	}
	if (n) v = __fadd_rn(v, w);
	return v;
}

// Replays the counted inputs of one slot (deterministic mode) in group order: group g adds its
// weight n_g times, one IEEE add at a time, as the reference's sequential deliver() calls do.
// All loops run over the compile-time bound kMaxGroups so every index is static (registers).
__device__ __forceinline__ void replay_words(PopDev const& P, const uint32_t (&x)[kMaxGroups], float& V, float& Gex,
                                             float& Gin) {
#pragma unroll
	for (int g = 0; g < kMaxGroups; g++) {
		if (g >= P.ngroups) break;
		uint32_t word = 0;
#pragma unroll
		for (int j = 0; j < kMaxGroups; j++)
			if (j == P.group_word[g]) word = x[j];
		uint32_t const n = P.group_bits[g] == 32 ? word : ((word >> P.group_shift[g]) & 0xffffu);
		if (n) {
			float const wt = P.group_weight[g];
			int const f    = P.group_field[g];
			float v        = add_n(f == 0 ? V : (f == 1 ? Gex : Gin), wt, n);
			if (f == 0) V = v;
			else if (f == 1) Gex = v;
			else Gin = v;
		}
	}
}

// Per-neuron window of a LIF population.  The inputs of every step of the window are complete
// already, so the input words of up to 16 consecutive slots are loaded together first; the step
// loop itself is kept rolled and small (instruction-cache friendly).  FAST: every input group adds to
// V through a 16-bit counter of word 0 (Brunel).
template <int MODE, bool FAST, bool HIST, class A>
__device__ __forceinline__ void window_neurons(A const& a, const PopDev* __restrict__ Pg, int p, int b) {
	int const N       = (int)Pg->size;
	int const i       = b * kThreads + threadIdx.x;
	bool const valid  = i < N;
	int const lane    = threadIdx.x & 31;
	int const word    = i >> 5;
	int const nwords  = Pg->nwords;
	bool const cond   = Pg->model == LIF_COND;
	float* const Vp   = Pg->V;
	int32_t* const Tp = Pg->T;
	uint32_t* const cnt = Pg->cnt;
	float* const acc  = Pg->acc;
	uint32_t* const bits = Pg->bits;
	int32_t* const list  = Pg->list;
	int const W = Pg->W, F = Pg->F;
	bool const zero     = Pg->zero_inputs != 0;
	float const vthres  = Pg->p0;
	int32_t const tref  = (int32_t)Pg->p1;
	float const tminv   = Pg->p2;
	float const w0 = Pg->group_weight[0], w1 = Pg->group_weight[1];
	float V = 0, Gex = 0, Gin = 0;
	int32_t T = 0;
	uint64_t* const hp = HIST ? Pg->hist : nullptr;
	uint64_t h         = 0;
	if (valid) {
		V = Vp[i];
		T = Tp[i];
		if (cond) {
			Gex = Pg->Gex[i];
			Gin = Pg->Gin[i];
		}
		if (HIST) h = hp[i];
	}
	int const D = (int)a.D, Hb = a.Hb;
	int slot  = a.slot0;   // (t0 - 1) mod D: inputs applied before the update of step t0
	int hslot = a.hslot0;  // t0 mod Hb
	int32_t* const count = a.counts + p;
	// pulled population (pull.cu): the inputs of step k are the weights of bins (k, f), in order
	bool const pulled  = Pg->pull != 0;
	int const pF       = Pg->pull_F;
	const int32_t* ko  = nullptr;
	int64_t pbase      = 0;
	int32_t ko0        = 0;
	if (pulled && valid) {
		ko    = Pg->pull_koff + (int64_t)i * (Pg->pull_nbins + 1);
		pbase = Pg->pull_base[i];
		ko0   = ko[0];
	}
	bool const word_in = MODE == 0 && W == 1 && !pulled;
	for (int k0 = 0; k0 < a.K; k0 += 16) {
		int const nk = min(16, a.K - k0);
		uint32_t xs[16];
		if (word_in) {
			int sl = slot;
#pragma unroll
			for (int u = 0; u < 16; u++) {
				xs[u] = (valid && u < nk) ? cnt[(int64_t)sl * N + i] : 0u;
				sl    = sl + 1 == D ? 0 : sl + 1;
			}
		}
#pragma unroll 1
		for (int u = 0; u < nk; u++) {
			int const k    = k0 + u;
			float const dt = a.dts[k];
			bool spike     = false;
			if (valid) {
				if (pulled) {
					if (ko0 >= 0) {
						for (int f = 0; f < pF; f++) {
							int const fi = Pg->pull_field[f];
							float v      = fi == 0 ? V : (fi == 1 ? Gex : Gin);
							int32_t const e1 = ko[k * pF + f + 1];
							for (int32_t e = ko[k * pF + f]; e < e1; e++) v = __fadd_rn(v, Pg->pull_G[pbase + e]);
							if (fi == 0) V = v;
							else if (fi == 1) Gex = v;
							else Gin = v;
						}
					} else {  // not grouped: the active synapses with step bit k, in order
						int32_t const nA = ko[1];
						for (int32_t e = 0; e < nA; e++) {
							uint64_t const av = Pg->pull_A[pbase + e];
							uint32_t const mf = (uint32_t)(av >> 32);
							if ((mf >> k) & 1u) {
								int const fi  = Pg->pull_field[mf >> 16];
								float const w = __uint_as_float((uint32_t)av);
								if (fi == 0) V = __fadd_rn(V, w);
								else if (fi == 1) Gex = __fadd_rn(Gex, w);
								else Gin = __fadd_rn(Gin, w);
							}
						}
					}
				} else if (word_in) {
					uint32_t const x = xs[u];
					if (x) {
						if (FAST) {
							uint32_t n0 = x & 0xffffu, n1 = x >> 16;
							for (; n0; n0--) V = __fadd_rn(V, w0);
							for (; n1; n1--) V = __fadd_rn(V, w1);
						} else {
							uint32_t xw[kMaxGroups] = {x};
							replay_words(*Pg, xw, V, Gex, Gin);
						}
						if (zero) cnt[(int64_t)slot * N + i] = 0;
					}
				} else if (MODE == 0) {
					uint32_t* w = cnt + ((int64_t)slot * N + i) * W;
					uint32_t xw[kMaxGroups];
					bool any = false;
#pragma unroll
					for (int j = 0; j < kMaxGroups; j++) {
						xw[j] = j < W ? w[j] : 0u;
						any |= xw[j] != 0;
					}
					if (any) {
						replay_words(*Pg, xw, V, Gex, Gin);
						if (zero) {
#pragma unroll
							for (int j = 0; j < kMaxGroups; j++)
								if (j < W) w[j] = 0;
						}
					}
				} else {
					float* ac = acc + ((int64_t)slot * N + i) * F;
#pragma unroll
					for (int f = 0; f < 3; f++) {
						int const sidx = Pg->field_slot[f];
						if (sidx < 0) continue;
						float const x = ac[sidx];
						if (x != 0.0f) {
							if (f == 0) V = __fadd_rn(V, x);
							else if (f == 1) Gex = __fadd_rn(Gex, x);
							else Gin = __fadd_rn(Gin, x);
							if (zero) ac[sidx] = 0.0f;
						}
					}
				}
				if (!cond)
					spike = lif_update(V, T, __fmaf_rn(-dt, tminv, 1.0f), vthres, tref);
				else
					spike = lifc_update(V, Gex, Gin, T, dt);
			}
			if (HIST) h = (h << 1) | (spike ? 1ull : 0ull);  // neuron_population.h:126-132
			unsigned const mask = __ballot_sync(0xffffffffu, spike);
			if (lane == 0 && word < nwords) bits[(int64_t)hslot * nwords + word] = mask;
			if (mask) {  // one list reservation per warp with spikes
				int base = 0;
				if (lane == 0) base = atomicAdd(count + k * a.npop, __popc(mask));
				base = __shfl_sync(0xffffffffu, base, 0);
				if (spike) list[(int64_t)(a.list_k0 + k) * N + base + __popc(mask & lanemask_lt())] = i;
			}
			slot  = slot + 1 == D ? 0 : slot + 1;
			hslot = hslot + 1 == Hb ? 0 : hslot + 1;
		}
	}
	if (valid) {
		Vp[i] = V;
		Tp[i] = T;
		if (cond) {
			Pg->Gex[i] = Gex;
			Pg->Gin[i] = Gin;
		}
		if (HIST) hp[i] = h;
	}
}

// v += w, n times, one IEEE add at a time, with a trip count common to the warp (its largest n):
// lanes past their own n keep v (predicated adds), so the loop has no divergent branches.  Every
// lane of the warp must call it.
__device__ __forceinline__ float add_n_warp(float v, float w, uint32_t n) {
	uint32_t const m = __reduce_max_sync(0xffffffffu, n);
	uint32_t j       = 0;
	for (; j + 2 <= m; j += 2) {
		v = j < n ? __fadd_rn(v, w) : v;
		v = j + 1 < n ? __fadd_rn(v, w) : v;
	}
	if (j < m) v = j < n ? __fadd_rn(v, w) : v;
	return v;
}

// Device span of a profiled launch (DeliverArgs::span, WindowArgs::span; null otherwise, both words
// zeroed before): the earliest CTA start (complemented: the max of ~t is the min of t) and the latest
// CTA end on the GPU's global nanosecond timer, so that the launch's own duration can be told from
// the fixed cost of the CUDA-event pair around it.  span_close is reached by every thread of the CTA.
__device__ __forceinline__ unsigned long long global_ns() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}
__device__ __forceinline__ void span_open(unsigned long long* sp) {
	if (sp && threadIdx.x == 0) atomicMax(sp, ~global_ns());
}
__device__ __forceinline__ void span_close(unsigned long long* sp) {
	if (sp) {  // uniform
		__syncthreads();
		if (threadIdx.x == 0) atomicMax(sp + 1, global_ns());
	}
}

// The Brunel LIF window (deterministic mode, every input group adds to V through a 16-bit counter
// of word 0): the input words of 16 consecutive slots are loaded up front, then the steps run.
// Same arithmetic, in the same order, as window_neurons<0, true, false>; dt comes from shared
// memory.  Variants (SPICE_TUNE_NEURON_VARIANT), identical results:
//   ROLLED = false: the words stay in registers and the 16 step bodies are unrolled (nothing is
//     indexed dynamically);
//   ROLLED = true: the words are parked in shared memory (one column per thread) and the step loop
//     stays rolled, a body small enough for the instruction cache;
//   UNIFORM: the count replay runs warp-uniform trip counts (add_n_warp) instead of per-lane loops.
template <bool ROLLED, bool UNIFORM, class A>
__device__ __forceinline__ void window_lif_fast(A const& a, const PopDev* __restrict__ Pg, int p, int b,
                                                const float* dts_sm, uint32_t (*xs_sm)[kThreads]) {
	int const N      = (int)Pg->size;
	int const i      = b * kThreads + threadIdx.x;
	bool const valid = i < N;
	int const lane   = threadIdx.x & 31;
	int const word   = i >> 5;
	int const nwords = Pg->nwords;
	uint32_t* const cnt  = Pg->cnt;
	bool const zero      = Pg->zero_inputs != 0;
	float const vthres   = Pg->p0;
	int32_t const tref   = (int32_t)Pg->p1;
	float const tminv    = Pg->p2;
	float const w0 = Pg->group_weight[0], w1 = Pg->group_weight[1];
	float V   = 0;
	int32_t T = 0;
	if (valid) {
		V = Pg->V[i];
		T = Pg->T[i];
	}
	int const D = (int)a.D, Hb = a.Hb, npop = a.npop;
	int slot  = a.slot0;
	int hslot = a.hslot0;
	uint32_t* const bits = Pg->bits;
	int32_t* const list  = Pg->list;
	int32_t* const count = a.counts + p;
	bool const wl = lane == 0 && word < nwords;
	auto step = [&](int k, uint32_t xx) {
		bool spike = false;
		if (UNIFORM) {
			uint32_t const n0 = valid ? xx & 0xffffu : 0u, n1 = valid ? xx >> 16 : 0u;
			V = add_n_warp(V, w0, n0);
			V = add_n_warp(V, w1, n1);
			if (valid) {
				if (zero && xx) cnt[(int64_t)slot * N + i] = 0;
				spike = lif_update(V, T, __fmaf_rn(-dts_sm[k], tminv, 1.0f), vthres, tref);
			}
		} else if (valid) {
			if (xx) {
				V = add_n(V, w0, xx & 0xffffu);
				V = add_n(V, w1, xx >> 16);
				if (zero) cnt[(int64_t)slot * N + i] = 0;
			}
			spike = lif_update(V, T, __fmaf_rn(-dts_sm[k], tminv, 1.0f), vthres, tref);
		}
		unsigned const mask = __ballot_sync(0xffffffffu, spike);
		if (wl) bits[(int64_t)hslot * nwords + word] = mask;
		if (mask) {
			int base = 0;
			if (lane == 0) base = atomicAdd(count + k * npop, __popc(mask));
			base = __shfl_sync(0xffffffffu, base, 0);
			if (spike) list[(int64_t)(a.list_k0 + k) * N + base + __popc(mask & lanemask_lt())] = i;
		}
		slot  = slot + 1 == D ? 0 : slot + 1;
		hslot = hslot + 1 == Hb ? 0 : hslot + 1;
	};
	for (int k0 = 0; k0 < a.K; k0 += 16) {
		int const nk = min(16, a.K - k0);
		int sl       = slot;
		if (ROLLED) {  // asynchronous copies into the thread's own shared-memory column
#pragma unroll
			for (int u = 0; u < 16; u++) {
				if (valid && u < nk) {
					unsigned const dst = (unsigned)__cvta_generic_to_shared(&xs_sm[u][threadIdx.x]);
					asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(cnt + (int64_t)sl * N + i)
					             : "memory");
				} else {
					xs_sm[u][threadIdx.x] = 0u;
				}
				sl = sl + 1 == D ? 0 : sl + 1;
			}
			asm volatile("cp.async.wait_all;" ::: "memory");
#pragma unroll 1
			for (int u = 0; u < nk; u++) step(k0 + u, xs_sm[u][threadIdx.x]);
		} else {
			uint32_t x[16];
#pragma unroll
			for (int u = 0; u < 16; u++) {
				x[u] = (valid && u < nk) ? cnt[(int64_t)sl * N + i] : 0u;
				sl   = sl + 1 == D ? 0 : sl + 1;
			}
#pragma unroll
			for (int u = 0; u < 16; u++)
				if (u < nk) step(k0 + u, x[u]);
		}
	}
	if (valid) {
		Pg->V[i] = V;
		Pg->T[i] = T;
	}
}

// v += w, n times, one IEEE add at a time, without branches: the adds of the 4-, 2- and 1-blocks of
// n's low bits are computed and kept by selects (all adds are the same operation, so their grouping
// does not change the result); counts of 8 or more, rare, loop first.
__device__ __forceinline__ float add_n_sel(float v, float w, uint32_t n) {
	for (; n >= 8; n -= 8)
		v = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(v, w), w), w), w), w), w), w), w);
	float const v4 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(v, w), w), w), w);
	v              = (n & 4u) ? v4 : v;
	float const v2 = __fadd_rn(__fadd_rn(v, w), w);
	v              = (n & 2u) ? v2 : v;
	float const v1 = __fadd_rn(v, w);
	return (n & 1u) ? v1 : v;
}

// As add_n_sel with the 4-, 2- and 1-blocks as predicated adds (one compare per block, the adds on
// the floating-point pipe) instead of computed-and-selected ones.
__device__ __forceinline__ float add_n_pred(float v, float w, uint32_t n) {
	for (; n >= 8; n -= 8)
		v = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(v, w), w), w), w), w), w), w), w);
	if (n & 4u) v = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(v, w), w), w), w);
	if (n & 2u) v = __fadd_rn(__fadd_rn(v, w), w);
	if (n & 1u) v = __fadd_rn(v, w);
	return v;
}

// The Brunel LIF window with the spike output deferred to the end of the window (variant 4): the
// step loop is rolled over input words staged in shared memory, replays counts without branches and
// only parks each step's warp ballot in shared memory; after the last step the warp writes its
// bitmap words (one lane per step) and reserves list entries for the steps that had spikes.  Same
// arithmetic and the same outputs as window_lif_fast (list order within a step is arbitrary in
// both: reservations are atomic).
template <bool PRED, bool LEAN, class A>
__device__ __forceinline__ void window_lif_deferred(A const& a, const PopDev* __restrict__ Pg, int p, int b,
                                                    const float* dts_sm, uint32_t (*xs_sm)[kThreads],
                                                    uint32_t (*masks_sm)[16]) {
	int const N      = (int)Pg->size;
	int const i      = b * kThreads + threadIdx.x;
	bool const valid = i < N;
	int const lane   = threadIdx.x & 31;
	int const warp   = threadIdx.x >> 5;
	int const word   = i >> 5;
	uint32_t* const cnt  = Pg->cnt;
	bool const zero      = Pg->zero_inputs != 0;
	float const vthres   = Pg->p0;
	int32_t const tref   = (int32_t)Pg->p1;
	float const tminv    = Pg->p2;
	float const w0 = Pg->group_weight[0], w1 = Pg->group_weight[1];
	float V   = 0;
	int32_t T = 0;
	if (valid) {  // written two launches back: loaded before waiting for the previous launch
		V = Pg->V[i];
		T = Pg->T[i];
	}
	griddep_wait();  // the input ring, counts and lists are the previous launches' output
	int const D = (int)a.D, Hb = a.Hb;
	for (int k0 = 0; k0 < a.K; k0 += 16) {
		int const nk    = min(16, a.K - k0);
		int const slot0 = (int)((a.slot0 + k0) % D);
		int sl          = slot0;
#pragma unroll
		for (int u = 0; u < 16; u++) {  // asynchronous copies into the thread's own shared-memory column
			if (valid && u < nk) {
				unsigned const dst = (unsigned)__cvta_generic_to_shared(&xs_sm[u][threadIdx.x]);
				asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(cnt + (int64_t)sl * N + i) : "memory");
			} else {
				xs_sm[u][threadIdx.x] = 0u;
			}
			sl = sl + 1 == D ? 0 : sl + 1;
		}
		asm volatile("cp.async.wait_all;" ::: "memory");
		uint32_t sbits = 0;  // this lane's spikes of the 16 steps
#pragma unroll 1
		for (int u = 0; u < nk; u++) {
			uint32_t const x = xs_sm[u][threadIdx.x];
			if (LEAN) {
				// both counts below 8 (the common case): the adds of the counts' 4-, 2- and 1-bits,
				// tested on the packed word; otherwise the general replay
				if ((x & 0xfff8fff8u) == 0) {
					float v4 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(V, w0), w0), w0), w0);
					V        = (x & 4u) ? v4 : V;
					float v2 = __fadd_rn(__fadd_rn(V, w0), w0);
					V        = (x & 2u) ? v2 : V;
					float v1 = __fadd_rn(V, w0);
					V        = (x & 1u) ? v1 : V;
					v4       = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(V, w1), w1), w1), w1);
					V        = (x & 0x40000u) ? v4 : V;
					v2       = __fadd_rn(__fadd_rn(V, w1), w1);
					V        = (x & 0x20000u) ? v2 : V;
					v1       = __fadd_rn(V, w1);
					V        = (x & 0x10000u) ? v1 : V;
				} else {
					V = add_n_sel(V, w0, x & 0xffffu);
					V = add_n_sel(V, w1, x >> 16);
				}
			} else {
				V = PRED ? add_n_pred(V, w0, x & 0xffffu) : add_n_sel(V, w0, x & 0xffffu);
				V = PRED ? add_n_pred(V, w1, x >> 16) : add_n_sel(V, w1, x >> 16);
			}
			if (zero && x) cnt[(int64_t)((slot0 + u) % D) * N + i] = 0;
			float const om   = LEAN ? dts_sm[k0 + u] : __fmaf_rn(-dts_sm[k0 + u], tminv, 1.0f);
			bool const spike = lif_update(V, T, om, vthres, tref) && valid;
			sbits |= (uint32_t)spike << u;
			unsigned const mask = __ballot_sync(0xffffffffu, spike);
			if (lane == 0) masks_sm[warp][u] = mask;
		}
		__syncwarp();
		if (lane < nk && word < Pg->nwords)
			Pg->bits[(int64_t)((a.hslot0 + k0 + lane) % Hb) * Pg->nwords + word] = masks_sm[warp][lane];
		unsigned const any = __ballot_sync(0xffffffffu, sbits != 0);
		if (any) {  // list reservations, one per step with spikes
			for (int u = 0; u < nk; u++) {
				unsigned const mask = masks_sm[warp][u];
				if (!mask) continue;
				int base = 0;
				if (lane == 0) base = atomicAdd(a.counts + (k0 + u) * a.npop + p, __popc(mask));
				base = __shfl_sync(0xffffffffu, base, 0);
				if ((sbits >> u) & 1u) Pg->list[(int64_t)(a.list_k0 + k0 + u) * N + base + __popc(mask & lanemask_lt())] = i;
			}
		}
		__syncwarp();
	}
	if (valid) {
		Pg->V[i] = V;
		Pg->T[i] = T;
	}
}

// The Brunel LIF window with fewer instructions per step (variant 7), same arithmetic and outputs
// as variant 6: the count replay takes its 4-, 2- and 1-blocks as predicated adds and falls back
// to the general replay by a warp-uniform test (a count of 8 or more anywhere in the warp); each
// step's warp ballot stays in the register of lane u; list entries are reserved only for the
// steps in which the warp spiked; the input words are staged by walking a pointer.
template <class A>
__device__ __forceinline__ void window_lif_lean(A const& a, const PopDev* __restrict__ Pg, int p, int b,
                                                const float* dts_sm, uint32_t (*xs_sm)[kThreads]) {
	int const N      = (int)Pg->size;
	int const i      = b * kThreads + threadIdx.x;
	bool const valid = i < N;
	int const lane   = threadIdx.x & 31;
	int const word   = i >> 5;
	uint32_t* const cnt = Pg->cnt;
	bool const zero     = Pg->zero_inputs != 0;
	float const vthres  = Pg->p0;
	int32_t const tref  = (int32_t)Pg->p1;
	float const w0 = Pg->group_weight[0], w1 = Pg->group_weight[1];
	float V   = 0;
	int32_t T = 0;
	if (valid) {  // written two launches back: loaded before waiting for the previous launch
		V = Pg->V[i];
		T = Pg->T[i];
	}
	griddep_wait();  // the input ring, counts and lists are the previous launches' output
	int const D = (int)a.D, Hb = a.Hb;
	for (int k0 = 0; k0 < a.K; k0 += 16) {
		int const nk    = min(16, a.K - k0);
		int const slot0 = (int)((a.slot0 + k0) % D);
		const uint32_t* src = cnt + (int64_t)slot0 * N + i;
		int const wrap      = D - slot0;  // step u >= wrap reads ring slot u - wrap
#pragma unroll
		for (int u = 0; u < 16; u++) {  // asynchronous copies into the thread's own shared-memory column
			if (u == wrap) src -= (int64_t)D * N;
			if (valid && u < nk) {
				unsigned const dst = (unsigned)__cvta_generic_to_shared(&xs_sm[u][threadIdx.x]);
				asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
			} else {
				xs_sm[u][threadIdx.x] = 0u;
			}
			src += N;
		}
		asm volatile("cp.async.wait_all;" ::: "memory");
		uint32_t sbits = 0;   // this lane's spikes of the 16 steps
		uint32_t mymask = 0;  // lane u: the warp's ballot of step u
#pragma unroll 1
		for (int u = 0; u < nk; u++) {
			uint32_t const x = xs_sm[u][threadIdx.x];
			if (__any_sync(0xffffffffu, (x & 0xfff8fff8u) != 0)) {  // a count of 8 or more in the warp
				V = add_n_sel(V, w0, x & 0xffffu);
				V = add_n_sel(V, w1, x >> 16);
			} else {
				if (x & 4u) V = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(V, w0), w0), w0), w0);
				if (x & 2u) V = __fadd_rn(__fadd_rn(V, w0), w0);
				if (x & 1u) V = __fadd_rn(V, w0);
				if (x & 0x40000u) V = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(V, w1), w1), w1), w1);
				if (x & 0x20000u) V = __fadd_rn(__fadd_rn(V, w1), w1);
				if (x & 0x10000u) V = __fadd_rn(V, w1);
			}
			if (zero && x) cnt[(int64_t)((slot0 + u) % D) * N + i] = 0;
			bool const spike = lif_update(V, T, dts_sm[k0 + u], vthres, tref) && valid;
			sbits |= (uint32_t)spike << u;
			unsigned const mask = __ballot_sync(0xffffffffu, spike);
			mymask              = lane == u ? mask : mymask;
		}
		if (lane < nk && word < Pg->nwords) Pg->bits[(int64_t)((a.hslot0 + k0 + lane) % Hb) * Pg->nwords + word] = mymask;
		// list reservations, one per step in which the warp spiked
		for (unsigned st = __reduce_or_sync(0xffffffffu, sbits); st; st &= st - 1) {
			int const u         = __ffs(st) - 1;
			unsigned const mask = __shfl_sync(0xffffffffu, mymask, u);
			int base = 0;
			if (lane == 0) base = atomicAdd(a.counts + (k0 + u) * a.npop + p, __popc(mask));
			base = __shfl_sync(0xffffffffu, base, 0);
			if ((sbits >> u) & 1u) Pg->list[(int64_t)(a.list_k0 + k0 + u) * N + base + __popc(mask & lanemask_lt())] = i;
		}
	}
	if (valid) {
		Pg->V[i] = V;
		Pg->T[i] = T;
	}
}

// Variant 9: variant 7 with the common step written as predicated PTX -- the count replay's
// 4-, 2- and 1-blocks of each group as adds under a predicate set from the packed input word, and
// the LIF step (lif_update) as compares feeding predicated multiply, reset and refractory load --
// so that no step contains a branch beyond the warp-uniform test for large counts.  Same IEEE
// operations in the same order as variant 7.
template <bool ZERO, class A>
__device__ __forceinline__ void window_lif_pred(A const& a, const PopDev* __restrict__ Pg, int p, int b,
                                                const float* dts_sm, uint32_t (*xs_sm)[kThreads]) {
	int const N      = (int)Pg->size;
	int const i      = b * kThreads + threadIdx.x;
	bool const valid = i < N;
	int const lane   = threadIdx.x & 31;
	int const word   = i >> 5;
	uint32_t* const cnt = Pg->cnt;
	float const vthres  = Pg->p0;
	int32_t const tref  = (int32_t)Pg->p1;
	float const w0 = Pg->group_weight[0], w1 = Pg->group_weight[1];
	float V   = 0;
	int32_t T = 0;
	if (valid) {  // written two launches back: loaded before waiting for the previous launch
		V = Pg->V[i];
		T = Pg->T[i];
	}
	uint32_t const vmask = valid ? 0xffffffffu : 0u;
	griddep_wait();  // the input ring, counts and lists are the previous launches' output
	int const D = (int)a.D, Hb = a.Hb;
	for (int k0 = 0; k0 < a.K; k0 += 16) {
		int const nk    = min(16, a.K - k0);
		int const slot0 = (int)((a.slot0 + k0) % D);
		const uint32_t* src = cnt + (int64_t)slot0 * N + i;
		int const wrap      = D - slot0;  // step u >= wrap reads ring slot u - wrap
#pragma unroll
		for (int u = 0; u < 16; u++) {  // asynchronous copies into the thread's own shared-memory column
			if (u == wrap) src -= (int64_t)D * N;
			if (valid && u < nk) {
				unsigned const dst = (unsigned)__cvta_generic_to_shared(&xs_sm[u][threadIdx.x]);
				asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
			} else {
				xs_sm[u][threadIdx.x] = 0u;
			}
			src += N;
		}
		asm volatile("cp.async.wait_all;" ::: "memory");
		uint32_t sbits = 0;   // this lane's spikes of the 16 steps
		uint32_t mymask = 0;  // lane u: the warp's ballot of step u
		uint32_t bit    = 1;  // 1 << u
#pragma unroll 1
		for (int u = 0; u < nk; u++, bit <<= 1) {
			uint32_t const x = xs_sm[u][threadIdx.x];
			if (__any_sync(0xffffffffu, (x & 0xfff8fff8u) != 0)) {  // a count of 8 or more in the warp
				V = add_n_sel(V, w0, x & 0xffffu);
				V = add_n_sel(V, w1, x >> 16);
			} else {
				asm("{\n\t.reg .pred q;\n\t.reg .b32 t;\n\t"
				    "and.b32 t, %1, 4;\n\tsetp.ne.u32 q, t, 0;\n\t"
				    "@q add.rn.f32 %0, %0, %2;\n\t@q add.rn.f32 %0, %0, %2;\n\t"
				    "@q add.rn.f32 %0, %0, %2;\n\t@q add.rn.f32 %0, %0, %2;\n\t"
				    "and.b32 t, %1, 2;\n\tsetp.ne.u32 q, t, 0;\n\t"
				    "@q add.rn.f32 %0, %0, %2;\n\t@q add.rn.f32 %0, %0, %2;\n\t"
				    "and.b32 t, %1, 1;\n\tsetp.ne.u32 q, t, 0;\n\t"
				    "@q add.rn.f32 %0, %0, %2;\n\t"
				    "and.b32 t, %1, 262144;\n\tsetp.ne.u32 q, t, 0;\n\t"
				    "@q add.rn.f32 %0, %0, %3;\n\t@q add.rn.f32 %0, %0, %3;\n\t"
				    "@q add.rn.f32 %0, %0, %3;\n\t@q add.rn.f32 %0, %0, %3;\n\t"
				    "and.b32 t, %1, 131072;\n\tsetp.ne.u32 q, t, 0;\n\t"
				    "@q add.rn.f32 %0, %0, %3;\n\t@q add.rn.f32 %0, %0, %3;\n\t"
				    "and.b32 t, %1, 65536;\n\tsetp.ne.u32 q, t, 0;\n\t"
				    "@q add.rn.f32 %0, %0, %3;\n\t}"
				    : "+f"(V)
				    : "r"(x), "f"(w0), "f"(w1));
			}
			if (ZERO && x) cnt[(int64_t)((slot0 + u) % D) * N + i] = 0;
			// lif_update: T -= 1; when T <= 0, either spike (V > Vthres: V = 0, T = Tref) or leak
			uint32_t spike;  // bit if the neuron spiked (and exists), else 0
			asm("{\n\t.reg .pred pr, ps, pl;\n\t"
			    "sub.s32 %1, %1, 1;\n\t"
			    "setp.le.s32 pr, %1, 0;\n\t"
			    "setp.gt.and.f32 ps, %0, %4, pr;\n\t"
			    "and.pred pl, pr, !ps;\n\t"
			    "@pl mul.rn.f32 %0, %0, %3;\n\t"
			    "@ps mov.f32 %0, 0f00000000;\n\t"
			    "@ps mov.b32 %1, %5;\n\t"
			    "selp.u32 %2, %6, 0, ps;\n\t}"
			    : "+f"(V), "+r"(T), "=r"(spike)
			    : "f"(dts_sm[k0 + u]), "f"(vthres), "r"(tref), "r"(vmask & bit));
			sbits |= spike;
			unsigned const mask = __ballot_sync(0xffffffffu, spike != 0);
			mymask              = lane == u ? mask : mymask;
		}
		if (lane < nk && word < Pg->nwords) Pg->bits[(int64_t)((a.hslot0 + k0 + lane) % Hb) * Pg->nwords + word] = mymask;
		// list reservations, one per step in which the warp spiked
		for (unsigned st = __reduce_or_sync(0xffffffffu, sbits); st; st &= st - 1) {
			int const u         = __ffs(st) - 1;
			unsigned const mask = __shfl_sync(0xffffffffu, mymask, u);
			int base = 0;
			if (lane == 0) base = atomicAdd(a.counts + (k0 + u) * a.npop + p, __popc(mask));
			base = __shfl_sync(0xffffffffu, base, 0);
			if ((sbits >> u) & 1u) Pg->list[(int64_t)(a.list_k0 + k0 + u) * N + base + __popc(mask & lanemask_lt())] = i;
		}
	}
	if (valid) {
		Pg->V[i] = V;
		Pg->T[i] = T;
	}
}

// Variant 8: variant 7 with two neurons per thread (neurons b*256 + tid and b*256 + 128 + tid of a
// 128-thread CTA): the step loop's control, the leak factor and the large-count test are shared by
// both, and the window's grid has half the neuron CTAs.  Same arithmetic and outputs per neuron.
template <class A>
__device__ __forceinline__ void window_lif_lean2(A const& a, const PopDev* __restrict__ Pg, int p, int b,
                                                 const float* dts_sm, uint32_t (*xs_sm)[2 * kThreads]) {
	int const N    = (int)Pg->size;
	int const lane = threadIdx.x & 31;
	int const i0   = b * 2 * kThreads + threadIdx.x, i1 = i0 + kThreads;
	bool const v0 = i0 < N, v1 = i1 < N;
	int const word0 = i0 >> 5, word1 = i1 >> 5;
	uint32_t* const cnt = Pg->cnt;
	bool const zero     = Pg->zero_inputs != 0;
	float const vthres  = Pg->p0;
	int32_t const tref  = (int32_t)Pg->p1;
	float const w0 = Pg->group_weight[0], w1 = Pg->group_weight[1];
	float V0 = 0, V1 = 0;
	int32_t T0 = 0, T1 = 0;
	if (v0) {  // written two launches back: loaded before waiting for the previous launch
		V0 = Pg->V[i0];
		T0 = Pg->T[i0];
	}
	if (v1) {
		V1 = Pg->V[i1];
		T1 = Pg->T[i1];
	}
	griddep_wait();  // the input ring, counts and lists are the previous launches' output
	int const D = (int)a.D, Hb = a.Hb;
	for (int k0 = 0; k0 < a.K; k0 += 16) {
		int const nk    = min(16, a.K - k0);
		int const slot0 = (int)((a.slot0 + k0) % D);
		const uint32_t* src = cnt + (int64_t)slot0 * N + i0;
		int const wrap      = D - slot0;  // step u >= wrap reads ring slot u - wrap
#pragma unroll
		for (int u = 0; u < 16; u++) {  // asynchronous copies into the thread's two shared-memory columns
			if (u == wrap) src -= (int64_t)D * N;
			unsigned const dst = (unsigned)__cvta_generic_to_shared(&xs_sm[u][threadIdx.x]);
			if (v0 && u < nk) asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
			else xs_sm[u][threadIdx.x] = 0u;
			if (v1 && u < nk)
				asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst + 4u * kThreads), "l"(src + kThreads) : "memory");
			else xs_sm[u][kThreads + threadIdx.x] = 0u;
			src += N;
		}
		asm volatile("cp.async.wait_all;" ::: "memory");
		uint32_t sb0 = 0, sb1 = 0;  // this thread's spikes of the 16 steps
		uint32_t my0 = 0, my1 = 0;  // lane u: the warp's ballots of step u
#pragma unroll 1
		for (int u = 0; u < nk; u++) {
			uint32_t const x0 = xs_sm[u][threadIdx.x], x1 = xs_sm[u][kThreads + threadIdx.x];
			if (__any_sync(0xffffffffu, ((x0 | x1) & 0xfff8fff8u) != 0)) {  // a count of 8 or more in the warp
				V0 = add_n_sel(V0, w0, x0 & 0xffffu);
				V0 = add_n_sel(V0, w1, x0 >> 16);
				V1 = add_n_sel(V1, w0, x1 & 0xffffu);
				V1 = add_n_sel(V1, w1, x1 >> 16);
			} else {
				if (x0 & 4u) V0 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(V0, w0), w0), w0), w0);
				if (x1 & 4u) V1 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(V1, w0), w0), w0), w0);
				if (x0 & 2u) V0 = __fadd_rn(__fadd_rn(V0, w0), w0);
				if (x1 & 2u) V1 = __fadd_rn(__fadd_rn(V1, w0), w0);
				if (x0 & 1u) V0 = __fadd_rn(V0, w0);
				if (x1 & 1u) V1 = __fadd_rn(V1, w0);
				if (x0 & 0x40000u) V0 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(V0, w1), w1), w1), w1);
				if (x1 & 0x40000u) V1 = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(V1, w1), w1), w1), w1);
				if (x0 & 0x20000u) V0 = __fadd_rn(__fadd_rn(V0, w1), w1);
				if (x1 & 0x20000u) V1 = __fadd_rn(__fadd_rn(V1, w1), w1);
				if (x0 & 0x10000u) V0 = __fadd_rn(V0, w1);
				if (x1 & 0x10000u) V1 = __fadd_rn(V1, w1);
			}
			if (zero) {
				int64_t const o = (int64_t)((slot0 + u) % D) * N;
				if (x0) cnt[o + i0] = 0;
				if (x1) cnt[o + i1] = 0;
			}
			float const om = dts_sm[k0 + u];
			bool const s0  = lif_update(V0, T0, om, vthres, tref) && v0;
			bool const s1  = lif_update(V1, T1, om, vthres, tref) && v1;
			sb0 |= (uint32_t)s0 << u;
			sb1 |= (uint32_t)s1 << u;
			unsigned const m0 = __ballot_sync(0xffffffffu, s0);
			unsigned const m1 = __ballot_sync(0xffffffffu, s1);
			my0 = lane == u ? m0 : my0;
			my1 = lane == u ? m1 : my1;
		}
		if (lane < nk) {
			int64_t const row = (int64_t)((a.hslot0 + k0 + lane) % Hb) * Pg->nwords;
			if (word0 < Pg->nwords) Pg->bits[row + word0] = my0;
			if (word1 < Pg->nwords) Pg->bits[row + word1] = my1;
		}
		// list reservations, one per step in which the warp spiked
		for (unsigned st = __reduce_or_sync(0xffffffffu, sb0 | sb1); st; st &= st - 1) {
			int const u    = __ffs(st) - 1;
			unsigned const mask0 = __shfl_sync(0xffffffffu, my0, u);
			unsigned const mask1 = __shfl_sync(0xffffffffu, my1, u);
			int base = 0;
			if (lane == 0) base = atomicAdd(a.counts + (k0 + u) * a.npop + p, __popc(mask0) + __popc(mask1));
			base = __shfl_sync(0xffffffffu, base, 0);
			int32_t* const out = Pg->list + (int64_t)(a.list_k0 + k0 + u) * N + base;
			if ((sb0 >> u) & 1u) out[__popc(mask0 & lanemask_lt())] = i0;
			if ((sb1 >> u) & 1u) out[__popc(mask0) + __popc(mask1 & lanemask_lt())] = i1;
		}
	}
	if (v0) {
		Pg->V[i0] = V0;
		Pg->T[i0] = T0;
	}
	if (v1) {
		Pg->V[i1] = V1;
		Pg->T[i1] = T1;
	}
}

// One step of a Poisson population (samples/brunel.cpp:27-30): thread c owns neurons
// [32c, 32c + 32), jumps to draw draw_offset + 32c of the step's stream and draws 32 numbers.
// The jump XORs the states T^i(s), i < 128, selected by the 128 bits of x^(offset) mod P; the step's
// jump table holds, for each byte of the polynomial, the XOR of every subset of its 8 states, so a
// jump is 16 independent table loads.
// canonical<float>(u) < thr with canonical = (u >> 40) * 2^-24 is evaluated exactly in integers:
// for an integer m < 2^24, m < thr * 2^24  <=>  m < ceil(thr * 2^24), and m < c <=> hi32(u) < 256 c.
template <class A>
__device__ void window_poisson(A const& a, const PopDev* __restrict__ Pg, int p, int b, int bps, int* red) {
	PopDev const P  = *Pg;
	int const k     = b / bps;
	int const cb    = b % bps;
	int const hslot = (a.hslot0 + k) % a.Hb;
	const u128* tab = a.tables + ((int64_t)P.net * a.tab_net_stride + k) * kJumpTable;
	int64_t const c  = (int64_t)cb * kThreads + threadIdx.x;
	float const thr  = __fmul_rn(P.p0, a.dts[k]);
	float const cthr = ceilf(thr * 16777216.0f);  // exact: scaling by 2^24
	uint64_t const lim = cthr <= 0.f ? 0ull : (cthr >= 16777216.f ? (1ull << 32) : (uint64_t)cthr << 8);
	unsigned mask = 0;
	if (c < P.nwords) {
		u128 const poly = P.chunk_poly[c];
		uint64_t s0 = 0, s1 = 0;
#pragma unroll
		for (int g = 0; g < 8; g++) {
			ulonglong2 const v = __ldg(reinterpret_cast<const ulonglong2*>(tab + g * 256 + ((poly.lo >> (8 * g)) & 255)));
			s0 ^= v.x;
			s1 ^= v.y;
		}
#pragma unroll
		for (int g = 0; g < 8; g++) {
			ulonglong2 const v = __ldg(reinterpret_cast<const ulonglong2*>(tab + (8 + g) * 256 + ((poly.hi >> (8 * g)) & 255)));
			s0 ^= v.x;
			s1 ^= v.y;
		}
		int const n = (int)(P.size - 32 * c < 32 ? P.size - 32 * c : 32);
		if (n == 32) {
#pragma unroll 8
			for (int r = 0; r < 32; r++) {
				uint64_t const u = xoro_next(s0, s1);
				mask |= (unsigned)((u >> 32) < lim) << r;
			}
		} else {
			for (int r = 0; r < n; r++) {
				uint64_t const u = xoro_next(s0, s1);
				mask |= (unsigned)((u >> 32) < lim) << r;
			}
		}
		P.bits[(int64_t)hslot * P.nwords + c] = mask;
	}
	// ascending append: CTA exclusive scan of the per-thread spike counts, one reservation
	int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int const mine = __popc(mask);
	int incl       = mine;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		int const v = __shfl_up_sync(0xffffffffu, incl, d);
		if (lane >= d) incl += v;
	}
	if (lane == 31) red[warp] = incl;
	__syncthreads();
	if (threadIdx.x == 0) {
		int tot = 0;
		for (int w = 0; w < kThreads / 32; w++) {
			int const v = red[w];
			red[w]      = tot;
			tot += v;
		}
		red[kThreads / 32] = tot ? atomicAdd(a.counts + k * a.npop + p, tot) : 0;
	}
	__syncthreads();
	if (!mask) return;
	int32_t* out = P.list + (int64_t)(a.list_k0 + k) * P.size + red[kThreads / 32] + red[warp] + (incl - mine);
	unsigned m   = mask;
	while (m) {
		int const r = __ffs(m) - 1;
		m &= m - 1;
		*out++ = (int32_t)(32 * c + r);
	}
}

// One step of an external population (samples/external_input.cpp:17-30).
template <class A>
__device__ void window_external(A const& a, const PopDev* __restrict__ Pg, int p, int k, int64_t ext_pos) {
	PopDev const P  = *Pg;
	uint32_t* bits  = P.bits + (int64_t)((a.hslot0 + k) % a.Hb) * P.nwords;
	for (int j = threadIdx.x; j < P.nwords; j += blockDim.x) bits[j] = 0;
	__syncthreads();
	if (P.ext_steps <= 0) return;
	int64_t const pos = (ext_pos + k) % P.ext_steps;
	int32_t const n   = P.ext_counts[pos];
	const int32_t* src = P.ext_idx + P.ext_off[pos];
	for (int j = threadIdx.x; j < n; j += blockDim.x) {
		int32_t const s = src[j];
		atomicOr(bits + (s >> 5), 1u << (s & 31));
		P.list[(int64_t)(a.list_k0 + k) * P.size + j] = s;
	}
	if (threadIdx.x == 0) a.counts[k * a.npop + p] = n;
}

// One CTA of the neuron update (block b of the window's neuron blocks).
template <int MODE, bool ONLY_FAST, int VAR>
__device__ __forceinline__ void neurons_block(WindowArgs const& a, int b) {
	constexpr bool ROLLED = VAR == 1 || VAR == 2 || VAR >= 4;  // 4 .. 8: deferred spike output
	__shared__ float dts_sm[kMaxWindow];
	__shared__ uint32_t xs_sm[ROLLED ? 16 : 1][VAR == 8 ? 2 * kThreads : kThreads];
	__shared__ uint32_t masks_sm[VAR >= 4 && VAR <= 6 ? kThreads / 32 : 1][16];
	int p = 0;
	while (p + 1 < a.npop && b >= a.blk_begin[p + 1]) p++;
	int const lb   = b - a.blk_begin[p];
	int const kind = a.blk_kind[p];
	if (VAR >= 6 && MODE == 0 && kind == 3) {  // the LIF leak factors of the window's steps
		float const tminv = a.pops[p].p2;
		for (int k = threadIdx.x; k < a.K; k += blockDim.x) dts_sm[k] = __fmaf_rn(-a.dts[k], tminv, 1.0f);
	} else {
		for (int k = threadIdx.x; k < a.K; k += blockDim.x) dts_sm[k] = a.dts[k];
	}
	__syncthreads();
	// window_lif_deferred waits for the previous launch after loading the state; the others first
	if (MODE == 0 && kind == 3) {
		if constexpr (VAR == 8) window_lif_lean2(a, a.pops + p, p, lb, dts_sm, xs_sm);
		else if constexpr (VAR == 7) window_lif_lean(a, a.pops + p, p, lb, dts_sm, xs_sm);
		else if constexpr (VAR == 9) {
			if (a.pops[p].zero_inputs) window_lif_pred<true>(a, a.pops + p, p, lb, dts_sm, xs_sm);
			else window_lif_pred<false>(a, a.pops + p, p, lb, dts_sm, xs_sm);
		}
		else if constexpr (VAR == 4) window_lif_deferred<false, false>(a, a.pops + p, p, lb, dts_sm, xs_sm, masks_sm);
		else if constexpr (VAR == 5) window_lif_deferred<true, false>(a, a.pops + p, p, lb, dts_sm, xs_sm, masks_sm);
		else if constexpr (VAR == 6) window_lif_deferred<false, true>(a, a.pops + p, p, lb, dts_sm, xs_sm, masks_sm);
		else {
			griddep_wait();
			window_lif_fast<ROLLED, VAR == 2 || VAR == 3>(a, a.pops + p, p, lb, dts_sm, xs_sm);
		}
		return;
	}
	griddep_wait();
	if (kind == 3) window_neurons<MODE, true, false>(a, a.pops + p, p, lb);
	else if (!ONLY_FAST) {
		if (kind == 0) window_neurons<MODE, false, false>(a, a.pops + p, p, lb);
		else if (kind == 3 + kHistKind) window_neurons<MODE, true, true>(a, a.pops + p, p, lb);
		else window_neurons<MODE, false, true>(a, a.pops + p, p, lb);
	}
}

// Per-neuron populations: one thread per neuron, K steps with the state in registers.
// ONLY_FAST: every population of the launch takes the FAST path, so the generic input replay is
// compiled out (fewer registers).  VAR: the LIF window variant (window_lif_fast), one kernel each so
// that each keeps its own register count.
template <int MODE, bool ONLY_FAST, int VAR>
__global__ void __launch_bounds__(kThreads, ONLY_FAST ? kNeuronBlocksPerSM : 1) k_neurons(const __grid_constant__ WindowArgs a) {
	span_open(a.span);
	neurons_block<MODE, ONLY_FAST, VAR>(a, (int)blockIdx.x);
	span_close(a.span);
}

// Populations without inputs (Poisson, external trains): one CTA per (step, chunk).  They depend on
// nothing but the step's random stream, so they run on a second stream, overlapped with the
// neuron update and the delivery of the previous window.
__device__ __forceinline__ void sources_block(WindowArgs const& a, int b) {
	__shared__ int red[kThreads / 32 + 1];
	griddep_wait();  // this parity's counts were cleared by the previous delivery
	int p = 0;
	while (p + 1 < a.npop && b >= a.blk_begin[p + 1]) p++;
	int const lb = b - a.blk_begin[p];
	if (a.blk_kind[p] == 1) {
		// the chunk's steps [k0, k0 + src_steps): src_steps > 1 keeps the window's grid within one wave
		int const bps = a.blk_per_step[p];
		int const S   = a.src_steps > 0 ? a.src_steps : 1;
		int const k0  = (lb / bps) * S, cb = lb % bps;
		for (int k = k0; k < min(a.K, k0 + S); k++) {
			if (k > k0) __syncthreads();  // red[] of the previous step is read
			window_poisson(a, a.pops + p, p, k * bps + cb, bps, red);
		}
	}
	else if (a.blk_kind[p] == 2) window_external(a, a.pops + p, p, lb, a.ext_pos[p]);
}

__global__ void __launch_bounds__(kThreads) k_sources(const __grid_constant__ WindowArgs a) {
	sources_block(a, (int)blockIdx.x);
}


// One window's neuron update and source populations in one grid: first (when recording) the
// raster blocks of the previous window `r`, whose bitmaps and counts are final, then nb neuron
// blocks of `a`, then the source blocks of `s`.  Launched as the programmatic dependent
// of the previous delivery, so its CTAs are resident, waiting, when that delivery ends.
__device__ void raster_block(RasterArgs const& a, int b);

template <int MODE, bool ONLY_FAST, int VAR, bool REC>
__global__ void __launch_bounds__(kThreads, ONLY_FAST ? kNeuronBlocksPerSM : 1) k_window(const __grid_constant__ WindowArgs a,
                                                                       const __grid_constant__ WindowArgs s, int nb,
                                                                       const __grid_constant__ RasterArgs r) {
	// each block kind waits for the previous launch where it first reads that launch's output; the
	// raster blocks read only final data (the previous window's bitmaps and counts)
	griddep_launch();
	span_open(a.span);
	int const nrb = REC ? r.K * r.npop : 0;  // raster blocks first: they start with the first wave
	int const b   = (int)blockIdx.x;
	if (REC && b < nrb) raster_block(r, b);  // the previous window's raster
	else if (b < nrb + nb) neurons_block<MODE, ONLY_FAST, VAR>(a, b - nrb);
	else sources_block(s, b - nrb - nb);
	span_close(a.span);
}

// Writes a finished shared-memory tile into ring slot sigma mod D: a plain store when this CTA is
// the slot's only writer, an add when the ring accumulates (mixed delays), reductions when several
// CTAs share the tile.
template <int MODE, class A>
__device__ __forceinline__ void flush_tile(A const& a, PopDev const& P, int tbase, int words, int64_t sigma,
                                           const uint32_t* tile_sm) {
	int64_t const slot = sigma % a.D;
	if (MODE == 0) {
		uint32_t* dst = P.cnt + (slot * P.size + tbase) * P.W;
		if (a.parts > 1) {
			for (int i = threadIdx.x; i < words; i += blockDim.x) {
				uint32_t const v = tile_sm[i];
				if (v) red_add_u32(dst + i, v);
			}
		} else if (P.zero_inputs) {
			for (int i = threadIdx.x; i < words; i += blockDim.x) {
				uint32_t const v = tile_sm[i];
				if (v) dst[i] += v;
			}
		} else {
			for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = tile_sm[i];
		}
	} else {
		float* dst      = P.acc + (slot * P.size + tbase) * P.F;
		const float* sm = reinterpret_cast<const float*>(tile_sm);
		if (a.parts > 1) {
			for (int i = threadIdx.x; i < words; i += blockDim.x) {
				float const v = sm[i];
				if (v != 0.0f) red_add_f32(dst + i, v);
			}
		} else if (P.zero_inputs) {
			for (int i = threadIdx.x; i < words; i += blockDim.x) {
				float const v = sm[i];
				if (v != 0.0f) dst[i] = __fadd_rn(dst[i], v);
			}
		} else {
			for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = sm[i];
		}
	}
}

// Block-wide event count of a delivery CTA into the net's counter.
__device__ __forceinline__ void add_events(unsigned long long* dst, unsigned long long mine, unsigned long long* ev_block) {
	for (int d = 16; d; d >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, d);
	if ((threadIdx.x & 31) == 0 && mine) atomicAdd(ev_block, mine);
	__syncthreads();
	if (threadIdx.x == 0 && *ev_block) atomicAdd(dst, *ev_block);
}

// Delivery of one (input slot sigma = slot_lo + si, target tile t of population P) work item:
// every connection into P whose spikes of the window reach slot sigma adds its events to the
// shared-memory tile, which is then flushed.  part: this CTA's share when `parts` CTAs split it.
// Warp-flattened mapping: a warp takes 32 spikes, prefix-sums their sub-row lengths and lanes walk
// the concatenated sub-rows (8 loads in flight per lane).
template <int MODE, class A>
__device__ __forceinline__ void deliver_flat(A const& a, PopDev const& P, int t, int si, int part) {
	extern __shared__ uint32_t tile_sm[];
	__shared__ unsigned long long ev_block;
	int const T     = P.tile;
	int const tbase = t * T;
	int const tn    = (int)min((int64_t)T, P.size - tbase);
	int const width = MODE == 0 ? P.W : P.F;
	int const words = tn * width;
	for (int i = threadIdx.x; i < words; i += blockDim.x) tile_sm[i] = 0;
	if (threadIdx.x == 0) ev_block = 0;
	__syncthreads();
	int64_t const sigma = a.slot_lo + si;
	int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
	unsigned long long my_events = 0;
	bool touched = false;
	for (int ci = P.in_begin; ci < P.in_end; ci++) {
		ConnDev const& C = a.conns[ci];
		int64_t const k  = sigma - (a.t0 + C.delay - 1);
		if (k < 0 || k >= a.K || C.plastic) continue;
		touched = true;
		int const n          = a.counts[k * a.npop + C.src];
		const int32_t* lst   = C.src_list + (a.list_k0 + k) * C.src_size;
		const int64_t* bnd   = C.bounds;
		int const stride     = P.ntiles + 1;
		const int32_t* nb    = C.nb;
		int const word       = MODE == 0 ? C.word : C.fslot;
		uint32_t const inc   = C.inc;
		float const w        = C.weight;
		int const jstride = a.parts * nwarps * 32;
		int j0            = (part * nwarps + warp) * 32;
		int s_next        = (j0 + lane < n) ? __ldg(lst + j0 + lane) : -1;
		while (j0 < n) {
			int const s = s_next;
			int64_t start = 0;
			int len       = 0;
			if (s >= 0) {
				const int64_t* bb = bnd + (int64_t)s * stride + t;
				start             = __ldg(bb);
				len               = (int)(__ldg(bb + 1) - start);
			}
			int const jn = j0 + jstride;  // prefetch the next batch's spike ids
			s_next       = (jn + lane < n) ? __ldg(lst + jn + lane) : -1;
			int incl = len;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				int const o = __shfl_up_sync(0xffffffffu, incl, d);
				if (lane >= d) incl += o;
			}
			int const total = __shfl_sync(0xffffffffu, incl, 31);
			int const excl  = incl - len;
			if (lane == 0) my_events += (unsigned long long)total;
			for (int base = 0; base < total; base += 32 * 8) {
				int32_t d[8];
#pragma unroll
				for (int u = 0; u < 8; u++) {
					int const e = base + u * 32 + lane;
					d[u]        = -1;
					// the spike q whose sub-row holds flattened event e: largest q with excl_q <= e
					int q = 0;
#pragma unroll
					for (int st = 16; st; st >>= 1) {
						int const cand = q + st;
						int const ex   = __shfl_sync(0xffffffffu, excl, cand & 31);
						if (cand < 32 && ex <= e) q = cand;
					}
					int64_t const sq = __shfl_sync(0xffffffffu, start, q);
					int const eq     = __shfl_sync(0xffffffffu, excl, q);
					if (e < total) d[u] = __ldg(nb + sq + (e - eq));
				}
#pragma unroll
				for (int u = 0; u < 8; u++)
					if (d[u] >= 0) {
						int const li = (d[u] - tbase) * width + word;
						if (MODE == 0)
							atomicAdd(tile_sm + li, inc);
						else
							atomicAdd(reinterpret_cast<float*>(tile_sm) + li, w);
					}
			}
			j0 = jn;
		}
	}
	add_events(a.events, my_events, &ev_block);
	if (!touched) return;
	flush_tile<MODE>(a, P, tbase, words, sigma, tile_sm);
}

// Thread-per-spike mapping: each thread walks the sub-row of one spike within the CTA's tile
// (8 loads in flight), no cross-lane work distribution.  VEC: 16-byte loads of the sub-row body.
template <int MODE, bool VEC, class A>
__device__ __forceinline__ void deliver_tps(A const& a, PopDev const& P, int t, int si, int part) {
	extern __shared__ uint32_t tile_sm[];
	__shared__ unsigned long long ev_block;
	int const tbase = t * P.tile;
	int const tn    = (int)min((int64_t)P.tile, P.size - tbase);
	int const width = MODE == 0 ? P.W : P.F;
	int const words = tn * width;
	for (int i = threadIdx.x; i < words; i += blockDim.x) tile_sm[i] = 0;
	if (threadIdx.x == 0) ev_block = 0;
	__syncthreads();
	int64_t const sigma = a.slot_lo + si;
	unsigned long long my_events = 0;
	bool touched = false;
	for (int ci = P.in_begin; ci < P.in_end; ci++) {
		ConnDev const& C = a.conns[ci];
		int64_t const k  = sigma - (a.t0 + C.delay - 1);
		if (k < 0 || k >= a.K || C.plastic) continue;
		touched = true;
		int const n        = a.counts[k * a.npop + C.src];
		const int32_t* lst = C.src_list + (a.list_k0 + k) * C.src_size;
		const int64_t* bnd = C.bounds;
		int const stride   = P.ntiles + 1;
		const int32_t* nb  = C.nb;
		int const word     = MODE == 0 ? C.word : C.fslot;
		uint32_t const inc = C.inc;
		float const w      = C.weight;
		auto add = [&](int32_t d) {
			int const li = (d - tbase) * width + word;
			if (MODE == 0) atomicAdd(tile_sm + li, inc);
			else atomicAdd(reinterpret_cast<float*>(tile_sm) + li, w);
		};
		for (int j = part * blockDim.x + threadIdx.x; j < n; j += a.parts * blockDim.x) {
			int const s        = __ldg(lst + j);
			const int64_t* bb  = bnd + (int64_t)s * stride + t;
			int64_t const e0   = __ldg(bb);
			int64_t const e1   = __ldg(bb + 1);
			my_events += (unsigned long long)(e1 - e0);
			if (!VEC) {
				for (int64_t e = e0; e < e1; e += 8) {
					int32_t d[8];
#pragma unroll
					for (int u = 0; u < 8; u++) d[u] = e + u < e1 ? __ldg(nb + e + u) : -1;
#pragma unroll
					for (int u = 0; u < 8; u++)
						if (d[u] >= 0) add(d[u]);
				}
				continue;
			}
			// the sub-row in 16-byte loads (4 targets each): scalar head up to a 4-aligned index,
			// aligned body two vectors at a time, scalar tail.  Fewer L1 sector lookups per event.
			int64_t const h = min(e1, (e0 + 3) & ~int64_t(3));
			for (int64_t e = e0; e < h; e++) add(__ldg(nb + e));
			int64_t const body_end = h + ((e1 - h) & ~int64_t(3));
			const int4* v = reinterpret_cast<const int4*>(nb + h);
			int64_t const nv = (body_end - h) >> 2;
			int64_t q = 0;
			for (; q + 2 <= nv; q += 2) {
				int4 const x = __ldg(v + q), y = __ldg(v + q + 1);
				add(x.x); add(x.y); add(x.z); add(x.w);
				add(y.x); add(y.y); add(y.z); add(y.w);
			}
			if (q < nv) {
				int4 const x = __ldg(v + q);
				add(x.x); add(x.y); add(x.z); add(x.w);
			}
			for (int64_t e = body_end; e < e1; e++) add(__ldg(nb + e));
		}
	}
	add_events(a.events, my_events, &ev_block);
	if (!touched) return;
	flush_tile<MODE>(a, P, tbase, words, sigma, tile_sm);
}

// Software-pipelined thread-per-spike mapping: while a thread walks the sub-row of its current
// spike (16 target loads in flight), the tile bounds of its next spike and the id of the one after
// are already on their way, so the list -> bounds -> targets chain is exposed once per thread
// instead of once per spike.
template <int MODE, class A>
__device__ __forceinline__ void deliver_tps_pipe(A const& a, PopDev const& P, int t, int si, int part) {
	extern __shared__ uint32_t tile_sm[];
	__shared__ unsigned long long ev_block;
	int const tbase = t * P.tile;
	int const tn    = (int)min((int64_t)P.tile, P.size - tbase);
	int const width = MODE == 0 ? P.W : P.F;
	int const words = tn * width;
	for (int i = threadIdx.x; i < words; i += blockDim.x) tile_sm[i] = 0;
	if (threadIdx.x == 0) ev_block = 0;
	__syncthreads();
	int64_t const sigma = a.slot_lo + si;
	unsigned long long my_events = 0;
	bool touched = false;
	for (int ci = P.in_begin; ci < P.in_end; ci++) {
		ConnDev const& C = a.conns[ci];
		int64_t const k  = sigma - (a.t0 + C.delay - 1);
		if (k < 0 || k >= a.K || C.plastic) continue;
		touched = true;
		int const n        = a.counts[k * a.npop + C.src];
		const int32_t* lst = C.src_list + (a.list_k0 + k) * C.src_size;
		const int64_t* bnd = C.bounds + t;
		int const stride   = P.ntiles + 1;
		const int32_t* nb  = C.nb;
		int const word     = MODE == 0 ? C.word : C.fslot;
		uint32_t const inc = C.inc;
		float const w      = C.weight;
		int const js       = a.parts * blockDim.x;
		int j              = part * blockDim.x + threadIdx.x;
		int s_next         = j + js < n ? __ldg(lst + j + js) : -1;
		int64_t e0 = 0, e1 = 0;
		if (j < n) {
			const int64_t* bb = bnd + (int64_t)__ldg(lst + j) * stride;
			e0                = __ldg(bb);
			e1                = __ldg(bb + 1);
		}
		while (j < n) {
			int64_t f0 = 0, f1 = 0;
			if (s_next >= 0) {
				const int64_t* bb = bnd + (int64_t)s_next * stride;
				f0                = __ldg(bb);
				f1                = __ldg(bb + 1);
			}
			int const j2 = j + 2 * js;
			s_next       = j2 < n ? __ldg(lst + j2) : -1;
			my_events += (unsigned long long)(e1 - e0);
			for (int64_t e = e0; e < e1; e += 16) {
				int32_t d[16];
#pragma unroll
				for (int u = 0; u < 16; u++) d[u] = e + u < e1 ? __ldg(nb + e + u) : -1;
#pragma unroll
				for (int u = 0; u < 16; u++)
					if (d[u] >= 0) {
						int const li = (d[u] - tbase) * width + word;
						if (MODE == 0) atomicAdd(tile_sm + li, inc);
						else atomicAdd(reinterpret_cast<float*>(tile_sm) + li, w);
					}
			}
			e0 = f0;
			e1 = f1;
			j += js;
		}
	}
	add_events(a.events, my_events, &ev_block);
	if (!touched) return;
	flush_tile<MODE>(a, P, tbase, words, sigma, tile_sm);
}

// Lane-group mapping: G consecutive lanes share one spike and walk its sub-row G targets at a time
// (U loads in flight per lane), so one warp load touches 32/G sub-rows -- about 32/G sectors --
// instead of 32: the thread-per-spike mapping is bound by L1 sector lookups, one per event.  The
// next spike's id and bounds are loaded while the current sub-row is processed.
template <int MODE, int G, class A>
__device__ __forceinline__ void deliver_groups(A const& a, PopDev const& P, int t, int si, int part) {
	constexpr int U = 4;
	extern __shared__ uint32_t tile_sm[];
	__shared__ unsigned long long ev_block;
	int const tbase = t * P.tile;
	int const tn    = (int)min((int64_t)P.tile, P.size - tbase);
	int const width = MODE == 0 ? P.W : P.F;
	int const words = tn * width;
	for (int i = threadIdx.x; i < words; i += blockDim.x) tile_sm[i] = 0;
	if (threadIdx.x == 0) ev_block = 0;
	__syncthreads();
	int64_t const sigma = a.slot_lo + si;
	int const gl = threadIdx.x & (G - 1);
	int const gi = threadIdx.x / G;
	int const ng = blockDim.x / G;
	unsigned long long my_events = 0;
	bool touched = false;
	for (int ci = P.in_begin; ci < P.in_end; ci++) {
		ConnDev const& C = a.conns[ci];
		int64_t const k  = sigma - (a.t0 + C.delay - 1);
		if (k < 0 || k >= a.K || C.plastic) continue;
		touched = true;
		int const n        = a.counts[k * a.npop + C.src];
		const int32_t* lst = C.src_list + (a.list_k0 + k) * C.src_size;
		const int64_t* bnd = C.bounds + t;
		int const stride   = P.ntiles + 1;
		const int32_t* nb  = C.nb;
		int const word     = MODE == 0 ? C.word : C.fslot;
		uint32_t const inc = C.inc;
		float const w      = C.weight;
		int const js       = a.parts * ng;
		int j              = part * ng + gi;
		int64_t e0 = 0, e1 = 0;
		if (j < n) {
			const int64_t* bb = bnd + (int64_t)__ldg(lst + j) * stride;
			e0                = __ldg(bb);
			e1                = __ldg(bb + 1);
		}
		int s_next = j + js < n ? __ldg(lst + j + js) : -1;
		while (j < n) {
			int64_t f0 = 0, f1 = 0;
			if (s_next >= 0) {
				const int64_t* bb = bnd + (int64_t)s_next * stride;
				f0                = __ldg(bb);
				f1                = __ldg(bb + 1);
			}
			int const j2 = j + 2 * js;
			s_next       = j2 < n ? __ldg(lst + j2) : -1;
			if (gl == 0) my_events += (unsigned long long)(e1 - e0);
			for (int64_t e = e0 + gl; e < e1; e += G * U) {
				int32_t d[U];
#pragma unroll
				for (int u = 0; u < U; u++) d[u] = e + u * G < e1 ? __ldg(nb + e + u * G) : -1;
#pragma unroll
				for (int u = 0; u < U; u++)
					if (d[u] >= 0) {
						int const li = (d[u] - tbase) * width + word;
						if (MODE == 0) atomicAdd(tile_sm + li, inc);
						else atomicAdd(reinterpret_cast<float*>(tile_sm) + li, w);
					}
			}
			e0 = f0;
			e1 = f1;
			j += js;
		}
	}
	add_events(a.events, my_events, &ev_block);
	if (!touched) return;
	flush_tile<MODE>(a, P, tbase, words, sigma, tile_sm);
}

// Staged lane-group mapping: the sub-row descriptors (start, length, connection) of up to kStage
// spikes -- of every connection into the tile's population that reaches this slot -- are first
// loaded by all threads at once (spike id, then tile bounds: many loads in flight) into shared
// memory; then 4-lane groups take pairs of sub-rows from a shared counter (balanced however the
// lengths vary) and walk both at once, so a spike's chain is one target load instead of
// id -> bounds -> targets.
constexpr int kStage     = 1024;
constexpr int kConnBatch = 16;

template <int MODE, int SF, class A>
__device__ __forceinline__ void deliver_staged(A const& a, PopDev const& P, int t, int si, int part) {
	constexpr int G = 4, U = 4;
	extern __shared__ uint32_t tile_sm[];
	__shared__ unsigned long long ev_block;
	__shared__ int64_t st_e0[kStage];
	__shared__ int32_t st_len[kStage];
	__shared__ uint8_t st_c[kStage];
	__shared__ int c_pre[kConnBatch + 1];
	__shared__ const int32_t* c_lst[kConnBatch];
	__shared__ const int64_t* c_bnd[kConnBatch];
	__shared__ const int32_t* c_nb[kConnBatch];
	__shared__ uint32_t c_inc[kConnBatch];
	__shared__ int c_word[kConnBatch];
	__shared__ float c_w[kConnBatch];
	__shared__ int s_nc, s_touched, s_next;
	int const tbase = t * P.tile;
	int const tn    = (int)min((int64_t)P.tile, P.size - tbase);
	int const width = MODE == 0 ? P.W : P.F;
	int const words = tn * width;
	for (int i = threadIdx.x; i < words; i += blockDim.x) tile_sm[i] = 0;
	if (threadIdx.x == 0) {
		ev_block  = 0;
		s_touched = 0;
	}
	int64_t const sigma = a.slot_lo + si;
	int const stride    = P.ntiles + 1;
	int const gl        = threadIdx.x & (G - 1);
	unsigned long long my_events = 0;
	for (int cb = P.in_begin; cb < P.in_end; cb += kConnBatch) {
		__syncthreads();
		if (threadIdx.x == 0) {  // the batch's connections that reach this slot, with this part's spikes
			int tot = 0, nc = 0;
			for (int ci = cb; ci < min(cb + kConnBatch, P.in_end); ci++) {
				ConnDev const& C = a.conns[ci];
				int64_t const k  = sigma - (a.t0 + C.delay - 1);
				if (k < 0 || k >= a.K || C.plastic) continue;
				s_touched    = 1;
				int const n  = a.counts[k * a.npop + C.src];
				int const pp = (n + a.parts - 1) / a.parts;
				int const lo = min(n, part * pp), hi = min(n, lo + pp);
				c_lst[nc]  = C.src_list + (a.list_k0 + k) * C.src_size + lo;
				c_bnd[nc]  = C.bounds + t;
				c_nb[nc]   = C.nb;
				c_inc[nc]  = C.inc;
				c_word[nc] = MODE == 0 ? C.word : C.fslot;
				c_w[nc]    = C.weight;
				c_pre[nc]  = tot;
				tot += hi - lo;
				nc++;
			}
			c_pre[nc] = tot;
			s_nc      = nc;
		}
		__syncthreads();
		int const nc    = s_nc;
		int const total = c_pre[nc];
		for (int c0 = 0; c0 < total; c0 += kStage) {
			int const m = min(kStage, total - c0);
			for (int q = threadIdx.x; q < m; q += blockDim.x) {
				int const g = c0 + q;
				int j       = 0;
				while (j + 1 < nc && c_pre[j + 1] <= g) j++;
				const int64_t* bb = c_bnd[j] + (int64_t)__ldg(c_lst[j] + (g - c_pre[j])) * stride;
				int64_t const b0  = __ldg(bb);
				st_e0[q]          = b0;
				st_len[q]         = (int32_t)(__ldg(bb + 1) - b0);
				st_c[q]           = (uint8_t)j;
			}
			if (threadIdx.x == 0) s_next = 0;
			__syncthreads();
			int const nsets = (m + SF - 1) / SF;
			while (true) {  // a warp takes 32 / G consecutive sets of SF sub-rows per fetch (warp-uniform exit)
				int base = 0;
				if ((threadIdx.x & 31) == 0) base = atomicAdd(&s_next, 32 / G);
				base = __shfl_sync(0xffffffffu, base, 0);
				if (base >= nsets) break;
				int const ps = base + ((threadIdx.x & 31) / G);
				if (ps >= nsets) continue;
				int64_t e[SF];
				int len[SF], cj[SF];
				int lmax = 0;
#pragma unroll
				for (int f = 0; f < SF; f++) {
					int const q = ps * SF + f;
					e[f]        = q < m ? st_e0[q] : 0;
					len[f]      = q < m ? st_len[q] : 0;
					cj[f]       = q < m ? st_c[q] : 0;
					lmax        = max(lmax, len[f]);
					if (gl == 0) my_events += (unsigned long long)len[f];
				}
				for (int o = gl; o < lmax; o += G * U) {
					int32_t d[SF][U];
#pragma unroll
					for (int f = 0; f < SF; f++) {
						const int32_t* nbf = c_nb[cj[f]];
#pragma unroll
						for (int u = 0; u < U; u++) {
							int const oo = o + u * G;
							d[f][u]      = oo < len[f] ? __ldg(nbf + e[f] + oo) : -1;
						}
					}
#pragma unroll
					for (int f = 0; f < SF; f++)
#pragma unroll
						for (int u = 0; u < U; u++)
							if (d[f][u] >= 0) {
								int const li = (d[f][u] - tbase) * width + c_word[cj[f]];
								if (MODE == 0) atomicAdd(tile_sm + li, c_inc[cj[f]]);
								else atomicAdd(reinterpret_cast<float*>(tile_sm) + li, c_w[cj[f]]);
							}
				}
			}
			__syncthreads();
		}
	}
	__syncthreads();
	bool const touched = s_touched != 0;
	add_events(a.events, my_events, &ev_block);
	if (!touched) return;
	flush_tile<MODE>(a, P, tbase, words, sigma, tile_sm);
}

// Staged mapping with whole sub-rows in one round trip: as deliver_staged, but a 4-lane group loads
// its SF sub-rows as aligned 16-byte blocks of the target array, U blocks per lane (4U*4 targets per
// sub-row) before the first shared-memory add, so a typical sub-row (<= 64 targets) costs one load
// latency instead of one per 16 targets.  Only blocks holding at least one target of the sub-row are
// read (target arrays are 16-byte aligned and padded to whole blocks); the targets of a block outside
// the sub-row are skipped.  Up to kStageV descriptors per round, so most CTAs stage once.
constexpr int kStageV = 2048;

template <int MODE, int SF, int U, class A>
__device__ __forceinline__ void deliver_staged_vec(A const& a, PopDev const& P, int t, int si, int part) {
	constexpr int G = 4;
	extern __shared__ uint32_t tile_sm[];
	__shared__ unsigned long long ev_block;
	__shared__ int64_t st_e0[kStageV];
	__shared__ int32_t st_len[kStageV];
	__shared__ uint8_t st_c[kStageV];
	__shared__ int c_pre[kConnBatch + 1];
	__shared__ const int32_t* c_lst[kConnBatch];
	__shared__ const int64_t* c_bnd[kConnBatch];
	__shared__ const int4* c_nb[kConnBatch];
	__shared__ uint32_t c_abase[kConnBatch];
	__shared__ uint32_t c_inc[kConnBatch];
	__shared__ float c_w[kConnBatch];
	__shared__ int s_nc, s_touched, s_next;
	int const tbase = t * P.tile;
	int const tn    = (int)min((int64_t)P.tile, P.size - tbase);
	int const width = MODE == 0 ? P.W : P.F;
	int const words = tn * width;
	int const lane  = threadIdx.x & 31;
	int64_t const sigma = a.slot_lo + si;
	int const stride    = P.ntiles + 1;
	int const gl        = threadIdx.x & (G - 1);
	uint32_t const tile_addr = (uint32_t)__cvta_generic_to_shared(tile_sm);
	uint32_t const mul       = 4u * (uint32_t)width;
	if (threadIdx.x == 0) {
		ev_block  = 0;
		s_touched = 0;
	}
	bool zeroed = false;
	unsigned long long my_events = 0;
	for (int cb = P.in_begin; cb < P.in_end; cb += kConnBatch) {
		__syncthreads();
		if (threadIdx.x < 32) {
			// warp 0: one lane per connection of the batch -- the connections' fields and spike
			// counts are loaded in parallel; a warp scan places their spikes in the stage
			int const ci = cb + lane;
			int n = 0;
			bool reach = false;
			const int32_t* lst = nullptr;
			const int4* nbp    = nullptr;
			const int64_t* bnp = nullptr;
			uint32_t ab = 0, ic = 0;
			float wt    = 0.0f;
			if (lane < kConnBatch && ci < P.in_end) {
				ConnDev const& C = a.conns[ci];
				int64_t const k  = sigma - (a.t0 + C.delay - 1);
				if (k >= 0 && k < a.K && !C.plastic) {
					int const cnt = a.counts[k * a.npop + C.src];
					int const pp  = (cnt + a.parts - 1) / a.parts;
					int const lo  = min(cnt, part * pp);
					reach         = true;
					n             = min(cnt, lo + pp) - lo;
					lst           = C.src_list + (a.list_k0 + k) * C.src_size + lo;
					nbp           = reinterpret_cast<const int4*>(C.nb);
					bnp           = C.bounds + t;
					ab            = tile_addr + 4u * (uint32_t)((MODE == 0 ? C.word : C.fslot) - tbase * width);
					ic            = C.inc;
					wt            = C.weight;
				}
			}
			unsigned const rm = __ballot_sync(0xffffffffu, reach);
			int incl          = n;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				int const o = __shfl_up_sync(0xffffffffu, incl, d);
				if (lane >= d) incl += o;
			}
			int const tot = __shfl_sync(0xffffffffu, incl, 31);
			if (reach) {  // the reaching connections, compacted to slots 0 .. nc-1 in batch order
				int const j = __popc(rm & lanemask_lt());
				c_pre[j]    = incl - n;
				c_lst[j]    = lst;
				c_nb[j]     = nbp;
				c_bnd[j]    = bnp;
				c_abase[j]  = ab;
				c_inc[j]    = ic;
				c_w[j]      = wt;
				s_touched   = 1;
			}
			if (lane == 0) {
				s_nc            = __popc(rm);
				c_pre[__popc(rm)] = tot;
			}
			if (blockDim.x == 32 && !zeroed)
				for (int i = lane; i < words; i += 32) tile_sm[i] = 0;
		} else if (!zeroed) {  // the other warps clear the tile meanwhile
			for (int i = threadIdx.x - 32; i < words; i += blockDim.x - 32) tile_sm[i] = 0;
		}
		zeroed = true;
		__syncthreads();
		int const nc    = s_nc;
		int const total = c_pre[nc];
		for (int c0 = 0; c0 < total; c0 += kStageV) {
			int const m = min(kStageV, total - c0);
			for (int q = threadIdx.x; q < m; q += blockDim.x) {
				int const g = c0 + q;
				int j       = 0;
				while (j + 1 < nc && c_pre[j + 1] <= g) j++;
				const int64_t* bb = c_bnd[j] + (int64_t)__ldg(c_lst[j] + (g - c_pre[j])) * stride;
				int64_t const b0  = __ldg(bb);
				st_e0[q]          = b0;
				st_len[q]         = (int32_t)(__ldg(bb + 1) - b0);
				st_c[q]           = (uint8_t)j;
			}
			if (threadIdx.x == 0) s_next = 0;
			__syncthreads();
			int const nsets = (m + SF - 1) / SF;
			while (true) {  // a warp takes 32 / G consecutive sets of SF sub-rows per fetch (warp-uniform exit)
				int base = 0;
				if (lane == 0) base = atomicAdd(&s_next, 32 / G);
				base = __shfl_sync(0xffffffffu, base, 0);
				if (base >= nsets) break;
				int const ps = base + lane / G;  // lanes past the last set take empty sub-rows
				const int4* nbf[SF];
				int lo[SF], hi[SF], nbk[SF], cj[SF];
				int nbw = 0;
#pragma unroll
				for (int f = 0; f < SF; f++) {
					int const q     = ps * SF + f;
					bool const ok   = ps < nsets && q < m;
					int64_t const e = ok ? st_e0[q] : 0;
					int const len   = ok ? st_len[q] : 0;
					cj[f]           = ok ? st_c[q] : 0;
					lo[f]           = (int)(e & 3);  // targets [lo, hi) of the 16-byte blocks from e / 4 on
					hi[f]           = lo[f] + len;
					nbk[f]          = (hi[f] + 3) >> 2;
					if (len == 0) nbk[f] = 0;
					nbf[f]          = c_nb[cj[f]] + (e >> 2);
					nbw             = max(nbw, nbk[f]);
					if (gl == 0) my_events += (unsigned long long)len;
				}
				nbw = __reduce_max_sync(0xffffffffu, nbw);  // the warp's longest sub-row, in blocks
				for (int o = 0; o < nbw; o += G * U) {
					int4 v[SF][U];
#pragma unroll
					for (int f = 0; f < SF; f++)
#pragma unroll
						for (int u = 0; u < U; u++) {
							int const ob = o + u * G + gl;
							if (ob < nbk[f]) v[f][u] = __ldg(nbf[f] + ob);
						}
#pragma unroll
					for (int f = 0; f < SF; f++) {
						uint32_t const abase = c_abase[cj[f]];
						uint32_t const inc   = c_inc[cj[f]];
						float const w        = c_w[cj[f]];
#pragma unroll
						for (int u = 0; u < U; u++) {
							if (o + u * G >= nbw) break;  // warp-uniform
							int const ob = o + u * G + gl;
							// targets [cl, ch) of this block belong to the sub-row; none when ob >= nbk
							int const cl     = lo[f] - 4 * ob, ch = hi[f] - 4 * ob;
							unsigned const m = (0xFu << max(cl, 0)) & (0xFu >> min(max(4 - ch, 0), 4));
							int const d[4]   = {v[f][u].x, v[f][u].y, v[f][u].z, v[f][u].w};
#pragma unroll
							for (int c = 0; c < 4; c++)
								if (m & (1u << c)) {
									uint32_t const addr = abase + (uint32_t)d[c] * mul;
									if (MODE == 0) asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(addr), "r"(inc) : "memory");
									else asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(addr), "f"(w) : "memory");
								}
						}
					}
				}
			}
			__syncthreads();
		}
	}
	__syncthreads();
	bool const touched = s_touched != 0;
	add_events(a.events, my_events, &ev_block);
	if (!touched) return;
	flush_tile<MODE>(a, P, tbase, words, sigma, tile_sm);
}

// Stores a finished tile like flush_tile; when the ring slot is overwritten by this CTA alone and
// both ends are 16-byte aligned, in 16-byte vectors (TMA: as bulk asynchronous copies).
template <int MODE, bool TMA, class A>
__device__ __forceinline__ void flush_tile_vec(A const& a, PopDev const& P, int tbase, int words, int64_t sigma,
                                               const uint32_t* tile_sm) {
	int64_t const slot = sigma % a.D;
	uint32_t* dst      = MODE == 0 ? P.cnt + (slot * P.size + tbase) * P.W
	                               : reinterpret_cast<uint32_t*>(P.acc + (slot * P.size + tbase) * P.F);
	if (a.parts == 1 && !P.zero_inputs && (words & 3) == 0 && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
		if (TMA) {
			// bulk copies by the tensor-memory-access unit: the first lane of up to 8 warps each copies
			// a 16-byte-aligned share, after a proxy fence that orders the CTA's shared-memory adds
			// (generic proxy) before the copies' reads (async proxy); each issuer waits for its writes
			int const nw     = min(8, (int)(blockDim.x >> 5));
			int const w      = threadIdx.x >> 5;
			int const blocks = words >> 2;  // 16-byte blocks of the tile
			int const per    = (blocks + nw - 1) / nw;
			if ((threadIdx.x & 31) == 0 && w < nw) {
				int const b0 = w * per, b1 = min(blocks, b0 + per);
				if (b0 < b1) {
					asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
					for (int c = b0; c < b1; c += 1024) {  // copies of at most 16 KiB
						uint32_t const src = (uint32_t)__cvta_generic_to_shared(tile_sm + 4 * c);
						asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
						             ::"l"(dst + 4 * c), "r"(src), "r"((uint32_t)(min(b1, c + 1024) - c) * 16u) : "memory");
					}
					asm volatile("cp.async.bulk.commit_group;" ::: "memory");
					asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
				}
			}
			return;
		}
		uint4* d4       = reinterpret_cast<uint4*>(dst);
		const uint4* s4 = reinterpret_cast<const uint4*>(tile_sm);
		for (int i = threadIdx.x; i < (words >> 2); i += blockDim.x) d4[i] = s4[i];
		return;
	}
	flush_tile<MODE>(a, P, tbase, words, sigma, tile_sm);
}

// Row mapping (algo 14): as deliver_staged_vec with one sub-row per 4-lane group and 8 blocks per
// lane, with everything a group needs per sub-row precomputed while staging -- the pointer to its
// first 16-byte block, its target range within the blocks, and the connection's shared-memory base
// and increment -- so the fetch loop is a few shared loads, 8 loads at immediate offsets from one
// pointer, and per target one compare, one multiply-add and one shared-memory reduction.
constexpr int kStageR = 2048;

template <int MODE, class A>
__device__ __forceinline__ void deliver_rows(A const& a, PopDev const& P, int t, int si, int part) {
	constexpr int G = 4, U = 8;
	extern __shared__ uint32_t tile_sm[];
	__shared__ unsigned long long ev_block;
	__shared__ const int4* st_ptr[kStageR];
	__shared__ uint32_t st_lohi[kStageR];  // lo (2 bits) | hi << 2: targets [lo, hi) of the blocks from st_ptr
	__shared__ uint2 st_ai[kStageR];       // shared-memory base of the connection's word, increment (or weight bits)
	__shared__ int c_pre[kConnBatch + 1];
	__shared__ const int32_t* c_lst[kConnBatch];
	__shared__ const int64_t* c_bnd[kConnBatch];
	__shared__ const int4* c_nb[kConnBatch];
	__shared__ uint2 c_ai[kConnBatch];
	__shared__ int s_nc, s_touched, s_next;
	int const tbase = t * P.tile;
	int const tn    = (int)min((int64_t)P.tile, P.size - tbase);
	int const width = MODE == 0 ? P.W : P.F;
	int const words = tn * width;
	int const lane  = threadIdx.x & 31;
	int64_t const sigma = a.slot_lo + si;
	int const stride    = P.ntiles + 1;
	int const gl        = threadIdx.x & (G - 1);
	uint32_t const tile_addr = (uint32_t)__cvta_generic_to_shared(tile_sm);
	uint32_t const mul       = 4u * (uint32_t)width;
	if (threadIdx.x == 0) {
		ev_block  = 0;
		s_touched = 0;
	}
	bool zeroed = false;
	unsigned long long my_events = 0;
	for (int cb = P.in_begin; cb < P.in_end; cb += kConnBatch) {
		__syncthreads();
		if (threadIdx.x < 32) {  // warp 0: one lane per connection of the batch
			int const ci = cb + lane;
			int n = 0;
			bool reach = false;
			const int32_t* lst = nullptr;
			const int4* nbp    = nullptr;
			const int64_t* bnp = nullptr;
			uint2 ai           = make_uint2(0u, 0u);
			if (lane < kConnBatch && ci < P.in_end) {
				ConnDev const& C = a.conns[ci];
				int64_t const k  = sigma - (a.t0 + C.delay - 1);
				if (k >= 0 && k < a.K && !C.plastic) {
					int const cnt = a.counts[k * a.npop + C.src];
					int const pp  = (cnt + a.parts - 1) / a.parts;
					int const lo  = min(cnt, part * pp);
					reach         = true;
					n             = min(cnt, lo + pp) - lo;
					lst           = C.src_list + (a.list_k0 + k) * C.src_size + lo;
					nbp           = reinterpret_cast<const int4*>(C.nb);
					bnp           = C.bounds + t;
					ai.x          = tile_addr + 4u * (uint32_t)((MODE == 0 ? C.word : C.fslot) - tbase * width);
					ai.y          = MODE == 0 ? C.inc : __float_as_uint(C.weight);
				}
			}
			unsigned const rm = __ballot_sync(0xffffffffu, reach);
			int incl          = n;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				int const o = __shfl_up_sync(0xffffffffu, incl, d);
				if (lane >= d) incl += o;
			}
			int const tot = __shfl_sync(0xffffffffu, incl, 31);
			if (reach) {
				int const j = __popc(rm & lanemask_lt());
				c_pre[j]    = incl - n;
				c_lst[j]    = lst;
				c_nb[j]     = nbp;
				c_bnd[j]    = bnp;
				c_ai[j]     = ai;
				s_touched   = 1;
			}
			if (lane == 0) {
				s_nc              = __popc(rm);
				c_pre[__popc(rm)] = tot;
			}
			if (blockDim.x == 32 && !zeroed)
				for (int i = lane; i < words; i += 32) tile_sm[i] = 0;
		} else if (!zeroed) {  // the other warps clear the tile meanwhile (16-byte stores, then the rest)
			uint4* t4 = reinterpret_cast<uint4*>(tile_sm);
			for (int i = threadIdx.x - 32; i < (words >> 2); i += blockDim.x - 32) t4[i] = make_uint4(0u, 0u, 0u, 0u);
			for (int i = (words & ~3) + threadIdx.x - 32; i < words; i += blockDim.x - 32) tile_sm[i] = 0;
		}
		zeroed = true;
		__syncthreads();
		int const nc    = s_nc;
		int const total = c_pre[nc];
		for (int c0 = 0; c0 < total; c0 += kStageR) {
			int const m = min(kStageR, total - c0);
			for (int q = threadIdx.x; q < m; q += blockDim.x) {
				int const g = c0 + q;
				int j       = 0;
				while (j + 1 < nc && c_pre[j + 1] <= g) j++;
				const int64_t* bb = c_bnd[j] + (int64_t)__ldg(c_lst[j] + (g - c_pre[j])) * stride;
				int64_t const b0  = __ldg(bb);
				int const len     = (int)(__ldg(bb + 1) - b0);
				st_ptr[q]         = c_nb[j] + (b0 >> 2);
				st_lohi[q]        = (uint32_t)(b0 & 3) | ((uint32_t)((int)(b0 & 3) + len) << 2);
				st_ai[q]          = c_ai[j];
			}
			if (threadIdx.x == 0) s_next = 0;
			__syncthreads();
			while (true) {  // a warp takes 8 consecutive sub-rows per fetch, one per 4-lane group
				int base = 0;
				if (lane == 0) base = atomicAdd(&s_next, 32 / G);
				base = __shfl_sync(0xffffffffu, base, 0);
				if (base >= m) break;
				int const q      = base + lane / G;
				bool const ok    = q < m;
				const int4* p    = ok ? st_ptr[q] : nullptr;
				uint32_t const lh = ok ? st_lohi[q] : 0u;
				uint2 const ai   = ok ? st_ai[q] : make_uint2(0u, 0u);
				int const lo     = (int)(lh & 3u), hi = (int)(lh >> 2);
				int const nb     = hi > lo ? (hi + 3) >> 2 : 0;  // 16-byte blocks of the sub-row
				if (gl == 0) my_events += (unsigned long long)(hi - lo);
				int const nbw = __reduce_max_sync(0xffffffffu, nb);
				for (int o = 0; o < nbw; o += G * U) {
					const int4* pb = p + (o + gl);
					int const lim  = nb - (o + gl);       // this lane's block u exists iff 4u < lim
					int const hr   = hi - 4 * (o + gl);   // target 16u + c of this lane is in the sub-row iff < hr
					int const lr   = lo - 4 * (o + gl);   // ... and, in block u = 0, iff c >= lr
					int4 v[U];
#pragma unroll
					for (int u = 0; u < U; u++)
						if (4 * u < lim) v[u] = __ldg(pb + 4 * u);
#pragma unroll
					for (int u = 0; u < U; u++) {
						if (o + 4 * u >= nbw) break;  // warp-uniform
						int const d[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
						for (int c = 0; c < 4; c++)
							if (16 * u + c < hr && (u > 0 || c >= lr)) {
								uint32_t const addr = ai.x + (uint32_t)d[c] * mul;
								if (MODE == 0) asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(addr), "r"(ai.y) : "memory");
								else asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(addr), "f"(__uint_as_float(ai.y)) : "memory");
							}
					}
				}
			}
			__syncthreads();
		}
	}
	__syncthreads();
	bool const touched = s_touched != 0;
	add_events(a.events, my_events, &ev_block);
	if (!touched) return;
	flush_tile_vec<MODE, false>(a, P, tbase, words, sigma, tile_sm);
}

// Compact-target row mapping (algos 15 .. 17): deliver_rows reading the 16-bit tile-local copy of
// the targets (ConnDev::nb16), so a sub-row costs half the bytes: one 16-byte block holds 8 targets,
// a group of 4 lanes takes SF sub-rows per fetch and covers 32 U targets of each per load round trip
// (all SF sub-rows' loads in flight together), and a target's shared-memory address is the
// connection's base plus index times the words per neuron.
template <int MODE, int SF, int U, bool TMA, int STAGE = kStageR, class A>
__device__ __forceinline__ void deliver_rows16(A const& a, PopDev const& P, int t, int si, int part) {
	constexpr int G = 4;
	extern __shared__ uint32_t tile_sm[];
	__shared__ unsigned long long ev_block;
	__shared__ const int4* st_ptr[STAGE];
	__shared__ uint32_t st_lohi[STAGE];  // lo (3 bits) | hi << 3: targets [lo, hi) of the blocks from st_ptr
	__shared__ uint2 st_ai[STAGE];       // shared-memory address of the connection's word of index 0, increment
	__shared__ int c_pre[kConnBatch + 1];
	__shared__ const int32_t* c_lst[kConnBatch];
	__shared__ const int64_t* c_bnd[kConnBatch];
	__shared__ const int4* c_nb[kConnBatch];
	__shared__ uint2 c_ai[kConnBatch];
	__shared__ int s_nc, s_touched, s_next;
	int const tbase = t * P.tile;
	int const tn    = (int)min((int64_t)P.tile, P.size - tbase);
	int const width = MODE == 0 ? P.W : P.F;
	int const words = tn * width;
	int const lane  = threadIdx.x & 31;
	int64_t const sigma = a.slot_lo + si;
	int const stride    = P.ntiles + 1;
	int const gl        = threadIdx.x & (G - 1);
	uint32_t const tile_addr = (uint32_t)__cvta_generic_to_shared(tile_sm);
	uint32_t const mul       = 4u * (uint32_t)width;
	if (threadIdx.x == 0) {
		ev_block  = 0;
		s_touched = 0;
	}
	bool zeroed = false;
	unsigned long long my_events = 0;
	for (int cb = P.in_begin; cb < P.in_end; cb += kConnBatch) {
		__syncthreads();
		if (threadIdx.x < 32) {  // warp 0: one lane per connection of the batch
			int const ci = cb + lane;
			int n = 0;
			bool reach = false;
			const int32_t* lst = nullptr;
			const int4* nbp    = nullptr;
			const int64_t* bnp = nullptr;
			uint2 ai           = make_uint2(0u, 0u);
			int64_t k = -1;
			int src = 0;
			if (lane < kConnBatch && ci < P.in_end) {  // the connection's fixed fields
				// every field is loaded before the reach test, so that all the loads are one round trip
				ConnDev const& C        = a.conns[ci];
				int const delay         = C.delay;
				int const plastic       = C.plastic;
				int const csrc          = C.src;
				const int32_t* const sl = C.src_list;
				int64_t const ssize     = C.src_size;
				const uint16_t* const n16 = C.nb16;
				const int64_t* const bd = C.bounds;
				int const wsel          = MODE == 0 ? C.word : C.fslot;
				uint32_t const incw     = MODE == 0 ? C.inc : __float_as_uint(C.weight);
				k = sigma - (a.t0 + delay - 1);
				if (k >= 0 && k < a.K && !plastic) {
					reach = true;
					src   = csrc;
					lst   = sl + (a.list_k0 + k) * ssize;
					nbp   = reinterpret_cast<const int4*>(n16);
					bnp   = bd + t;
					ai.x  = tile_addr + 4u * (uint32_t)wsel;
					ai.y  = incw;
				}
			}
			if (cb == P.in_begin) {  // spike counts and lists: the previous launch's output
				griddep_wait();
				griddep_launch();
			}
			if (reach) {
				int const cnt = a.counts[k * a.npop + src];
				int const pp  = (cnt + a.parts - 1) / a.parts;
				int const lo  = min(cnt, part * pp);
				n             = min(cnt, lo + pp) - lo;
				lst += lo;
			}
			unsigned const rm = __ballot_sync(0xffffffffu, reach);
			int incl          = n;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				int const o = __shfl_up_sync(0xffffffffu, incl, d);
				if (lane >= d) incl += o;
			}
			int const tot = __shfl_sync(0xffffffffu, incl, 31);
			if (reach) {
				int const j = __popc(rm & lanemask_lt());
				c_pre[j]    = incl - n;
				c_lst[j]    = lst;
				c_nb[j]     = nbp;
				c_bnd[j]    = bnp;
				c_ai[j]     = ai;
				s_touched   = 1;
			}
			if (lane == 0) {
				s_nc              = __popc(rm);
				c_pre[__popc(rm)] = tot;
			}
			if (blockDim.x == 32 && !zeroed)
				for (int i = lane; i < words; i += 32) tile_sm[i] = 0;
		} else if (!zeroed) {
			uint4* t4 = reinterpret_cast<uint4*>(tile_sm);
			for (int i = threadIdx.x - 32; i < (words >> 2); i += blockDim.x - 32) t4[i] = make_uint4(0u, 0u, 0u, 0u);
			for (int i = (words & ~3) + threadIdx.x - 32; i < words; i += blockDim.x - 32) tile_sm[i] = 0;
			griddep_wait();
			griddep_launch();
		}
		zeroed = true;
		__syncthreads();
		int const nc    = s_nc;
		int const total = c_pre[nc];
		for (int c0 = 0; c0 < total; c0 += STAGE) {
			int const m = min(STAGE, total - c0);
			// A thread stages up to R sub-rows per pass with all their loads in flight together: the
			// R spike-list loads, then the 2 R bound loads that depend on them -- two load round trips
			// per pass (one pass when STAGE <= R * blockDim.x) instead of two per sub-row.
			constexpr int R = STAGE > 1024 ? 3 : 2;
			for (int q0 = threadIdx.x; q0 < m; q0 += R * blockDim.x) {
				int jr[R];
				int32_t sr[R];
#pragma unroll
				for (int r = 0; r < R; r++) {
					int const q = q0 + r * (int)blockDim.x;
					int j       = 0;
					sr[r]       = 0;
					if (q < m) {
						int const g = c0 + q;
						while (j + 1 < nc && c_pre[j + 1] <= g) j++;
						sr[r] = __ldg(c_lst[j] + (g - c_pre[j]));
					}
					jr[r] = j;
				}
				int64_t b0[R], b1[R];
#pragma unroll
				for (int r = 0; r < R; r++) {
					b0[r] = b1[r] = 0;
					if (q0 + r * (int)blockDim.x < m) {
						const int64_t* bb = c_bnd[jr[r]] + (int64_t)sr[r] * stride;
						b0[r]             = __ldg(bb);
						b1[r]             = __ldg(bb + 1);
					}
				}
#pragma unroll
				for (int r = 0; r < R; r++) {
					int const q = q0 + r * (int)blockDim.x;
					if (q < m) {
						int const len = (int)(b1[r] - b0[r]);
						st_ptr[q]     = c_nb[jr[r]] + (b0[r] >> 3);
						st_lohi[q]    = (uint32_t)(b0[r] & 7) | ((uint32_t)((int)(b0[r] & 7) + len) << 3);
						st_ai[q]      = c_ai[jr[r]];
					}
				}
			}
			if (threadIdx.x == 0) s_next = 0;
			__syncthreads();
			while (true) {  // a warp takes 8 SF consecutive sub-rows per fetch, SF per 4-lane group
				int base = 0;
				if (lane == 0) base = atomicAdd(&s_next, 32 / G * SF);
				base = __shfl_sync(0xffffffffu, base, 0);
				if (base >= m) break;
				const int4* p[SF];
				uint2 ai[SF];
				int lo[SF], hi[SF], nb[SF];
				int nbw = 0;
#pragma unroll
				for (int f = 0; f < SF; f++) {
					int const q       = base + (lane / G) * SF + f;
					bool const ok     = q < m;
					p[f]              = ok ? st_ptr[q] : nullptr;
					uint32_t const lh = ok ? st_lohi[q] : 0u;
					ai[f]             = ok ? st_ai[q] : make_uint2(0u, 0u);
					lo[f]             = (int)(lh & 7u);
					hi[f]             = (int)(lh >> 3);
					nb[f]             = hi[f] > lo[f] ? (hi[f] + 7) >> 3 : 0;  // 16-byte blocks of the sub-row
					nbw               = max(nbw, nb[f]);
					if (gl == 0) my_events += (unsigned long long)(hi[f] - lo[f]);
				}
				nbw = __reduce_max_sync(0xffffffffu, nbw);
				for (int o = 0; o < nbw; o += G * U) {
					int4 v[SF][U];
#pragma unroll
					for (int f = 0; f < SF; f++) {
						const int4* pb = p[f] + (o + gl);
						int const lim  = nb[f] - (o + gl);  // this lane's block u exists iff 4u < lim
#pragma unroll
						for (int u = 0; u < U; u++)
							if (4 * u < lim) v[f][u] = __ldg(pb + 4 * u);
					}
#pragma unroll
					for (int f = 0; f < SF; f++) {
						int const hr = hi[f] - 8 * (o + gl);  // target 32u + c of this lane is in the sub-row iff < hr
						int const lr = lo[f] - 8 * (o + gl);  // ... and, in block u = 0, iff c >= lr
#pragma unroll
						for (int u = 0; u < U; u++) {
							if (o + 4 * u >= nbw) break;  // warp-uniform
							uint32_t const x[4] = {(uint32_t)v[f][u].x, (uint32_t)v[f][u].y, (uint32_t)v[f][u].z,
							                       (uint32_t)v[f][u].w};
#pragma unroll
							for (int c = 0; c < 8; c++)
								if (32 * u + c < hr && (u > 0 || c >= lr)) {
									uint32_t const d    = (c & 1) ? x[c >> 1] >> 16 : x[c >> 1] & 0xffffu;
									uint32_t const addr = ai[f].x + d * mul;
									if (MODE == 0) asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(addr), "r"(ai[f].y) : "memory");
									else asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(addr), "f"(__uint_as_float(ai[f].y)) : "memory");
								}
						}
					}
				}
			}
			__syncthreads();
		}
	}
	__syncthreads();
	griddep_wait();  // (no-op when done above) the ring slot is read by the previous launch
	griddep_launch();
	bool const touched = s_touched != 0;
	add_events(a.events, my_events, &ev_block);
	if (!touched) return;
	flush_tile_vec<MODE, TMA>(a, P, tbase, words, sigma, tile_sm);
}

// Warp-per-spike mapping: a warp takes 32 spikes, loads their sub-row bounds lane-parallel, then
// streams 8 sub-rows at a time with lanes spanning each sub-row (coalesced loads, 8 in flight per
// lane, no cross-lane search).
template <int MODE, class A>
__device__ __forceinline__ void deliver_wps(A const& a, PopDev const& P, int t, int si, int part) {
	extern __shared__ uint32_t tile_sm[];
	__shared__ unsigned long long ev_block;
	int const tbase = t * P.tile;
	int const tn    = (int)min((int64_t)P.tile, P.size - tbase);
	int const width = MODE == 0 ? P.W : P.F;
	int const words = tn * width;
	for (int i = threadIdx.x; i < words; i += blockDim.x) tile_sm[i] = 0;
	if (threadIdx.x == 0) ev_block = 0;
	__syncthreads();
	int64_t const sigma = a.slot_lo + si;
	int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
	unsigned long long my_events = 0;
	bool touched = false;
	for (int ci = P.in_begin; ci < P.in_end; ci++) {
		ConnDev const& C = a.conns[ci];
		int64_t const k  = sigma - (a.t0 + C.delay - 1);
		if (k < 0 || k >= a.K || C.plastic) continue;
		touched = true;
		int const n        = a.counts[k * a.npop + C.src];
		const int32_t* lst = C.src_list + (a.list_k0 + k) * C.src_size;
		const int64_t* bnd = C.bounds + t;
		int const stride   = P.ntiles + 1;
		const int32_t* nb  = C.nb;
		int const word     = MODE == 0 ? C.word : C.fslot;
		uint32_t const inc = C.inc;
		float const w      = C.weight;
		for (int j0 = (part * nwarps + warp) * 32; j0 < n; j0 += a.parts * nwarps * 32) {
			int64_t start = 0;
			int len       = 0;
			if (j0 + lane < n) {
				int const s       = __ldg(lst + j0 + lane);
				const int64_t* bb = bnd + (int64_t)s * stride;
				start             = __ldg(bb);
				len               = (int)(__ldg(bb + 1) - start);
			}
			my_events += (unsigned long long)len;
			int const nq = min(32, n - j0);
			for (int q0 = 0; q0 < nq; q0 += 8) {
				int32_t d[8];
#pragma unroll
				for (int u = 0; u < 8; u++) {
					int64_t const st = __shfl_sync(0xffffffffu, start, (q0 + u) & 31);
					int const ln     = __shfl_sync(0xffffffffu, len, (q0 + u) & 31);
					d[u]             = (q0 + u < nq && lane < ln) ? __ldg(nb + st + lane) : -1;
				}
#pragma unroll
				for (int u = 0; u < 8; u++)
					if (d[u] >= 0) {
						int const li = (d[u] - tbase) * width + word;
						if (MODE == 0) atomicAdd(tile_sm + li, inc);
						else atomicAdd(reinterpret_cast<float*>(tile_sm) + li, w);
					}
				// sub-rows longer than a warp (large tiles): the rest, spike by spike
#pragma unroll 1
				for (int u = 0; u < 8; u++) {
					int64_t const st = __shfl_sync(0xffffffffu, start, (q0 + u) & 31);
					int const ln     = __shfl_sync(0xffffffffu, len, (q0 + u) & 31);
					if (q0 + u >= nq || ln <= 32) continue;
					for (int e = 32 + lane; e < ln; e += 32) {
						int const li = (__ldg(nb + st + e) - tbase) * width + word;
						if (MODE == 0) atomicAdd(tile_sm + li, inc);
						else atomicAdd(reinterpret_cast<float*>(tile_sm) + li, w);
					}
				}
			}
		}
	}
	add_events(a.events, my_events, &ev_block);
	if (!touched) return;
	flush_tile<MODE>(a, P, tbase, words, sigma, tile_sm);
}

__device__ __forceinline__ void span_begin(DeliverArgs const& a) { span_open(a.span); }
__device__ __forceinline__ void span_end(DeliverArgs const& a) { span_close(a.span); }

// Plain-net delivery kernels: block -> (part, slot si, tile g over all target populations).
struct DeliverItem {
	int part, si, Q, t;
};
// The spike counts of the other parity (fully delivered) are cleared for the window after next.
__device__ __forceinline__ void clear_counts_next(DeliverArgs const& a) {
	if (blockIdx.x == 0)
		for (int j = threadIdx.x; j < a.counts_next_len; j += blockDim.x) a.counts_next[j] = 0;
}

// The work item of a plain delivery CTA.  WAIT: wait for the previous launch (and clear the other
// parity's counts) first; otherwise the caller waits, releases the dependents and clears the counts
// once its independent prologue is done.
// The dependents are released only after the wait: the next window's grid reads the neuron state
// of this window's neuron update (complete once this launch has waited for it) before it waits.
template <bool WAIT = true>
__device__ __forceinline__ DeliverItem deliver_item(DeliverArgs const& a) {
	if (WAIT) {
		griddep_wait();
		griddep_launch();
	}
	DeliverItem it;
	it.part    = blockIdx.x % a.parts;
	int const b = blockIdx.x / a.parts;
	it.si      = b / a.ntiles_total;
	int const g = b - it.si * a.ntiles_total;
	int Q       = 0;
	while (Q + 1 < a.npop && g >= a.tile_begin[Q + 1]) Q++;
	it.Q = Q;
	it.t = g - a.tile_begin[Q];
	if (WAIT) clear_counts_next(a);
	return it;
}

template <int MODE>
__global__ void __launch_bounds__(1024) k_deliver(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item(a);
	deliver_flat<MODE>(a, a.pops[it.Q], it.t, it.si, it.part);
	span_end(a);
}

template <int MODE, bool VEC>
__global__ void k_deliver_tps(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item(a);
	deliver_tps<MODE, VEC>(a, a.pops[it.Q], it.t, it.si, it.part);
	span_end(a);
}

template <int MODE>
__global__ void k_deliver_pipe(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item(a);
	deliver_tps_pipe<MODE>(a, a.pops[it.Q], it.t, it.si, it.part);
	span_end(a);
}

template <int MODE, int G>
__global__ void k_deliver_groups(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item(a);
	deliver_groups<MODE, G>(a, a.pops[it.Q], it.t, it.si, it.part);
	span_end(a);
}

template <int MODE, int SF>
__global__ void k_deliver_staged(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item(a);
	deliver_staged<MODE, SF>(a, a.pops[it.Q], it.t, it.si, it.part);
	span_end(a);
}

template <int MODE, int SF, int U>
__global__ void __launch_bounds__(SF > 2 || SF * U > 8 ? 768 : 1024, 1) k_deliver_staged_vec(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item(a);
	deliver_staged_vec<MODE, SF, U>(a, a.pops[it.Q], it.t, it.si, it.part);
	span_end(a);
}

template <int MODE>
__global__ void __launch_bounds__(1024, 1) k_deliver_rows(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item(a);
	deliver_rows<MODE>(a, a.pops[it.Q], it.t, it.si, it.part);
	span_end(a);
}

template <int MODE, int SF, int U, bool TMA>
__global__ void __launch_bounds__(SF > 1 ? 768 : 1024, 1) k_deliver_rows16(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item<false>(a);  // deliver_rows16 waits after its prologue
	deliver_rows16<MODE, SF, U, TMA>(a, a.pops[it.Q], it.t, it.si, it.part);
	clear_counts_next(a);
	span_end(a);
}

// The compact-target row mapping at two 512-thread CTAs per SM (at most 64 registers, 1024 staged
// sub-rows): one CTA's staging, barriers and flush overlap the other's reductions.
template <int MODE, int SF, int U>
__global__ void __launch_bounds__(512, 2) k_deliver_rows16_occ(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item<false>(a);
	deliver_rows16<MODE, SF, U, false, 1024>(a, a.pops[it.Q], it.t, it.si, it.part);
	clear_counts_next(a);
	span_end(a);
}

// The 4-lane mapping with at most 32 registers per thread: four 512-thread CTAs (all 64 warps)
// resident per SM, for windows whose (slot, tile) items fit one wave at that occupancy.
template <int MODE>
__global__ void __launch_bounds__(512, 4) k_deliver_groups_occ(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item(a);
	deliver_groups<MODE, 4>(a, a.pops[it.Q], it.t, it.si, it.part);
	span_end(a);
}

template <int MODE>
__global__ void __launch_bounds__(1024) k_deliver_wps(const __grid_constant__ DeliverArgs a) {
	span_begin(a);
	DeliverItem const it = deliver_item(a);
	deliver_wps<MODE>(a, a.pops[it.Q], it.t, it.si, it.part);
	span_end(a);
}

// Targets as indices within their delivery tile (tile <= 65536 neurons), in CSR order.
__global__ void k_compact_targets(const int32_t* __restrict__ nb, int64_t synapses, int tile, uint16_t* __restrict__ nb16) {
	for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < synapses; e += (int64_t)gridDim.x * blockDim.x)
		nb16[e] = (uint16_t)(nb[e] % tile);
}

__global__ void k_tile_bounds(const int64_t* __restrict__ off, const int32_t* __restrict__ nb, int64_t rows, int tile,
                              int ntiles, int64_t* __restrict__ bounds) {
	int64_t const r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (r >= rows) return;
	int64_t pos       = off[r];
	int64_t const end = off[r + 1];
	int64_t* out = bounds + r * (ntiles + 1);
	for (int t = 0; t <= ntiles; t++) {
		int64_t const lim = (int64_t)t * tile;
		while (pos < end && nb[pos] < lim) pos++;
		out[t] = t == ntiles ? end : pos;
	}
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

// Per step t: the states T^i(seed_t), i < 128, then for each of the 16 bytes of a jump polynomial
// the XOR of every subset of the byte's 8 states: tables[t][g][m] = XOR_{q: bit q of m} T^(8g+q)(s).
__global__ void k_jump_tables(const u128* __restrict__ seeds, int64_t nsteps, u128* __restrict__ tables) {
	__shared__ u128 basis[kBasis];
	int64_t const t = blockIdx.x;
	if (t >= nsteps) return;
	if (threadIdx.x == 0) {
		uint64_t s0 = seeds[t].lo, s1 = seeds[t].hi;
		for (int i = 0; i < kBasis; i++) {
			basis[i] = {s0, s1};
			xoro_next(s0, s1);
		}
	}
	__syncthreads();
	u128* out = tables + t * kJumpTable;
	for (int e = threadIdx.x; e < kJumpTable; e += blockDim.x) {
		int const g = e >> 8, m = e & 255;
		uint64_t lo = 0, hi = 0;
#pragma unroll
		for (int q = 0; q < 8; q++)
			if ((m >> q) & 1) {
				lo ^= basis[8 * g + q].lo;
				hi ^= basis[8 * g + q].hi;
			}
		out[e] = {lo, hi};
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

// One (step, population) pair of a window's raster (block b of the window's K npop raster blocks).
__device__ void raster_block(RasterArgs const& a, int b) {
	__shared__ int64_t off;
	int const k = b / a.npop, p = b % a.npop;
	PopDev const& P = a.pops[p];
	if (threadIdx.x == 0) {
		int64_t o = a.base[a.parity];
		for (int j = 0; j < k * a.npop + p; j++) o += a.counts[j];
		off = o;
		a.step_counts[(a.row0 + k) * a.npop + p] = a.counts[k * a.npop + p];
		if (b == 0) {  // where the next window's raster starts
			int64_t tot = 0;
			for (int j = 0; j < a.K * a.npop; j++) tot += a.counts[j];
			a.base[a.parity ^ 1] = a.base[a.parity] + tot;
		}
	}
	// each warp extracts a contiguous range of bitmap words: counts first, one block-wide prefix over
	// the warps, then warp-level scans only
	__shared__ int64_t warp_cnt[32];
	const uint32_t* bits = P.bits + ((a.t0 + k) % a.Hb) * P.nwords;
	int const lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
	int const per  = (P.nwords + nw - 1) / nw;
	int const w0 = min(P.nwords, w * per), w1 = min(P.nwords, w0 + per);
	int c = 0;
	for (int i = w0 + lane; i < w1; i += 32) c += __popc(bits[i]);
	for (int d = 16; d; d >>= 1) c += __shfl_xor_sync(0xffffffffu, c, d);
	if (lane == 0) warp_cnt[w] = c;
	__syncthreads();
	int64_t pos = off;
	for (int j = 0; j < w; j++) pos += warp_cnt[j];
	for (int i0 = w0; i0 < w1; i0 += 32) {
		int const i      = i0 + lane;
		uint32_t const m = i < w1 ? bits[i] : 0u;
		int const pc     = __popc(m);
		int incl         = pc;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			int const o = __shfl_up_sync(0xffffffffu, incl, d);
			if (lane >= d) incl += o;
		}
		int64_t p2 = pos + incl - pc;
		uint32_t mm = m;
		while (mm) {
			int const r = __ffs(mm) - 1;
			mm &= mm - 1;
			if (p2 < a.capacity) a.out[p2] = 32 * i + r;
			p2++;
		}
		pos += __shfl_sync(0xffffffffu, incl, 31);
	}
}

__global__ void k_raster(const __grid_constant__ RasterArgs a) {
	griddep_wait();
	griddep_launch();
	raster_block(a, (int)blockIdx.x);
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


// ---------------------------------------------------------------------------------------------
// Plastic synapses: the lazy per-synapse catch-up of synapse_population::_update
// (synapse_population.h:82-140).  A synapse's state is current as of the step recorded in its
// source's `ages` word; at each delivery of the source's spike and every 64 steps it replays the
// steps since: the pending pre update of the last delivery (bit 63), then every post spike in
// the target's 64-step history with skip() over the quiet steps between them.
// ---------------------------------------------------------------------------------------------

struct SynState {
	float W, A, B;
};

// iSTDP (Vogels et al. 2011) and the counting model of the reference's tests.
__device__ __forceinline__ void syn_update(ConnDev const& C, SynState& s, bool pre, bool post) {
	if (C.plastic == SPICE_SYNAPSE_COUNT) {
		s.W = __fadd_rn(s.W, 1.0f);
		return;
	}
	if (pre) {
		float const w = __fadd_rn(s.W, __fmul_rn(C.eta, __fsub_rn(s.B, C.alpha)));
		s.W           = w > 0.0f ? w : 0.0f;
	}
	if (post) s.W = __fadd_rn(s.W, __fmul_rn(C.eta, s.A));
	s.A = __fadd_rn(s.A, pre ? 1.0f : 0.0f);
	s.B = __fadd_rn(s.B, post ? 1.0f : 0.0f);
	s.A = __fsub_rn(s.A, __fmul_rn(s.A, C.cdt));
	s.B = __fsub_rn(s.B, __fmul_rn(s.B, C.cdt));
}

// skip(n): the traces decay by (1 - dt/tau)^n, a double, each trace rounded back to float
// (synapse_population.h:118-139); mul_f32_f64_rn gives the bits of that double multiply without
// the FP64 pipe (the traces are never negative).
__device__ __forceinline__ void syn_skip(ConnDev const& C, SynState& s, int64_t n) {
	if (C.plastic == SPICE_SYNAPSE_COUNT) {
		s.W = __fadd_rn(s.W, (float)n);
		return;
	}
	uint64_t const f = __ldg(C.skip_pk + (n + 64));
	s.A              = mul_f32_f64_rn(s.A, f);
	s.B              = mul_f32_f64_rn(s.B, f);
}

// The catch-up of one edge to step `time` (synapse_population.h:88-116).  The reference computes
// ~0 >> prefix with prefix up to 64 (pre set and time == age); x86-64 shifts by prefix mod 64, and
// that is what is computed here.
__device__ __forceinline__ void catch_up(ConnDev const& C, SynState& s, int64_t time, uint64_t ages, uint64_t hist) {
	int const pre     = (int)(ages >> 63);
	int64_t const age = (int64_t)(ages & ~(1ull << 63));
	if (!(time >= age)) return;
	int64_t const prefix = 63 + pre - time + age;
	uint64_t const mask  = ~0ull >> (prefix & 63);
	if (pre) syn_update(C, s, true, (hist & (1ull << ((time - age) & 63))) != 0);
	hist &= mask;
	int64_t p = prefix;
	while (hist) {
		int const lz = __clzll((long long)hist);
		syn_skip(C, s, lz - p);
		syn_update(C, s, false, true);
		hist ^= 1ull << (63 - lz);
		p = lz + 1;
	}
	syn_skip(C, s, 64 - p);
}

// The catch-up of synapses [e0, e1) of one plastic row to step `time` and, with `deliver`, their
// weights into ring slot `slot`: lanes take every 32nd synapse, four at a time with their loads in
// flight together (the per-synapse body of k_plastic_deliver / k_plastic_update_all).
__device__ __forceinline__ void plastic_row_chunk(ConnDev const& C, int64_t e0, int64_t e1, int64_t time, uint64_t ages,
                                                  int64_t slot, bool deliver, int lane) {
	constexpr int U = 4;
	for (int64_t eb = e0 + lane; eb < e1; eb += 32 * U) {
		SynState st[U];
		int32_t j[U];
		uint64_t h[U];
#pragma unroll
		for (int u = 0; u < U; u++) {
			int64_t const e = eb + 32 * u;
			if (e < e1) {
				st[u] = SynState{C.sW[e], C.sA[e], C.sB[e]};
				j[u]  = C.nb[e];
			}
		}
#pragma unroll
		for (int u = 0; u < U; u++)
			if (eb + 32 * u < e1) h[u] = C.dst_hist[j[u]];
#pragma unroll
		for (int u = 0; u < U; u++) {
			int64_t const e = eb + 32 * u;
			if (e >= e1) break;
			catch_up(C, st[u], time, ages, h[u]);
			C.sW[e] = st[u].W;
			C.sA[e] = st[u].A;
			C.sB[e] = st[u].B;
			if (deliver) {
				float const v = C.plastic == SPICE_SYNAPSE_COUNT ? __fmul_rn(C.weight, st[u].W) : st[u].W;
				red_add_f32(C.dst_acc + (slot * C.dst_size + j[u]) * C.F + C.fslot, v);
			}
		}
	}
}

// Every 64 steps (snn.cpp:17-19): every synapse of the connection catches up; a warp per source.
__global__ void __launch_bounds__(256) k_plastic_update_all(const __grid_constant__ ConnDev C, int64_t time) {
	int const lane = threadIdx.x & 31;
	int64_t const src = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
	if (src >= C.src_size) return;
	uint64_t const ages = C.ages[src];
	for (int64_t e = C.off[src] + lane; e < C.off[src + 1]; e += 32) {  // one synapse per lane at a time
		SynState st{C.sW[e], C.sA[e], C.sB[e]};                           // (more in flight lowered the
		catch_up(C, st, time, ages, C.dst_hist[C.nb[e]]);                  // occupancy and lost)
		C.sW[e] = st.W;
		C.sA[e] = st.A;
		C.sB[e] = st.B;
	}
	__syncwarp();
	if (lane == 0) C.ages[src] = (uint64_t)(time + 1);
}

// Delivery of the spikes of step time - delay + 1 through a plastic connection (synapse_population
// .h:82-140): CTA (w, c) takes chunk c (kPlasticChunk synapses, a thread each) of the row of every
// spiking source of bitmap word w: catch up, then deliver W into input ring slot `slot` (atomic-mode
// sums; COUNT with scale 0 and any model in deterministic mode deliver nothing).  Every chunk of a
// row catches up from the source's `ages` word as it was at launch; the row's last chunk to finish
// (a per-source counter) writes the new value.
constexpr int kPlasticChunk = 256;

__global__ void __launch_bounds__(kPlasticChunk) k_plastic_deliver(const __grid_constant__ ConnDev C, int64_t time,
                                                                   int hslot, int64_t slot, int deliver,
                                                                   unsigned long long* events) {
	int const w = blockIdx.x;
	uint32_t bits = C.src_bits[(int64_t)hslot * C.src_nwords + w];
	unsigned long long ev = 0;
	while (bits) {
		int const r       = __ffs(bits) - 1;
		bits &= bits - 1;
		int64_t const src = 32 * (int64_t)w + r;
		int64_t const e0 = C.off[src], e1 = C.off[src + 1];
		int64_t const nchunks = (e1 - e0 + kPlasticChunk - 1) / kPlasticChunk;
		if (blockIdx.y == 0 && threadIdx.x == 0) ev += (unsigned long long)(e1 - e0);
		for (int64_t c = blockIdx.y; c < nchunks; c += gridDim.y) {
		uint64_t const ages = C.ages[src];
		int64_t const e = e0 + c * kPlasticChunk + threadIdx.x;
		if (e < e1) {
			SynState st{C.sW[e], C.sA[e], C.sB[e]};
			int32_t const j = C.nb[e];
			catch_up(C, st, time, ages, C.dst_hist[j]);
			C.sW[e] = st.W;
			C.sA[e] = st.A;
			C.sB[e] = st.B;
			if (deliver) {
				float const v = C.plastic == SPICE_SYNAPSE_COUNT ? __fmul_rn(C.weight, st.W) : st.W;
				red_add_f32(C.dst_acc + (slot * C.dst_size + j) * C.F + C.fslot, v);
			}
		}
		__syncthreads();  // every thread of this chunk has read `ages`
		if (threadIdx.x == 0) {
			__threadfence();
			if (atomicAdd(C.chunks_done + src, 1u) == (uint32_t)(nchunks - 1)) {  // the row's last chunk
				C.ages[src]        = (uint64_t)(time + 1) | (1ull << 63);
				C.chunks_done[src] = 0;
			}
		}
		__syncthreads();
		}
	}
	if (threadIdx.x == 0 && ev) atomicAdd(events, ev);
}

// ---------------------------------------------------------------------------------------------
// Batched networks: the populations and connections of many independent nets (same dt, delay
// ring, window and time) are concatenated and one launch per kernel kind steps all of them.  The
// window's time-dependent values live in a device clock that k_batch_prologue advances, so every
// launch of a window has fixed arguments and a window (or several) can be replayed as a CUDA graph.
// ---------------------------------------------------------------------------------------------

// Largest p < n with begin[p] <= x (begin ascending; empty segments are skipped).
__device__ __forceinline__ int find_segment(const int* __restrict__ begin, int n, int x) {
	int lo = 0, hi = n - 1;
	while (lo < hi) {
		int const mid = (lo + hi + 1) >> 1;
		if (__ldg(begin + mid) <= x) lo = mid;
		else hi = mid - 1;
	}
	return lo;
}

__device__ __forceinline__ WinCtx batch_win_ctx(BatchArgs const& b, BatchClock const& c) {
	WinCtx w;
	w.K              = c.k;
	w.slot0          = (int)((c.t0 - 1 + b.D) % b.D);
	w.hslot0         = (int)(c.t0 % b.Hb);
	w.Hb             = b.Hb;
	w.npop           = b.npop;
	w.list_k0        = c.parity * b.K;
	w.D              = b.D;
	w.dts            = b.dts;
	w.tables         = b.tables;
	w.tab_net_stride = b.K;
	w.counts         = b.counts + (int64_t)c.parity * b.K * b.npop;
	return w;
}

// One CTA: advances the clock to the next window of k steps, computes the window's dt (Kahan, as
// kahan_next on the host: kahan_sum<float> then the reset at >= 1 s) and every net's step seeds
// (seed_seq post-increment, one per step), and clears this window's spike counters.
__global__ void k_batch_prologue(const __grid_constant__ BatchArgs b, int k) {
	BatchClock* clk    = b.clock;
	int64_t const t0   = clk->next_t0;
	int const parity   = clk->next_parity;
	__syncthreads();
	if (threadIdx.x == 0) {
		clk->t0          = t0;
		clk->parity      = parity;
		clk->k           = k;
		clk->next_t0     = t0 + k;
		clk->next_parity = parity ^ 1;
		float c = clk->kahan_c, sum = clk->kahan_sum;
		for (int j = 0; j < k; j++) {
			float const y = __fsub_rn(b.dt, c);
			float const t = __fadd_rn(sum, y);
			c             = __fsub_rn(__fsub_rn(t, sum), y);
			sum           = t >= 1.0f ? 0.0f : t;
			b.dts[j]      = y;
		}
		clk->kahan_c   = c;
		clk->kahan_sum = sum;
	}
	int32_t* counts = b.counts + (int64_t)parity * b.K * b.npop;
	for (int i = threadIdx.x; i < b.K * b.npop; i += blockDim.x) counts[i] = 0;
	for (int n = threadIdx.x; n < b.nnets; n += blockDim.x) {
		u128 s = b.seed_state[n];
		for (int j = 0; j < k; j++) {
			b.step_seeds[(int64_t)n * b.K + j] = s;
			s = murmur3_u128(s);
		}
		b.seed_state[n] = s;
	}
}

// Source populations of all nets: grid (Poisson chunk CTAs of one step, steps of the window).
__global__ void __launch_bounds__(kThreads) k_batch_sources(const __grid_constant__ BatchArgs b) {
	__shared__ int red[kThreads / 32 + 1];
	BatchClock const c = *b.clock;
	int const x   = blockIdx.x;
	int const p   = find_segment(b.sblk_begin, b.npop, x);
	int const bps = __ldg(b.sblk_begin + p + 1) - __ldg(b.sblk_begin + p);
	WinCtx const w = batch_win_ctx(b, c);
	window_poisson(w, b.pops + p, p, (int)blockIdx.y * bps + (x - __ldg(b.sblk_begin + p)), bps, red);
}

// Per-neuron populations of all nets, K steps each with the state in registers.
template <int MODE, bool ONLY_FAST>
__global__ void __launch_bounds__(kThreads, ONLY_FAST ? kNeuronBlocksPerSM : 1) k_batch_neurons(const __grid_constant__ BatchArgs b) {
	BatchClock const c = *b.clock;
	int const x        = blockIdx.x;
	int const p        = find_segment(b.nblk_begin, b.npop, x);
	int const lb       = x - __ldg(b.nblk_begin + p);
	WinCtx const w     = batch_win_ctx(b, c);
	__shared__ float dts_sm[kMaxWindow];
	__shared__ uint32_t xs_sm[MODE == 0 ? 16 : 1][kThreads];
	__shared__ uint32_t masks_sm[MODE == 0 ? kThreads / 32 : 1][16];
	for (int k = threadIdx.x; k < w.K; k += blockDim.x) dts_sm[k] = b.dts[k];
	__syncthreads();
	if (MODE == 0 && __ldg(b.nblk_kind + p) == 3) window_lif_deferred<false, false>(w, b.pops + p, p, lb, dts_sm, xs_sm, masks_sm);
	else if (MODE != 0 && __ldg(b.nblk_kind + p) == 3) window_neurons<MODE, true, false>(w, b.pops + p, p, lb);
	else if (!ONLY_FAST) window_neurons<MODE, false, false>(w, b.pops + p, p, lb);
}

// Delivery of all nets: grid (target tiles x parts, input slots of the window).
template <int MODE, int ALGO>
__global__ void k_batch_deliver(const __grid_constant__ BatchArgs b) {
	BatchClock const c = *b.clock;
	int const part     = blockIdx.x % b.parts;
	int const g        = blockIdx.x / b.parts;
	int const Q        = find_segment(b.tile_begin, b.npop, g);
	PopDev const& P    = b.pops[Q];
	DelCtx a;
	a.t0      = c.t0;
	a.D       = b.D;
	a.slot_lo = c.t0 + b.dmin - 1;
	a.K       = c.k;
	a.npop    = b.npop;
	a.list_k0 = c.parity * b.K;
	a.parts   = b.parts;
	a.conns   = b.conns;
	a.counts  = b.counts + (int64_t)c.parity * b.K * b.npop;
	a.events  = b.net_events[P.net];
	int const t = g - __ldg(b.tile_begin + Q);
	if (ALGO == 0) deliver_flat<MODE>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 1) deliver_tps<MODE, false>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 2) deliver_wps<MODE>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 3) deliver_tps<MODE, true>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 4) deliver_tps_pipe<MODE>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 5 || ALGO == 7) deliver_groups<MODE, 4>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 6) deliver_groups<MODE, 8>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 8) deliver_staged<MODE, 2>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 9) deliver_staged<MODE, 4>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 10) deliver_staged_vec<MODE, 2, 4>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 11) deliver_staged_vec<MODE, 4, 2>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 12) deliver_staged_vec<MODE, 1, 8>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 13) deliver_staged_vec<MODE, 2, 6>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 14) deliver_rows<MODE>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 15) deliver_rows16<MODE, 1, 8, false>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 16) deliver_rows16<MODE, 4, 2, false>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 17) deliver_rows16<MODE, 2, 4, false>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 18) deliver_rows16<MODE, 1, 8, true>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 19) deliver_rows16<MODE, 2, 4, true>(a, P, t, (int)blockIdx.y, part);
	else if (ALGO == 20) deliver_rows16<MODE, 1, 8, false, 1024>(a, P, t, (int)blockIdx.y, part);
	else deliver_rows16<MODE, 2, 4, false, 1024>(a, P, t, (int)blockIdx.y, part);
}

// ---------------------------------------------------------------------------------------------
// Persistent steps: a network whose windows are one step long (plastic connections, or a minimum
// delay of one step) pays three to four launches per step in the window design, each mostly
// launch latency.  Here one cooperative launch runs every step of a chunk; the phases of a step
// are separated by grid-wide barriers:
//   A  the neuron update and source populations of step t (the window bodies with K = 1)
//   C  the deliveries of step t (snn.cpp:21-25) -- each fixed-weight connection's spikes of step t
//      into ring slot (t + d - 1) mod D, and each plastic connection's spikes of step t - d + 1
//      (catch-up, then the synapse's weight into slot t mod D; with delay 1 from the step's spike
//      list, else from the bitmap), with global reductions, in work units of a warp and at most
//      kPersistChunk (plastic: kPersistPlasticChunk) synapses of one row; the raster of step t; the
//      other parity's spike counts cleared.  At t mod 64 == 0 the plastic units cover every row:
//      the periodic catch-up of every synapse (snn.cpp:17-19) and, for a spiking source, the
//      delivery right after it -- the reference's order per synapse, with no barrier between.  A
//      plastic source's `ages` word is written in phase A of the next step, when every unit of its
//      row has read the old value.
// Deterministic mode adds integer counts (exact in any order); atomic mode adds floats as the
// window design does.
// ---------------------------------------------------------------------------------------------
constexpr long long kBarrierCycles = 2000000000ll;  // ~1 s at the SM clock, then the wait gives up

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
	unsigned v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

// Grid-wide barrier over a monotonic arrival counter (every CTA calls it the same number of times;
// `target` is this CTA's running count of expected arrivals).  Returns false once any wait has
// given up: the caller stops.
__device__ __forceinline__ bool grid_barrier(unsigned* count, unsigned& target, int* status) {
	__syncthreads();
	target += gridDim.x;
	if (threadIdx.x == 0) {
		__threadfence();
		atomicAdd(count, 1u);
		long long const start = clock64();
		while (ld_acquire(count) < target) {
			if (clock64() - start > kBarrierCycles || *(volatile int*)status != 0) {
				atomicExch(status, 1);
				break;
			}
			__nanosleep(32);
		}
		__threadfence();
	}
	__syncthreads();
	return *(volatile int*)status == 0;
}

// The ages of plastic sources after the deliveries of step t (phase C): every source caught up to
// t + 1 when t mod 64 == 0 (unless that catch-up ran as its own kernel, which set them), and the
// sources delivered at t with the pending pre update (bit 63).
__device__ __forceinline__ void plastic_ages_after(PersistArgs const& a, int64_t t) {
	bool const full = t % 64 == 0 && !a.external_full;
	for (int c = 0; c < a.nconn; c++) {
		ConnDev const& C = a.conns[c];
		if (!C.plastic) continue;
		bool const delivered = t >= C.delay - 1;
		const uint32_t* bits = C.src_bits + ((t - C.delay + 1 + a.Hb) % a.Hb) * C.src_nwords;
		for (int64_t wd = blockIdx.x * (int64_t)kPersistThreads + threadIdx.x; wd < C.src_nwords;
		     wd += (int64_t)gridDim.x * kPersistThreads) {
			uint32_t const m = delivered ? bits[wd] : 0u;
			if (full) {
				int64_t const s0 = 32 * wd, s1 = min(C.src_size, s0 + 32);
				for (int64_t sidx = s0; sidx < s1; sidx++)
					C.ages[sidx] = (uint64_t)(t + 1) | ((uint64_t)((m >> (sidx - s0)) & 1u) << 63);
			} else {
				for (uint32_t x = m; x; x &= x - 1) C.ages[32 * wd + __ffs(x) - 1] = (uint64_t)(t + 1) | (1ull << 63);
			}
		}
	}
}

template <int MODE>
__global__ void __launch_bounds__(kPersistThreads) k_persist(const __grid_constant__ PersistArgs a) {
	__shared__ int red[kPersistThreads / 32 + 1];
	__shared__ int64_t u_begin[kMaxConns + 1];  // phase C: first unit of each connection
	__shared__ unsigned long long ev_block;
	int const lane = threadIdx.x & 31;
	int const wib  = threadIdx.x >> 5;
	constexpr int WPB = kPersistThreads / 32;
	int64_t const gwarp  = (int64_t)blockIdx.x * WPB + wib;
	int64_t const nwarps = (int64_t)gridDim.x * WPB;
	unsigned target = 0;
	if (threadIdx.x == 0) ev_block = 0;
	for (int s = 0; s < a.nsteps; s++) {
		int64_t const t = a.t0 + s;
		int const q     = (a.parity0 + s) & 1;
		WinCtx w;
		w.K              = 1;
		w.D              = a.D;
		w.slot0          = (int)((t - 1 + a.D) % a.D);
		w.hslot0         = (int)(t % a.Hb);
		w.Hb             = a.Hb;
		w.npop           = a.npop;
		w.list_k0        = q;
		w.dts            = a.dts + s;
		w.tables         = a.tables ? a.tables + (int64_t)s * kJumpTable : nullptr;
		w.tab_net_stride = 0;
		w.counts         = a.counts + q * a.npop;
		bool const do_a  = !(s == 0 && a.start_at_c);
		bool const do_c  = !(s == a.nsteps - 1 && a.end_after_a);
		// ---- A: the update of step t; the ages of the previous step's plastic deliveries ----
		for (int vb = do_a ? (int)blockIdx.x : a.nblk; vb < a.nblk; vb += gridDim.x) {
			int p = 0;
			while (p + 1 < a.npop && vb >= a.blk_begin[p + 1]) p++;
			int const lb   = vb - a.blk_begin[p];
			int const kind = a.blk_kind[p];
			if (kind == 1) window_poisson(w, a.pops + p, p, lb, a.blk_per_step[p], red);
			else if (kind == 2) window_external(w, a.pops + p, p, 0, a.ext_pos[p] + s);
			else if ((kind & 7) == 3) {
				if (kind & kHistKind) window_neurons<MODE, true, true>(w, a.pops + p, p, lb);
				else window_neurons<MODE, true, false>(w, a.pops + p, p, lb);
			} else {
				if (kind & kHistKind) window_neurons<MODE, false, true>(w, a.pops + p, p, lb);
				else window_neurons<MODE, false, false>(w, a.pops + p, p, lb);
			}
			__syncthreads();  // shared scratch of the bodies is reused by the next item
		}
		if (do_a && a.any_plastic && t > a.t0) plastic_ages_after(a, t - 1);  // the deliveries of step t - 1
		if (!do_c) break;  // the periodic catch-up kernel and the next launch follow
		if (do_a && !grid_barrier(a.barrier, target, a.status)) return;
		// ---- C: deliveries of step t, raster, counts of the other parity ----
		bool const full = a.any_plastic && t % 64 == 0 && !a.external_full;  // every plastic row catches up
		if (threadIdx.x == 0) {
			int64_t acc = 0;
			for (int c = 0; c < a.nconn; c++) {
				ConnDev const& C = a.conns[c];
				u_begin[c] = acc;
				if (C.plastic) {
					if (full) acc += C.src_size * a.chunks[c];
					else if (C.delay == 1) acc += (int64_t)a.counts[q * a.npop + C.src] * a.chunks[c];
					else if (t >= C.delay - 1) acc += (int64_t)C.src_nwords * a.chunks[c];
				} else {
					acc += (int64_t)a.counts[q * a.npop + C.src] * a.chunks[c];
				}
			}
			u_begin[a.nconn] = acc;
		}
		if (blockIdx.x == 0 && threadIdx.x < a.npop) a.counts[(q ^ 1) * a.npop + threadIdx.x] = 0;
		__syncthreads();
		if (a.record && blockIdx.x < a.npop) {
			RasterArgs r = a.raster;
			r.t0     = t;
			r.K      = 1;
			r.counts = a.counts + q * a.npop;
			r.parity = (a.rec_parity0 + s) & 1;
			r.row0   = a.raster.row0 + s;
			raster_block(r, blockIdx.x);
		}
		int64_t const total = u_begin[a.nconn];
		unsigned long long ev = 0;
		int c = 0;
		for (int64_t u = gwarp; u < total; u += nwarps) {
			while (c + 1 < a.nconn && u >= u_begin[c + 1]) c++;
			while (c > 0 && u < u_begin[c]) c--;
			ConnDev const& C = a.conns[c];
			int64_t const r  = u - u_begin[c];
			int64_t const ch = r % a.chunks[c];
			if (C.plastic) {
				bool const delivers  = t >= C.delay - 1;
				bool const weight_in = MODE == 1 && (C.plastic == SPICE_SYNAPSE_ISTDP || C.weight != 0.0f);
				int64_t const slot   = t % a.D;
				const uint32_t* bits = C.src_bits + ((t - C.delay + 1 + a.Hb) % a.Hb) * C.src_nwords;
				constexpr int64_t L = kPersistPlasticChunk;
				if (full) {  // unit: (source, chunk) of every row: catch-up, then the delivery if it spiked
					int64_t const src = r / a.chunks[c];
					bool const spiked = delivers && ((bits[src >> 5] >> (src & 31)) & 1u);
					int64_t const e0 = C.off[src] + ch * L, e1 = min(C.off[src + 1], e0 + L);
					if (spiked && ch == 0 && lane == 0) ev += (unsigned long long)(C.off[src + 1] - C.off[src]);
					plastic_row_chunk(C, e0, e1, t, C.ages[src], slot, spiked && weight_in, lane);
				} else if (C.delay == 1) {  // unit: (spike, chunk) of step t, from the step's spike list
					int32_t const src = C.src_list[(int64_t)q * C.src_size + r / a.chunks[c]];
					int64_t const e0 = C.off[src] + ch * L, e1 = min(C.off[src + 1], e0 + L);
					if (ch == 0 && lane == 0) ev += (unsigned long long)(C.off[src + 1] - C.off[src]);
					plastic_row_chunk(C, e0, e1, t, C.ages[src], slot, weight_in, lane);
				} else {  // unit: (bitmap word, chunk) of the spikes of step t - d + 1
					int64_t const wd = r / a.chunks[c];
					for (uint32_t m = bits[wd]; m; m &= m - 1) {
						int64_t const src = 32 * wd + __ffs(m) - 1;
						int64_t const e0 = C.off[src] + ch * L, e1 = min(C.off[src + 1], e0 + L);
						if (ch == 0 && lane == 0) ev += (unsigned long long)(C.off[src + 1] - C.off[src]);
						plastic_row_chunk(C, e0, e1, t, C.ages[src], slot, weight_in, lane);
					}
				}
			} else {  // unit: (spike, chunk) of step t
				int32_t const src = C.src_list[(int64_t)q * C.src_size + r / a.chunks[c]];
				int64_t const e0 = C.off[src] + ch * kPersistChunk, e1 = min(C.off[src + 1], e0 + kPersistChunk);
				if (ch == 0 && lane == 0) ev += (unsigned long long)(C.off[src + 1] - C.off[src]);
				int64_t const slot = (t + C.delay - 1) % a.D;
				if (MODE == 0) {
					uint32_t* const base = C.dst_cnt + slot * C.dst_size * C.W + C.word;
					for (int64_t e = e0 + lane; e < e1; e += 32) red_add_u32(base + (int64_t)C.nb[e] * C.W, C.inc);
				} else {
					float* const base = C.dst_acc + slot * C.dst_size * C.F + C.fslot;
					for (int64_t e = e0 + lane; e < e1; e += 32) red_add_f32(base + (int64_t)C.nb[e] * C.F, C.weight);
				}
			}
		}
		if (lane == 0 && ev) atomicAdd(&ev_block, ev);
		if (!grid_barrier(a.barrier, target, a.status)) return;
	}
	if (a.any_plastic && !a.end_after_a) plastic_ages_after(a, a.t0 + a.nsteps - 1);  // the last step's deliveries
	__syncthreads();
	if (threadIdx.x == 0 && ev_block) atomicAdd(a.events, ev_block);
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

cudaError_t scan_row_lengths_into(cudaStream_t stream, const int32_t* lens, int64_t n, int64_t* offsets,
                                  int64_t* block_sums) {
	if (n <= 0) return cudaMemsetAsync(offsets, 0, sizeof(int64_t), stream);
	int64_t const nb = (n + kScanItems - 1) / kScanItems;
	k_scan_local<<<(unsigned)nb, kScanItems, 0, stream>>>(lens, n, offsets, block_sums);
	k_scan_sums<<<1, kScanItems, 0, stream>>>(block_sums, nb);
	k_scan_add<<<(unsigned)nb, kScanItems, 0, stream>>>(offsets, n, block_sums);
	return cudaGetLastError();
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

cudaError_t launch_jump_tables(cudaStream_t stream, const u128* seeds, int64_t nsteps, u128* tables) {
	if (nsteps <= 0) return cudaSuccess;
	k_jump_tables<<<(unsigned)nsteps, 256, 0, stream>>>(seeds, nsteps, tables);
	return cudaGetLastError();
}

cudaError_t launch_neurons(cudaStream_t stream, WindowArgs const& a, int nblocks) {
	if (nblocks <= 0) return cudaSuccess;
	bool only_fast = true;
	for (int p = 0; p < a.npop; p++) only_fast &= a.blk_kind[p] != 0 && a.blk_kind[p] < kHistKind;
	if (a.mode == 0) {
		if (!only_fast) k_neurons<0, false, 0><<<nblocks, kThreads, 0, stream>>>(a);
		else if (a.variant == 1) k_neurons<0, true, 1><<<nblocks, kThreads, 0, stream>>>(a);
		else if (a.variant == 2) k_neurons<0, true, 2><<<nblocks, kThreads, 0, stream>>>(a);
		else if (a.variant == 3) k_neurons<0, true, 3><<<nblocks, kThreads, 0, stream>>>(a);
		else if (a.variant == 4) k_neurons<0, true, 4><<<nblocks, kThreads, 0, stream>>>(a);
		else if (a.variant == 5) k_neurons<0, true, 5><<<nblocks, kThreads, 0, stream>>>(a);
		else if (a.variant == 6) k_neurons<0, true, 6><<<nblocks, kThreads, 0, stream>>>(a);
		else if (a.variant == 7) k_neurons<0, true, 7><<<nblocks, kThreads, 0, stream>>>(a);
		else if (a.variant == 8) k_neurons<0, true, 8><<<nblocks, kThreads, 0, stream>>>(a);
		else if (a.variant == 9) k_neurons<0, true, 9><<<nblocks, kThreads, 0, stream>>>(a);
		else k_neurons<0, true, 0><<<nblocks, kThreads, 0, stream>>>(a);
	} else {
		if (only_fast) k_neurons<1, true, 0><<<nblocks, kThreads, 0, stream>>>(a);
		else k_neurons<1, false, 0><<<nblocks, kThreads, 0, stream>>>(a);
	}
	return cudaGetLastError();
}

cudaError_t launch_window(cudaStream_t stream, WindowArgs const& a, int nblocks, WindowArgs const& s, int nsrc_blocks,
                          RasterArgs const* r, bool pdl) {
	int const nrb = r ? r->K * r->npop : 0;
	if (nblocks + nsrc_blocks + nrb <= 0) return cudaSuccess;
	bool only_fast = true;
	for (int p = 0; p < a.npop; p++) only_fast &= a.blk_kind[p] != 0 && a.blk_kind[p] < kHistKind;
	void const* fns[2][12] = {{(void const*)k_window<0, false, 0, false>, (void const*)k_window<0, true, 0, false>,
	                           (void const*)k_window<0, true, 1, false>, (void const*)k_window<0, true, 2, false>,
	                           (void const*)k_window<0, true, 3, false>, (void const*)k_window<0, true, 4, false>,
	                           (void const*)k_window<0, true, 5, false>, (void const*)k_window<0, true, 6, false>,
	                           (void const*)k_window<0, true, 7, false>, (void const*)k_window<0, true, 8, false>,
	                           (void const*)k_window<0, true, 9, false>, (void const*)k_window<1, true, 0, false>},
	                          {(void const*)k_window<0, false, 0, true>, (void const*)k_window<0, true, 0, true>,
	                           (void const*)k_window<0, true, 1, true>, (void const*)k_window<0, true, 2, true>,
	                           (void const*)k_window<0, true, 3, true>, (void const*)k_window<0, true, 4, true>,
	                           (void const*)k_window<0, true, 5, true>, (void const*)k_window<0, true, 6, true>,
	                           (void const*)k_window<0, true, 7, true>, (void const*)k_window<0, true, 8, true>,
	                           (void const*)k_window<0, true, 9, true>, (void const*)k_window<1, true, 0, true>}};
	void const* fk_atomic_generic[2] = {(void const*)k_window<1, false, 0, false>, (void const*)k_window<1, false, 0, true>};
	int const rec = nrb > 0 ? 1 : 0;
	void const* fn = nullptr;
	if (a.mode == 0) fn = !only_fast ? fns[rec][0] : fns[rec][1 + (a.variant >= 0 && a.variant <= 9 ? a.variant : 0)];
	else fn = only_fast ? fns[rec][11] : fk_atomic_generic[rec];
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim          = dim3((unsigned)(nblocks + nsrc_blocks + nrb));
	cfg.blockDim         = dim3((unsigned)kThreads);
	cfg.dynamicSmemBytes = 0;
	cfg.stream           = stream;
	cudaLaunchAttribute at[1];
	at[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
	cfg.attrs    = at;
	cfg.numAttrs = 1;
	int nb = nblocks;
	RasterArgs rr{};
	if (r) rr = *r;
	void* args[] = {const_cast<WindowArgs*>(&a), const_cast<WindowArgs*>(&s), &nb, &rr};
	return cudaLaunchKernelExC(&cfg, fn, args);
}

cudaError_t launch_sources(cudaStream_t stream, WindowArgs const& a, int nblocks) {
	if (nblocks <= 0) return cudaSuccess;
	k_sources<<<nblocks, kThreads, 0, stream>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_deliver(cudaStream_t stream, DeliverArgs const& a, int threads) {
	int64_t const nblocks = (int64_t)a.nslots * a.ntiles_total * a.parts;
	if (nblocks <= 0) {
		if (a.counts_next_len > 0) return cudaMemsetAsync(a.counts_next, 0, sizeof(int32_t) * a.counts_next_len, stream);
		return cudaSuccess;
	}
	static int configured[kDeliverFns] = {};
	int const m = (a.mode == 0 ? 0 : 1) + 2 * a.algo;
	void const* fns[kDeliverFns] = {(void const*)k_deliver<0>,            (void const*)k_deliver<1>,
	                       (void const*)k_deliver_tps<0, false>, (void const*)k_deliver_tps<1, false>,
	                       (void const*)k_deliver_wps<0>,        (void const*)k_deliver_wps<1>,
	                       (void const*)k_deliver_tps<0, true>,  (void const*)k_deliver_tps<1, true>,
	                       (void const*)k_deliver_pipe<0>,       (void const*)k_deliver_pipe<1>,
	                       (void const*)k_deliver_groups<0, 4>,  (void const*)k_deliver_groups<1, 4>,
	                       (void const*)k_deliver_groups<0, 8>,  (void const*)k_deliver_groups<1, 8>,
	                       (void const*)k_deliver_groups_occ<0>, (void const*)k_deliver_groups_occ<1>,
	                       (void const*)k_deliver_staged<0, 2>,  (void const*)k_deliver_staged<1, 2>,
	                       (void const*)k_deliver_staged<0, 4>,  (void const*)k_deliver_staged<1, 4>,
	                       (void const*)k_deliver_staged_vec<0, 2, 4>, (void const*)k_deliver_staged_vec<1, 2, 4>,
	                       (void const*)k_deliver_staged_vec<0, 4, 2>, (void const*)k_deliver_staged_vec<1, 4, 2>,
	                       (void const*)k_deliver_staged_vec<0, 1, 8>, (void const*)k_deliver_staged_vec<1, 1, 8>,
	                       (void const*)k_deliver_staged_vec<0, 2, 6>, (void const*)k_deliver_staged_vec<1, 2, 6>,
	                       (void const*)k_deliver_rows<0>,             (void const*)k_deliver_rows<1>,
	                       (void const*)k_deliver_rows16<0, 1, 8, false>, (void const*)k_deliver_rows16<1, 1, 8, false>,
	                       (void const*)k_deliver_rows16<0, 4, 2, false>, (void const*)k_deliver_rows16<1, 4, 2, false>,
	                       (void const*)k_deliver_rows16<0, 2, 4, false>, (void const*)k_deliver_rows16<1, 2, 4, false>,
	                       (void const*)k_deliver_rows16<0, 1, 8, true>,  (void const*)k_deliver_rows16<1, 1, 8, true>,
	                       (void const*)k_deliver_rows16<0, 2, 4, true>,  (void const*)k_deliver_rows16<1, 2, 4, true>,
	                       (void const*)k_deliver_rows16_occ<0, 1, 8>,   (void const*)k_deliver_rows16_occ<1, 1, 8>,
	                       (void const*)k_deliver_rows16_occ<0, 2, 4>,   (void const*)k_deliver_rows16_occ<1, 2, 4>};
	void const* fn = fns[m];
	cudaFuncAttributes fa;
	if (cudaFuncGetAttributes(&fa, fn) == cudaSuccess && threads > fa.maxThreadsPerBlock)
		threads = fa.maxThreadsPerBlock / 32 * 32;  // the launch shape never changes results
	if (configured[m] < a.smem_bytes) {
		cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, a.smem_bytes);
		if (e != cudaSuccess) return e;
		configured[m] = a.smem_bytes;
	}
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim          = dim3((unsigned)nblocks);
	cfg.blockDim         = dim3((unsigned)threads);
	cfg.dynamicSmemBytes = (size_t)a.smem_bytes;
	cfg.stream           = stream;
	cudaLaunchAttribute at[1];
	at[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = a.pdl ? 1 : 0;
	cfg.attrs    = at;
	cfg.numAttrs = 1;
	void* args[] = {const_cast<DeliverArgs*>(&a)};
	cudaError_t const e = cudaLaunchKernelExC(&cfg, fn, args);
	if (e != cudaSuccess) return e;
	return cudaGetLastError();
}

cudaError_t launch_compact_targets(cudaStream_t stream, const int32_t* nb, int64_t synapses, int tile, uint16_t* nb16) {
	if (synapses <= 0) return cudaSuccess;
	k_compact_targets<<<1216, 256, 0, stream>>>(nb, synapses, tile, nb16);
	return cudaGetLastError();
}

cudaError_t launch_tile_bounds(cudaStream_t stream, const int64_t* off, const int32_t* nb, int64_t rows, int tile,
                               int ntiles, int64_t* bounds) {
	if (rows <= 0) return cudaSuccess;
	k_tile_bounds<<<(unsigned)((rows + 255) / 256), 256, 0, stream>>>(off, nb, rows, tile, ntiles, bounds);
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

cudaError_t launch_batch_prologue(cudaStream_t stream, BatchArgs const& b, int k) {
	k_batch_prologue<<<1, 256, 0, stream>>>(b, k);
	return cudaGetLastError();
}

cudaError_t launch_batch_sources(cudaStream_t stream, BatchArgs const& b, int k) {
	if (b.sblk_total <= 0 || k <= 0) return cudaSuccess;
	k_batch_sources<<<dim3((unsigned)b.sblk_total, (unsigned)k), kThreads, 0, stream>>>(b);
	return cudaGetLastError();
}

cudaError_t launch_batch_neurons(cudaStream_t stream, BatchArgs const& b) {
	if (b.nblk_total <= 0) return cudaSuccess;
	if (b.mode == 0) {
		if (b.only_fast) k_batch_neurons<0, true><<<b.nblk_total, kThreads, 0, stream>>>(b);
		else k_batch_neurons<0, false><<<b.nblk_total, kThreads, 0, stream>>>(b);
	} else {
		if (b.only_fast) k_batch_neurons<1, true><<<b.nblk_total, kThreads, 0, stream>>>(b);
		else k_batch_neurons<1, false><<<b.nblk_total, kThreads, 0, stream>>>(b);
	}
	return cudaGetLastError();
}

namespace {
void const* batch_deliver_fn(BatchArgs const& b) {
	int const m = (b.mode == 0 ? 0 : 1) + 2 * b.algo;
	void const* fns[kDeliverFns] = {(void const*)k_batch_deliver<0, 0>, (void const*)k_batch_deliver<1, 0>,
	                       (void const*)k_batch_deliver<0, 1>, (void const*)k_batch_deliver<1, 1>,
	                       (void const*)k_batch_deliver<0, 2>, (void const*)k_batch_deliver<1, 2>,
	                       (void const*)k_batch_deliver<0, 3>, (void const*)k_batch_deliver<1, 3>,
	                       (void const*)k_batch_deliver<0, 4>, (void const*)k_batch_deliver<1, 4>,
	                       (void const*)k_batch_deliver<0, 5>, (void const*)k_batch_deliver<1, 5>,
	                       (void const*)k_batch_deliver<0, 6>, (void const*)k_batch_deliver<1, 6>,
	                       (void const*)k_batch_deliver<0, 7>, (void const*)k_batch_deliver<1, 7>,
	                       (void const*)k_batch_deliver<0, 8>, (void const*)k_batch_deliver<1, 8>,
	                       (void const*)k_batch_deliver<0, 9>, (void const*)k_batch_deliver<1, 9>,
	                       (void const*)k_batch_deliver<0, 10>, (void const*)k_batch_deliver<1, 10>,
	                       (void const*)k_batch_deliver<0, 11>, (void const*)k_batch_deliver<1, 11>,
	                       (void const*)k_batch_deliver<0, 12>, (void const*)k_batch_deliver<1, 12>,
	                       (void const*)k_batch_deliver<0, 13>, (void const*)k_batch_deliver<1, 13>,
	                       (void const*)k_batch_deliver<0, 14>, (void const*)k_batch_deliver<1, 14>,
	                       (void const*)k_batch_deliver<0, 15>, (void const*)k_batch_deliver<1, 15>,
	                       (void const*)k_batch_deliver<0, 16>, (void const*)k_batch_deliver<1, 16>,
	                       (void const*)k_batch_deliver<0, 17>, (void const*)k_batch_deliver<1, 17>,
	                       (void const*)k_batch_deliver<0, 18>, (void const*)k_batch_deliver<1, 18>,
	                       (void const*)k_batch_deliver<0, 19>, (void const*)k_batch_deliver<1, 19>,
	                       (void const*)k_batch_deliver<0, 20>, (void const*)k_batch_deliver<1, 20>,
	                       (void const*)k_batch_deliver<0, 21>, (void const*)k_batch_deliver<1, 21>};
	return fns[m];
}
}  // namespace

cudaError_t configure_batch_deliver(BatchArgs const& b) {
	return cudaFuncSetAttribute(batch_deliver_fn(b), cudaFuncAttributeMaxDynamicSharedMemorySize, b.smem_bytes);
}

cudaError_t launch_batch_deliver(cudaStream_t stream, BatchArgs const& b, int k, int threads) {
	int const nslots = k + b.dmax - b.dmin;
	if (b.ntiles_total <= 0 || nslots <= 0) return cudaSuccess;
	cudaFuncAttributes fa;
	if (cudaFuncGetAttributes(&fa, batch_deliver_fn(b)) == cudaSuccess && threads > fa.maxThreadsPerBlock)
		threads = fa.maxThreadsPerBlock / 32 * 32;  // the launch shape never changes results
	dim3 const grid((unsigned)(b.ntiles_total * b.parts), (unsigned)nslots);
	switch ((b.mode == 0 ? 0 : 1) + 2 * b.algo) {
		case 0: k_batch_deliver<0, 0><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 1: k_batch_deliver<1, 0><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 2: k_batch_deliver<0, 1><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 3: k_batch_deliver<1, 1><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 4: k_batch_deliver<0, 2><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 5: k_batch_deliver<1, 2><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 6: k_batch_deliver<0, 3><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 7: k_batch_deliver<1, 3><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 8: k_batch_deliver<0, 4><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 9: k_batch_deliver<1, 4><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 10: k_batch_deliver<0, 5><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 11: k_batch_deliver<1, 5><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 12: k_batch_deliver<0, 6><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 13: k_batch_deliver<1, 6><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 14: k_batch_deliver<0, 7><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 15: k_batch_deliver<1, 7><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 16: k_batch_deliver<0, 8><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 17: k_batch_deliver<1, 8><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 18: k_batch_deliver<0, 9><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 19: k_batch_deliver<1, 9><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 20: k_batch_deliver<0, 10><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 21: k_batch_deliver<1, 10><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 22: k_batch_deliver<0, 11><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 23: k_batch_deliver<1, 11><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 24: k_batch_deliver<0, 12><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 25: k_batch_deliver<1, 12><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 26: k_batch_deliver<0, 13><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 27: k_batch_deliver<1, 13><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 28: k_batch_deliver<0, 14><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 29: k_batch_deliver<1, 14><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 30: k_batch_deliver<0, 15><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 31: k_batch_deliver<1, 15><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 32: k_batch_deliver<0, 16><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 33: k_batch_deliver<1, 16><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 34: k_batch_deliver<0, 17><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 35: k_batch_deliver<1, 17><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 36: k_batch_deliver<0, 18><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 37: k_batch_deliver<1, 18><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 38: k_batch_deliver<0, 19><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 39: k_batch_deliver<1, 19><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 40: k_batch_deliver<0, 20><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 41: k_batch_deliver<1, 20><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 42: k_batch_deliver<0, 21><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		case 43: k_batch_deliver<1, 21><<<grid, threads, b.smem_bytes, stream>>>(b); break;
		default: return cudaErrorInvalidValue;  // a delivery mapping without a batched kernel
	}
	static_assert(kDeliverFns == 44, "every delivery mapping has a case above");
	return cudaGetLastError();
}

namespace {
// Self-test of mul_f32_f64_rn against the double multiply: random finite a >= 0 (every exponent,
// subnormals included) and random f in [2^-4, 2^5) (products overflowing float included).
__global__ void k_selftest_mulround(int64_t count, uint64_t seed, unsigned long long* mismatches,
                                    unsigned long long* first) {
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
		uint64_t x = seed ^ (0x9e3779b97f4a7c15ull * (uint64_t)(i + 1));
		x ^= x >> 31;
		x *= 0xbf58476d1ce4e5b9ull;
		x ^= x >> 29;
		x *= 0x94d049bb133111ebull;
		x ^= x >> 32;
		uint32_t ab = (uint32_t)x & 0x7fffffffu;
		if ((ab >> 23) == 0xffu) ab &= 0x7f7fffffu;  // finite
		if ((i & 7) == 0) ab &= 0x007fffffu;      // every eighth a subnormal
		uint64_t y = x * 0xd1342543de82ef95ull + 1;
		y ^= y >> 33;
		int const ex  = (int)(y % 9) - 4;
		double const f = ldexp(1.0 + (double)(y >> 12) * 0x1p-52, ex);
		float const a  = __uint_as_float(ab);
		float const r1 = __double2float_rn(__dmul_rn((double)a, f));
		// pack f on the device as pack_f64 does on the host
		uint64_t const fb = (uint64_t)__double_as_longlong(f);
		int const e       = (int)((fb >> 52) & 0x7ff) - 1023;  // f = 1.m 2^e
		uint64_t const pk = ((fb & ((1ull << 52) - 1)) | (1ull << 52)) | ((uint64_t)(e - 52 + 1100) << 53);
		float const r2    = mul_f32_f64_rn(a, pk);
		if (__float_as_uint(r1) != __float_as_uint(r2)) {
			if (atomicAdd(mismatches, 1ull) == 0) {
				first[0] = ab;
				first[1] = fb;
			}
		}
	}
}
}  // namespace

cudaError_t launch_selftest_mulround(cudaStream_t stream, int64_t count, uint64_t seed, unsigned long long* mismatches,
                                     unsigned long long* first) {
	k_selftest_mulround<<<1216, 256, 0, stream>>>(count, seed, mismatches, first);
	return cudaGetLastError();
}

cudaError_t launch_plastic_update_all(cudaStream_t stream, ConnDev const& c, int64_t time) {
	if (c.src_size <= 0) return cudaSuccess;
	k_plastic_update_all<<<(unsigned)((c.src_size + 7) / 8), 256, 0, stream>>>(c, time);
	return cudaGetLastError();
}

cudaError_t launch_plastic_deliver(cudaStream_t stream, ConnDev const& c, int64_t time, int hslot, int64_t slot,
                                   bool deliver, unsigned long long* events) {
	if (c.src_nwords <= 0 || c.max_row <= 0) return cudaSuccess;
	dim3 const grid((unsigned)c.src_nwords,
	                (unsigned)std::min<int64_t>(65535, (c.max_row + kPlasticChunk - 1) / kPlasticChunk));
	k_plastic_deliver<<<grid, kPlasticChunk, 0, stream>>>(c, time, hslot, slot, deliver ? 1 : 0, events);
	return cudaGetLastError();
}

cudaError_t persist_occupancy(int mode, int* blocks_per_sm) {
	void const* f = mode == 0 ? (void const*)k_persist<0> : (void const*)k_persist<1>;
	return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, kPersistThreads, 0);
}

// A cooperative launch: every CTA of the grid is resident at once (the barriers wait on each other).
cudaError_t launch_persist(cudaStream_t stream, PersistArgs const& a, int grid) {
	if (a.nsteps <= 0) return cudaSuccess;
	void const* f = a.mode == 0 ? (void const*)k_persist<0> : (void const*)k_persist<1>;
	void* args[]  = {const_cast<PersistArgs*>(&a)};
	return cudaLaunchCooperativeKernel(f, dim3((unsigned)grid), dim3((unsigned)kPersistThreads), args, 0, stream);
}

cudaError_t launch_raster(cudaStream_t stream, RasterArgs const& a) {
	if (a.K * a.npop <= 0) return cudaSuccess;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim  = dim3((unsigned)(a.K * a.npop));
	cfg.blockDim = dim3(1024u);
	cfg.stream   = stream;
	cudaLaunchAttribute at[1];
	at[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = a.pdl ? 1 : 0;
	cfg.attrs    = at;
	cfg.numAttrs = 1;
	void* args[] = {const_cast<RasterArgs*>(&a)};
	return cudaLaunchKernelExC(&cfg, (void const*)k_raster, args);
}

}  // namespace spice_gb300
