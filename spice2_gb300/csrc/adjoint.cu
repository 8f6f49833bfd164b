// adjoint.cu -- a differentiable recurrent LIF layer: forward and adjoint (backward-in-time)
// kernels behind spice_lif_* (include/spice_gb300.h).  No counterpart in the reference.
//
// Model (one sample; n_in inputs x_t in {0,1}, n recurrent neurons, delay 1 step, t = 1..T):
//   u_t = beta (.) v_{t-1} + W_in^T x_{t-1} + W_rec^T s_{t-1}          v_0 = 0, s_0 = 0
//   s_t = H(u_t - theta)                 (relaxed: s_t = g(u_t - theta), g(x) = (1 + kx/(1+k|x|))/2)
//   v_t = u_t - theta (.) s_t            (reset by subtraction)
//   counts = sum_t s_t;  the caller's loss gives dL/dcounts.
// Backward (reverse mode through time; sigma'(x) = 1/(1+k|x|)^2 is the fast-sigmoid surrogate of
// H', and g' = (k/2) sigma' is exact for the relaxed forward):
//   vbar_t = beta (.) ubar_{t+1}
//   sbar_t = dL/dcounts + W_rec ubar_{t+1} - theta (.) vbar_t
//   ubar_t = vbar_t + sigma'(u_t - theta) (.) sbar_t                      ubar_{T+1} = 0
//   dW_rec[i->j] = sum_t s_{t-1,i} ubar_{t,j}    dW_in[k->j] = sum_t x_{t-1,k} ubar_{t,j}
//   dbeta = sum_t v_{t-1} (.) ubar_t              dtheta = -sum_t (sigma'_t (.) sbar_t + s_t (.) vbar_t)
//
// One CTA per sample runs all T steps (the layer's state lives in shared memory).  The forward
// delivers input and recurrent events by scattering each active source's CSR row into per-neuron
// 64-bit fixed-point accumulators (2^-32 units; integer sums do not depend on the order of the
// shared-memory atomics, so every run is bit-reproducible).  The forward stores s_t and, every
// `checkpoint_every` steps, v_t; the backward walks the segments last to first, recomputes each
// segment's u_t and s_t from its checkpoint into shared memory, then runs the adjoint recursion
// through it.  Weight gradients are event driven (only sources active at t-1 touch their row);
// per-sample partials are summed over samples in a fixed order by k_lif_reduce.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "spice_gb300.h"
#include "internal.h"

using namespace spice_gb300;

struct spice_lif_layer {
	int n_in = 0, n = 0;
	int64_t in_syn = 0, rec_syn = 0;
	int64_t* in_off = nullptr;   // CSR by source, device
	int32_t* in_nb  = nullptr;
	int64_t* rec_off = nullptr;
	int32_t* rec_nb  = nullptr;
	long long* wq = nullptr;     // fixed-point weights: [in_syn] then [rec_syn]
	// the recurrent rows again as a column-major ELL matrix (entry q of row i at q * n + i) for the
	// backward's dense gather W_rec ubar: thread i walks row i, a warp's loads are coalesced
	int dmax = 0;
	int32_t* deg = nullptr;      // [n] row lengths
	int32_t* ell_nb = nullptr;   // [dmax][n] targets (0 past the row's end)
	float* ell_w = nullptr;      // [dmax][n] weights, refreshed from w_rec by each backward call
	float* partial = nullptr;    // per-sample gradient partials
	int64_t partial_cap = 0;     // floats
};

namespace {

constexpr int kLifThreads = 1024;
constexpr int kRowChunk   = 8;  // row entries per lane loaded before use
constexpr double kFix     = 4294967296.0;  // 2^32

struct LifArgs {
	int n_in, n, nw_in, T, ck, relaxed;
	float slope, sg_scale;  // sg_scale: 1 (surrogate) or slope / 2 (exact derivative of the relaxed g)
	const int64_t* in_off;
	const int32_t* in_nb;
	const int64_t* rec_off;
	const int32_t* rec_nb;
	const long long* wq_in;
	const long long* wq_rec;
	const uint32_t* x;      // [B][T][nw_in] bits of x_t (bit k of word k / 32)
	const float* w_in;
	const float* w_rec;
	const float* theta;
	const float* beta;
	float* counts;          // [B][n]
	float* spikes;          // [B][T][n]: s_t at index t - 1
	float* vck;             // [B][nck][n]: v at t = c * ck
	const float* gcounts;   // [B][n]
	float* part;            // [B][in_syn + rec_syn + 2 n]
	int64_t in_syn, rec_syn;
	const int32_t* deg;     // ELL view of the recurrent rows
	const int32_t* ell_nb;
	const float* ell_w;
};

__device__ __forceinline__ float relaxed_g(float x, float k) {
	return __fmul_rn(0.5f, __fadd_rn(1.0f, __fdiv_rn(__fmul_rn(k, x), __fadd_rn(1.0f, __fmul_rn(k, fabsf(x))))));
}

__device__ __forceinline__ float surrogate(float x, float k, float scale) {
	float const d = __fadd_rn(1.0f, __fmul_rn(k, fabsf(x)));
	return __fdiv_rn(scale, __fmul_rn(d, d));
}

// Shared-memory working set of one step (offsets in floats / words set up by the kernels).
struct StepSmem {
	unsigned long long* acc;  // [n] fixed-point input of the step
	int* list_in;             // [n_in] active inputs
	int* list_s;              // [n] active sources (s != 0)
	int* nact;                // [2] list lengths
	uint32_t* xb;             // [nw_in] x bits
};

__device__ __forceinline__ void load_x(LifArgs const& a, int b, int t_minus_1, uint32_t* xb) {
	const uint32_t* src = a.x + ((int64_t)b * a.T + t_minus_1) * a.nw_in;
	for (int w = threadIdx.x; w < a.nw_in; w += blockDim.x) xb[w] = src[w];
}

// Lists of the inputs set in xb and of the sources with s != 0 (unordered).
__device__ __forceinline__ void build_lists(LifArgs const& a, StepSmem const& m, const float* s) {
	for (int k = threadIdx.x; k < a.n_in; k += blockDim.x)
		if ((m.xb[k >> 5] >> (k & 31)) & 1u) m.list_in[atomicAdd(m.nact, 1)] = k;
	for (int i = threadIdx.x; i < a.n; i += blockDim.x)
		if (s[i] != 0.0f) m.list_s[atomicAdd(m.nact + 1, 1)] = i;
}

// One forward step t (1-based).  xb holds x_{t-1}; s_prev = s_{t-1}; v = v_{t-1} on entry and
// v_t on return; u_out (optional) and s_out receive u_t and s_t.  Ends with a barrier.
__device__ void lif_step(LifArgs const& a, StepSmem const& m, const float* s_prev, float* v, float* u_out,
                         float* s_out) {
	int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
	for (int j = threadIdx.x; j < a.n; j += blockDim.x) m.acc[j] = 0ull;
	if (threadIdx.x < 2) m.nact[threadIdx.x] = 0;
	__syncthreads();
	build_lists(a, m, s_prev);
	__syncthreads();
	int const ni = m.nact[0], ns = m.nact[1];
	// scatter: one warp per active source row, lanes over the row (coalesced); each chunk of up to
	// kRowChunk entries per lane is loaded before its atomics so the loads overlap
	for (int q = warp; q < ni + ns; q += nwarps) {
		bool const inp    = q < ni;
		int const src     = inp ? m.list_in[q] : m.list_s[q - ni];
		int64_t const e0  = inp ? __ldg(a.in_off + src) : __ldg(a.rec_off + src);
		int64_t const e1  = inp ? __ldg(a.in_off + src + 1) : __ldg(a.rec_off + src + 1);
		const int32_t* nb = inp ? a.in_nb : a.rec_nb;
		const long long* wq = inp ? a.wq_in : a.wq_rec;
		float const sv    = inp ? 1.0f : s_prev[src];
		for (int64_t base = e0; base < e1; base += 32 * kRowChunk) {
			int32_t d[kRowChunk];
			long long w[kRowChunk];
#pragma unroll
			for (int u = 0; u < kRowChunk; u++) {
				int64_t const e = base + u * 32 + lane;
				bool const ok   = e < e1;
				d[u]            = ok ? __ldg(nb + e) : -1;
				if (sv == 1.0f) w[u] = ok ? __ldg(wq + e) : 0;
				else w[u] = ok ? __double2ll_rn((double)__ldg(a.w_rec + e) * (double)sv * kFix) : 0;
			}
#pragma unroll
			for (int u = 0; u < kRowChunk; u++)
				if (d[u] >= 0) atomicAdd(m.acc + d[u], (unsigned long long)w[u]);
		}
	}
	__syncthreads();
	for (int j = threadIdx.x; j < a.n; j += blockDim.x) {
		float const I  = (float)((double)(long long)m.acc[j] * (1.0 / kFix));
		float const u  = __fadd_rn(__fmul_rn(a.beta[j], v[j]), I);
		float const th = a.theta[j];
		float const x  = __fsub_rn(u, th);
		float const s  = a.relaxed ? relaxed_g(x, a.slope) : (x > 0.0f ? 1.0f : 0.0f);
		v[j]           = __fsub_rn(u, __fmul_rn(th, s));
		if (u_out) u_out[j] = u;
		s_out[j] = s;
	}
	__syncthreads();
}

__global__ void __launch_bounds__(kLifThreads, 1) k_lif_forward(const __grid_constant__ LifArgs a) {
	extern __shared__ __align__(16) unsigned char sm[];
	int const b = blockIdx.x, n = a.n;
	unsigned long long* acc = reinterpret_cast<unsigned long long*>(sm);
	float* v    = reinterpret_cast<float*>(acc + n);
	float* sA   = v + n;
	float* sB   = sA + n;
	float* cnt  = sB + n;
	int* list_s = reinterpret_cast<int*>(cnt + n);
	int* list_in = list_s + n;
	int* nact   = list_in + a.n_in;
	uint32_t* xb = reinterpret_cast<uint32_t*>(nact + 2);
	StepSmem const m{acc, list_in, list_s, nact, xb};
	int const nck = (a.T + a.ck - 1) / a.ck + 1;
	float* vck    = a.vck + (int64_t)b * nck * n;
	for (int j = threadIdx.x; j < n; j += blockDim.x) {
		v[j]   = 0.0f;
		sA[j]  = 0.0f;
		cnt[j] = 0.0f;
		vck[j] = 0.0f;
	}
	float* s_prev = sA;
	float* s_cur  = sB;
	for (int t = 1; t <= a.T; t++) {
		load_x(a, b, t - 1, xb);
		lif_step(a, m, s_prev, v, nullptr, s_cur);
		float* out = a.spikes + ((int64_t)b * a.T + (t - 1)) * n;
		bool const ckpt = t % a.ck == 0 || t == a.T;
		for (int j = threadIdx.x; j < n; j += blockDim.x) {
			float const s = s_cur[j];
			out[j]        = s;
			cnt[j]        = __fadd_rn(cnt[j], s);
			if (ckpt) vck[(int64_t)((t + a.ck - 1) / a.ck) * n + j] = v[j];
		}
		float* tmp = s_prev;
		s_prev     = s_cur;
		s_cur      = tmp;
	}
	__syncthreads();
	for (int j = threadIdx.x; j < n; j += blockDim.x) a.counts[(int64_t)b * n + j] = cnt[j];
}

__global__ void __launch_bounds__(kLifThreads, 1) k_lif_backward(const __grid_constant__ LifArgs a) {
	extern __shared__ __align__(16) unsigned char sm[];
	int const b = blockIdx.x, n = a.n, ck = a.ck;
	int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
	unsigned long long* acc = reinterpret_cast<unsigned long long*>(sm);
	float* useg  = reinterpret_cast<float*>(acc + n);  // [ck][n]
	float* sseg  = useg + (int64_t)ck * n;             // [ck][n]
	float* v     = sseg + (int64_t)ck * n;
	float* s0    = v + n;      // s at the segment start
	float* ubA   = s0 + n;
	float* ubB   = ubA + n;
	float* thb   = ubB + n;
	float* beb   = thb + n;
	int* list_s  = reinterpret_cast<int*>(beb + n);
	int* list_in = list_s + n;
	int* nact    = list_in + a.n_in;
	uint32_t* xb = reinterpret_cast<uint32_t*>(nact + 2);
	StepSmem const m{acc, list_in, list_s, nact, xb};
	int const nck      = (a.T + ck - 1) / ck + 1;
	const float* vck   = a.vck + (int64_t)b * nck * n;
	const float* gc    = a.gcounts + (int64_t)b * n;
	int64_t const pstride = a.in_syn + a.rec_syn + 2 * (int64_t)n;
	float* pw_in  = a.part + (int64_t)b * pstride;
	float* pw_rec = pw_in + a.in_syn;
	float* pth    = pw_rec + a.rec_syn;
	float* pbe    = pth + n;
	for (int64_t e = threadIdx.x; e < a.in_syn + a.rec_syn; e += blockDim.x) pw_in[e] = 0.0f;
	for (int j = threadIdx.x; j < n; j += blockDim.x) {
		ubA[j] = 0.0f;  // ubar_{T+1}
		thb[j] = 0.0f;
		beb[j] = 0.0f;
	}
	float* ub_next = ubA;
	float* ub_cur  = ubB;
	int const nseg = (a.T + ck - 1) / ck;
	for (int c = nseg - 1; c >= 0; c--) {
		int const t0 = c * ck, t1 = min(a.T, t0 + ck);
		// ---- recompute u_t, s_t of steps t0+1 .. t1 from the checkpoint v_{t0} ----
		__syncthreads();
		for (int j = threadIdx.x; j < n; j += blockDim.x) {
			v[j]  = vck[(int64_t)c * n + j];
			s0[j] = t0 == 0 ? 0.0f : a.spikes[((int64_t)b * a.T + (t0 - 1)) * n + j];
		}
		for (int t = t0 + 1; t <= t1; t++) {
			int const idx = t - t0 - 1;
			load_x(a, b, t - 1, xb);
			lif_step(a, m, idx == 0 ? s0 : sseg + (int64_t)(idx - 1) * n, v, useg + (int64_t)idx * n,
			         sseg + (int64_t)idx * n);
		}
		// ---- adjoint through the segment, t = t1 .. t0+1 ----
		for (int t = t1; t >= t0 + 1; t--) {
			int const idx      = t - t0 - 1;
			const float* u_t   = useg + (int64_t)idx * n;
			const float* s_t   = sseg + (int64_t)idx * n;
			const float* s_tm1 = idx == 0 ? s0 : sseg + (int64_t)(idx - 1) * n;
			load_x(a, b, t - 1, xb);
			if (threadIdx.x < 2) nact[threadIdx.x] = 0;
			// per neuron i: r_i = sum_j W_rec[i->j] ubar_{t+1, j} along row i of the ELL matrix (CSR
			// order, one fused multiply-add per entry), then the adjoint update of neuron i
			for (int i = threadIdx.x; i < n; i += blockDim.x) {
				int const d = __ldg(a.deg + i);
				float acc   = 0.0f;
				int q       = 0;
				for (; q + 4 <= d; q += 4) {
					int32_t j[4];
					float w[4];
#pragma unroll
					for (int u = 0; u < 4; u++) {
						j[u] = __ldg(a.ell_nb + (int64_t)(q + u) * n + i);
						w[u] = __ldg(a.ell_w + (int64_t)(q + u) * n + i);
					}
#pragma unroll
					for (int u = 0; u < 4; u++) acc = __fmaf_rn(w[u], ub_next[j[u]], acc);
				}
				for (; q < d; q++)
					acc = __fmaf_rn(__ldg(a.ell_w + (int64_t)q * n + i), ub_next[__ldg(a.ell_nb + (int64_t)q * n + i)], acc);
				float const th   = a.theta[i];
				float const vbar = __fmul_rn(a.beta[i], ub_next[i]);
				float const sbar = __fsub_rn(__fadd_rn(gc[i], acc), __fmul_rn(th, vbar));
				float const sg   = surrogate(__fsub_rn(u_t[i], th), a.slope, a.sg_scale);
				float const ubar = __fadd_rn(vbar, __fmul_rn(sg, sbar));
				ub_cur[i]        = ubar;
				thb[i] = __fsub_rn(thb[i], __fadd_rn(__fmul_rn(sg, sbar), __fmul_rn(s_t[i], vbar)));
				float const vprev = idx == 0 ? vck[(int64_t)c * n + i]
				                             : __fsub_rn(useg[(int64_t)(idx - 1) * n + i],
				                                         __fmul_rn(th, sseg[(int64_t)(idx - 1) * n + i]));
				beb[i] = __fadd_rn(beb[i], __fmul_rn(vprev, ubar));
			}
			__syncthreads();  // xb and nact ready; every thread is done reading ub_next's neighbours
			build_lists(a, m, s_tm1);
			__syncthreads();
			// event-driven weight gradients of step t: rows of the sources active at t - 1
			int const ni = nact[0], ns = nact[1];
			for (int q = warp; q < ni + ns; q += nwarps) {
				bool const inp    = q < ni;
				int const src     = inp ? list_in[q] : list_s[q - ni];
				float const sv    = inp ? 1.0f : s_tm1[src];
				int64_t const e0  = inp ? __ldg(a.in_off + src) : __ldg(a.rec_off + src);
				int64_t const e1  = inp ? __ldg(a.in_off + src + 1) : __ldg(a.rec_off + src + 1);
				const int32_t* nb = inp ? a.in_nb : a.rec_nb;
				float* pw         = inp ? pw_in : pw_rec;
				for (int64_t base = e0; base < e1; base += 32 * kRowChunk) {
					float g[kRowChunk], old[kRowChunk];
#pragma unroll
					for (int u = 0; u < kRowChunk; u++) {
						int64_t const e = base + u * 32 + lane;
						bool const ok   = e < e1;
						int32_t const d = ok ? __ldg(nb + e) : 0;
						old[u]          = ok ? pw[e] : 0.0f;
						g[u]            = ok ? __fmul_rn(sv, ub_cur[d]) : 0.0f;
					}
#pragma unroll
					for (int u = 0; u < kRowChunk; u++) {
						int64_t const e = base + u * 32 + lane;
						if (e < e1) pw[e] = __fadd_rn(old[u], g[u]);
					}
				}
			}
			__syncthreads();
			float* tmp = ub_next;
			ub_next    = ub_cur;
			ub_cur     = tmp;
		}
	}
	__syncthreads();
	for (int j = threadIdx.x; j < n; j += blockDim.x) {
		pth[j] = thb[j];
		pbe[j] = beb[j];
	}
}

// out[e] = sum over samples b = 0..B-1 (in order) of part[b][e].
__global__ void k_lif_reduce(const float* __restrict__ part, int B, int64_t stride, int64_t len, float* __restrict__ out) {
	for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < len; e += (int64_t)gridDim.x * blockDim.x) {
		float s = 0.0f;
		for (int b = 0; b < B; b++) s = __fadd_rn(s, part[(int64_t)b * stride + e]);
		out[e] = s;
	}
}

__global__ void k_lif_quantize(const float* __restrict__ w, int64_t n, long long* __restrict__ q) {
	for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
		q[e] = __double2ll_rn((double)w[e] * kFix);
}

int lfail(int code, std::string const& msg) { return set_last_error(code, msg); }

#define L_CUDA_TRY(x)                                                                                     \
	do {                                                                                                  \
		cudaError_t const e_ = (x);                                                                       \
		if (e_ != cudaSuccess) return lfail(SPICE_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
	} while (0)

size_t forward_smem(int n, int n_in) {
	int const nw = (n_in + 31) / 32;
	return 8 * (size_t)n + 4 * (size_t)(4 * n) + 4 * (size_t)(n + n_in + 2) + 4 * (size_t)nw + 16;
}

size_t backward_smem(int n, int n_in, int ck) {
	int const nw = (n_in + 31) / 32;
	return 8 * (size_t)n + 4 * (size_t)(2 * (size_t)ck * n + 6 * (size_t)n) + 4 * (size_t)(n + n_in + 2) +
	       4 * (size_t)nw + 16;
}

// ell_w[q][i] = w_rec[off[i] + q] for q < deg[i], else 0.
__global__ void k_lif_ell_weights(const float* __restrict__ w_rec, const int64_t* __restrict__ off,
                                  const int32_t* __restrict__ deg, int n, int dmax, float* __restrict__ ell_w) {
	int64_t const total = (int64_t)dmax * n;
	for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
		int const q = (int)(e / n), i = (int)(e - (int64_t)q * n);
		ell_w[e]    = q < __ldg(deg + i) ? __ldg(w_rec + __ldg(off + i) + q) : 0.0f;
	}
}

int check_common(spice_lif_layer* L, int batch, int steps, int ck, float slope) {
	if (!L) return lfail(SPICE_EINVAL, "layer must not be NULL");
	if (batch <= 0 || steps <= 0) return lfail(SPICE_EINVAL, "batch and steps must be > 0");
	if (ck <= 0) return lfail(SPICE_EINVAL, "checkpoint_every must be > 0");
	if (!(slope > 0)) return lfail(SPICE_EINVAL, "slope must be > 0");
	return SPICE_OK;
}

int max_optin_smem(int* out) {
	int dev = 0;
	L_CUDA_TRY(cudaGetDevice(&dev));
	L_CUDA_TRY(cudaDeviceGetAttribute(out, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
	return SPICE_OK;
}

LifArgs make_args(spice_lif_layer* L, int steps, int ck, int relaxed, float slope, const uint32_t* x,
                  const float* w_in, const float* w_rec, const float* theta, const float* beta) {
	LifArgs a{};
	a.n_in    = L->n_in;
	a.n       = L->n;
	a.nw_in   = (L->n_in + 31) / 32;
	a.T       = steps;
	a.ck      = ck;
	a.relaxed = relaxed ? 1 : 0;
	a.slope   = slope;
	a.sg_scale = relaxed ? 0.5f * slope : 1.0f;
	a.in_off  = L->in_off;
	a.in_nb   = L->in_nb;
	a.rec_off = L->rec_off;
	a.rec_nb  = L->rec_nb;
	a.wq_in   = L->wq;
	a.wq_rec  = L->wq + L->in_syn;
	a.x       = x;
	a.w_in    = w_in;
	a.w_rec   = w_rec;
	a.theta   = theta;
	a.beta    = beta;
	a.in_syn  = L->in_syn;
	a.rec_syn = L->rec_syn;
	a.deg     = L->deg;
	a.ell_nb  = L->ell_nb;
	a.ell_w   = L->ell_w;
	return a;
}

cudaError_t quantize(spice_lif_layer* L, const float* w_in, const float* w_rec, cudaStream_t st) {
	if (L->in_syn) k_lif_quantize<<<256, 256, 0, st>>>(w_in, L->in_syn, L->wq);
	if (L->rec_syn) k_lif_quantize<<<256, 256, 0, st>>>(w_rec, L->rec_syn, L->wq + L->in_syn);
	return cudaGetLastError();
}

}  // namespace

extern "C" int spice_lif_layer_create(int n_in, int n_rec, const int64_t* in_off, const int32_t* in_nb,
                                      const int64_t* rec_off, const int32_t* rec_nb, spice_lif_layer** out) {
	if (!out) return lfail(SPICE_EINVAL, "out must not be NULL");
	*out = nullptr;
	if (n_in < 0 || n_rec <= 0) return lfail(SPICE_EINVAL, "n_in must be >= 0 and n_rec > 0");
	if (!in_off || !rec_off || (!in_nb && in_off[n_in] > 0) || (!rec_nb && rec_off[n_rec] > 0))
		return lfail(SPICE_EINVAL, "CSR arrays must not be NULL");
	int64_t const in_syn = in_off[n_in], rec_syn = rec_off[n_rec];
	for (int64_t e = 0; e < in_syn; e++)
		if (in_nb[e] < 0 || in_nb[e] >= n_rec) return lfail(SPICE_EINVAL, "input CSR target out of range");
	for (int64_t e = 0; e < rec_syn; e++)
		if (rec_nb[e] < 0 || rec_nb[e] >= n_rec) return lfail(SPICE_EINVAL, "recurrent CSR target out of range");
	for (int i = 0; i < n_in; i++)
		if (in_off[i + 1] < in_off[i]) return lfail(SPICE_EINVAL, "input CSR offsets must not decrease");
	for (int i = 0; i < n_rec; i++)
		if (rec_off[i + 1] < rec_off[i]) return lfail(SPICE_EINVAL, "recurrent CSR offsets must not decrease");
	auto* L    = new spice_lif_layer();
	L->n_in    = n_in;
	L->n       = n_rec;
	L->in_syn  = in_syn;
	L->rec_syn = rec_syn;
	cudaError_t e = cudaMalloc(&L->in_off, sizeof(int64_t) * (n_in + 1));
	if (e == cudaSuccess) e = cudaMalloc(&L->in_nb, sizeof(int32_t) * std::max<int64_t>(in_syn, 1));
	if (e == cudaSuccess) e = cudaMalloc(&L->rec_off, sizeof(int64_t) * (n_rec + 1));
	if (e == cudaSuccess) e = cudaMalloc(&L->rec_nb, sizeof(int32_t) * std::max<int64_t>(rec_syn, 1));
	if (e == cudaSuccess) e = cudaMalloc(&L->wq, sizeof(long long) * std::max<int64_t>(in_syn + rec_syn, 1));
	if (e == cudaSuccess) e = cudaMemcpy(L->in_off, in_off, sizeof(int64_t) * (n_in + 1), cudaMemcpyHostToDevice);
	if (e == cudaSuccess && in_syn) e = cudaMemcpy(L->in_nb, in_nb, sizeof(int32_t) * in_syn, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(L->rec_off, rec_off, sizeof(int64_t) * (n_rec + 1), cudaMemcpyHostToDevice);
	if (e == cudaSuccess && rec_syn) e = cudaMemcpy(L->rec_nb, rec_nb, sizeof(int32_t) * rec_syn, cudaMemcpyHostToDevice);
	// ELL view of the recurrent rows
	std::vector<int32_t> deg(n_rec);
	int dmax = 0;
	for (int i = 0; i < n_rec; i++) {
		deg[i] = (int32_t)(rec_off[i + 1] - rec_off[i]);
		dmax   = std::max(dmax, deg[i]);
	}
	L->dmax = dmax;
	std::vector<int32_t> ell((size_t)std::max(dmax, 1) * n_rec, 0);
	for (int i = 0; i < n_rec; i++)
		for (int q = 0; q < deg[i]; q++) ell[(size_t)q * n_rec + i] = rec_nb[rec_off[i] + q];
	if (e == cudaSuccess) e = cudaMalloc(&L->deg, sizeof(int32_t) * n_rec);
	if (e == cudaSuccess) e = cudaMalloc(&L->ell_nb, sizeof(int32_t) * ell.size());
	if (e == cudaSuccess) e = cudaMalloc(&L->ell_w, sizeof(float) * ell.size());
	if (e == cudaSuccess) e = cudaMemcpy(L->deg, deg.data(), sizeof(int32_t) * n_rec, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(L->ell_nb, ell.data(), sizeof(int32_t) * ell.size(), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) {
		spice_lif_layer_destroy(L);
		return lfail(e == cudaErrorMemoryAllocation ? SPICE_ENOMEM : SPICE_ECUDA,
		             std::string("layer allocation: ") + cudaGetErrorString(e));
	}
	*out = L;
	return SPICE_OK;
}

extern "C" int spice_lif_layer_destroy(spice_lif_layer* L) {
	if (!L) return SPICE_OK;
	cudaDeviceSynchronize();
	cudaFree(L->in_off);
	cudaFree(L->in_nb);
	cudaFree(L->rec_off);
	cudaFree(L->rec_nb);
	cudaFree(L->wq);
	cudaFree(L->deg);
	cudaFree(L->ell_nb);
	cudaFree(L->ell_w);
	cudaFree(L->partial);
	delete L;
	return SPICE_OK;
}

extern "C" int spice_lif_layer_synapses(spice_lif_layer* L, int64_t* in_syn, int64_t* rec_syn) {
	if (!L) return lfail(SPICE_EINVAL, "layer must not be NULL");
	if (in_syn) *in_syn = L->in_syn;
	if (rec_syn) *rec_syn = L->rec_syn;
	return SPICE_OK;
}

extern "C" int spice_lif_forward(spice_lif_layer* L, int batch, int steps, int checkpoint_every, int relaxed,
                                 float slope, const uint32_t* x_bits, const float* w_in, const float* w_rec,
                                 const float* theta, const float* beta, float* counts, float* spikes, float* v_ckpt,
                                 void* stream) {
	int r = check_common(L, batch, steps, checkpoint_every, slope);
	if (r != SPICE_OK) return r;
	if (!x_bits || !w_rec || !theta || !beta || !counts || !spikes || !v_ckpt || (!w_in && L->in_syn))
		return lfail(SPICE_EINVAL, "device arrays must not be NULL");
	size_t const smem = forward_smem(L->n, L->n_in);
	int optin         = 0;
	if ((r = max_optin_smem(&optin)) != SPICE_OK) return r;
	if (smem > (size_t)optin) return lfail(SPICE_EINVAL, "layer too large for one CTA's shared memory");
	auto const st = (cudaStream_t)stream;
	L_CUDA_TRY(quantize(L, w_in, w_rec, st));
	LifArgs a  = make_args(L, steps, checkpoint_every, relaxed, slope, x_bits, w_in, w_rec, theta, beta);
	a.counts   = counts;
	a.spikes   = spikes;
	a.vck      = v_ckpt;
	L_CUDA_TRY(cudaFuncSetAttribute(k_lif_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	k_lif_forward<<<batch, kLifThreads, smem, st>>>(a);
	L_CUDA_TRY(cudaGetLastError());
	return SPICE_OK;
}

extern "C" int spice_lif_backward(spice_lif_layer* L, int batch, int steps, int checkpoint_every, int relaxed,
                                  float slope, const uint32_t* x_bits, const float* w_in, const float* w_rec,
                                  const float* theta, const float* beta, const float* spikes, const float* v_ckpt,
                                  const float* grad_counts, float* grad_w_in, float* grad_w_rec, float* grad_theta,
                                  float* grad_beta, void* stream) {
	int r = check_common(L, batch, steps, checkpoint_every, slope);
	if (r != SPICE_OK) return r;
	if (!x_bits || !w_rec || !theta || !beta || !spikes || !v_ckpt || !grad_counts || !grad_w_rec || !grad_theta ||
	    !grad_beta || ((!w_in || !grad_w_in) && L->in_syn))
		return lfail(SPICE_EINVAL, "device arrays must not be NULL");
	size_t const smem = backward_smem(L->n, L->n_in, checkpoint_every);
	int optin         = 0;
	if ((r = max_optin_smem(&optin)) != SPICE_OK) return r;
	if (smem > (size_t)optin)
		return lfail(SPICE_EINVAL, "checkpoint segment too large for one CTA's shared memory (lower checkpoint_every)");
	int64_t const stride = L->in_syn + L->rec_syn + 2 * (int64_t)L->n;
	int64_t const need   = stride * batch;
	auto const st        = (cudaStream_t)stream;
	if (need > L->partial_cap) {
		L_CUDA_TRY(cudaStreamSynchronize(st));
		cudaFree(L->partial);
		L->partial     = nullptr;
		L->partial_cap = 0;
		L_CUDA_TRY(cudaMalloc(&L->partial, sizeof(float) * need));
		L->partial_cap = need;
	}
	L_CUDA_TRY(quantize(L, w_in, w_rec, st));
	if (L->dmax > 0) k_lif_ell_weights<<<256, 256, 0, st>>>(w_rec, L->rec_off, L->deg, L->n, L->dmax, L->ell_w);
	LifArgs a = make_args(L, steps, checkpoint_every, relaxed, slope, x_bits, w_in, w_rec, theta, beta);
	a.spikes  = const_cast<float*>(spikes);
	a.vck     = const_cast<float*>(v_ckpt);
	a.gcounts = grad_counts;
	a.part    = L->partial;
	L_CUDA_TRY(cudaFuncSetAttribute(k_lif_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	k_lif_backward<<<batch, kLifThreads, smem, st>>>(a);
	L_CUDA_TRY(cudaGetLastError());
	if (L->in_syn) k_lif_reduce<<<512, 256, 0, st>>>(L->partial, batch, stride, L->in_syn, grad_w_in);
	if (L->rec_syn) k_lif_reduce<<<512, 256, 0, st>>>(L->partial + L->in_syn, batch, stride, L->rec_syn, grad_w_rec);
	k_lif_reduce<<<8, 256, 0, st>>>(L->partial + L->in_syn + L->rec_syn, batch, stride, L->n, grad_theta);
	k_lif_reduce<<<8, 256, 0, st>>>(L->partial + L->in_syn + L->rec_syn + L->n, batch, stride, L->n, grad_beta);
	L_CUDA_TRY(cudaGetLastError());
	return SPICE_OK;
}
