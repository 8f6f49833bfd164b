// gen.cu -- fixed_probability adjacency generated on the GPU, bit-identical to the reference.
//
// The reference (spice/src/topology.cpp:78-112) walks ONE serial xoroshiro128+ stream per
// projection: row by row, a double `noise` restarts at 0, accumulates exponential gaps
// -scale*log(u) (u = canonical<double, left-open>, scale = 1/p - 1), and emits
// dst = index + round(noise) until dst >= dst_count or index >= max_degree; the stopping draw is
// consumed.  The GPU splits that into
//   1. gaps    -- counter-based: thread j of super-chunk m jumps straight to draw 65536 m + 256 j
//                 with a GF(2) jump polynomial (rng.h) and writes 256 gaps.  All draws that any
//                 row can consume (src * (max_degree + 1)) are generated in parallel.  Each gap is
//                 also rounded to a fixed-point integer (2^-s units) and prefix-summed; integer
//                 sums are associative, so F[d] - F[d'] is the exact sum of the rounded gaps.
//   2. rows    -- the only serial part: a row's first draw depends on where the previous row
//                 stopped.  One warp per projection finds each row's stop index with a 32-way
//                 search on F (two rounds for rows up to 1024 draws).  The search answer equals
//                 the reference's (sequential double sums) unless a running sum lies within the
//                 proven error bound of a .5 rounding tie at the stop index; such rows are redone
//                 by one lane with the reference's exact sequential double loop.
//   3. offsets -- exclusive scan of the row lengths (int64, csr.h:97).
//   4. fill    -- one thread per row re-adds that row's gaps in order and writes its neighbours.
// Every double addition happens in the reference's order, so the neighbour lists are identical
// whenever the device log agrees with the host C library's log on which side of .5 a running
// sum falls (ties are not observed; the parity tests compare whole CSRs and checksums).
#include <math.h>

#include <algorithm>
#include <vector>

#include "internal.h"
#include "kernels.h"

namespace spice_gb300 {

namespace {

constexpr int kSuper    = 65536;  // draws per super-chunk
constexpr int kSubDraws = 256;    // draws per thread
constexpr int kGenThreads = 256;  // kSuper = kGenThreads * kSubDraws

__device__ __forceinline__ void basis_xor(const u128* basis, u128 poly, uint64_t& s0, uint64_t& s1) {
	uint64_t a0 = 0, a1 = 0;
#pragma unroll 4
	for (int i = 0; i < 64; i++)
		if ((poly.lo >> i) & 1) {
			a0 ^= basis[i].lo;
			a1 ^= basis[i].hi;
		}
#pragma unroll 4
	for (int i = 0; i < 64; i++)
		if ((poly.hi >> i) & 1) {
			a0 ^= basis[64 + i].lo;
			a1 ^= basis[64 + i].hi;
		}
	s0 = a0;
	s1 = a1;
}

// Start states of every super-chunk: T^(65536 m)(s) for m < nsuper.
__global__ void k_superstates(u128 seed, const u128* __restrict__ polys, int64_t nsuper,
                              u128* __restrict__ out) {
	__shared__ u128 basis[kBasis];
	if (threadIdx.x == 0) {
		uint64_t s0 = seed.lo, s1 = seed.hi;
		for (int i = 0; i < kBasis; i++) {
			basis[i] = {s0, s1};
			xoro_next(s0, s1);
		}
	}
	__syncthreads();
	for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < nsuper;
	     m += (int64_t)gridDim.x * blockDim.x) {
		uint64_t s0, s1;
		basis_xor(basis, polys[m], s0, s1);
		out[m] = {s0, s1};
	}
}

// gaps[d] = -scale * log(canonical<double, true>(draw d)) for d < ndraws; F[d] = the thread's
// inclusive prefix of round(gap * 2^s) over its 256 draws; tot[chunk] = that chunk's sum.
__global__ void __launch_bounds__(kGenThreads) k_gaps(const u128* __restrict__ superstates,
                                                      const u128* __restrict__ subpolys, double scale,
                                                      double fx_scale, int64_t ndraws, double* __restrict__ gaps,
                                                      uint64_t* __restrict__ F, uint64_t* __restrict__ tot) {
	__shared__ u128 basis[kBasis];
	int64_t const m = blockIdx.x;
	if (threadIdx.x == 0) {
		uint64_t s0 = superstates[m].lo, s1 = superstates[m].hi;
		for (int i = 0; i < kBasis; i++) {
			basis[i] = {s0, s1};
			xoro_next(s0, s1);
		}
	}
	__syncthreads();
	int64_t const first = m * kSuper + (int64_t)threadIdx.x * kSubDraws;
	if (first >= ndraws) return;
	uint64_t s0, s1;
	basis_xor(basis, subpolys[threadIdx.x], s0, s1);
	int64_t const n = min((int64_t)kSubDraws, ndraws - first);
	double* out     = gaps + first;
	uint64_t* fo    = F + first;
	uint64_t acc    = 0;
	for (int r = 0; r < n; r++) {
		uint64_t const u = xoro_next(s0, s1);
		double const g   = -scale * log(canonical_f64_leftopen(u));
		out[r]           = g;
		acc += (uint64_t)__double2ll_rn(g * fx_scale);
		fo[r] = acc;
	}
	tot[first / kSubDraws] = acc;
}

// Exclusive scan (wrapping uint64) of the chunk totals, one CTA.
__global__ void k_scan_u64(uint64_t* __restrict__ v, int64_t n) {
	__shared__ uint64_t warp_sums[32];
	__shared__ uint64_t carry_s;
	int const lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
	uint64_t carry = 0;
	for (int64_t b0 = 0; b0 < n; b0 += blockDim.x) {
		int64_t const i = b0 + threadIdx.x;
		uint64_t const x = i < n ? v[i] : 0;
		uint64_t incl    = x;
		for (int d = 1; d < 32; d <<= 1) {
			uint64_t const o = __shfl_up_sync(0xffffffffu, incl, d);
			if (lane >= d) incl += o;
		}
		if (lane == 31) warp_sums[wid] = incl;
		__syncthreads();
		if (wid == 0) {
			uint64_t const sv = lane < nw ? warp_sums[lane] : 0;
			uint64_t si       = sv;
			for (int d = 1; d < 32; d <<= 1) {
				uint64_t const o = __shfl_up_sync(0xffffffffu, si, d);
				if (lane >= d) si += o;
			}
			warp_sums[lane] = si - sv;
			if (lane == nw - 1) carry_s = si;
		}
		__syncthreads();
		if (i < n) v[i] = carry + warp_sums[wid] + incl - x;
		carry += carry_s;
		__syncthreads();
	}
}

// F[d] += prefix of the chunks before d's chunk: F becomes the global inclusive prefix.
__global__ void k_add_chunk_prefix(uint64_t* __restrict__ F, const uint64_t* __restrict__ cp, int64_t n) {
	for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < n; d += (int64_t)gridDim.x * blockDim.x)
		F[d] += cp[d / kSubDraws];
}

// The row chain: one warp per projection.
struct RowJob {
	const double* gaps;
	const uint64_t* F;   // global inclusive prefix of the fixed-point gaps
	int64_t ndraws;
	int64_t src_count;
	int64_t dst_count;
	int64_t max_degree;
	int shift;           // fixed-point gaps are round(gap * 2^shift)
	int32_t* row_len;
	unsigned long long* fallbacks;
};

// The reference's row loop (topology.cpp:93-110) for one row starting at draw D.
__device__ int64_t exact_row(RowJob const& job, int64_t D) {
	double noise = 0;
	for (int64_t j = 0;; j++) {
		noise += job.gaps[D + j];
		int64_t const dst = j + (int64_t)(int32_t)round(noise);
		if ((dst >= job.dst_count) | (j >= job.max_degree)) return j;
	}
}

__global__ void __launch_bounds__(32) k_rows(const RowJob* __restrict__ jobs) {
	RowJob const job = jobs[blockIdx.x];
	int const lane   = threadIdx.x;
	int64_t const md = job.max_degree;
	int64_t const dc = job.dst_count;
	double const ulp_fac = 1.1102230246251565e-16;  // 2^-53
	unsigned long long fb = 0;
	int64_t D = 0;
	for (int64_t r = 0; r < job.src_count; r++) {
		uint64_t const base = D > 0 ? __ldg(job.F + D - 1) : 0ull;
		// C(j): gap sum over draws D..D+j >= dst - j - 0.5, in fixed point:
		//        S(j) >= (2 (dst - j) - 1) 2^(shift-1)
		auto S = [&](int64_t j) -> int64_t { return (int64_t)(__ldg(job.F + D + j) - base); };
		auto T = [&](int64_t j) -> int64_t { return (2 * (dc - j) - 1) * (1ll << (job.shift - 1)); };
		int64_t lo = 0, hi = md, L = md;
		while (true) {
			int64_t const n = hi - lo;
			if (n <= 32) {
				bool const c = lane < n && S(lo + lane) >= T(lo + lane);
				unsigned const mk = __ballot_sync(0xffffffffu, c);
				L = mk ? lo + __ffs(mk) - 1 : hi;
				break;
			}
			// probe the right end of 32 sub-intervals; probes past the range test hi - 1
			int64_t const step = (n + 31) / 32;
			int64_t const j    = min(lo + (lane + 1) * step - 1, hi - 1);
			bool const c       = S(j) >= T(j);
			unsigned const mk  = __ballot_sync(0xffffffffu, c);
			if (!mk) {  // C(hi - 1) is false, so C is false below hi
				L = hi;
				break;
			}
			int const f         = __ffs(mk) - 1;
			int64_t const jf    = __shfl_sync(0xffffffffu, j, f);
			int64_t const jprev = __shfl_sync(0xffffffffu, j, f > 0 ? f - 1 : 0);
			hi = jf;                       // C(jf) is true
			lo = f > 0 ? jprev + 1 : lo;   // C is false up to the previous probe
		}
		// the answer is exact unless S is within the error bound of the threshold at L or L-1:
		// |seq. double sum - exact sum| <= (j+1) sum * 2^-53, |fixed - exact| <= (j+1)/2 units
		bool amb = false;
		if (lane == 0) {
			for (int q = 0; q < 2; q++) {
				int64_t const j = q == 0 ? L : L - 1;
				if (j < 0 || (q == 0 && L >= md)) continue;
				int64_t const sj = S(j);
				double const margin = 2.0 * (double)(j + 1) * (0.5 + fabs((double)sj) * ulp_fac) + 4.0;
				if (fabs((double)(sj - T(j))) <= margin) amb = true;
			}
			if (amb) {
				L = exact_row(job, D);
				fb++;
			}
		}
		L = __shfl_sync(0xffffffffu, L, 0);
		if (lane == 0) job.row_len[r] = (int32_t)L;
		D += L + 1;
	}
	if (lane == 0 && fb) atomicAdd(job.fallbacks, fb);
}

// Thread per row: re-add the row's gaps in order and write its neighbours.
__global__ void k_fill(const double* __restrict__ gaps, const int64_t* __restrict__ off,
                       int64_t src_count, int32_t* __restrict__ nb) {
	int64_t const r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (r >= src_count) return;
	int64_t const o0 = off[r], o1 = off[r + 1];
	const double* g  = gaps + o0 + r;  // row r starts at draw off[r] + r (one stop draw per row)
	double noise     = 0;
	for (int64_t j = 0; j < o1 - o0; j++) {
		noise += g[j];
		nb[o0 + j] = (int32_t)j + (int32_t)round(noise);
	}
}

}  // namespace

// Host side ------------------------------------------------------------------------------------

unsigned long long g_gen_fallbacks = 0;

int64_t fp_max_degree(int64_t dst_count, double p) {
	// fixed_probability::size() / src_count (topology.cpp:75-78, 90)
	double const m = (double)dst_count * p;
	return (int64_t)(m + 3 * sqrt(m * (1 - p)));
}

cudaError_t generate_fixed_probability(cudaStream_t stream, std::vector<GenRequest>& reqs) {
	cudaError_t err = cudaSuccess;
#define CK(x)                         \
	do {                              \
		err = (x);                    \
		if (err != cudaSuccess) goto fail; \
	} while (0)
	std::vector<double*> gaps(reqs.size(), nullptr);
	std::vector<uint64_t*> fxs(reqs.size(), nullptr);
	std::vector<uint64_t*> tots(reqs.size(), nullptr);
	unsigned long long* d_fallbacks = nullptr;
	std::vector<int32_t*> lens(reqs.size(), nullptr);
	std::vector<u128*> sstates(reqs.size(), nullptr);
	std::vector<RowJob> jobs;
	std::vector<int> job_req;
	RowJob* d_jobs   = nullptr;
	u128* d_subpolys = nullptr;
	std::vector<u128*> d_polys(reqs.size(), nullptr);
	{
		// x^(256 j) mod P, j < 256: the offsets of the threads inside a super-chunk
		std::vector<u128> sub(kGenThreads);
		u128 const step = gf2_xpow(kSubDraws);
		sub[0]          = {1, 0};
		for (int j = 1; j < kGenThreads; j++) sub[j] = gf2_mulmod(sub[j - 1], step);
		CK(cudaMalloc(&d_subpolys, sizeof(u128) * kGenThreads));
		CK(cudaMemcpyAsync(d_subpolys, sub.data(), sizeof(u128) * kGenThreads, cudaMemcpyHostToDevice, stream));
		CK(cudaStreamSynchronize(stream));
	}
	for (size_t q = 0; q < reqs.size(); q++) {
		GenRequest& r = reqs[q];
		r.offsets     = nullptr;
		r.neighbors   = nullptr;
		r.synapses    = 0;
		CK(cudaMalloc(&r.offsets, sizeof(int64_t) * (r.src + 1)));
		CK(cudaMemsetAsync(r.offsets, 0, sizeof(int64_t) * (r.src + 1), stream));
		if (r.src == 0 || r.dst == 0 || r.p == 0) continue;
		int64_t const md = fp_max_degree(r.dst, r.p);
		int64_t const nd = r.src * (md + 1);  // every row consumes at most max_degree + 1 draws
		int64_t const nsuper = (nd + kSuper - 1) / kSuper;
		CK(cudaMalloc(&gaps[q], sizeof(double) * nd));
		CK(cudaMalloc(&fxs[q], sizeof(uint64_t) * nd));
		int64_t const nchunks = (nd + kSubDraws - 1) / kSubDraws;
		CK(cudaMalloc(&tots[q], sizeof(uint64_t) * nchunks));
		// fixed-point scale: row sums stay below dst + 36.74 * scale (-log u <= 53 ln 2) + slack
		double const bound = (double)r.dst + 36.75 * (1 / r.p - 1) + 4;
		int shift = 61 - (int)ceil(log2(bound));
		shift     = std::min(40, std::max(shift, 8));
		CK(cudaMalloc(&lens[q], sizeof(int32_t) * r.src));
		CK(cudaMemsetAsync(lens[q], 0, sizeof(int32_t) * r.src, stream));
		CK(cudaMalloc(&sstates[q], sizeof(u128) * nsuper));
		std::vector<u128> polys(nsuper);
		u128 const stride = gf2_xpow(kSuper);
		polys[0]          = {1, 0};
		for (int64_t m = 1; m < nsuper; m++) polys[m] = gf2_mulmod(polys[m - 1], stride);
		CK(cudaMalloc(&d_polys[q], sizeof(u128) * nsuper));
		CK(cudaMemcpyAsync(d_polys[q], polys.data(), sizeof(u128) * nsuper, cudaMemcpyHostToDevice, stream));
		k_superstates<<<(unsigned)std::min<int64_t>((nsuper + 255) / 256, 1024), 256, 0, stream>>>(r.seed, d_polys[q], nsuper,
		                                                                                     sstates[q]);
		k_gaps<<<(unsigned)nsuper, kGenThreads, 0, stream>>>(sstates[q], d_subpolys, 1 / r.p - 1, ldexp(1.0, shift),
		                                                     nd, gaps[q], fxs[q], tots[q]);
		k_scan_u64<<<1, 1024, 0, stream>>>(tots[q], nchunks);
		k_add_chunk_prefix<<<1216, 256, 0, stream>>>(fxs[q], tots[q], nd);
		CK(cudaGetLastError());
		CK(cudaStreamSynchronize(stream));  // the host-side polys vector goes out of scope
		if (!d_fallbacks) {
			CK(cudaMalloc(&d_fallbacks, sizeof(unsigned long long)));
			CK(cudaMemsetAsync(d_fallbacks, 0, sizeof(unsigned long long), stream));
		}
		jobs.push_back({gaps[q], fxs[q], nd, r.src, r.dst, md, shift, lens[q], d_fallbacks});
		job_req.push_back((int)q);
	}
	if (!jobs.empty()) {
		CK(cudaMalloc(&d_jobs, sizeof(RowJob) * jobs.size()));
		CK(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(RowJob) * jobs.size(), cudaMemcpyHostToDevice, stream));
		k_rows<<<(unsigned)jobs.size(), 32, 0, stream>>>(d_jobs);
		CK(cudaGetLastError());
		for (size_t j = 0; j < jobs.size(); j++) {
			GenRequest& r = reqs[job_req[j]];
			CK(scan_row_lengths(stream, lens[job_req[j]], r.src, r.offsets));
		}
		CK(cudaStreamSynchronize(stream));
		for (size_t j = 0; j < jobs.size(); j++) {
			GenRequest& r = reqs[job_req[j]];
			CK(cudaMemcpy(&r.synapses, r.offsets + r.src, sizeof(int64_t), cudaMemcpyDeviceToHost));
			// whole 16-byte blocks: delivery reads targets as aligned int4 blocks
			CK(cudaMalloc(&r.neighbors, sizeof(int32_t) * ((r.synapses + 3) / 4 * 4 + 4)));
			k_fill<<<(unsigned)((r.src + 255) / 256), 256, 0, stream>>>(gaps[job_req[j]], r.offsets, r.src,
			                                                            r.neighbors);
			CK(cudaGetLastError());
		}
		CK(cudaStreamSynchronize(stream));
	}
	for (size_t q = 0; q < reqs.size(); q++)
		if (!reqs[q].neighbors) CK(cudaMalloc(&reqs[q].neighbors, sizeof(int32_t)));
fail:
	cudaStreamSynchronize(stream);
	for (auto* g : gaps) cudaFree(g);
	for (auto* f : fxs) cudaFree(f);
	for (auto* t : tots) cudaFree(t);
	if (d_fallbacks) {
		unsigned long long fb = 0;
		cudaMemcpy(&fb, d_fallbacks, sizeof(fb), cudaMemcpyDeviceToHost);
		g_gen_fallbacks += fb;
		cudaFree(d_fallbacks);
	}
	for (auto* l : lens) cudaFree(l);
	for (auto* s : sstates) cudaFree(s);
	for (auto* p : d_polys) cudaFree(p);
	cudaFree(d_jobs);
	cudaFree(d_subpolys);
	if (err != cudaSuccess)
		for (auto& r : reqs) {
			cudaFree(r.offsets);
			cudaFree(r.neighbors);
			r.offsets   = nullptr;
			r.neighbors = nullptr;
		}
	return err;
#undef CK
}

}  // namespace spice_gb300

namespace spice_gb300 {

// The generator pipeline of generate_fixed_probability for one projection, with every scratch
// buffer supplied by the caller (GenScratch) and the neighbours written to a caller buffer of
// `capacity` entries.  Allocates nothing.  Synchronises `stream` once, to read the synapse count.
cudaError_t generate_fixed_probability_into(cudaStream_t stream, int64_t src, int64_t dst, double p, u128 seed,
                                            GenScratch const& sc, int64_t* offsets, int32_t* neighbors,
                                            int64_t capacity, int64_t* synapses) {
	*synapses = 0;
	if (src == 0 || dst == 0 || p == 0) return cudaMemsetAsync(offsets, 0, sizeof(int64_t) * (src + 1), stream);
	int64_t const md     = fp_max_degree(dst, p);
	int64_t const nd     = src * (md + 1);
	int64_t const nsuper = (nd + kSuper - 1) / kSuper;
	int64_t const nchunk = (nd + kSubDraws - 1) / kSubDraws;
	if (nd > sc.max_draws || src > sc.max_src || nsuper > sc.max_super) return cudaErrorInvalidValue;
	// jump polynomials: x^(65536 m) and x^(256 j) mod P, computed once per process on the host
	struct Polys {
		u128 sub[kGenThreads];
		u128 sup[64];
	};
	static Polys const polys = [] {  // thread-safe one-time initialisation
		Polys q;
		u128 const step = gf2_xpow(kSubDraws), stride = gf2_xpow(kSuper);
		q.sub[0] = {1, 0};
		for (int j = 1; j < kGenThreads; j++) q.sub[j] = gf2_mulmod(q.sub[j - 1], step);
		q.sup[0] = {1, 0};
		for (int m = 1; m < 64; m++) q.sup[m] = gf2_mulmod(q.sup[m - 1], stride);
		return q;
	}();
	if (nsuper > 64) return cudaErrorInvalidValue;
	cudaError_t e = cudaMemcpyAsync(sc.subpolys, polys.sub, sizeof(polys.sub), cudaMemcpyHostToDevice, stream);
	if (e == cudaSuccess) e = cudaMemcpyAsync(sc.polys, polys.sup, sizeof(u128) * nsuper, cudaMemcpyHostToDevice, stream);
	if (e != cudaSuccess) return e;
	double const bound = (double)dst + 36.75 * (1 / p - 1) + 4;
	int shift          = 61 - (int)ceil(log2(bound));
	shift              = std::min(40, std::max(shift, 8));
	k_superstates<<<1, 256, 0, stream>>>(seed, sc.polys, nsuper, sc.superstates);
	k_gaps<<<(unsigned)nsuper, kGenThreads, 0, stream>>>(sc.superstates, sc.subpolys, 1 / p - 1, ldexp(1.0, shift), nd,
	                                                     sc.gaps, sc.fx, sc.tots);
	k_scan_u64<<<1, 1024, 0, stream>>>(sc.tots, nchunk);
	k_add_chunk_prefix<<<1216, 256, 0, stream>>>(sc.fx, sc.tots, nd);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	RowJob const job = {sc.gaps, sc.fx, nd, src, dst, md, shift, sc.lens, sc.fallbacks};
	if ((e = cudaMemsetAsync(sc.lens, 0, sizeof(int32_t) * src, stream)) != cudaSuccess) return e;
	if ((e = cudaMemsetAsync(sc.fallbacks, 0, sizeof(unsigned long long), stream)) != cudaSuccess) return e;
	if ((e = cudaMemcpyAsync(sc.job, &job, sizeof(RowJob), cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
	k_rows<<<1, 32, 0, stream>>>(reinterpret_cast<const RowJob*>(sc.job));
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	if ((e = scan_row_lengths_into(stream, sc.lens, src, offsets, sc.block_sums)) != cudaSuccess) return e;
	int64_t total = 0;
	if ((e = cudaMemcpyAsync(&total, offsets + src, sizeof(int64_t), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
	if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
	*synapses = total;
	if (total > capacity) return cudaErrorInvalidValue;
	k_fill<<<(unsigned)((src + 255) / 256), 256, 0, stream>>>(sc.gaps, offsets, src, neighbors);
	return cudaGetLastError();
}

size_t gen_row_job_bytes() { return sizeof(RowJob); }

namespace {
// w[e] = wmax * canonical<float>(draw e) for e < n: the PerSynapseInit stream of a weighted
// synapse (synapse_population.h:34-41), one draw per synapse in CSR order; thread j of super-chunk
// m jumps to draw 65536 m + 256 j like k_gaps.
__global__ void __launch_bounds__(kGenThreads) k_init_weights(const u128* __restrict__ superstates,
                                                              const u128* __restrict__ subpolys, float wmax, int64_t n,
                                                              float* __restrict__ w) {
	__shared__ u128 basis[kBasis];
	int64_t const m = blockIdx.x;
	if (threadIdx.x == 0) {
		uint64_t s0 = superstates[m].lo, s1 = superstates[m].hi;
		for (int i = 0; i < kBasis; i++) {
			basis[i] = {s0, s1};
			xoro_next(s0, s1);
		}
	}
	__syncthreads();
	int64_t const first = m * kSuper + (int64_t)threadIdx.x * kSubDraws;
	if (first >= n) return;
	uint64_t s0, s1;
	basis_xor(basis, subpolys[threadIdx.x], s0, s1);
	int64_t const cnt = min((int64_t)kSubDraws, n - first);
	for (int r = 0; r < cnt; r++) w[first + r] = __fmul_rn(wmax, canonical_f32(xoro_next(s0, s1)));
}
}  // namespace

cudaError_t init_synapse_weights(cudaStream_t stream, u128 seed, int64_t n, float wmax, float* w) {
	if (n <= 0) return cudaSuccess;
	int64_t const nsuper = (n + kSuper - 1) / kSuper;
	std::vector<u128> polys(nsuper), sub(kGenThreads);
	u128 const stride = gf2_xpow(kSuper), step = gf2_xpow(kSubDraws);
	polys[0] = {1, 0};
	for (int64_t m = 1; m < nsuper; m++) polys[m] = gf2_mulmod(polys[m - 1], stride);
	sub[0] = {1, 0};
	for (int j = 1; j < kGenThreads; j++) sub[j] = gf2_mulmod(sub[j - 1], step);
	u128 *d_polys = nullptr, *d_sub = nullptr, *d_states = nullptr;
	cudaError_t e = cudaMalloc(&d_polys, sizeof(u128) * nsuper);
	if (e == cudaSuccess) e = cudaMalloc(&d_sub, sizeof(u128) * kGenThreads);
	if (e == cudaSuccess) e = cudaMalloc(&d_states, sizeof(u128) * nsuper);
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_polys, polys.data(), sizeof(u128) * nsuper, cudaMemcpyHostToDevice, stream);
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_sub, sub.data(), sizeof(u128) * kGenThreads, cudaMemcpyHostToDevice, stream);
	if (e == cudaSuccess) {
		k_superstates<<<(unsigned)std::min<int64_t>((nsuper + 255) / 256, 1024), 256, 0, stream>>>(seed, d_polys, nsuper,
		                                                                                     d_states);
		k_init_weights<<<(unsigned)nsuper, kGenThreads, 0, stream>>>(d_states, d_sub, wmax, n, w);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(stream);  // the host vectors go out of scope
	cudaFree(d_polys);
	cudaFree(d_sub);
	cudaFree(d_states);
	return e;
}

}  // namespace spice_gb300
