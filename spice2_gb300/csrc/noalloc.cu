// noalloc.cu -- fixed_probability generation for callers that cannot allocate device memory.
//
// Some hosts of this library must not call cudaMalloc: real-time loops whose device memory is
// fixed up front (an allocation can block and can fail at any time), and runtimes that hand the
// library a fixed arena of buffers because they own every device allocation themselves (a
// framework's caching allocator, a JNI/cgo host with its own pool).  spice_fixed_probability_noalloc
// gives them the GPU generator of fixed_probability adjacency with every intermediate buffer
// (exponential gaps, their fixed-point prefix, row lengths, scan sums, jump polynomials) placed in
// one file-scope static device array of fixed size.  The caller passes only the output buffers.
// The call synchronises its stream once (it reads the synapse count back to the host before the
// adjacency is filled).
#include <stdint.h>

#include <cuda.h>

#include <mutex>
#include <string>

#include "internal.h"
#include "kernels.h"
#include "spice_gb300.h"

namespace spice_gb300 {
int set_last_error(int code, std::string const& msg);
}

using namespace spice_gb300;

namespace {

constexpr int64_t kMaxDraws = int64_t(1) << 18;  // src * (max_degree + 1)
constexpr int64_t kMaxSrc   = int64_t(1) << 16;  // rows
constexpr int64_t kMaxSuper = 64;                // 65536-draw super-chunks (covers kMaxDraws)

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kOffGaps   = 0;
constexpr size_t kOffFx     = kOffGaps + align256(sizeof(double) * kMaxDraws);
constexpr size_t kOffTots   = kOffFx + align256(sizeof(uint64_t) * kMaxDraws);
constexpr size_t kOffLens   = kOffTots + align256(sizeof(uint64_t) * (kMaxDraws / 256 + 1));
constexpr size_t kOffSuper  = kOffLens + align256(sizeof(int32_t) * kMaxSrc);
constexpr size_t kOffPolys  = kOffSuper + align256(sizeof(u128) * kMaxSuper);
constexpr size_t kOffSub    = kOffPolys + align256(sizeof(u128) * kMaxSuper);
constexpr size_t kOffSums   = kOffSub + align256(sizeof(u128) * 256);
constexpr size_t kOffJob    = kOffSums + align256(sizeof(int64_t) * (kMaxSrc / 1024 + 2));
constexpr size_t kOffFb     = kOffJob + 1024;
constexpr size_t kScratchBytes = kOffFb + 256;  // about 4.3 MiB

// The scratch of every call on this device.  Every GPU that loads the library holds it until the
// process exits.  Calls share it: two calls whose work overlaps on the GPU race.
static __device__ __align__(256) unsigned char g_gen_scratch[kScratchBytes];

constexpr int kMaxDevices = 256;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices]  = {};
CUcontext g_scratch_ctx[kMaxDevices] = {};  // the context the address was looked up in

// cuCtxGetCurrent, reached through the runtime (the library does not link the driver API).
using ctx_get_fn = CUresult (*)(CUcontext*);
ctx_get_fn ctx_get_current() {
	static ctx_get_fn fn = [] {
		void* f = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
		    q != cudaDriverEntryPointSuccess)
			f = nullptr;
		return reinterpret_cast<ctx_get_fn>(f);
	}();
	return fn;
}

// Host code cannot use &g_gen_scratch (that is a host-side stand-in, not a device address): the
// device address is looked up with the device current, the first time a device is used and again
// whenever the calling thread's current context is not the one of the last lookup (after a
// cudaDeviceReset the old address belongs to a destroyed context; the lookup itself creates the new
// primary context).
int scratch_address(void** out) {
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return set_last_error(SPICE_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
	if (dev < 0 || dev >= kMaxDevices) return set_last_error(SPICE_EINVAL, "device ordinal out of range");
	ctx_get_fn const get = ctx_get_current();
	CUcontext ctx = nullptr;
	if (get && get(&ctx) != CUDA_SUCCESS) ctx = nullptr;
	std::lock_guard<std::mutex> lock(g_setup_mutex);
	if (!g_scratch_ptr[dev] || !ctx || ctx != g_scratch_ctx[dev]) {
		void* p = nullptr;
		e       = cudaGetSymbolAddress(&p, g_gen_scratch);
		if (e != cudaSuccess || !p)
			return set_last_error(SPICE_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
		if (get && get(&ctx) != CUDA_SUCCESS) ctx = nullptr;
		g_scratch_ptr[dev] = p;
		g_scratch_ctx[dev] = ctx;
	}
	*out = g_scratch_ptr[dev];
	return SPICE_OK;
}

}  // namespace

extern "C" int spice_fixed_probability_noalloc(int64_t src_count, int64_t dst_count, double p, uint64_t seed_lo,
                                               uint64_t seed_hi, int64_t* offsets, int32_t* neighbors,
                                               int64_t neighbors_capacity, int64_t* synapses_out, void* stream) {
	if (synapses_out) *synapses_out = 0;
	if (!offsets || (!neighbors && neighbors_capacity > 0) || !synapses_out)
		return set_last_error(SPICE_EINVAL, "offsets, neighbors and synapses_out must not be NULL");
	if (!(0 <= p && p <= 1))
		return set_last_error(SPICE_EINVAL, "spice_fixed_probability_noalloc: p must be in [0, 1]");
	if (src_count < 0 || dst_count < 0 || src_count >= INT32_MAX || dst_count >= INT32_MAX)
		return set_last_error(SPICE_EINVAL, "spice_fixed_probability_noalloc: src_count and dst_count must be in [0, 2^31 - 1)");
	if (src_count > kMaxSrc)
		return set_last_error(SPICE_EINVAL, "spice_fixed_probability_noalloc: src_count " + std::to_string(src_count) +
		                                         " exceeds the static scratch limit of " + std::to_string(kMaxSrc) + " rows");
	int64_t const draws = (src_count > 0 && dst_count > 0 && p > 0) ? src_count * (fp_max_degree(dst_count, p) + 1) : 0;
	if (draws > kMaxDraws)
		return set_last_error(SPICE_EINVAL, "spice_fixed_probability_noalloc: src_count * (max_degree + 1) = " +
		                                         std::to_string(draws) + " draws exceeds the static scratch limit of " +
		                                         std::to_string(kMaxDraws));
	void* base = nullptr;
	int r      = scratch_address(&base);
	if (r != SPICE_OK) return r;
	unsigned char* b = static_cast<unsigned char*>(base);
	GenScratch sc;
	sc.gaps        = reinterpret_cast<double*>(b + kOffGaps);
	sc.fx          = reinterpret_cast<uint64_t*>(b + kOffFx);
	sc.tots        = reinterpret_cast<uint64_t*>(b + kOffTots);
	sc.lens        = reinterpret_cast<int32_t*>(b + kOffLens);
	sc.superstates = reinterpret_cast<u128*>(b + kOffSuper);
	sc.polys       = reinterpret_cast<u128*>(b + kOffPolys);
	sc.subpolys    = reinterpret_cast<u128*>(b + kOffSub);
	sc.block_sums  = reinterpret_cast<int64_t*>(b + kOffSums);
	sc.job         = b + kOffJob;
	sc.fallbacks   = reinterpret_cast<unsigned long long*>(b + kOffFb);
	sc.max_draws   = kMaxDraws;
	sc.max_src     = kMaxSrc;
	sc.max_super   = kMaxSuper;
	if (gen_row_job_bytes() > 1024) return set_last_error(SPICE_ESTATE, "row job descriptor larger than its scratch slot");
	int64_t syn = 0;
	cudaError_t e = generate_fixed_probability_into(static_cast<cudaStream_t>(stream), src_count, dst_count, p,
	                                               u128{seed_lo, seed_hi}, sc, offsets, neighbors,
	                                               neighbors_capacity, &syn);
	*synapses_out = syn;
	if (e == cudaErrorInvalidValue && syn > neighbors_capacity)
		return set_last_error(SPICE_EOVERFLOW, "neighbors buffer holds " + std::to_string(neighbors_capacity) +
		                                           " entries, the adjacency has " + std::to_string(syn));
	if (e != cudaSuccess)
		return set_last_error(SPICE_ECUDA, std::string("fixed_probability generation failed: ") + cudaGetErrorString(e));
	return SPICE_OK;
}
