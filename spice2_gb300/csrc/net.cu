// net.cu -- the C ABI (include/spice_gb300.h): network construction, the step loop, readback.
//
// Host-side order of the reference is kept exactly: seeds are consumed in the order of
// snn::add_population (stateful populations, neuron_population.h:56-60), snn::connect (one per
// connection, synapse_population.h:30-31) and snn::step (one per step, snn.cpp:12); the per-step
// dt is the Kahan-compensated increment (numeric.h:9-15, snn.cpp:8-10).  Construction is lazy:
// the adjacency of every fixed_probability connection is generated on the GPU together, the first
// time the network steps or a CSR is read.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cstring>
#include <thread>
#include <cstdio>
#include <string>
#include <vector>

#include "spice_gb300.h"
#include "internal.h"
#include "mulround.h"
#include "kernels.h"

using namespace spice_gb300;

namespace {

thread_local std::string g_err;

int fail(int code, std::string msg) {
	g_err = std::move(msg);
	return code;
}

// The reference's precondition failure text (spice/src/util/assert.cpp:8-15).
int pre_failed(const char* file_line, const char* cond) {
	return fail(SPICE_EINVAL, std::string("Assertion failed (") + file_line + "): " + cond);
}

#define CUDA_TRY(x)                                                                                  \
	do {                                                                                             \
		cudaError_t const e_ = (x);                                                                  \
		if (e_ != cudaSuccess) return fail(SPICE_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
	} while (0)

#define TRY(x)                    \
	do {                          \
		int const r_ = (x);       \
		if (r_ != SPICE_OK) return r_; \
	} while (0)

constexpr int64_t kRunCap = 1024;  // steps of dt / seed / jump tables prepared per chunk

// memcpy of a large host buffer, split over a few threads (host memory bandwidth is per core).
void parallel_copy(void* dst, const void* src, size_t bytes) {
	constexpr size_t kChunk = size_t(4) << 20;
	int const nt = (int)std::min<size_t>(8, (bytes + kChunk - 1) / kChunk);
	if (nt <= 1) {
		std::memcpy(dst, src, bytes);
		return;
	}
	size_t const per = (bytes / nt + 63) & ~size_t(63);
	std::vector<std::thread> th;
	size_t done = per;  // [0, per) is copied by this thread; parts no thread could be started for too
	for (int i = 1; i < nt; i++) {
		size_t const o = per * i;
		if (o >= bytes) break;
		try {
			th.emplace_back([=] { std::memcpy((char*)dst + o, (const char*)src + o, std::min(per, bytes - o)); });
			done = std::min(bytes, o + per);
		} catch (...) {
			break;
		}
	}
	std::memcpy(dst, src, std::min(per, bytes));
	if (done < bytes) std::memcpy((char*)dst + done, (const char*)src + done, bytes - done);
	for (auto& x : th) x.join();
}

template <class T>
int dalloc(spice_net* n, T** p, size_t count, bool zero = true) {
	size_t const bytes = sizeof(T) * (count > 0 ? count : 1);
	cudaError_t e      = cudaMalloc((void**)p, bytes);
	if (e != cudaSuccess) {
		*p = nullptr;
		return fail(e == cudaErrorMemoryAllocation ? SPICE_ENOMEM : SPICE_ECUDA,
		            std::string("cudaMalloc(") + std::to_string(bytes) + " bytes): " + cudaGetErrorString(e));
	}
	n->allocations.push_back(*p);
	if (zero) CUDA_TRY(cudaMemsetAsync(*p, 0, bytes, n->stream));
	return SPICE_OK;
}

bool stateful_model(int m) { return m == LIF || m == LIF_COND; }

u128 seed_next(spice_net* n) {  // seed_seq::operator++(int) (random.h:163-167)
	u128 const r = n->seed;
	n->seed      = murmur3_u128(n->seed);
	return r;
}

float kahan_next(spice_net* n) {  // kahan_sum<float>::operator+= then the reset at >= 1 s
	volatile float y = n->dt - n->kahan_c;
	volatile float t = n->kahan_sum + y;
	n->kahan_c       = (t - n->kahan_sum) - y;
	n->kahan_sum     = t;
	if (n->kahan_sum >= 1) n->kahan_sum = 0;
	return y;
}

// ---- profiling ----
constexpr size_t kEventPool = 4096;  // CUDA events of the profiling pool (two per launch)

// Reads every recorded pair (complete once the streams are idle) into the per-kind statistics, with
// the device spans of the delivery launches, and empties the pool.
int harvest(spice_net* n) {
	if (n->ev_pending.empty()) return SPICE_OK;
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	if (n->stream_src) CUDA_TRY(cudaStreamSynchronize(n->stream_src));
	std::vector<unsigned long long> span;
	if (n->d_span) {
		span.resize(kEventPool);
		CUDA_TRY(cudaMemcpy(span.data(), n->d_span, sizeof(unsigned long long) * kEventPool, cudaMemcpyDeviceToHost));
	}
	for (auto const& pr : n->ev_pending) {
		float ms = 0;
		CUDA_TRY(cudaEventElapsedTime(&ms, n->ev_pool[pr.second], n->ev_pool[pr.second + 1]));
		KernelStat& st = n->stats[pr.first];
		st.ms += ms;
		st.launches++;
		if (!span.empty() && pr.second + 1 < (int)kEventPool && span[pr.second] && span[pr.second + 1]) {
			unsigned long long const t0 = ~span[pr.second], t1 = span[pr.second + 1];  // start kept complemented
			if (t1 >= t0) {
				st.span_ms += (double)(t1 - t0) * 1e-6;
				st.span_launches++;
			}
		}
	}
	n->ev_pending.clear();
	n->ev_used = 0;
	if (n->d_span) CUDA_TRY(cudaMemsetAsync(n->d_span, 0, sizeof(unsigned long long) * kEventPool, n->stream));
	return SPICE_OK;
}

int ev_begin(spice_net* n, int kind, int* slot, cudaStream_t st = nullptr) {
	*slot = -1;
	if (!n->profiling) return SPICE_OK;
	if (n->ev_used + 2 > n->ev_pool.size()) {
		TRY(harvest(n));
		while (n->ev_pool.size() < kEventPool) {
			cudaEvent_t e;
			CUDA_TRY(cudaEventCreate(&e));
			n->ev_pool.push_back(e);
		}
	}
	*slot = (int)n->ev_used;
	n->ev_used += 2;
	n->ev_pending.push_back({kind, *slot});
	CUDA_TRY(cudaEventRecord(n->ev_pool[*slot], st ? st : n->stream));
	return SPICE_OK;
}

int ev_end(spice_net* n, int slot, cudaStream_t st = nullptr) {
	if (slot >= 0) CUDA_TRY(cudaEventRecord(n->ev_pool[slot + 1], st ? st : n->stream));
	return SPICE_OK;
}

}  // namespace

namespace spice_gb300 {
// Records the calling thread's last error for spice_last_error() (for other translation units).
int set_last_error(int code, std::string const& msg) { return fail(code, msg); }

// k_neurons CTA kind of a per-neuron population: 3 for a LIF whose every input group adds to V
// through a 16-bit counter of word 0 (the fast replay), else 0.
int neuron_block_kind(PopDev const& P) {
	bool fast = P.model == LIF && P.W == 1 && P.ngroups <= 2 && !P.pull;
	for (int g = 0; g < P.ngroups && fast; g++)
		fast = P.group_field[g] == 0 && P.group_bits[g] == 16 && P.group_word[g] == 0 && P.group_shift[g] == 16 * g;
	return fast ? 3 : 0;
}
}  // namespace spice_gb300

// ------------------------------------------------------------------------------------------------
// construction
// ------------------------------------------------------------------------------------------------

extern "C" const char* spice_last_error(void) { return g_err.c_str(); }

extern "C" int spice_net_create(float dt, float max_delay, const uint32_t* seeds, int nseeds, spice_net** out) {
	if (!out) return fail(SPICE_EINVAL, "out must not be NULL");
	*out = nullptr;
	if (nseeds <= 0 || !seeds)
		return pre_failed("random.h:151", "il.size() > 0 && \"Please provide at least 1 seed to seed_seq\"");
	auto* n = new spice_net();
	n->dt   = dt;
	// _max_delay(std::round(max_delay / dt)) (snn.h:18-19)
	n->max_delay = (int64_t)roundf(max_delay / dt);
	n->seed      = murmur3_bytes(seeds, 4ull * (uint64_t)nseeds);
	cudaError_t e = cudaGetDevice(&n->device);
	if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking);
	if (e != cudaSuccess) {
		delete n;
		return fail(SPICE_ECUDA, std::string("no usable CUDA device: ") + cudaGetErrorString(e));
	}
	int r = dalloc(n, &n->d_events, 1);
	if (r != SPICE_OK) {
		spice_net_destroy(n);
		return r;
	}
	*out = n;
	return SPICE_OK;
}

extern "C" int spice_net_destroy(spice_net* n) {
	if (!n) return SPICE_OK;
	if (n->stream) cudaStreamSynchronize(n->stream);
	for (void* p : n->allocations) cudaFree(p);
	for (auto& c : n->conns) {
		cudaFree((void*)c.d.off);
		cudaFree((void*)c.d.nb);
		if (c.nb16) cudaFree(c.nb16);
	}
	if (n->h_dt) cudaFreeHost(n->h_dt);
	if (n->h_raster) cudaFreeHost(n->h_raster);
	if (n->h_rcounts) cudaFreeHost(n->h_rcounts);
	if (n->h_seeds) cudaFreeHost(n->h_seeds);
	if (n->h_pstatus) cudaFreeHost(n->h_pstatus);
	for (auto e : n->ev_pool) cudaEventDestroy(e);
	if (n->stream_src) {
		cudaStreamSynchronize(n->stream_src);
		cudaStreamDestroy(n->stream_src);
	}
	if (n->ev_tab) cudaEventDestroy(n->ev_tab);
	for (int b = 0; b < 2; b++)
		if (n->ev_chunk[b]) cudaEventDestroy(n->ev_chunk[b]);
	for (int q = 0; q < 2; q++) {
		if (n->ev_src[q]) cudaEventDestroy(n->ev_src[q]);
		if (n->ev_free[q]) cudaEventDestroy(n->ev_free[q]);
	}
	if (n->stream) cudaStreamDestroy(n->stream);
	delete n;
	return SPICE_OK;
}

namespace {
// A negative population size as the reference's neuron adapters meet it: a stateless adapter checks
// the size (neuron_population.h:35), a per-population one too (:92), and a stateful one's
// std::vector<neuron>(size) throws std::length_error (a std::logic_error) before its own check.
// kind: 0 stateless, 1 stateful, 2 per-population update.
int negative_size(int kind) {
	if (kind == 0) return pre_failed("neuron_population.h:35", "size >= 0");
	if (kind == 2) return pre_failed("neuron_population.h:92", "size >= 0");
	return fail(SPICE_EINVAL, "cannot create std::vector larger than max_size()");
}
}  // namespace

extern "C" int spice_add_population(spice_net* n, int model, int64_t size, const float* params, int np,
                                    int* pop_out) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (n->prepared) return fail(SPICE_ESTATE, "populations must be added before the network first steps");
	if (model < POISSON || model > EXTERNAL) return fail(SPICE_EINVAL, "unknown neuron model");
	if (!(size >= 0)) return negative_size(model == POISSON ? 0 : model == EXTERNAL ? 2 : 1);
	if (!(n->max_delay >= 1)) return pre_failed("neuron_population.h:108", "max_delay >= 1");
	if (size >= INT32_MAX) return pre_failed("topology.cpp:35", "0 <= src_count_ && src_count_ < std::numeric_limits<Int32>::max()");
	if ((int)n->pops.size() >= kMaxPops) return fail(SPICE_EINVAL, "too many populations");
	if (np < 0 || (np > 0 && !params)) return fail(SPICE_EINVAL, "bad params");
	Pop p{};
	PopDev& d = p.d;
	memset(&d, 0, sizeof d);
	d.model  = model;
	d.size   = size;
	d.nwords = (int)((size + 31) / 32);
	for (int f = 0; f < 3; f++) d.field_slot[f] = -1;
	if (model == POISSON) {
		d.p0 = np > 0 ? params[0] : 20.0f;
	} else if (model == LIF) {
		d.p0 = np > 0 ? params[0] : 0.02f;
		d.p1 = np > 1 ? params[1] : 20.0f;
		d.p2 = np > 2 ? params[2] : 50.0f;
	}
	p.stateful = stateful_model(model);
	if (p.stateful) {
		p.seed = seed_next(n);  // stateful_neuron_adapter: rng(seed++) (neuron_population.h:56-60)
		TRY(dalloc(n, &d.V, size));
		TRY(dalloc(n, &d.T, size));
		if (model == LIF_COND) {
			TRY(dalloc(n, &d.Gex, size));
			TRY(dalloc(n, &d.Gin, size));
			std::vector<float> v0(size, -0.06f);  // samples/vogels.cpp:12
			CUDA_TRY(cudaMemcpyAsync(d.V, v0.data(), sizeof(float) * size, cudaMemcpyHostToDevice, n->stream));
			CUDA_TRY(cudaStreamSynchronize(n->stream));
		}
	}
	n->pops.push_back(std::move(p));
	n->ext_t_set.push_back(0);
	if (pop_out) *pop_out = (int)n->pops.size() - 1;
	return SPICE_OK;
}

extern "C" int spice_add_user_population(spice_net* n, int64_t size, int stateful, int neuron_bytes,
                                         const void* init_neuron, spice_user_update_fn fn, void* ctx, int* pop_out) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (n->prepared) return fail(SPICE_ESTATE, "populations must be added before the network first steps");
	if (!fn) return fail(SPICE_EINVAL, "a user population needs an update function");
	if (!(size >= 0)) return negative_size(stateful ? 1 : 0);
	if (size >= INT32_MAX) return pre_failed("topology.cpp:35", "0 <= src_count_ && src_count_ < std::numeric_limits<Int32>::max()");
	if ((int)n->pops.size() >= kMaxPops) return fail(SPICE_EINVAL, "too many populations");
	if (stateful && (neuron_bytes <= 0 || !init_neuron))
		return fail(SPICE_EINVAL, "a stateful user model needs its neuron struct size and initial value");
	Pop p{};
	PopDev& d = p.d;
	memset(&d, 0, sizeof d);
	d.model  = USER;
	d.size   = size;
	d.nwords = (int)((size + 31) / 32);
	for (int f = 0; f < 3; f++) d.field_slot[f] = -1;
	p.stateful = stateful != 0;
	p.ufn      = (void*)fn;
	p.uctx     = ctx;
	if (p.stateful) {
		p.seed   = seed_next(n);  // stateful_neuron_adapter: rng(seed++) (neuron_population.h:56-60)
		d.ubytes = neuron_bytes;
		char* st = nullptr;
		TRY(dalloc(n, &st, (size_t)std::max<int64_t>(size, 1) * neuron_bytes, false));
		std::vector<char> h((size_t)std::max<int64_t>(size, 1) * neuron_bytes);
		for (int64_t i = 0; i < std::max<int64_t>(size, 1); i++)
			memcpy(h.data() + i * neuron_bytes, init_neuron, (size_t)neuron_bytes);
		CUDA_TRY(cudaMemcpy(st, h.data(), h.size(), cudaMemcpyHostToDevice));
		d.ustate = st;
	}
	n->pops.push_back(std::move(p));
	n->ext_t_set.push_back(0);
	if (pop_out) *pop_out = (int)n->pops.size() - 1;
	return SPICE_OK;
}

extern "C" int spice_user_field(spice_net* n, int pop, int byte_offset, int* field_out) {
	if (!n || !field_out) return fail(SPICE_EINVAL, "NULL argument");
	if (pop < 0 || pop >= (int)n->pops.size() || n->pops[pop].d.model != USER || !n->pops[pop].stateful)
		return fail(SPICE_EINVAL, "not a stateful user population");
	Pop& P = n->pops[pop];
	if (byte_offset < 0 || byte_offset % 4 || byte_offset + 4 > P.d.ubytes)
		return fail(SPICE_EINVAL, "a field must be a float member of the neuron struct");
	for (int f = 0; f < P.nfields; f++)
		if (P.field_offset[f] == byte_offset) {
			*field_out = f;
			return SPICE_OK;
		}
	if (n->prepared) return fail(SPICE_ESTATE, "fields must be registered before the network first steps");
	if (P.nfields >= 3) return fail(SPICE_EINVAL, "at most 3 fields of a user neuron can be synapse targets");
	P.field_offset[P.nfields] = byte_offset;
	*field_out                = P.nfields++;
	return SPICE_OK;
}

namespace {
int parse_synapse(spice_net* n, int dst, int synapse, const float* params, int np, Conn& c) {
	float* w   = &c.d.weight;
	int* field = &c.d.field;
	if (synapse == SPICE_SYNAPSE_FIXED_WEIGHT) {
		if (np < 1 || !params) return fail(SPICE_EINVAL, "fixed_weight needs params {weight[, field]}");
	} else if (synapse == SPICE_SYNAPSE_ISTDP) {
		if (np < 5 || !params) return fail(SPICE_EINVAL, "istdp needs params {w0, field, eta, rho0, tau}");
		if (!(params[4] > 0)) return fail(SPICE_EINVAL, "istdp tau must be > 0");
		c.w0   = params[0];
		c.rho0 = params[3];
		c.tau  = params[4];
		c.d.eta = params[2];
	} else if (synapse == SPICE_SYNAPSE_COUNT) {
		if (np < 1 || !params) return fail(SPICE_EINVAL, "count needs params {scale[, field]}");
		c.tau = 1.0f;
	} else if (synapse == SPICE_SYNAPSE_USER_PLASTIC) {
		if (np < 3 || !params) return fail(SPICE_EINVAL, "user plastic synapses need params {field, synapse_bytes, weight_word}");
		c.ubytes      = (int)params[1];
		c.weight_word = (int)params[2];
		c.init_seed   = np > 3 && params[3] != 0.0f;  // PerSynapseInit: the ctor's rng(seed++)
		if (c.ubytes <= 0 || c.ubytes % 4 || c.weight_word < 0 || 4 * c.weight_word + 4 > c.ubytes)
			return fail(SPICE_EINVAL, "a user synapse struct is a multiple of 4 bytes and holds its weight word");
		c.d.plastic = synapse;
		c.d.weight  = 0.0f;
		c.d.field   = (int)params[0];
		c.tau       = 1.0f;
		int const m = n->pops[dst].d.model;
		if (m == USER ? (c.d.field < 0 || c.d.field >= n->pops[dst].nfields) : (c.d.field < 0 || c.d.field > 2 || (m == LIF && c.d.field != 0)))
			return fail(SPICE_EINVAL, "the synapse's target field does not exist in the target neuron model");
		return SPICE_OK;
	} else if (synapse == SPICE_SYNAPSE_USER_DELIVER) {
		if (np < 2 || !params) return fail(SPICE_EINVAL, "user deliver synapses need params {synapse_bytes, reads_source[, init]}");
		if (n->pops[dst].d.model != USER || !n->pops[dst].stateful)
			return fail(SPICE_EINVAL, "a synapse with its own deliver() code targets a stateful user population");
		c.ubytes       = (int)params[0];
		c.reads_source = params[1] != 0.0f;
		c.init_seed    = np > 2 && params[2] != 0.0f;
		if (c.ubytes < 0) return fail(SPICE_EINVAL, "synapse struct size must be >= 0");
		c.d.plastic = 0;
		c.d.weight  = 0.0f;
		c.d.field   = 0;
		c.udeliver  = true;
		return SPICE_OK;
	} else if (synapse == SPICE_SYNAPSE_WEIGHTED) {
		if (np < 1 || !params) return fail(SPICE_EINVAL, "weighted needs params {wmax[, field[, source]]}");
		c.weighted = true;
		c.wmax     = params[0];
		c.wsource  = np > 2 ? (int)params[2] : 0;
		if (c.wsource < 0 || c.wsource > 2) return fail(SPICE_EINVAL, "weighted source must be 0, 1 or 2");
	} else {
		return fail(SPICE_EINVAL, "unknown synapse model");
	}
	c.d.plastic = synapse == SPICE_SYNAPSE_WEIGHTED ? 0 : synapse;
	*w          = c.weighted ? 0.0f : params[0];
	*field      = np > 1 ? (int)params[1] : 0;
	int const m = n->pops[dst].d.model;
	if (m == USER ? (*field < 0 || *field >= n->pops[dst].nfields) : (*field < 0 || *field > 2 || (m == LIF && *field != 0)))
		return fail(SPICE_EINVAL, "the synapse's target field does not exist in the target neuron model");
	return SPICE_OK;
}

int conn_common(spice_net* n, int src, int dst, float delay, int* d_out) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (n->prepared) return fail(SPICE_ESTATE, "connections must be added before the network first steps");
	if (src < 0 || src >= (int)n->pops.size() || dst < 0 || dst >= (int)n->pops.size())
		return fail(SPICE_EINVAL, "population id out of range");
	if (!n->pops[dst].stateful)
		return fail(SPICE_EINVAL, "the target population of a connection must be stateful (StatefulNeuron<DstNeur>, snn.h:29-31)");
	if ((int)n->conns.size() >= kMaxConns) return fail(SPICE_EINVAL, "too many connections");
	// Int const d = std::round(delay / _dt) (snn.h:33-38)
	int64_t const d = (int64_t)roundf(delay / n->dt);
	if (!(d >= 1)) return pre_failed("snn.h:35", "d >= 1 && \"The delay must be at least 1dt.\"");
	if (!(d <= n->max_delay))
		return pre_failed("snn.h:36", "d <= _max_delay && \"The delay of a synapse population may not exceed the maximum delay of the network.\"");
	*d_out = (int)d;
	return SPICE_OK;
}
}  // namespace

extern "C" int spice_connect_fixed_probability(spice_net* n, int src, int dst, double p, float delay, int synapse,
                                               const float* params, int np, int* conn_out) {
	int d = 0;
	TRY(conn_common(n, src, dst, delay, &d));
	if (!(0 <= p && p <= 1)) return pre_failed("topology.cpp:73", "0 <= p && p <= 1");
	// the csr of an empty source has no offsets (csr.h:70), which generate refuses (topology.cpp:82)
	if (n->pops[src].d.size == 0) return pre_failed("topology.cpp:82", "offsets.size() > src_count");
	Conn c{};
	memset(&c.d, 0, sizeof c.d);
	TRY(parse_synapse(n, dst, synapse, params, np, c));
	c.d.src = src;
	c.d.dst = dst;
	c.d.delay  = d;
	c.d.src_size = n->pops[src].d.size;
	c.d.dst_size = n->pops[dst].d.size;
	n->conns.push_back(c);
	// synapse_population ctor: _graph(c, seed++) (synapse_population.h:30-31)
	n->conns.back().gseed = seed_next(n);
	n->gen_pending.push_back({(int)n->conns.size() - 1, n->conns.back().gseed, p});
	// PerSynapseInit: rng(seed++) after the adjacency's (synapse_population.h:34-41)
	if ((c.weighted && c.wsource != 2) || c.init_seed) n->conns.back().wseed = seed_next(n);
	if (conn_out) *conn_out = (int)n->conns.size() - 1;
	return SPICE_OK;
}

extern "C" int spice_connect_adj_list(spice_net* n, int src, int dst, const int32_t* pairs, int64_t npairs, float delay,
                                      int synapse, const float* params, int np, int* conn_out) {
	int d = 0;
	TRY(conn_common(n, src, dst, delay, &d));
	if (npairs < 0 || (npairs > 0 && !pairs)) return fail(SPICE_EINVAL, "bad pairs");
	// the csr of an empty source has no offsets (csr.h:70), which Topology::generate refuses (topology.cpp:48)
	if (n->pops[src].d.size == 0) return pre_failed("topology.cpp:48", "offsets.size() > src_count");
	Conn c{};
	memset(&c.d, 0, sizeof c.d);
	TRY(parse_synapse(n, dst, synapse, params, np, c));
	int64_t const S = n->pops[src].d.size, Dn = n->pops[dst].d.size;
	// adj_list::connect checks each edge (topology.cpp:56-58); adj_list::generate sorts src<<32|dst and
	// streams the edges into offsets of S + 1 entries (topology.cpp:15-32, 65-71), with the stream's
	// checks in its order: an edge from row S or beyond fails them, as in the reference
	std::vector<uint64_t> e((size_t)npairs);
	for (int64_t i = 0; i < npairs; i++) {
		int32_t const a = pairs[2 * i], b = pairs[2 * i + 1];
		if (a < 0) return pre_failed("topology.cpp:57", "0 <= src && src < std::numeric_limits<Int32>::max()");
		if (b < 0) return pre_failed("topology.cpp:58", "0 <= dst && dst < std::numeric_limits<Int32>::max()");
		e[i] = ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
	}
	std::sort(e.begin(), e.end());
	{
		int64_t at = 0;  // edge_stream::_src
		for (uint64_t const x : e) {
			int64_t const first = (int64_t)(x >> 32);
			if (!(at < S + 1)) return pre_failed("topology.cpp:16", "_src < _offsets.size()");
			if (!(first < S + 1)) return pre_failed("topology.cpp:18", "edge.first < _offsets.size()");
			if (at <= first) at = first + 1;
		}
		if (!(at < S + 1)) return pre_failed("topology.cpp:29", "_src < _offsets.size()");  // flush
	}
	for (uint64_t const x : e)  // every source row is now below S
		if ((int64_t)(x & 0xffffffffu) >= Dn) return pre_failed("synapse_population.h:119", "edge.first < dst_neurons.size()");
	std::vector<int64_t> off((size_t)S + 1, 0);
	std::vector<int32_t> nb((size_t)npairs);
	int64_t s = 0;
	for (int64_t i = 0; i < npairs; i++) {
		int64_t const es = (int64_t)(e[i] >> 32);
		while (s <= es) off[s++] = i;
		nb[i] = (int32_t)(e[i] & 0xffffffffu);
	}
	while (s <= S) off[s++] = npairs;
	c.d.src = src;
	c.d.dst = dst;
	c.d.delay    = d;
	c.d.src_size = S;
	c.d.dst_size = Dn;
	c.synapses   = npairs;
	c.adj        = true;
	int64_t* doff = nullptr;
	int32_t* dnb  = nullptr;
	CUDA_TRY(cudaMalloc(&doff, sizeof(int64_t) * (S + 1)));
	if (cudaMalloc(&dnb, sizeof(int32_t) * ((npairs + 3) / 4 * 4 + 4)) != cudaSuccess) {  // whole 16-byte blocks
		cudaFree(doff);
		return fail(SPICE_ENOMEM, "cudaMalloc failed for adjacency");
	}
	CUDA_TRY(cudaMemcpyAsync(doff, off.data(), sizeof(int64_t) * (S + 1), cudaMemcpyHostToDevice, n->stream));
	if (npairs > 0)
		CUDA_TRY(cudaMemcpyAsync(dnb, nb.data(), sizeof(int32_t) * npairs, cudaMemcpyHostToDevice, n->stream));
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	c.d.off = doff;
	c.d.nb  = dnb;
	n->conns.push_back(c);
	n->conns.back().gseed = seed_next(n);  // the synapse_population ctor consumes a seed for every topology
	if ((c.weighted && c.wsource != 2) || c.init_seed) n->conns.back().wseed = seed_next(n);  // PerSynapseInit (synapse_population.h:34-41)
	if (conn_out) *conn_out = (int)n->conns.size() - 1;
	return SPICE_OK;
}

extern "C" int spice_set_external_input(spice_net* n, int pop, int nsteps, const int32_t* counts,
                                        const int32_t* indices) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (pop < 0 || pop >= (int)n->pops.size() || n->pops[pop].d.model != EXTERNAL)
		return fail(SPICE_EINVAL, "population is not an external-input population");
	if (nsteps < 0 || (nsteps > 0 && !counts)) return fail(SPICE_EINVAL, "bad train");
	Pop& P          = n->pops[pop];
	int64_t const S = P.d.size;
	std::vector<int64_t> off((size_t)nsteps + 1, 0);
	for (int i = 0; i < nsteps; i++) {
		if (counts[i] < 0 || counts[i] > S) return fail(SPICE_EINVAL, "train step has more spikes than neurons");
		off[i + 1] = off[i] + counts[i];
	}
	for (int i = 0; i < nsteps; i++)
		for (int64_t j = off[i]; j < off[i + 1]; j++) {
			if (indices[j] < 0 || indices[j] >= S) return fail(SPICE_EINVAL, "train spike index out of range");
			if (j > off[i] && indices[j] <= indices[j - 1])
				return fail(SPICE_EINVAL, "each step of an external train must list strictly ascending neuron indices");
		}
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	int32_t* dc = nullptr;
	int64_t* doff = nullptr;
	int32_t* di = nullptr;
	TRY(dalloc(n, &dc, nsteps + 1, false));
	TRY(dalloc(n, &doff, nsteps + 1, false));
	TRY(dalloc(n, &di, off[nsteps] + 1, false));
	if (nsteps > 0) CUDA_TRY(cudaMemcpy(dc, counts, sizeof(int32_t) * nsteps, cudaMemcpyHostToDevice));
	CUDA_TRY(cudaMemcpy(doff, off.data(), sizeof(int64_t) * (nsteps + 1), cudaMemcpyHostToDevice));
	if (off[nsteps] > 0) CUDA_TRY(cudaMemcpy(di, indices, sizeof(int32_t) * off[nsteps], cudaMemcpyHostToDevice));
	P.d.ext_counts = dc;
	P.d.ext_off    = doff;
	P.d.ext_idx    = di;
	P.d.ext_steps  = nsteps;
	n->ext_t_set[pop] = n->time;
	if (n->prepared) CUDA_TRY(cudaMemcpy(n->d_pops + pop, &P.d, sizeof(PopDev), cudaMemcpyHostToDevice));
	return SPICE_OK;
}

extern "C" int spice_set_mode(spice_net* n, int mode) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (mode != SPICE_MODE_DETERMINISTIC && mode != SPICE_MODE_ATOMIC) return fail(SPICE_EINVAL, "unknown mode");
	if (n->prepared && mode != n->mode) return fail(SPICE_ESTATE, "the delivery mode is fixed once the network steps");
	n->mode = mode;
	return SPICE_OK;
}

extern "C" int spice_set_window(spice_net* n, int w) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (w < 0) return fail(SPICE_EINVAL, "window must be >= 0");
	if (n->prepared && w > n->K) return fail(SPICE_ESTATE, "the window can only shrink once the network steps");
	n->max_window = w;
	return SPICE_OK;
}

// ------------------------------------------------------------------------------------------------
// preparation
// ------------------------------------------------------------------------------------------------
namespace {

int generate_pending(spice_net* n) {
	auto& pend = n->gen_pending;
	if (pend.empty()) return SPICE_OK;
	std::vector<GenRequest> reqs;
	for (auto const& g : pend) {
		Conn const& c = n->conns[g.conn];
		reqs.push_back({c.d.src_size, c.d.dst_size, g.p, g.seed, nullptr, nullptr, 0});
	}
	cudaError_t e = generate_fixed_probability(n->stream, reqs);
	if (e != cudaSuccess)
		return fail(e == cudaErrorMemoryAllocation ? SPICE_ENOMEM : SPICE_ECUDA,
		            std::string("fixed_probability generation failed: ") + cudaGetErrorString(e));
	for (size_t i = 0; i < pend.size(); i++) {
		Conn& c     = n->conns[pend[i].conn];
		c.d.off     = reqs[i].offsets;
		c.d.nb      = reqs[i].neighbors;
		c.synapses  = reqs[i].synapses;
	}
	n->launches += 8 * (int64_t)pend.size();
	pend.clear();
	return SPICE_OK;
}

// The per-synapse weights of weighted connections (their adjacency generated), drawn from each
// connection's PerSynapseInit stream in CSR order.
int init_weights(spice_net* n) {
	for (size_t ci = 0; ci < n->conns.size(); ci++) {
		Conn& c = n->conns[ci];
		if (!c.weighted || c.d.wts) continue;
		if (c.wsource != 0)
			return fail(SPICE_ESTATE, "connection " + std::to_string(ci) +
			                              ": its per-synapse weights come from the host (spice_set_synapse_weights) and were not set");
		float* w = nullptr;
		TRY(dalloc(n, &w, (size_t)std::max<int64_t>(c.synapses, 1), false));
		CUDA_TRY(init_synapse_weights(n->stream, c.wseed, c.synapses, c.wmax, w));
		n->launches += 2;
		c.d.wts = w;
	}
	return SPICE_OK;
}

// The CSC of connection ci (built once).
int ensure_csc(spice_net* n, int ci) {
	Conn& c = n->conns[ci];
	if (c.d.csc_off) return SPICE_OK;
	int64_t* off = nullptr;
	int32_t* src = nullptr;
	float* w     = nullptr;
	TRY(dalloc(n, &off, (size_t)c.d.dst_size + 1, false));
	TRY(dalloc(n, &src, (size_t)std::max<int64_t>(c.synapses, 1), false));
	if (c.d.wts) TRY(dalloc(n, &w, (size_t)std::max<int64_t>(c.synapses, 1), false));
	CUDA_TRY(build_csc(n->stream, c.d.off, c.d.nb, c.d.wts, c.d.src_size, c.d.dst_size, c.synapses, off, src, w));
	n->launches += 5;
	c.d.csc_off = off;
	c.d.csc_src = src;
	c.d.csc_w   = w;
	return SPICE_OK;
}

// The delivery mapping when the caller set none: the compact-target rows (17), unless the tile
// leaves too little shared memory for its staged sub-rows (then one thread per spike, 1).
void default_algo(spice_net* n) {
	if (!n->algo_set) n->deliver_algo = n->tile_bytes <= kCompactMaxTileBytes ? 17 : 1;
}

// The launch shape of a network whose caller set none (the values an autotuner run on large and
// small Brunel networks converges to): the compact-target row mapping with two sub-rows per lane
// group (17), the predicated LIF window (variant 9), and the tile size that gives the most delivery CTAs
// per window -- input slots times target tiles -- within one wave of one CTA per SM, the largest
// such tile (fewest sub-rows per spike), at most 100 KiB; threads by tile size.
void default_shape(spice_net* n) {
	if (!n->variant_set) n->neuron_variant = 9;
	default_algo(n);
	if (n->tile_set && n->threads_set) return;
	int dmin = (int)n->max_delay, dmax = 1;
	for (auto const& c : n->conns) {
		dmin = std::min(dmin, c.d.delay);
		dmax = std::max(dmax, c.d.delay);
	}
	int64_t const nslots = n->conns.empty() ? 0 : (int64_t)n->K + dmax - dmin;
	std::vector<std::pair<int64_t, int>> targets;  // (size, words per neuron) of tiled populations
	for (int pi = 0; pi < (int)n->pops.size(); pi++) {
		PopDev const& d = n->pops[pi].d;
		bool in = false;
		for (auto const& c : n->conns) in |= c.d.dst == pi;
		if (in && d.size > 0 && !d.pull && !d.direct)
			targets.push_back({d.size, std::max(n->mode == SPICE_MODE_DETERMINISTIC ? d.W : d.F, 1)});
	}
	int constexpr kMaxTile = 100 * 1024, kMinTile = 4 * 1024;
	int tb = kMaxTile;
	if (!n->tile_set && nslots > 0 && !targets.empty()) {
		auto ctas = [&](int bytes) {
			int64_t m = 0;
			for (auto const& [size, width] : targets) {
				int64_t const tile = std::max(32, bytes / (4 * width) / 32 * 32);
				m += (size + tile - 1) / tile;
			}
			return nslots * m;
		};
		int64_t best = -1;
		for (int bytes = kMaxTile; bytes >= kMinTile; bytes -= 128) {  // CTAs grow as tiles shrink
			int64_t const m = ctas(bytes);
			if (m > n->sm_count) break;
			if (m > best) {
				best = m;
				tb   = bytes;
			}
		}
		n->tile_bytes = tb;
	}
	if (!n->threads_set) n->deliver_threads = n->tile_bytes >= 64 * 1024 ? 768 : n->tile_bytes >= 24 * 1024 ? 512 : 256;
	default_algo(n);
}

// Tile sizes of the delivery kernel, the by-target connection order and the per-row positions
// where each tile starts.  Called at preparation and again when the launch shape is re-tuned.
int setup_tiles(spice_net* n, bool first) {
	int const np = (int)n->pops.size();
	// tiled delivery: tile sizes, the by-target connection order, per-row tile start positions
	n->dmin = (int)n->max_delay;
	n->dmax = 1;
	for (auto const& c : n->conns) {
		n->dmin = std::min(n->dmin, c.d.delay);
		n->dmax = std::max(n->dmax, c.d.delay);
	}
	if (n->conns.empty()) n->dmin = n->dmax = 1;
	std::vector<int> by_dst;
	for (int pi = 0; pi < np; pi++) {
		PopDev& d   = n->pops[pi].d;
		d.in_begin  = (int)by_dst.size();
		int dfirst = -1;
		bool mixed = false;
		for (int ci = 0; ci < (int)n->conns.size(); ci++)
			if (n->conns[ci].d.dst == pi) {
				by_dst.push_back(ci);
				if (dfirst < 0) dfirst = n->conns[ci].d.delay;
				mixed |= n->conns[ci].d.delay != dfirst;
				mixed |= n->conns[ci].d.plastic != 0;  // plastic deliveries add into the ring
			}
		d.in_end      = (int)by_dst.size();
		// slots are overwritten by one delivery CTA unless delays differ, tiles are split or the
		// persistent steps deliver (they add into the ring)
		d.zero_inputs = (mixed || n->deliver_parts > 1 || n->persist_ok) ? 1 : 0;
		int const width = n->mode == SPICE_MODE_DETERMINISTIC ? d.W : d.F;
		int tile        = n->tile_bytes / (4 * std::max(width, 1));
		tile            = std::max(32, tile / 32 * 32);
		d.tile          = tile;
		d.ntiles        = (d.in_end > d.in_begin && d.size > 0 && !d.pull && !d.direct) ? (int)((d.size + tile - 1) / tile) : 0;
	}
	for (auto& c : n->conns) {
		ConnDev& d      = c.d;
		PopDev const& T = n->pops[d.dst].d;
		int64_t* bnd    = nullptr;
		if (T.pull || T.direct) continue;  // gathered over the CSC: no tiles
		if (!first && d.bounds) {
			CUDA_TRY(cudaStreamSynchronize(n->stream));
			cudaFree((void*)d.bounds);
			n->allocations.erase(std::find(n->allocations.begin(), n->allocations.end(), (void*)d.bounds));
		}
		TRY(dalloc(n, &bnd, (size_t)d.src_size * (T.ntiles + 1), false));
		CUDA_TRY(launch_tile_bounds(n->stream, d.off, d.nb, d.src_size, T.tile, T.ntiles, bnd));
		n->launches++;
		d.bounds = bnd;
		// the compact-target mapping reads targets as 16-bit indices within their tile
		if (compact_algo(n->deliver_algo) && !d.plastic && c.synapses > 0 && c.nb16_tile != T.tile) {
			if (!c.nb16) {  // whole 16-byte blocks plus one, as the target array
				size_t const bytes = sizeof(uint16_t) * (size_t)((c.synapses + 7) / 8 * 8 + 8);
				if (cudaMalloc((void**)&c.nb16, bytes) != cudaSuccess)
					return fail(SPICE_ENOMEM, "cudaMalloc failed for the compact targets (" + std::to_string(bytes) + " bytes)");
			}
			CUDA_TRY(launch_compact_targets(n->stream, d.nb, c.synapses, T.tile, c.nb16));
			n->launches++;
			c.nb16_tile = T.tile;
		}
		d.nb16 = c.nb16_tile == T.tile ? c.nb16 : nullptr;
	}
	n->by_dst = by_dst;
	return SPICE_OK;
}

// Pulled populations: the CSC of their incoming connections, region starts, active-list, grouped
// and bin-offset buffers; one window-mask set per (source population, delay); event jobs.
int setup_pull(spice_net* n) {
	int const np = (int)n->pops.size();
	n->pull_pops.clear();
	n->pull_sets.clear();
	n->pull_ev.clear();
	std::vector<int> blk(1, 0);
	for (int pi = 0; pi < np; pi++) {
		PopDev& d = n->pops[pi].d;
		if (!d.pull) continue;
		std::vector<const int64_t*> offs;
		d.pull_F = 0;
		for (int b = d.in_begin; b < d.in_end; b++) {
			int const ci = n->by_dst[b];
			TRY(ensure_csc(n, ci));
			Conn& c = n->conns[ci];
			offs.push_back(c.d.csc_off);
			bool seen = false;
			for (int f = 0; f < d.pull_F; f++) seen |= d.pull_field[f] == c.d.field;
			if (!seen) d.pull_field[d.pull_F++] = c.d.field;
			// the window masks of (source, delay)
			int set = -1;
			for (int q = 0; q < (int)n->pull_sets.size(); q++)
				if (n->pull_sets[q].src == c.d.src && n->pull_sets[q].delay == c.d.delay) set = q;
			if (set < 0) {
				PopDev const& S = n->pops[c.d.src].d;
				PullSet ps{};
				ps.src    = c.d.src;
				ps.delay  = c.d.delay;
				ps.nwords = S.nwords;
				ps.size   = S.size;
				ps.bits   = S.bits;
				TRY(dalloc(n, &ps.orb, (size_t)std::max(S.nwords, 1)));
				TRY(dalloc(n, &ps.wm, (size_t)std::max<int64_t>(S.size, 1)));
				TRY(dalloc(n, &ps.act, (size_t)std::max<int64_t>(S.size, 1), false));
				TRY(dalloc(n, &ps.nact, 1));  // zero
				set = (int)n->pull_sets.size();
				n->pull_sets.push_back(ps);
			}
			c.d.pull_orb  = n->pull_sets[set].orb;
			c.d.pull_wm   = n->pull_sets[set].wm;
			c.d.pull_act  = n->pull_sets[set].act;
			c.d.pull_nact = n->pull_sets[set].nact;
			n->pull_ev.push_back({n->pops[c.d.src].d.nwords, n->pops[c.d.src].d.bits, c.d.off});
		}
		for (int f = d.pull_F; f < 3; f++) d.pull_field[f] = 0;
		d.pull_nbins = n->K * d.pull_F;
		const int64_t** d_offs = nullptr;
		TRY(dalloc(n, &d_offs, offs.size(), false));
		CUDA_TRY(cudaMemcpy(d_offs, offs.data(), sizeof(void*) * offs.size(), cudaMemcpyHostToDevice));
		int64_t* base = nullptr;
		TRY(dalloc(n, &base, (size_t)d.size + 1, false));
		CUDA_TRY(pull_region_bases(n->stream, d_offs, (int)offs.size(), d.size, base));
		n->launches++;
		int64_t total = 0;
		CUDA_TRY(cudaMemcpyAsync(&total, base + d.size, sizeof(int64_t), cudaMemcpyDeviceToHost, n->stream));
		CUDA_TRY(cudaStreamSynchronize(n->stream));
		d.pull_base = base;
		TRY(dalloc(n, &d.pull_A, (size_t)std::max<int64_t>(total, 1), false));
		TRY(dalloc(n, &d.pull_G, (size_t)std::max<int64_t>(total, 1), false));
		TRY(dalloc(n, &d.pull_koff, (size_t)std::max<int64_t>(d.size, 1) * (d.pull_nbins + 1)));  // zero: no inputs yet
		TRY(dalloc(n, &d.pull_fill, (size_t)std::max<int64_t>(d.size, 1)));
		n->pull_pops.push_back(pi);
		blk.push_back(blk.back() + pull_blocks_for(d.size));
	}
	n->pull_blocks = blk.back();
	{  // push-and-sort gather: units (pulled connection, spiking source); rows must fit the sort key
		std::vector<int> ps_conn, ps_pop;
		std::vector<int64_t> ps_begin(1, 0);  // source bitmap words per connection (their sum: the flag)
		bool ok = !n->pull_pops.empty();
		for (int pi : n->pull_pops) {
			PopDev const& d = n->pops[pi].d;
			for (int b = d.in_begin; b < d.in_end && ok; b++) {
				ConnDev const& c = n->conns[n->by_dst[b]].d;
				std::vector<int64_t> off((size_t)c.src_size + 1);
				if (c.src_size > 0)
					CUDA_TRY(cudaMemcpy(off.data(), c.off, sizeof(int64_t) * off.size(), cudaMemcpyDeviceToHost));
				for (int64_t r = 0; r < c.src_size && ok; r++) ok = off[r + 1] - off[r] < kPushSortMaxRow;
				ps_conn.push_back(b);
				ps_pop.push_back(pi);
				ps_begin.push_back(ps_begin.back() + n->pops[c.src].d.nwords);
			}
		}
		n->ps_ok    = ok;
		n->ps_nconn = (int)ps_conn.size();
		// (pulled populations without neurons have nothing to gather: no lists are kept for them,
		// since k_ps_sort, which empties the lists, runs only over target blocks)
		n->ps_units = (ok && blk.back() > 0) ? ps_begin.back() : 0;
		if (ok) {
			for (int pi : n->pull_pops) {  // the targets' entry slots
				PopDev& d = n->pops[pi].d;
				TRY(dalloc(n, &d.ps_slot, (size_t)std::max<int64_t>(d.size, 1) * kPushSortSlots, false));
			}
			TRY(dalloc(n, &n->d_ps_conn, std::max<size_t>(ps_conn.size(), 1), false));
			TRY(dalloc(n, &n->d_ps_pop, std::max<size_t>(ps_pop.size(), 1), false));
			CUDA_TRY(cudaMemcpy(n->d_ps_conn, ps_conn.data(), sizeof(int) * ps_conn.size(), cudaMemcpyHostToDevice));
			CUDA_TRY(cudaMemcpy(n->d_ps_pop, ps_pop.data(), sizeof(int) * ps_pop.size(), cudaMemcpyHostToDevice));
		}
	}
	TRY(dalloc(n, &n->d_pull_pops, std::max<size_t>(n->pull_pops.size(), 1), false));
	TRY(dalloc(n, &n->d_pull_blk, blk.size(), false));
	TRY(dalloc(n, &n->d_pull_sets, std::max<size_t>(n->pull_sets.size(), 1), false));
	TRY(dalloc(n, &n->d_pull_ev, std::max<size_t>(n->pull_ev.size(), 1), false));
	if (!n->pull_pops.empty())
		CUDA_TRY(cudaMemcpy(n->d_pull_pops, n->pull_pops.data(), sizeof(int) * n->pull_pops.size(), cudaMemcpyHostToDevice));
	CUDA_TRY(cudaMemcpy(n->d_pull_blk, blk.data(), sizeof(int) * blk.size(), cudaMemcpyHostToDevice));
	if (!n->pull_sets.empty())
		CUDA_TRY(cudaMemcpy(n->d_pull_sets, n->pull_sets.data(), sizeof(PullSet) * n->pull_sets.size(), cudaMemcpyHostToDevice));
	if (!n->pull_ev.empty())
		CUDA_TRY(cudaMemcpy(n->d_pull_ev, n->pull_ev.data(), sizeof(PullEvJob) * n->pull_ev.size(), cudaMemcpyHostToDevice));
	return SPICE_OK;
}

// USER_DELIVER targets: the CSC of every incoming connection (with CSR positions for synapse state)
// and the user synapses' state.
int setup_direct(spice_net* n) {
	for (size_t ci = 0; ci < n->conns.size(); ci++) {
		Conn& c = n->conns[ci];
		if (!n->pops[c.d.dst].d.direct) continue;
		if (c.reads_source && (n->pops[c.d.src].d.model != USER || !n->pops[c.d.src].stateful))
			return fail(SPICE_EINVAL, "a deliver() that reads the source neuron needs a stateful user source population");
		if (c.udeliver && c.ubytes > 0 && !c.csc_pos) {  // CSR positions: build this connection's CSC with them
			int64_t* pos = nullptr;
			TRY(dalloc(n, &pos, (size_t)std::max<int64_t>(c.synapses, 1), false));
			c.csc_pos = pos;
			if (c.d.csc_off) return fail(SPICE_ESTATE, "internal: CSC built without positions");
			int64_t* off = nullptr;
			int32_t* src = nullptr;
			TRY(dalloc(n, &off, (size_t)c.d.dst_size + 1, false));
			TRY(dalloc(n, &src, (size_t)std::max<int64_t>(c.synapses, 1), false));
			CUDA_TRY(build_csc(n->stream, c.d.off, c.d.nb, nullptr, c.d.src_size, c.d.dst_size, c.synapses, off, src, nullptr, pos));
			n->launches += 5;
			c.d.csc_off = off;
			c.d.csc_src = src;
		}
		TRY(ensure_csc(n, (int)ci));
		if (c.udeliver && c.ubytes > 0 && !c.ustate) {
			char* st = nullptr;
			size_t const bytes = (size_t)std::max<int64_t>(c.synapses, 1) * c.ubytes;
			TRY(dalloc(n, &st, bytes, false));
			if (!c.uhost.empty()) {
				CUDA_TRY(cudaMemcpy(st, c.uhost.data(), c.uhost.size(), cudaMemcpyHostToDevice));
				c.uhost.clear();
			} else {
				std::vector<char> h(bytes);
				for (size_t q = 0; q + c.ubytes <= bytes; q += c.ubytes) memcpy(h.data() + q, c.uinit.data(), c.ubytes);
				CUDA_TRY(cudaMemcpy(st, h.data(), bytes, cudaMemcpyHostToDevice));
			}
			c.ustate = st;
		}
	}
	return SPICE_OK;
}

// The deliveries into USER_DELIVER targets at the end of step n->time, connection by connection in
// connect order (snn.cpp:21-25).
int deliver_direct(spice_net* n) {
	for (auto const& c : n->conns) {
		PopDev const& T = n->pops[c.d.dst].d;
		if (!T.direct || n->time < c.d.delay - 1) continue;
		int const hs = (int)((n->time - c.d.delay + 1) % n->Hb);
		if (c.udeliver) {
			spice_user_deliver_call u;
			memset(&u, 0, sizeof u);
			u.version         = SPICE_USER_DELIVER_ABI_VERSION;
			u.time            = n->time;
			u.dt              = n->dt;
			u.hslot           = hs;
			u.src_size        = c.d.src_size;
			u.dst_size        = c.d.dst_size;
			u.off             = c.d.off;
			u.nb              = c.d.nb;
			u.col_off         = c.d.csc_off;
			u.col_src         = c.d.csc_src;
			u.col_pos         = c.csc_pos;
			u.src_bits        = c.d.src_bits;
			u.src_nwords      = c.d.src_nwords;
			u.src_state       = n->pops[c.d.src].d.ustate;
			u.dst_state       = T.ustate;
			u.synapse_state   = c.ustate;
			u.same_population = c.d.src == c.d.dst;
			u.events          = n->d_events;
			int const r = reinterpret_cast<spice_user_deliver_fn>(c.ufn)(&u, (void*)n->stream, c.uctx);
			if (r != 0) return fail(SPICE_ECUDA, "the deliver() kernels of a user connection failed (" + std::to_string(r) + ")");
		} else {
			CUDA_TRY(launch_direct_add(n->stream, c.d, hs, T.ustate, T.ubytes, n->pops[c.d.dst].field_offset[c.d.field],
			                           n->d_events));
		}
		n->launches++;
	}
	return SPICE_OK;
}

int prepare(spice_net* n) {
	if (n->prepared) return SPICE_OK;
	TRY(generate_pending(n));
	TRY(init_weights(n));
	int const np = (int)n->pops.size();
	int64_t const D = n->max_delay;
	if (D < 1) return pre_failed("neuron_population.h:108", "max_delay >= 1");
	// plastic connections: per-step catch-up timing, so windows of one step
	n->plastic = false;
	for (auto const& c : n->conns) {
		if (!c.d.plastic) continue;
		n->plastic = true;
		bool const delivers = c.d.plastic == SPICE_SYNAPSE_ISTDP || c.d.plastic == SPICE_SYNAPSE_USER_PLASTIC ||
		                      c.d.weight != 0.0f;
		if (c.d.plastic == SPICE_SYNAPSE_USER_PLASTIC && !c.ufn)
			return fail(SPICE_ESTATE, "a user plastic connection needs its kernels (spice_user_plastic) before the network steps");
		if (delivers && n->mode != SPICE_MODE_ATOMIC)
			return fail(SPICE_EINVAL, "plastic synapses that deliver per-synapse weights need SPICE_MODE_ATOMIC "
			                          "(their per-step sums are order-dependent)");
	}
	// populations receiving user deliver() code get every input directly at the end of each step
	n->any_direct = false;
	for (int pi = 0; pi < np; pi++) {
		n->pops[pi].d.direct = 0;
		bool udel = false, plastic_in = false;
		for (auto const& c : n->conns)
			if (c.d.dst == pi) {
				udel |= c.udeliver;
				plastic_in |= c.d.plastic != 0;
			}
		if (!udel) continue;
		if (plastic_in)
			return fail(SPICE_EINVAL, "population " + std::to_string(pi) +
			                              ": plastic synapses into a population with user deliver() code are not supported");
		for (auto const& c : n->conns)
			if (c.udeliver && !c.ufn)
				return fail(SPICE_ESTATE, "a user deliver connection needs its kernels (spice_user_deliver) before the network steps");
		n->pops[pi].d.direct = 1;
		n->any_direct        = true;
	}
	// pulled populations: inputs with per-synapse weights, the pull knob, or (deterministic mode)
	// more distinct input weights than the count replay keeps apart
	n->any_pull = false;
	for (int pi = 0; pi < np; pi++) {
		Pop& P = n->pops[pi];
		P.d.pull = 0;
		bool has_in = false, weighted_in = false, plastic_in = false;
		int groups = 0, last_of_field[3] = {-1, -1, -1};
		std::vector<float> gw;
		for (auto const& c : n->conns) {
			if (c.d.dst != pi) continue;
			has_in = true;
			weighted_in |= c.weighted;
			plastic_in |= c.d.plastic != 0;
			if (c.d.plastic || c.weighted) continue;
			int const g = last_of_field[c.d.field];
			if (g < 0 || memcmp(&gw[g], &c.d.weight, sizeof(float)) != 0) {
				gw.push_back(c.d.weight);
				last_of_field[c.d.field] = groups++;
			}
		}
		if (!P.stateful || !has_in || P.d.direct) continue;
		bool const pull = weighted_in || (P.d.model != USER && n->pull_all) ||
		                  (P.d.model != USER && n->mode == SPICE_MODE_DETERMINISTIC && groups > kMaxGroups);
		if (!pull) continue;
		if (plastic_in)
			return fail(SPICE_EINVAL, "population " + std::to_string(pi) +
			                              ": plastic synapses into a population whose inputs are pulled (weighted synapses, "
			                              "more than 4 distinct weights, or the pull knob) are not supported");
		P.d.pull    = 1;
		n->any_pull = true;
	}
	// window: the minimum delay (every delay is >= 1)
	int K = kMaxWindow;
	for (auto const& c : n->conns) K = std::min<int>(K, c.d.delay);
	if (n->max_window > 0) K = std::min(K, n->max_window);
	if (n->plastic || n->any_direct) K = 1;  // per-step catch-up, or deliveries at the end of each step
	// the delivery kernel keeps a (step, connection) prefix of K * nconn entries in shared memory
	if (!n->conns.empty()) K = std::min<int>(K, std::max<int>(1, 4096 / (int)n->conns.size()));
	if (n->any_pull) K = std::min(K, kPullMaxWindow);  // step masks of 16 bits
	n->K  = std::max(K, 1);
	// bitmaps: the last D steps for spikes(age), and two windows in flight (sources run ahead);
	// the pull reads the D steps before the next window while sources may already write it
	n->Hb = (int)std::max<int64_t>(D, 2 * n->K) + 1 + (n->any_pull ? n->K : 0);
	// persistent steps: windows of one step, built-in models and synapses, pushed deliveries
	n->persist_ok = n->persist_knob != 0 && n->K == 1 && !n->any_pull && !n->any_direct &&
	                np <= kMaxPops && n->conns.size() <= (size_t)kMaxConns;
	for (auto const& p : n->pops) n->persist_ok &= p.d.model != USER;
	for (auto const& c : n->conns)
		n->persist_ok &= !c.weighted && !c.udeliver && c.d.plastic != SPICE_SYNAPSE_USER_PLASTIC;
	if (n->persist_ok) {
		int coop = 0, sms = 0, per_sm = 0;
		CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, n->device));
		CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, n->device));
		CUDA_TRY(persist_occupancy(n->mode == SPICE_MODE_DETERMINISTIC ? 0 : 1, &per_sm));
		n->persist_grid = sms * per_sm;  // the most resident CTAs (the knob may ask for fewer per SM)
		n->persist_ok   = coop != 0 && n->persist_grid > 0;
	}
	// draw offsets in the step's shared stream (populations in add order, snn.cpp:14-15)
	int64_t draws = 0;
	for (auto& p : n->pops) {
		p.d.draw_offset = draws;
		if (p.d.model == POISSON || (p.d.model == USER && !p.stateful)) draws += p.d.size;
		if (p.d.model == USER && p.stateful) draws += p.d.size * p.udraws;  // declared draws per update
	}
	n->total_draws = draws;
	for (auto& p : n->pops) {
		PopDev& d = p.d;
		TRY(dalloc(n, &d.bits, (size_t)n->Hb * std::max(d.nwords, 1)));
		TRY(dalloc(n, &d.list, (size_t)2 * n->K * std::max<int64_t>(d.size, 1), false));
		bool const drawing_user = d.model == USER && p.stateful && p.udraws > 0;
		if ((d.model == POISSON || (d.model == USER && !p.stateful) || drawing_user) && d.nwords > 0) {
			std::vector<u128> polys(d.nwords);
			u128 const step = gf2_xpow((uint64_t)kPoissonChunk * (drawing_user ? p.udraws : 1));
			polys[0]        = gf2_xpow((uint64_t)d.draw_offset);
			for (int c = 1; c < d.nwords; c++) polys[c] = gf2_mulmod(polys[c - 1], step);
			u128* dp = nullptr;
			TRY(dalloc(n, &dp, d.nwords, false));
			CUDA_TRY(cudaMemcpy(dp, polys.data(), sizeof(u128) * d.nwords, cudaMemcpyHostToDevice));
			d.chunk_poly = dp;
		}
	}
	// input groups per target population: connections in connect order; a connection joins the
	// latest group of its field when the weights are bit-identical (same sequence of adds)
	std::vector<std::vector<int>> group_conns(np * kMaxGroups);
	for (int pi = 0; pi < np; pi++) {
		PopDev& d = n->pops[pi].d;
		if (!n->pops[pi].stateful) continue;
		if (d.pull || d.direct) {  // inputs gathered by the pull kernel, or applied directly: no input ring
			d.ngroups = 0;
			d.W = d.F = 1;
			continue;
		}
		int last_of_field[3] = {-1, -1, -1};
		d.ngroups = 0;
		for (int ci = 0; ci < (int)n->conns.size(); ci++) {
			ConnDev& c = n->conns[ci].d;
			if (c.dst != pi || c.plastic || n->conns[ci].weighted) continue;
			int g = last_of_field[c.field];
			// deterministic mode replays counts per weight; atomic mode sums weights per field
			bool const new_group = g < 0 || (n->mode == SPICE_MODE_DETERMINISTIC &&
			                                 memcmp(&d.group_weight[g], &c.weight, sizeof(float)) != 0);
			if (new_group) {
				if (d.ngroups >= kMaxGroups)
					return fail(SPICE_EINVAL, "too many distinct input weights into one population (max 4)");
				g                 = d.ngroups++;
				d.group_field[g]  = c.field;
				d.group_weight[g] = c.weight;
				last_of_field[c.field] = g;
			}
			c.group = g;
			group_conns[pi * kMaxGroups + g].push_back(ci);
		}
		// counter widths from the maximum in-degree of each group
		uint32_t* scratch = nullptr;
		uint32_t* dmax    = nullptr;
		CUDA_TRY(cudaMalloc(&scratch, sizeof(uint32_t) * (d.size > 0 ? d.size : 1)));
		CUDA_TRY(cudaMalloc(&dmax, sizeof(uint32_t)));
		int word = 0, half = 0;
		for (int g = 0; g < d.ngroups; g++) {
			std::vector<const int32_t*> nbs;
			std::vector<int64_t> ns;
			for (int ci : group_conns[pi * kMaxGroups + g]) {
				nbs.push_back(n->conns[ci].d.nb);
				ns.push_back(n->conns[ci].synapses);
			}
			uint32_t mx = 0;
			cudaError_t e = max_indegree(n->stream, nbs.data(), ns.data(), (int)nbs.size(), d.size, scratch, dmax);
			if (e == cudaSuccess) e = cudaMemcpyAsync(&mx, dmax, sizeof(uint32_t), cudaMemcpyDeviceToHost, n->stream);
			if (e == cudaSuccess) e = cudaStreamSynchronize(n->stream);
			n->launches += (int64_t)nbs.size() + 1;
			if (e != cudaSuccess) {
				cudaFree(scratch);
				cudaFree(dmax);
				return fail(SPICE_ECUDA, std::string("in-degree count failed: ") + cudaGetErrorString(e));
			}
			if (mx < 65536u) {
				if (half == 1) {
					d.group_word[g]  = word - 1;
					d.group_shift[g] = 16;
					half             = 0;
				} else {
					d.group_word[g]  = word++;
					d.group_shift[g] = 0;
					half             = 1;
				}
				d.group_bits[g] = 16;
			} else {
				d.group_word[g]  = word++;
				d.group_shift[g] = 0;
				d.group_bits[g]  = 32;
				half             = 0;
			}
		}
		cudaFree(scratch);
		cudaFree(dmax);
		d.W = std::max(word, 1);
		int F = 0;
		for (int g = 0; g < d.ngroups; g++)
			if (d.field_slot[d.group_field[g]] < 0) d.field_slot[d.group_field[g]] = F++;
		for (auto const& cc : n->conns)  // plastic deliveries add into the atomic-mode sums
			if (cc.d.dst == pi && cc.d.plastic && n->mode == SPICE_MODE_ATOMIC && d.field_slot[cc.d.field] < 0)
				d.field_slot[cc.d.field] = F++;
		d.F = std::max(F, 1);
		if (n->mode == SPICE_MODE_DETERMINISTIC)
			TRY(dalloc(n, &d.cnt, (size_t)D * d.size * d.W));
		else
			TRY(dalloc(n, &d.acc, (size_t)D * d.size * d.F));
	}
	CUDA_TRY(cudaDeviceGetAttribute(&n->sm_count, cudaDevAttrMultiProcessorCount, n->device));
	default_shape(n);
	TRY(setup_tiles(n, true));
	for (auto& c : n->conns) {
		ConnDev& d      = c.d;
		PopDev const& S = n->pops[d.src].d;
		PopDev const& T = n->pops[d.dst].d;
		d.src_list = S.list;
		d.dst_cnt  = T.cnt;
		d.dst_acc  = T.acc;
		d.W        = T.W;
		d.word     = T.group_word[d.group];
		d.inc      = 1u << T.group_shift[d.group];
		d.F        = T.F;
		d.fslot    = T.field_slot[d.field];
	}
	for (auto& p : n->pops) p.d.net = 0;
	// plastic connections: per-synapse state, per-source ages, the targets' post history
	for (auto& c : n->conns) {
		ConnDev& d = c.d;
		if (!d.plastic) continue;
		PopDev& T = n->pops[d.dst].d;
		PopDev const& S = n->pops[d.src].d;
		if (!T.hist) TRY(dalloc(n, &T.hist, (size_t)std::max<int64_t>(T.size, 1)));
		if (d.plastic == SPICE_SYNAPSE_USER_PLASTIC) {  // the user's structs, initial value or host state
			char* st = nullptr;
			size_t const bytes = (size_t)std::max<int64_t>(c.synapses, 1) * c.ubytes;
			TRY(dalloc(n, &st, bytes, false));
			if (!c.uhost.empty()) {
				CUDA_TRY(cudaMemcpy(st, c.uhost.data(), c.uhost.size(), cudaMemcpyHostToDevice));
				c.uhost.clear();
			} else {
				std::vector<char> h(bytes);
				for (size_t q = 0; q + c.ubytes <= bytes; q += c.ubytes) memcpy(h.data() + q, c.uinit.data(), c.ubytes);
				CUDA_TRY(cudaMemcpy(st, h.data(), bytes, cudaMemcpyHostToDevice));
			}
			c.ustate = st;
		} else {
			TRY(dalloc(n, &d.sW, (size_t)std::max<int64_t>(c.synapses, 1), false));
			TRY(dalloc(n, &d.sA, (size_t)std::max<int64_t>(c.synapses, 1)));
			TRY(dalloc(n, &d.sB, (size_t)std::max<int64_t>(c.synapses, 1)));
		}
		TRY(dalloc(n, &d.ages, (size_t)std::max<int64_t>(S.size, 1)));
		TRY(dalloc(n, &d.chunks_done, (size_t)std::max<int64_t>(S.size, 1)));
		{  // the longest row sizes the plastic delivery's grid
			std::vector<int64_t> off((size_t)S.size + 1);
			CUDA_TRY(cudaMemcpy(off.data(), d.off, sizeof(int64_t) * off.size(), cudaMemcpyDeviceToHost));
			d.max_row = 0;
			for (int64_t r = 0; r < S.size; r++) d.max_row = std::max(d.max_row, off[r + 1] - off[r]);
		}
		if (d.sW) {
			std::vector<float> w0((size_t)std::max<int64_t>(c.synapses, 1), d.plastic == SPICE_SYNAPSE_ISTDP ? c.w0 : 0.0f);
			CUDA_TRY(cudaMemcpy(d.sW, w0.data(), sizeof(float) * w0.size(), cudaMemcpyHostToDevice));
		}
		d.alpha = 2.0f * c.rho0 * c.tau;
		d.cdt   = n->dt * (1.0f / c.tau);
		std::vector<double> tab(129);
		float const base = 1.0f - d.cdt;
		for (int k = -64; k <= 64; k++) tab[k + 64] = pow((double)base, (double)k);
		double* dt = nullptr;
		TRY(dalloc(n, &dt, tab.size(), false));
		CUDA_TRY(cudaMemcpy(dt, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice));
		d.skip_tab   = dt;
		std::vector<uint64_t> pk(tab.size());
		for (size_t q = 0; q < tab.size(); q++) pk[q] = pack_f64(tab[q]);
		uint64_t* dpk = nullptr;
		TRY(dalloc(n, &dpk, pk.size(), false));
		CUDA_TRY(cudaMemcpy(dpk, pk.data(), sizeof(uint64_t) * pk.size(), cudaMemcpyHostToDevice));
		d.skip_pk = dpk;
		d.src_bits   = S.bits;
		d.src_nwords = S.nwords;
	}
	for (auto& c : n->conns)
		if (c.d.plastic) c.d.dst_hist = n->pops[c.d.dst].d.hist;
	if (n->any_pull) TRY(setup_pull(n));
	for (size_t ci = 0; ci < n->conns.size(); ci++) {  // every connection: its source's bitmap ring
		n->conns[ci].d.src_bits   = n->pops[n->conns[ci].d.src].d.bits;
		n->conns[ci].d.src_nwords = n->pops[n->conns[ci].d.src].d.nwords;
	}
	if (n->any_direct) TRY(setup_direct(n));
	TRY(dalloc(n, &n->d_counts, (size_t)2 * n->K * std::max(np, 1)));
	TRY(dalloc(n, &n->d_pops, std::max(np, 1), false));
	TRY(dalloc(n, &n->d_conns, std::max<size_t>(n->conns.size(), 1), false));
	std::vector<PopDev> hp;
	for (auto& p : n->pops) hp.push_back(p.d);
	std::vector<ConnDev> hc;
	for (auto& c : n->conns) hc.push_back(c.d);
	if (np) CUDA_TRY(cudaMemcpy(n->d_pops, hp.data(), sizeof(PopDev) * np, cudaMemcpyHostToDevice));
	if (!hc.empty()) CUDA_TRY(cudaMemcpy(n->d_conns, hc.data(), sizeof(ConnDev) * hc.size(), cudaMemcpyHostToDevice));
	{
		std::vector<ConnDev> hb;
		for (int ci : n->by_dst) hb.push_back(n->conns[ci].d);
		TRY(dalloc(n, &n->d_conns_by_dst, std::max<size_t>(hb.size(), 1), false));
		if (!hb.empty())
			CUDA_TRY(cudaMemcpy(n->d_conns_by_dst, hb.data(), sizeof(ConnDev) * hb.size(), cudaMemcpyHostToDevice));
	}
	n->run_cap = kRunCap;
	CUDA_TRY(cudaDeviceGetAttribute(&n->sm_count, cudaDevAttrMultiProcessorCount, n->device));
	if (n->persist_ok) {  // delivery units: a warp and at most kPersistChunk (plastic: kPersistPlasticChunk)
		                  // synapses of one row
		n->persist_chunks.assign(n->conns.size(), 1);
		for (size_t ci = 0; ci < n->conns.size(); ci++) {
			ConnDev const& d = n->conns[ci].d;
			int64_t mr = d.max_row;
			if (!d.plastic && d.src_size > 0) {
				std::vector<int64_t> off((size_t)d.src_size + 1);
				CUDA_TRY(cudaMemcpy(off.data(), d.off, sizeof(int64_t) * off.size(), cudaMemcpyDeviceToHost));
				mr = 0;
				for (int64_t r = 0; r < d.src_size; r++) mr = std::max(mr, off[r + 1] - off[r]);
			}
			int64_t const len     = d.plastic ? kPersistPlasticChunk : kPersistChunk;
			n->persist_chunks[ci] = std::max<int64_t>(1, (mr + len - 1) / len);
		}
		TRY(dalloc(n, &n->d_barrier, 1));
		TRY(dalloc(n, &n->d_pstatus, 1));
		CUDA_TRY(cudaMallocHost(&n->h_pstatus, sizeof(int)));
		*n->h_pstatus = 0;
	}
	// two chunk buffers: the host prepares one chunk while the GPU still steps the previous one
	TRY(dalloc(n, &n->d_dt, 2 * kRunCap, false));
	TRY(dalloc(n, &n->d_seeds, 2 * kRunCap, false));
	if (n->total_draws > 0) TRY(dalloc(n, &n->d_tables, (size_t)2 * kRunCap * kJumpTable, false));
	CUDA_TRY(cudaMallocHost(&n->h_dt, sizeof(float) * 2 * kRunCap));
	CUDA_TRY(cudaMallocHost(&n->h_seeds, sizeof(u128) * 2 * kRunCap));
	for (int b = 0; b < 2; b++) {
		CUDA_TRY(cudaEventCreateWithFlags(&n->ev_chunk[b], cudaEventDisableTiming));
		CUDA_TRY(cudaEventRecord(n->ev_chunk[b], n->stream));
	}
	int64_t maxN = 1;
	for (auto& p : n->pops) maxN = std::max(maxN, p.d.size);
	TRY(dalloc(n, &n->d_tmp, maxN, false));
	TRY(dalloc(n, &n->d_tmp_n, 1));
	for (auto& p : n->pops) {
		n->has_sources |= p.d.model == POISSON || p.d.model == EXTERNAL || (p.d.model == USER && !p.stateful);
		n->user_seeds |= p.d.model == USER && p.stateful;  // their counter-based streams read the step seeds
	}
	CUDA_TRY(cudaStreamCreateWithFlags(&n->stream_src, cudaStreamNonBlocking));
	CUDA_TRY(cudaEventCreateWithFlags(&n->ev_tab, cudaEventDisableTiming));
	for (int q = 0; q < 2; q++) {
		CUDA_TRY(cudaEventCreateWithFlags(&n->ev_src[q], cudaEventDisableTiming));
		CUDA_TRY(cudaEventCreateWithFlags(&n->ev_free[q], cudaEventDisableTiming));
		CUDA_TRY(cudaEventRecord(n->ev_free[q], n->stream));
	}
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	n->prepared = true;
	return SPICE_OK;
}

// The window of a user population, as its update kernel sees it (spice_user_window).
spice_user_window user_window(spice_net* n, int pi, WindowArgs const& wa, int64_t j, bool apply_only) {
	Pop const& P    = n->pops[pi];
	PopDev const& d = P.d;
	spice_user_window w;
	memset(&w, 0, sizeof w);
	w.version    = SPICE_USER_ABI_VERSION;
	w.apply_only = apply_only ? 1 : 0;
	w.t0         = wa.t0;
	w.K          = apply_only ? 0 : wa.K;
	w.slot0      = wa.slot0;
	w.hslot0     = wa.hslot0;
	w.Hb         = wa.Hb;
	w.list_k0    = wa.list_k0;
	w.npop       = wa.npop;
	w.pop        = pi;
	w.mode       = n->mode;
	w.D          = wa.D;
	w.dts        = wa.dts;
	w.tables     = (const void*)wa.tables;
	w.chunk_poly = d.chunk_poly;
	w.draw_offset = d.draw_offset;
	w.state      = d.ustate;
	w.size       = d.size;
	w.neuron_bytes = d.ubytes;
	w.nwords     = d.nwords;
	w.bits       = d.bits;
	w.list       = d.list;
	w.counts     = wa.counts;
	w.cnt        = d.cnt;
	w.acc        = d.acc;
	w.W          = d.W;
	w.F          = d.F;
	w.ngroups    = d.ngroups;
	w.zero_inputs = d.zero_inputs;
	for (int g = 0; g < kMaxGroups; g++) {
		w.group_word[g]   = d.group_word[g];
		w.group_shift[g]  = d.group_shift[g];
		w.group_bits[g]   = d.group_bits[g];
		w.group_field[g]  = d.group_field[g];
		w.group_weight[g] = d.group_weight[g];
	}
	for (int f = 0; f < 3; f++) {
		w.field_offset[f] = P.field_offset[f];
		w.field_slot[f]   = d.field_slot[f];
	}
	w.step_seeds = wa.seeds;
	w.draws      = P.stateful ? P.udraws : 0;
	w.pull       = d.pull;
	w.pull_F     = d.pull_F;
	w.pull_nbins = d.pull_nbins;
	for (int f = 0; f < 3; f++) w.pull_field[f] = d.pull_field[f];
	w.pull_base = d.pull_base;
	w.pull_A    = d.pull_A;
	w.pull_G    = d.pull_G;
	w.pull_koff = d.pull_koff;
	w.hist      = d.hist;
	w.direct    = d.direct;
	return w;
}

// Calls the update callbacks of the stateful (or stateless) user populations on `st`.
int launch_user_pops(spice_net* n, WindowArgs const& wa, int64_t j, bool stateful, bool apply_only, cudaStream_t st) {
	for (int pi = 0; pi < (int)n->pops.size(); pi++) {
		Pop const& P = n->pops[pi];
		if (P.d.model != USER || P.stateful != stateful || P.d.size == 0) continue;
		spice_user_window const w = user_window(n, pi, wa, j, apply_only);
		int const r = reinterpret_cast<spice_user_update_fn>(P.ufn)(&w, (void*)st, P.uctx);
		if (r != 0) return fail(SPICE_ECUDA, "the update function of user population " + std::to_string(pi) +
		                                          " failed (" + std::to_string(r) + ")");
		n->launches++;
	}
	return SPICE_OK;
}

// One call of a user plastic connection's kernels (spice_user_plastic_call).
int call_user_plastic(spice_net* n, Conn const& c, int what, int hslot, int64_t slot, bool deliver) {
	spice_user_plastic_call u;
	memset(&u, 0, sizeof u);
	u.version       = SPICE_USER_PLASTIC_ABI_VERSION;
	u.what          = what;
	u.time          = n->time;
	u.dt            = n->dt;  // synapses see the raw dt (snn.cpp:19, 23)
	u.hslot         = hslot;
	u.slot          = slot;
	u.deliver       = deliver ? 1 : 0;
	u.src_size      = c.d.src_size;
	u.dst_size      = c.d.dst_size;
	u.off           = c.d.off;
	u.nb            = c.d.nb;
	u.state         = c.ustate;
	u.synapse_bytes = c.ubytes;
	u.weight_word   = c.weight_word;
	u.ages          = c.d.ages;
	u.chunks_done   = c.d.chunks_done;
	u.max_row       = c.d.max_row;
	u.dst_hist      = c.d.dst_hist;
	u.src_bits      = c.d.src_bits;
	u.src_nwords    = c.d.src_nwords;
	u.dst_acc       = c.d.dst_acc;
	u.F             = c.d.F;
	u.fslot         = c.d.fslot;
	u.events        = n->d_events;
	int const r     = reinterpret_cast<spice_user_plastic_fn>(c.ufn)(&u, (void*)n->stream, c.uctx);
	if (r != 0) return fail(SPICE_ECUDA, "the kernels of a user plastic connection failed (" + std::to_string(r) + ")");
	n->launches++;
	return SPICE_OK;
}

// A grid barrier of an earlier persistent launch that gave up waiting leaves its steps incomplete.
int check_persist(spice_net* n) {
	if (n->h_pstatus && *(volatile int*)n->h_pstatus != 0)
		return fail(SPICE_ECUDA, "a grid-wide barrier of the persistent step kernel gave up waiting; the network state "
		                         "is invalid");
	return SPICE_OK;
}

// The steps [time, time + chunk) of a network whose windows are one step long, as cooperative
// launches of k_persist (step.cu): one per chunk; with plastic connections the launches are split at
// every step t with t mod 64 == 0, whose catch-up of every plastic synapse (snn.cpp:17-19) runs
// between its update and its deliveries as its own kernel at full occupancy.
int run_persist(spice_net* n, int64_t chunk, const float* d_dt, const u128* d_tables, bool record, int64_t rows,
                int64_t rec_windows) {
	int const np = (int)n->pops.size();
	PersistArgs pa{};
	pa.D           = (int)n->max_delay;
	pa.Hb          = n->Hb;
	pa.npop        = np;
	pa.nconn       = (int)n->conns.size();
	pa.mode        = n->mode;
	pa.pops        = n->d_pops;
	pa.conns       = n->d_conns;
	pa.counts      = n->d_counts;
	pa.events      = n->d_events;
	pa.barrier     = n->d_barrier;
	pa.status      = n->d_pstatus;
	pa.any_plastic = n->plastic ? 1 : 0;
	pa.external_full = n->plastic ? 1 : 0;
	int nb = 0;
	for (int p = 0; p < np; p++) {
		PopDev const& P = n->pops[p].d;
		pa.blk_begin[p] = nb;
		if (P.model == POISSON) {
			pa.blk_kind[p]     = 1;
			pa.blk_per_step[p] = (P.nwords + kNeuronThreads - 1) / kNeuronThreads;
			nb += pa.blk_per_step[p];
		} else if (P.model == EXTERNAL) {
			pa.blk_kind[p] = 2;
			nb += 1;
		} else {
			pa.blk_kind[p] = neuron_block_kind(P) + (P.hist ? kHistKind : 0);
			nb += (int)((P.size + kNeuronThreads - 1) / kNeuronThreads);
		}
	}
	pa.blk_begin[np] = nb;
	pa.nblk          = nb;
	for (size_t ci = 0; ci < n->conns.size(); ci++) pa.chunks[ci] = n->persist_chunks[ci];
	pa.record = record ? 1 : 0;
	if (record) {
		RasterArgs& ra = pa.raster;
		ra.Hb          = n->Hb;
		ra.npop        = np;
		ra.pops        = n->d_pops;
		ra.base        = n->d_raster_base;
		ra.out         = n->rec_out;
		ra.capacity    = n->rec_cap;
		ra.step_counts = n->rec_counts;
	}
	int const per_sm = n->persist_knob >= 2 ? n->persist_knob : kPersistBlocksPerSM;
	int const grid   = std::min(n->persist_grid, n->sm_count * per_sm);
	// one launch over steps [s, e) of the chunk: start_at_c -- step s's update ran in the previous
	// launch; end_after_a -- step e - 1 stops after its update
	auto launch = [&](int64_t s, int64_t e, bool start_at_c, bool end_after_a) -> int {
		int64_t const t0 = n->time + s;
		pa.t0          = t0;
		pa.nsteps      = (int)(e - s);
		pa.parity0     = (n->parity + (int)(s & 1)) & 1;
		pa.dts         = d_dt + s;
		pa.tables      = n->total_draws > 0 ? d_tables + s * kJumpTable : nullptr;
		pa.start_at_c  = start_at_c ? 1 : 0;
		pa.end_after_a = end_after_a ? 1 : 0;
		pa.rec_parity0 = (int)((rec_windows + s) & 1);
		pa.raster.row0 = rows + s;
		for (int p = 0; p < np; p++)
			if (n->pops[p].d.model == EXTERNAL) {
				int64_t const ns = n->pops[p].d.ext_steps;
				pa.ext_pos[p] = ns > 0 ? ((t0 - n->ext_t_set[p]) % ns + ns) % ns : 0;
			}
		CUDA_TRY(cudaMemsetAsync(n->d_barrier, 0, sizeof(unsigned), n->stream));
		int slot = -1;
		TRY(ev_begin(n, 0, &slot));
		CUDA_TRY(launch_persist(n->stream, pa, grid));
		TRY(ev_end(n, slot));
		n->launches++;
		return SPICE_OK;
	};
	if (!n->plastic) {
		TRY(launch(0, chunk, false, false));
	} else {
		int64_t s       = 0;
		bool start_at_c = false;
		while (s < chunk) {
			// the next step f > s (or s itself, not yet updated) whose catch-up runs as its own kernel
			int64_t f = s + (start_at_c ? 1 : 0);
			while (f < chunk && (n->time + f) % 64 != 0) f++;
			if (f >= chunk) {  // no catch-up in the rest of the chunk
				TRY(launch(s, chunk, start_at_c, false));
				break;
			}
			TRY(launch(s, f + 1, start_at_c, true));  // ... up to step f's update
			for (auto const& c : n->conns)
				if (c.d.plastic) {
					CUDA_TRY(launch_plastic_update_all(n->stream, c.d, n->time + f));
					n->launches++;
				}
			s          = f;
			start_at_c = true;
		}
	}
	CUDA_TRY(cudaMemcpyAsync(n->h_pstatus, n->d_pstatus, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
	return SPICE_OK;
}

int run_steps(spice_net* n, int64_t steps, bool record, int64_t* rows_done_out) {
	TRY(prepare(n));
	int const np   = (int)n->pops.size();
	int64_t rows   = 0;
	int64_t rec_windows = 0;  // recorded windows: parity of the raster base
	// fused launches extract a window's raster in the next window's grid; the last one is pending
	bool raster_pending = false;
	RasterArgs pending{};
	int slot_last = -1;
	while (steps > 0) {
		int64_t const chunk = std::min<int64_t>(steps, n->run_cap);
		// chunk buffer cb (pinned staging, device dt / seeds / jump tables) was last used by the chunk
		// before the previous one: wait for that chunk only (its end is recorded on the main stream,
		// which joins the source stream before every delivery)
		int const cb = n->chunk_buf;
		n->chunk_buf ^= 1;
		CUDA_TRY(cudaEventSynchronize(n->ev_chunk[cb]));
		TRY(check_persist(n));
		float* const h_dt          = n->h_dt + (size_t)cb * kRunCap;
		u128* const h_seeds        = n->h_seeds + (size_t)cb * kRunCap;
		float* const d_dt          = n->d_dt + (size_t)cb * kRunCap;
		u128* const d_seeds        = n->d_seeds + (size_t)cb * kRunCap;
		u128* const d_tables       = n->d_tables ? n->d_tables + (size_t)cb * kRunCap * kJumpTable : nullptr;
		for (int64_t j = 0; j < chunk; j++) {
			h_dt[j]    = kahan_next(n);
			h_seeds[j] = seed_next(n);  // xoroshiro64_128p rng(_seed++) (snn.cpp:12)
		}
		CUDA_TRY(cudaMemcpyAsync(d_dt, h_dt, sizeof(float) * chunk, cudaMemcpyHostToDevice, n->stream));
		if (n->total_draws > 0 || n->user_seeds) {
			CUDA_TRY(cudaMemcpyAsync(d_seeds, h_seeds, sizeof(u128) * chunk, cudaMemcpyHostToDevice, n->stream));
		}
		if (n->total_draws > 0) {
			CUDA_TRY(launch_jump_tables(n->stream, d_seeds, chunk, d_tables));
			n->launches++;
		}
		if (n->persist_ok && n->persist_knob) {  // every step of the chunk in one cooperative launch
			TRY(run_persist(n, chunk, d_dt, d_tables, record, rows, rec_windows));
			n->parity ^= (int)(chunk & 1);
			n->time += chunk;
			rows += chunk;
			rec_windows += chunk;
			steps -= chunk;
			CUDA_TRY(cudaEventRecord(n->ev_chunk[cb], n->stream));
			continue;
		}
		// the source kernels of this chunk read dt and the jump tables written above
		CUDA_TRY(cudaEventRecord(n->ev_tab, n->stream));
		CUDA_TRY(cudaStreamWaitEvent(n->stream_src, n->ev_tab, 0));
		int64_t j = 0;
		while (j < chunk) {
			int const k = (int)std::min<int64_t>(n->K, chunk - j);
			int const q = n->parity;
			WindowArgs wa{};
			wa.t0      = n->time;
			wa.K       = k;
			wa.slot0   = (int)((n->time - 1 + n->max_delay) % n->max_delay);
			wa.hslot0  = (int)(n->time % n->Hb);
			wa.D       = n->max_delay;
			wa.Hb      = n->Hb;
			wa.npop    = np;
			wa.mode    = n->mode;
			wa.pops    = n->d_pops;
			wa.dts     = d_dt + j;
			wa.tables  = d_tables ? d_tables + j * kJumpTable : nullptr;
			wa.seeds   = d_seeds + j;
			wa.counts  = n->d_counts + (size_t)q * n->K * np;
			wa.list_k0 = q * n->K;
			wa.variant = n->neuron_variant;
			WindowArgs ws = wa;  // sources
			int nb = 0, nbs = 0;
			// neurons per neuron-update CTA: 2 per thread with LIF window variant 8, which applies when
			// every per-neuron population takes the fast LIF path (deterministic mode)
			bool only_fast = n->mode == SPICE_MODE_DETERMINISTIC;
			for (auto const& P : n->pops)
				if (P.d.model != POISSON && P.d.model != EXTERNAL)
					only_fast &= P.d.model != USER && neuron_block_kind(P.d) == 3 && !P.d.hist;
			int const lif_per_cta = (only_fast && n->neuron_variant == 8) ? 2 * kNeuronThreads : kNeuronThreads;
			for (int p = 0; p < np; p++) {
				PopDev const& P = n->pops[p].d;
				wa.blk_begin[p] = nb;
				ws.blk_begin[p] = nbs;
				if (P.model == POISSON) {
					ws.blk_kind[p]     = 1;
					ws.blk_per_step[p] = (P.nwords + kNeuronThreads - 1) / kNeuronThreads;
					wa.blk_kind[p] = 1;
				} else if (P.model == USER) {
					ws.blk_kind[p] = 0;  // launched by the user's callback
					wa.blk_kind[p] = 0;
				} else if (P.model == EXTERNAL) {
					ws.blk_kind[p]     = 2;
					ws.blk_per_step[p] = 1;
					nbs += k;
					int64_t const ns = P.ext_steps;
					ws.ext_pos[p] = ns > 0 ? ((n->time - n->ext_t_set[p]) % ns + ns) % ns : 0;
					wa.blk_kind[p] = 2;
				} else {
					wa.blk_kind[p] = neuron_block_kind(P) + (P.hist ? kHistKind : 0);
					ws.blk_kind[p] = wa.blk_kind[p];
					nb += (int)((P.size + lif_per_cta - 1) / lif_per_cta);
				}
			}
			// Poisson CTAs: src_steps consecutive steps each -- by default the fewest that keep the
			// window's grid (neuron, source and raster CTAs) within one wave of resident CTAs
			int poisson_bps = 0;
			for (int p = 0; p < np; p++)
				if (n->pops[p].d.model == POISSON) poisson_bps += ws.blk_per_step[p];
			int S = n->src_steps > 0 ? std::min(n->src_steps, k) : 1;
			if (n->src_steps == 0 && poisson_bps > 0) {
				int const wave = n->sm_count * kNeuronBlocksPerSM - (record ? k * np : 0);
				while (S < k && nb + nbs + poisson_bps * ((k + S - 1) / S) > wave) S++;
			}
			ws.src_steps = S;
			{  // source block ranges with the chosen steps per CTA
				int acc = 0;
				for (int p = 0; p < np; p++) {
					PopDev const& P = n->pops[p].d;
					ws.blk_begin[p] = acc;
					if (P.model == POISSON) acc += ws.blk_per_step[p] * ((k + S - 1) / S);
					else if (P.model == EXTERNAL) acc += k;
				}
				nbs = acc;
			}
			wa.blk_begin[np] = nb;
			ws.blk_begin[np] = nbs;
			int slot = -1;
			cudaStream_t const ss = n->overlap_sources ? n->stream_src : n->stream;
			bool user_src = false, user_st = false;
			for (auto const& P : n->pops)
				if (P.d.model == USER) (P.stateful ? user_st : user_src) = true;
			bool const any_src = nbs > 0 || user_src;
			// one stream, one grid for neurons and sources, each launch the programmatic dependent
			// of the previous one (its CTAs wait on the device instead of being launched after it)
			// (plastic kernels stay plain launches between them: a plain kernel releases its dependents
			// when it completes)
			bool const fused = n->launch_mode == 1 && !user_src && !user_st;
			if (fused) {
				TRY(ev_begin(n, 0, &slot));
				wa.span = (slot >= 0 && n->d_span) ? n->d_span + slot : nullptr;  // profiled: the grid's device span
				// the first window of a chunk follows the chunk's host-to-device copies: a plain launch
				CUDA_TRY(launch_window(n->stream, wa, nb, ws, nbs, raster_pending ? &pending : nullptr, j > 0));
				wa.span = nullptr;
				TRY(ev_end(n, slot));
				if (nb + nbs > 0 || raster_pending) n->launches++;
				raster_pending = false;
			} else if (any_src) {
				// sources of this window may start once the lists of this parity are free
				CUDA_TRY(cudaStreamWaitEvent(ss, n->ev_free[q], 0));
				TRY(ev_begin(n, 3, &slot, ss));
				if (nbs > 0) {
					CUDA_TRY(launch_sources(ss, ws, nbs));
					n->launches++;
				}
				if (user_src) TRY(launch_user_pops(n, wa, j, false, false, ss));
				TRY(ev_end(n, slot, ss));
				CUDA_TRY(cudaEventRecord(n->ev_src[q], ss));
			}
			if (!fused) {
				TRY(ev_begin(n, 0, &slot));
				wa.span = (slot >= 0 && n->d_span && !user_st) ? n->d_span + slot : nullptr;  // profiled
				CUDA_TRY(launch_neurons(n->stream, wa, nb));
				wa.span = nullptr;
				if (user_st) TRY(launch_user_pops(n, wa, j, true, false, n->stream));
				TRY(ev_end(n, slot));
				if (nb > 0) n->launches++;
			}
			if (n->plastic && n->time % 64 == 0)  // snn.cpp:17-19 (windows are one step long)
				for (auto const& c : n->conns)
					if (c.d.plastic == SPICE_SYNAPSE_USER_PLASTIC) {
						TRY(call_user_plastic(n, c, 0, 0, 0, false));
					} else if (c.d.plastic) {
						CUDA_TRY(launch_plastic_update_all(n->stream, c.d, n->time));
						n->launches++;
					}
			if (any_src && !fused) CUDA_TRY(cudaStreamWaitEvent(n->stream, n->ev_src[q], 0));
			DeliverArgs da{};
			da.t0     = n->time;
			da.K      = k;
			da.D      = n->max_delay;
			da.nconn  = (int)n->conns.size();
			da.npop   = np;
			da.mode   = n->mode;
			da.conns  = n->d_conns_by_dst;
			da.pops   = n->d_pops;
			da.counts = wa.counts;
			// the other parity's counts (its window is fully delivered) are cleared by the delivery
			// kernel for the window after this one
			da.counts_next     = n->d_counts + (size_t)(q ^ 1) * n->K * np;
			da.counts_next_len = n->K * np;
			da.list_k0         = q * n->K;
			da.events = n->d_events;
			da.slot_lo = n->time + n->dmin - 1;
			da.nslots  = k + n->dmax - n->dmin;
			int tb = 0, smem = 0;
			for (int p = 0; p < np; p++) {
				PopDev const& P = n->pops[p].d;
				da.tile_begin[p] = tb;
				tb += P.ntiles;
				if (P.ntiles) smem = std::max(smem, 4 * P.tile * (n->mode == 0 ? P.W : P.F));
			}
			da.tile_begin[np] = tb;
			da.ntiles_total   = tb;
			da.smem_bytes     = std::max(smem, 4);
			da.parts          = n->deliver_parts;
			da.algo           = n->deliver_algo;
			da.pdl            = fused ? 1 : 0;
			TRY(ev_begin(n, 1, &slot));
			da.span = (slot >= 0 && n->d_span) ? n->d_span + slot : nullptr;  // profiled: the launch's device span
			CUDA_TRY(launch_deliver(n->stream, da, n->deliver_threads));
			if (n->plastic)  // spikes of age d - 1 (snn.cpp:21-25), from the source's bitmap ring
				for (auto const& c : n->conns)
					if (c.d.plastic && n->time >= c.d.delay - 1) {
						int const hs = (int)((n->time - c.d.delay + 1) % n->Hb);
						bool const delivers = n->mode == SPICE_MODE_ATOMIC &&
						                      (c.d.plastic == SPICE_SYNAPSE_ISTDP || c.d.plastic == SPICE_SYNAPSE_USER_PLASTIC ||
						                       c.d.weight != 0.0f);
						if (c.d.plastic == SPICE_SYNAPSE_USER_PLASTIC) {
							TRY(call_user_plastic(n, c, 1, hs, n->time % n->max_delay, delivers));
						} else {
							CUDA_TRY(launch_plastic_deliver(n->stream, c.d, n->time, hs, n->time % n->max_delay, delivers,
							                                n->d_events));
							n->launches++;
						}
					}
			TRY(ev_end(n, slot));
			n->launches++;
			if (n->any_pull) {  // the pulled populations' inputs of the next window, steps [time + k, time + k + K)
				PullArgs pa{};
				pa.t           = n->time + k;
				pa.K           = n->K;
				pa.Hb          = n->Hb;
				pa.nsets       = (int)n->pull_sets.size();
				pa.sets        = n->d_pull_sets;
				pa.nev         = (int)n->pull_ev.size();
				pa.ev          = n->d_pull_ev;
				pa.t_emit0     = n->time;
				pa.k_emit      = k;
				pa.events      = n->d_events;
				pa.npull       = (int)n->pull_pops.size();
				pa.pull_pops   = n->d_pull_pops;
				pa.pull_blk    = n->d_pull_blk;
				pa.pull_blocks = n->pull_blocks;
				pa.pops        = n->d_pops;
				pa.conns       = n->d_conns_by_dst;
				pa.ps_nconn    = n->ps_nconn;
				pa.ps_conn     = n->d_ps_conn;
				pa.ps_pop      = n->d_ps_pop;
				pa.ps_units    = n->ps_units;
				pa.ps_grid     = 5 * std::max(n->sm_count, 1);
				TRY(ev_begin(n, 4, &slot));
				CUDA_TRY(launch_pull(n->stream, pa, n->pull_sets, n->pull_ev));
				TRY(ev_end(n, slot));
				n->launches += n->ps_units > 0 ? 3 : 2;
			}
			if (n->any_direct) TRY(deliver_direct(n));  // windows of one step: the end of step n->time
			if (!fused) CUDA_TRY(cudaEventRecord(n->ev_free[q ^ 1], n->stream));  // the other parity's counts are clear
			if (record) {
				RasterArgs ra{};
				ra.t0          = n->time;
				ra.K           = k;
				ra.Hb          = n->Hb;
				ra.npop        = np;
				ra.pops        = n->d_pops;
				ra.counts      = wa.counts;
				ra.base        = n->d_raster_base;
				ra.parity      = (int)(rec_windows++ & 1);
				ra.out         = n->rec_out;
				ra.capacity    = n->rec_cap;
				ra.step_counts = n->rec_counts;
				ra.row0        = rows;
				ra.pdl         = fused ? 1 : 0;
				if (fused) {  // extracted by the next window's grid, or after the last window
					pending        = ra;
					raster_pending = true;
				} else {
					TRY(ev_begin(n, 2, &slot));
					CUDA_TRY(launch_raster(n->stream, ra));
					TRY(ev_end(n, slot));
					n->launches++;
				}
			}
			n->parity ^= 1;
			n->time += k;
			rows += k;
			j += k;
		}
		steps -= chunk;
		if (raster_pending && steps == 0) {  // the last window's raster
			TRY(ev_begin(n, 2, &slot_last));
			CUDA_TRY(launch_raster(n->stream, pending));
			TRY(ev_end(n, slot_last));
			n->launches++;
			raster_pending = false;
		}
		CUDA_TRY(cudaEventRecord(n->ev_chunk[cb], n->stream));
	}
	if (rows_done_out) *rows_done_out = rows;
	return SPICE_OK;
}

// Applies inputs waiting for the next update so that state reads match the reference's state
// after step() (which has already delivered them).
int flush_pending(spice_net* n) {
	if (!n->prepared || n->time == 0) return SPICE_OK;
	std::vector<int> st;
	std::vector<PopDev> hp;
	bool user = false;
	for (int i = 0; i < (int)n->pops.size(); i++) {
		hp.push_back(n->pops[i].d);
		if (n->pops[i].stateful && n->pops[i].d.model != USER && !n->pops[i].d.pull) st.push_back(i);
		user |= n->pops[i].stateful && n->pops[i].d.model == USER;
	}
	for (int i : n->pull_pops) {  // the pulled inputs of the next step (user models: their callback)
		if (n->pops[i].d.model == USER) continue;
		CUDA_TRY(launch_pull_apply_first(n->stream, n->pops[i].d));
		n->launches++;
	}
	CUDA_TRY(launch_apply_pending(n->stream, n->d_pops, (int)hp.size(), st.data(), (int)st.size(), hp, n->time,
	                              n->max_delay, n->mode));
	n->launches += (int64_t)st.size();
	if (user) {
		WindowArgs wa{};
		wa.t0     = n->time;
		wa.slot0  = (int)((n->time - 1 + n->max_delay) % n->max_delay);
		wa.hslot0 = (int)(n->time % n->Hb);
		wa.Hb     = n->Hb;
		wa.D      = n->max_delay;
		wa.npop   = (int)n->pops.size();
		wa.dts    = n->d_dt;
		wa.counts = n->d_counts;
		TRY(launch_user_pops(n, wa, 0, true, true, n->stream));
	}
	return SPICE_OK;
}

}  // namespace

// ------------------------------------------------------------------------------------------------
// stepping and readback
// ------------------------------------------------------------------------------------------------

extern "C" int spice_step(spice_net* n) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	return run_steps(n, 1, false, nullptr);
}

extern "C" int spice_run(spice_net* n, int64_t steps) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (steps < 0) return fail(SPICE_EINVAL, "steps must be >= 0");
	return run_steps(n, steps, false, nullptr);
}

extern "C" int spice_run_record(spice_net* n, int64_t steps, int64_t* counts_out, int32_t* spikes_out, int64_t capacity,
                                int64_t* total_out) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (steps < 0 || capacity < 0) return fail(SPICE_EINVAL, "steps and capacity must be >= 0");
	TRY(prepare(n));
	int const np = (int)n->pops.size();
	int64_t const need_counts = std::max<int64_t>(steps * np, 1);
	// caller buffers in pinned host memory: the GPU writes the raster into them directly
	auto device_view = [](void* p) -> void* {
		if (!p) return nullptr;
		cudaPointerAttributes at{};
		if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
			cudaGetLastError();  // pageable memory of an older runtime: clear the error
			return nullptr;
		}
		return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
	};
	int32_t* const direct_out  = static_cast<int32_t*>(device_view(spikes_out));
	int64_t* const direct_cnt  = static_cast<int64_t*>(device_view(counts_out));
	bool const direct          = direct_out && direct_cnt;
	// otherwise mapped pinned staging buffers (grown on demand), copied to the caller's at the end
	if (!direct && (n->raster_cap < std::max<int64_t>(capacity, 1) || n->rcounts_cap < need_counts)) {
		CUDA_TRY(cudaStreamSynchronize(n->stream));
		if (n->raster_cap < std::max<int64_t>(capacity, 1)) {
			if (n->h_raster) cudaFreeHost(n->h_raster);
			n->h_raster   = nullptr;
			n->raster_cap = 0;
			CUDA_TRY(cudaHostAlloc((void**)&n->h_raster, sizeof(int32_t) * std::max<int64_t>(capacity, 1), cudaHostAllocMapped));
			n->raster_cap = std::max<int64_t>(capacity, 1);
		}
		if (n->rcounts_cap < need_counts) {
			if (n->h_rcounts) cudaFreeHost(n->h_rcounts);
			n->h_rcounts   = nullptr;
			n->rcounts_cap = 0;
			CUDA_TRY(cudaHostAlloc((void**)&n->h_rcounts, sizeof(int64_t) * need_counts, cudaHostAllocMapped));
			n->rcounts_cap = need_counts;
		}
	}
	if (!n->d_raster_base) TRY(dalloc(n, &n->d_raster_base, 2));
	CUDA_TRY(cudaMemsetAsync(n->d_raster_base, 0, sizeof(int64_t) * 2, n->stream));
	n->rec_out    = direct ? direct_out : n->h_raster;
	n->rec_cap    = direct ? capacity : n->raster_cap;
	n->rec_counts = direct ? direct_cnt : n->h_rcounts;
	int64_t rows = 0;
	int const rc = run_steps(n, steps, true, &rows);
	n->rec_out    = nullptr;
	n->rec_counts = nullptr;
	if (rc != SPICE_OK) {
		// kernels launched before the failure may still write the caller's buffers: let them finish
		if (direct) cudaStreamSynchronize(n->stream);
		return rc;
	}
	int64_t base[2] = {0, 0};
	CUDA_TRY(cudaMemcpyAsync(base, n->d_raster_base, sizeof(base), cudaMemcpyDeviceToHost, n->stream));
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	// the raster ends where the window after the last recorded one would start
	int64_t const total = std::max(base[0], base[1]);
	if (total_out) *total_out = total;
	if (total > capacity)
		return fail(SPICE_EOVERFLOW, "raster needs " + std::to_string(total) + " entries, capacity is " +
		                                 std::to_string(capacity));
	if (direct) return SPICE_OK;  // written in place
	if (counts_out && steps * np > 0) std::memcpy(counts_out, n->h_rcounts, sizeof(int64_t) * steps * np);
	if (spikes_out && total > 0) parallel_copy(spikes_out, n->h_raster, sizeof(int32_t) * (size_t)total);
	return SPICE_OK;
}

namespace {
int age_check(spice_net* n, int pop, int64_t age) {
	if (pop < 0 || pop >= (int)n->pops.size()) return fail(SPICE_EINVAL, "population id out of range");
	int64_t const recorded = std::min<int64_t>(n->time, n->max_delay);
	if (!(0 <= age && age < recorded))
		return pre_failed("neuron_population.h:148", "0 <= age && age < _spike_counts.size()");
	return SPICE_OK;
}
}  // namespace

extern "C" int spice_spikes(spice_net* n, int pop, int64_t age, int32_t* out, int64_t capacity, int64_t* n_out) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	TRY(age_check(n, pop, age));
	PopDev const& P   = n->pops[pop].d;
	int64_t const t   = n->time - 1 - age;
	const uint32_t* b = P.bits + (t % n->Hb) * P.nwords;
	CUDA_TRY(launch_extract(n->stream, b, P.nwords, n->d_tmp, n->d_tmp_n));
	n->launches++;
	int64_t cnt = 0;
	CUDA_TRY(cudaMemcpyAsync(&cnt, n->d_tmp_n, sizeof(int64_t), cudaMemcpyDeviceToHost, n->stream));
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	if (n_out) *n_out = cnt;
	if (cnt > capacity) return fail(SPICE_EOVERFLOW, "spike buffer too small");
	if (cnt && out) CUDA_TRY(cudaMemcpy(out, n->d_tmp, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost));
	return SPICE_OK;
}

extern "C" int spice_spike_count(spice_net* n, int pop, int64_t age, int64_t* n_out) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	TRY(age_check(n, pop, age));
	int64_t cnt = 0;
	int const r = spice_spikes(n, pop, age, nullptr, INT64_MAX, &cnt);
	if (n_out) *n_out = cnt;
	return r;
}

namespace {
int field_ptr(spice_net* n, int pop, int field, void** p) {
	if (pop < 0 || pop >= (int)n->pops.size()) return fail(SPICE_EINVAL, "population id out of range");
	PopDev const& P = n->pops[pop].d;
	if (!n->pops[pop].stateful)
		return fail(SPICE_EINVAL, "Can only return collections of stateful neurons. (neuron_population.h:143)");
	void* f = nullptr;
	switch (field) {
		case SPICE_FIELD_V: f = P.V; break;
		case SPICE_FIELD_GEX: f = P.Gex; break;
		case SPICE_FIELD_GIN: f = P.Gin; break;
		case SPICE_FIELD_TREF: f = P.T; break;
	}
	if (!f) return fail(SPICE_EINVAL, "the neuron model has no such state field");
	*p = f;
	return SPICE_OK;
}
}  // namespace

namespace {
// Field f of a stateful user population: a float member at field_offset[f] of every struct.
int user_field_copy(spice_net* n, int pop, int field, void* host, bool to_host) {
	Pop const& P = n->pops[pop];
	if (!P.stateful) return fail(SPICE_EINVAL, "Can only return collections of stateful neurons. (neuron_population.h:143)");
	if (field < 0 || field >= P.nfields) return fail(SPICE_EINVAL, "the neuron model has no such state field");
	TRY(flush_pending(n));
	char* base = static_cast<char*>(P.d.ustate) + P.field_offset[field];
	if (P.d.size > 0) {
		if (to_host)
			CUDA_TRY(cudaMemcpy2DAsync(host, 4, base, P.d.ubytes, 4, P.d.size, cudaMemcpyDeviceToHost, n->stream));
		else
			CUDA_TRY(cudaMemcpy2DAsync(base, P.d.ubytes, host, 4, 4, P.d.size, cudaMemcpyHostToDevice, n->stream));
	}
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	return SPICE_OK;
}
}  // namespace

extern "C" int spice_get_user_state(spice_net* n, int pop, void* host_out) {
	if (!n || !host_out) return fail(SPICE_EINVAL, "NULL argument");
	if (pop < 0 || pop >= (int)n->pops.size() || n->pops[pop].d.model != USER || !n->pops[pop].stateful)
		return fail(SPICE_EINVAL, "not a stateful user population");
	TRY(flush_pending(n));
	PopDev const& P = n->pops[pop].d;
	CUDA_TRY(cudaMemcpyAsync(host_out, P.ustate, (size_t)P.size * P.ubytes, cudaMemcpyDeviceToHost, n->stream));
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	return SPICE_OK;
}

extern "C" int spice_set_user_state(spice_net* n, int pop, const void* host_in) {
	if (!n || !host_in) return fail(SPICE_EINVAL, "NULL argument");
	if (pop < 0 || pop >= (int)n->pops.size() || n->pops[pop].d.model != USER || !n->pops[pop].stateful)
		return fail(SPICE_EINVAL, "not a stateful user population");
	TRY(flush_pending(n));
	PopDev const& P = n->pops[pop].d;
	CUDA_TRY(cudaMemcpyAsync(P.ustate, host_in, (size_t)P.size * P.ubytes, cudaMemcpyHostToDevice, n->stream));
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	return SPICE_OK;
}

extern "C" int spice_get_state(spice_net* n, int pop, int field, void* host_out) {
	if (!n || !host_out) return fail(SPICE_EINVAL, "NULL argument");
	if (pop >= 0 && pop < (int)n->pops.size() && n->pops[pop].d.model == USER)
		return user_field_copy(n, pop, field, host_out, true);
	void* f = nullptr;
	TRY(field_ptr(n, pop, field, &f));
	TRY(flush_pending(n));
	CUDA_TRY(cudaMemcpyAsync(host_out, f, 4 * n->pops[pop].d.size, cudaMemcpyDeviceToHost, n->stream));
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	return SPICE_OK;
}

extern "C" int spice_set_state(spice_net* n, int pop, int field, const void* host_in) {
	if (!n || !host_in) return fail(SPICE_EINVAL, "NULL argument");
	if (pop >= 0 && pop < (int)n->pops.size() && n->pops[pop].d.model == USER)
		return user_field_copy(n, pop, field, const_cast<void*>(host_in), false);
	void* f = nullptr;
	TRY(field_ptr(n, pop, field, &f));
	TRY(flush_pending(n));
	CUDA_TRY(cudaMemcpyAsync(f, host_in, 4 * n->pops[pop].d.size, cudaMemcpyHostToDevice, n->stream));
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	return SPICE_OK;
}

extern "C" int spice_pop_size(spice_net* n, int pop, int64_t* size_out) {
	if (!n || !size_out) return fail(SPICE_EINVAL, "NULL argument");
	if (pop < 0 || pop >= (int)n->pops.size()) return fail(SPICE_EINVAL, "population id out of range");
	*size_out = n->pops[pop].d.size;
	return SPICE_OK;
}

extern "C" int spice_time(spice_net* n, int64_t* t) {
	if (!n || !t) return fail(SPICE_EINVAL, "NULL argument");
	*t = n->time;
	return SPICE_OK;
}

extern "C" int spice_events(spice_net* n, uint64_t* ev) {
	if (!n || !ev) return fail(SPICE_EINVAL, "NULL argument");
	unsigned long long v = 0;
	CUDA_TRY(cudaMemcpyAsync(&v, n->d_events, sizeof(v), cudaMemcpyDeviceToHost, n->stream));
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	*ev = v;
	return SPICE_OK;
}

extern "C" int spice_conn_size(spice_net* n, int conn, int64_t* src_out, int64_t* syn_out) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (conn < 0 || conn >= (int)n->conns.size()) return fail(SPICE_EINVAL, "connection id out of range");
	TRY(generate_pending(n));
	if (src_out) *src_out = n->conns[conn].d.src_size;
	if (syn_out) *syn_out = n->conns[conn].synapses;
	return SPICE_OK;
}

extern "C" int spice_get_csr(spice_net* n, int conn, int64_t* off, int32_t* nb) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (conn < 0 || conn >= (int)n->conns.size()) return fail(SPICE_EINVAL, "connection id out of range");
	TRY(generate_pending(n));
	Conn const& c = n->conns[conn];
	if (off) CUDA_TRY(cudaMemcpy(off, c.d.off, sizeof(int64_t) * (c.d.src_size + 1), cudaMemcpyDeviceToHost));
	if (nb && c.synapses) CUDA_TRY(cudaMemcpy(nb, c.d.nb, sizeof(int32_t) * c.synapses, cudaMemcpyDeviceToHost));
	return SPICE_OK;
}

extern "C" int spice_get_csc(spice_net* n, int conn, int64_t* col_off, int32_t* src) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (conn < 0 || conn >= (int)n->conns.size()) return fail(SPICE_EINVAL, "connection id out of range");
	TRY(generate_pending(n));
	TRY(init_weights(n));
	TRY(ensure_csc(n, conn));
	Conn const& c = n->conns[conn];
	if (col_off) CUDA_TRY(cudaMemcpy(col_off, c.d.csc_off, sizeof(int64_t) * (c.d.dst_size + 1), cudaMemcpyDeviceToHost));
	if (src && c.synapses) CUDA_TRY(cudaMemcpy(src, c.d.csc_src, sizeof(int32_t) * c.synapses, cudaMemcpyDeviceToHost));
	return SPICE_OK;
}

extern "C" int spice_set_profiling(spice_net* n, int on) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	TRY(harvest(n));
	n->profiling = on != 0;
	for (auto& s : n->stats) s = KernelStat{};
	if (n->profiling) {
		while (n->ev_pool.size() < kEventPool) {
			cudaEvent_t e;
			CUDA_TRY(cudaEventCreate(&e));
			n->ev_pool.push_back(e);
		}
		if (!n->d_span) TRY(dalloc(n, &n->d_span, kEventPool));  // zeroed
	}
	return SPICE_OK;
}

extern "C" int spice_get_synapse_state(spice_net* n, int conn, int field, float* out) {
	if (!n || !out) return fail(SPICE_EINVAL, "NULL argument");
	if (conn < 0 || conn >= (int)n->conns.size()) return fail(SPICE_EINVAL, "connection id out of range");
	if (field < 0 || field > 2) return fail(SPICE_EINVAL, "field must be 0 (W), 1 (x_pre) or 2 (x_post)");
	if (!n->conns[conn].d.plastic && !(n->conns[conn].weighted && field == 0))
		return fail(SPICE_EINVAL, "not a plastic connection (a weighted connection has field 0, its weights)");
	TRY(prepare(n));
	ConnDev const& d = n->conns[conn].d;
	const float* src = n->conns[conn].weighted ? d.wts : (field == 0 ? d.sW : (field == 1 ? d.sA : d.sB));
	int64_t const m  = n->conns[conn].synapses;
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	if (m > 0) CUDA_TRY(cudaMemcpy(out, src, sizeof(float) * m, cudaMemcpyDeviceToHost));
	return SPICE_OK;
}

extern "C" int spice_kernel_stats(spice_net* n, int kind, int64_t* launches, double* ms) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (kind < 0 || kind > 4) return fail(SPICE_EINVAL, "unknown kernel kind");
	TRY(harvest(n));
	if (launches) *launches = n->stats[kind].launches;
	if (ms) *ms = n->stats[kind].ms;
	return SPICE_OK;
}

extern "C" int spice_kernel_span(spice_net* n, int kind, int64_t* launches, double* ms) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (kind < 0 || kind > 4) return fail(SPICE_EINVAL, "unknown kernel kind");
	TRY(harvest(n));
	if (launches) *launches = n->stats[kind].span_launches;
	if (ms) *ms = n->stats[kind].span_ms;
	return SPICE_OK;
}

extern "C" int spice_launch_count(spice_net* n, int64_t* out) {
	if (!n || !out) return fail(SPICE_EINVAL, "NULL argument");
	*out = n->launches;
	return SPICE_OK;
}

extern "C" int spice_set_tuning(spice_net* n, int knob, int64_t value) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	switch (knob) {
		case SPICE_TUNE_TILE_BYTES:
			if (value < 1024 || value > 220 * 1024) return fail(SPICE_EINVAL, "tile bytes must be in [1 KiB, 220 KiB]");
			n->tile_set = true;
			if (n->tile_bytes == (int)value) return SPICE_OK;
			n->tile_bytes = (int)value;
			default_algo(n);  // a tile too large for the default mapping's staging
			if (n->prepared) {  // re-tile: the input ring layout does not depend on the tile size
				TRY(setup_tiles(n, false));
				std::vector<PopDev> hp;
				for (auto& p : n->pops) hp.push_back(p.d);
				CUDA_TRY(cudaMemcpy(n->d_pops, hp.data(), sizeof(PopDev) * hp.size(), cudaMemcpyHostToDevice));
				std::vector<ConnDev> hb;
				for (int ci : n->by_dst) hb.push_back(n->conns[ci].d);
				if (!hb.empty())
					CUDA_TRY(cudaMemcpy(n->d_conns_by_dst, hb.data(), sizeof(ConnDev) * hb.size(), cudaMemcpyHostToDevice));
			}
			return SPICE_OK;
		case SPICE_TUNE_DELIVER_THREADS:
			if (value < 32 || value > 1024 || value % 32) return fail(SPICE_EINVAL, "threads must be a multiple of 32 in [32, 1024]");
			n->deliver_threads = (int)value;
			n->threads_set     = true;
			return SPICE_OK;
		case SPICE_TUNE_DELIVER_ALGO:
			if (value < 0 || value >= kDeliverAlgos)
				return fail(SPICE_EINVAL, "delivery algorithm must be 0 .. " + std::to_string(kDeliverAlgos - 1));
			n->deliver_algo = (int)value;
			n->algo_set     = true;
			if (n->prepared && compact_algo((int)value)) {  // build the compact targets for the current tiles
				TRY(setup_tiles(n, false));
				std::vector<PopDev> hp;
				for (auto& p : n->pops) hp.push_back(p.d);
				CUDA_TRY(cudaMemcpy(n->d_pops, hp.data(), sizeof(PopDev) * hp.size(), cudaMemcpyHostToDevice));
				std::vector<ConnDev> hb;
				for (int ci : n->by_dst) hb.push_back(n->conns[ci].d);
				if (!hb.empty())
					CUDA_TRY(cudaMemcpy(n->d_conns_by_dst, hb.data(), sizeof(ConnDev) * hb.size(), cudaMemcpyHostToDevice));
			}
			return SPICE_OK;
		case SPICE_TUNE_LAUNCH:
			if (value < 0 || value > 1) return fail(SPICE_EINVAL, "launch mode must be 0 or 1");
			if (n->prepared && n->launch_mode != (int)value) {  // the streams hand over at a quiet point
				CUDA_TRY(cudaStreamSynchronize(n->stream));
				if (n->stream_src) CUDA_TRY(cudaStreamSynchronize(n->stream_src));
				for (int q = 0; q < 2; q++) CUDA_TRY(cudaEventRecord(n->ev_free[q], n->stream));
			}
			n->launch_mode = (int)value;
			return SPICE_OK;
		case SPICE_TUNE_SOURCE_STEPS:
			if (value < 0 || value > kMaxWindow) return fail(SPICE_EINVAL, "source steps must be in [0, 64]");
			n->src_steps = (int)value;
			return SPICE_OK;
		case SPICE_TUNE_PULL:
			if (value < 0 || value > 1) return fail(SPICE_EINVAL, "pull must be 0 or 1");
			if (n->prepared && n->pull_all != (value != 0))
				return fail(SPICE_ESTATE, "the delivery path of a population is fixed once the network steps");
			n->pull_all = value != 0;
			return SPICE_OK;
		case SPICE_TUNE_PERSISTENT:
			if (value < 0 || value > 32) return fail(SPICE_EINVAL, "persistent must be 0 (off), 1 (on) or 2 .. 32 (on, CTAs per SM)");
			if (n->prepared && value != 0 && !n->persist_ok)
				return fail(SPICE_ESTATE, "persistent steps are set up when the network first steps (this network "
				                          "was prepared without them, or is not eligible)");
			n->persist_knob = (int)value;
			return SPICE_OK;
		case SPICE_TUNE_NEURON_VARIANT:
			if (value < 0 || value > 9) return fail(SPICE_EINVAL, "neuron variant must be 0 .. 9");
			n->neuron_variant = (int)value;
			n->variant_set    = true;
			return SPICE_OK;
		case SPICE_TUNE_OVERLAP_SOURCES:
			if (value < 0 || value > 1) return fail(SPICE_EINVAL, "overlap must be 0 or 1");
			if (n->prepared) {
				CUDA_TRY(cudaStreamSynchronize(n->stream));
				if (n->stream_src) CUDA_TRY(cudaStreamSynchronize(n->stream_src));
			}
			n->overlap_sources = (int)value;
			return SPICE_OK;
		case SPICE_TUNE_DELIVER_PARTS: {
			if (value < 1 || value > 64) return fail(SPICE_EINVAL, "parts must be in [1, 64]");
			if (n->deliver_parts == (int)value) return SPICE_OK;
			bool const was_split = n->deliver_parts > 1;
			n->deliver_parts      = (int)value;
			if (n->prepared && was_split != (value > 1)) {
				// Overwritten slots (one delivery CTA per tile) are not cleared after use; slots that
				// several CTAs accumulate into must start at zero.  Going from the first to the second
				// convention, clear every slot that holds no pending input: for a population whose
				// inputs all have delay d, slots t+d-1 .. t+D-2 (mod D).
				std::vector<int> was_zeroing;
				for (auto& p : n->pops) was_zeroing.push_back(p.d.zero_inputs);
				TRY(setup_tiles(n, false));
				for (size_t pi = 0; pi < n->pops.size(); pi++) {
					PopDev& d = n->pops[pi].d;
					if (was_zeroing[pi] || !d.zero_inputs || d.in_end == d.in_begin) continue;
					int const dl = n->conns[n->by_dst[d.in_begin]].d.delay;
					for (int64_t sg = n->time + dl - 1; sg <= n->time + n->max_delay - 2; sg++) {
						int64_t const sl = sg % n->max_delay;
						if (d.cnt) CUDA_TRY(cudaMemsetAsync(d.cnt + sl * d.size * d.W, 0, sizeof(uint32_t) * d.size * d.W, n->stream));
						if (d.acc) CUDA_TRY(cudaMemsetAsync(d.acc + sl * d.size * d.F, 0, sizeof(float) * d.size * d.F, n->stream));
					}
				}
				std::vector<PopDev> hp;
				for (auto& p : n->pops) hp.push_back(p.d);
				CUDA_TRY(cudaMemcpy(n->d_pops, hp.data(), sizeof(PopDev) * hp.size(), cudaMemcpyHostToDevice));
				std::vector<ConnDev> hb;
				for (int ci : n->by_dst) hb.push_back(n->conns[ci].d);
				if (!hb.empty())
					CUDA_TRY(cudaMemcpy(n->d_conns_by_dst, hb.data(), sizeof(ConnDev) * hb.size(), cudaMemcpyHostToDevice));
			}
			return SPICE_OK;
		}
	}
	return fail(SPICE_EINVAL, "unknown tuning knob");
}

extern "C" int spice_get_tuning(spice_net* n, int knob, int64_t* value) {
	if (!n || !value) return fail(SPICE_EINVAL, "NULL argument");
	switch (knob) {
		case SPICE_TUNE_TILE_BYTES: *value = n->tile_bytes; return SPICE_OK;
		case SPICE_TUNE_DELIVER_THREADS: *value = n->deliver_threads; return SPICE_OK;
		case SPICE_TUNE_DELIVER_PARTS: *value = n->deliver_parts; return SPICE_OK;
		case SPICE_TUNE_DELIVER_ALGO: *value = n->deliver_algo; return SPICE_OK;
		case SPICE_TUNE_OVERLAP_SOURCES: *value = n->overlap_sources; return SPICE_OK;
		case SPICE_TUNE_NEURON_VARIANT: *value = n->neuron_variant; return SPICE_OK;
		case SPICE_TUNE_LAUNCH: *value = n->launch_mode; return SPICE_OK;
		case SPICE_TUNE_PULL: *value = n->pull_all ? 1 : 0; return SPICE_OK;
		case SPICE_TUNE_SOURCE_STEPS: *value = n->src_steps; return SPICE_OK;
		case SPICE_TUNE_PERSISTENT: *value = n->persist_knob; return SPICE_OK;
	}
	return fail(SPICE_EINVAL, "unknown tuning knob (graph windows belong to batches)");
}

extern "C" int spice_get_stream(spice_net* n, void** out) {
	if (!n || !out) return fail(SPICE_EINVAL, "NULL argument");
	*out = (void*)n->stream;
	return SPICE_OK;
}

extern "C" int spice_synchronize(spice_net* n) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	return check_persist(n);
}

extern "C" int spice_selftest_skip_rounding(int64_t count, uint64_t seed, int64_t* mismatches,
                                            uint32_t* first_a, double* first_f) {
	if (count < 0 || !mismatches) return fail(SPICE_EINVAL, "count must be >= 0 and mismatches not NULL");
	unsigned long long* d = nullptr;
	CUDA_TRY(cudaMalloc(&d, sizeof(unsigned long long) * 3));
	cudaError_t e = cudaMemset(d, 0, sizeof(unsigned long long) * 3);
	if (e == cudaSuccess) e = launch_selftest_mulround(nullptr, count, seed, d, d + 1);
	unsigned long long h[3] = {0, 0, 0};
	if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
	cudaFree(d);
	if (e != cudaSuccess) return fail(SPICE_ECUDA, cudaGetErrorString(e));
	*mismatches = (int64_t)h[0];
	if (first_a) *first_a = (uint32_t)h[1];
	if (first_f) memcpy(first_f, &h[2], sizeof(double));
	return SPICE_OK;
}

extern "C" int spice_user_draws(spice_net* n, int pop, int draws) {
	if (!n) return fail(SPICE_EINVAL, "net must not be NULL");
	if (pop < 0 || pop >= (int)n->pops.size() || n->pops[pop].d.model != USER || !n->pops[pop].stateful)
		return fail(SPICE_EINVAL, "not a stateful user population");
	if (draws < 0 || draws > 1024) return fail(SPICE_EINVAL, "draws per update must be in [0, 1024]");
	if (n->prepared) return fail(SPICE_ESTATE, "draws must be declared before the network first steps");
	n->pops[pop].udraws = draws;
	return SPICE_OK;
}

extern "C" int spice_population_seed(spice_net* n, int pop, uint64_t* lo, uint64_t* hi) {
	if (!n || !lo || !hi) return fail(SPICE_EINVAL, "NULL argument");
	if (pop < 0 || pop >= (int)n->pops.size()) return fail(SPICE_EINVAL, "population id out of range");
	if (!n->pops[pop].stateful) return fail(SPICE_EINVAL, "a stateless population consumes no seed");
	*lo = n->pops[pop].seed.lo;
	*hi = n->pops[pop].seed.hi;
	return SPICE_OK;
}

extern "C" int spice_connection_seeds(spice_net* n, int conn, uint64_t* out) {
	if (!n || !out) return fail(SPICE_EINVAL, "NULL argument");
	if (conn < 0 || conn >= (int)n->conns.size()) return fail(SPICE_EINVAL, "connection id out of range");
	Conn const& c = n->conns[conn];
	out[0] = c.gseed.lo;
	out[1] = c.gseed.hi;
	out[2] = c.wseed.lo;
	out[3] = c.wseed.hi;
	return SPICE_OK;
}

extern "C" int spice_set_synapse_weights(spice_net* n, int conn, const float* w) {
	if (!n || !w) return fail(SPICE_EINVAL, "NULL argument");
	if (conn < 0 || conn >= (int)n->conns.size()) return fail(SPICE_EINVAL, "connection id out of range");
	Conn& c = n->conns[conn];
	if (!c.weighted || c.wsource == 0) return fail(SPICE_EINVAL, "not a weighted connection with host weights");
	if (n->prepared) return fail(SPICE_ESTATE, "weights must be set before the network first steps");
	TRY(generate_pending(n));
	if (!c.d.wts) {
		float* d = nullptr;
		TRY(dalloc(n, &d, (size_t)std::max<int64_t>(c.synapses, 1), false));
		c.d.wts = d;
	}
	if (c.synapses > 0) CUDA_TRY(cudaMemcpy((void*)c.d.wts, w, sizeof(float) * c.synapses, cudaMemcpyHostToDevice));
	return SPICE_OK;
}

extern "C" int spice_user_plastic(spice_net* n, int conn, spice_user_plastic_fn fn, void* ctx, const void* init_syn) {
	if (!n || !fn || !init_syn) return fail(SPICE_EINVAL, "NULL argument");
	if (conn < 0 || conn >= (int)n->conns.size()) return fail(SPICE_EINVAL, "connection id out of range");
	Conn& c = n->conns[conn];
	if (c.d.plastic != SPICE_SYNAPSE_USER_PLASTIC) return fail(SPICE_EINVAL, "not a user plastic connection");
	if (n->prepared) return fail(SPICE_ESTATE, "user plastic kernels are registered before the network first steps");
	c.ufn  = (void*)fn;
	c.uctx = ctx;
	c.uinit.assign(static_cast<const char*>(init_syn), static_cast<const char*>(init_syn) + c.ubytes);
	return SPICE_OK;
}

extern "C" int spice_user_deliver(spice_net* n, int conn, spice_user_deliver_fn fn, void* ctx, const void* init_syn) {
	if (!n || !fn) return fail(SPICE_EINVAL, "NULL argument");
	if (conn < 0 || conn >= (int)n->conns.size()) return fail(SPICE_EINVAL, "connection id out of range");
	Conn& c = n->conns[conn];
	if (!c.udeliver) return fail(SPICE_EINVAL, "not a user deliver connection");
	if (n->prepared) return fail(SPICE_ESTATE, "user deliver kernels are registered before the network first steps");
	if (c.ubytes > 0 && !init_syn) return fail(SPICE_EINVAL, "a stateful synapse needs its initial state");
	c.ufn  = (void*)fn;
	c.uctx = ctx;
	if (c.ubytes > 0) c.uinit.assign(static_cast<const char*>(init_syn), static_cast<const char*>(init_syn) + c.ubytes);
	return SPICE_OK;
}

extern "C" int spice_set_user_synapse_state(spice_net* n, int conn, const void* in) {
	if (!n || !in) return fail(SPICE_EINVAL, "NULL argument");
	if (conn < 0 || conn >= (int)n->conns.size()) return fail(SPICE_EINVAL, "connection id out of range");
	Conn& c = n->conns[conn];
	if (c.d.plastic != SPICE_SYNAPSE_USER_PLASTIC && !(c.udeliver && c.ubytes > 0))
		return fail(SPICE_EINVAL, "not a connection of user synapse structs");
	if (n->prepared) return fail(SPICE_ESTATE, "the initial synapse state is set before the network first steps");
	TRY(generate_pending(n));
	c.uhost.assign(static_cast<const char*>(in), static_cast<const char*>(in) + (size_t)c.synapses * c.ubytes);
	return SPICE_OK;
}

extern "C" int spice_get_user_synapse_state(spice_net* n, int conn, void* out) {
	if (!n || !out) return fail(SPICE_EINVAL, "NULL argument");
	if (conn < 0 || conn >= (int)n->conns.size()) return fail(SPICE_EINVAL, "connection id out of range");
	Conn const& c = n->conns[conn];
	if (c.d.plastic != SPICE_SYNAPSE_USER_PLASTIC && !(c.udeliver && c.ubytes > 0))
		return fail(SPICE_EINVAL, "not a connection of user synapse structs");
	TRY(prepare(n));
	CUDA_TRY(cudaStreamSynchronize(n->stream));
	if (c.synapses > 0) CUDA_TRY(cudaMemcpy(out, c.ustate, (size_t)c.synapses * c.ubytes, cudaMemcpyDeviceToHost));
	return SPICE_OK;
}

namespace spice_gb300 {
// Generates pending adjacency and allocates the device state (batch.cu prepares its members).
int net_prepare(spice_net* n) { return prepare(n); }
}  // namespace spice_gb300
