// rng.h -- seed chain, xoroshiro128+ and GF(2) jump-ahead, shared by host and device code.
//
// The reference draws every random number from xoroshiro128+ (rotations 24/16/37) seeded by a
// murmur3-based seed_seq (spice/include/spice/util/random.h:32-175, 222-234).  Its streams are
// serial; the GPU engine reproduces them in parallel by jumping each thread to its position in
// the stream.  The state transition T of xoroshiro128+ is linear over GF(2), so with P(x) the
// characteristic polynomial of T and  x^n mod P(x) = sum_i a_i x^i,
//   T^n(s) = sum_i a_i T^i(s)                          (Cayley-Hamilton)
// i.e. a jump by n is an XOR of the states s, T(s), ..., T^127(s) selected by the 128 bits
// a_i.  P is computed from the generator's definition by Berlekamp-Massey (rng_host.cpp).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define SPICE_HD __host__ __device__ __forceinline__
#else
#define SPICE_HD inline
#endif

namespace spice_gb300 {

struct u128 {
	uint64_t lo, hi;
};

SPICE_HD uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

// xoroshiro64_128p::operator() (random.h:222-234); s0 = seed.lo, s1 = seed.hi (random.h:188-192).
SPICE_HD uint64_t xoro_next(uint64_t& s0, uint64_t& s1) {
	uint64_t const r = s0 + s1;
	uint64_t const t = s0 ^ s1;
	s0               = rotl64(s0, 24) ^ t ^ (t << 16);
	s1               = rotl64(t, 37);
	return r;
}

// generate_canonical<float, false> on a 64-bit engine (random.h:236-247).
SPICE_HD float canonical_f32(uint64_t u) { return (float)(u >> 40) * (1.0f / 16777216.0f); }
// generate_canonical<double, true> (random.h:236-247): ((u >> 11) + 1) / 2^53 in (0, 1].
SPICE_HD double canonical_f64_leftopen(uint64_t u) {
	return (double)((u >> 11) + 1) * (1.0 / 9007199254740992.0);
}

// ---- MurmurHash3-x64-128 with the reference's fixed seed (random.h:19-139) ----
namespace mm3 {
constexpr uint64_t C1 = 0x87c37b91114253d5ULL;
constexpr uint64_t C2 = 0x4cf5ad432745937fULL;
constexpr uint64_t H0_LO = 0x2E4016967F18E81ULL, H0_HI = 0x447567949F9AA86ULL;

SPICE_HD uint64_t fmix64(uint64_t k) {  // random.h:19-26
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdULL;
	k ^= k >> 33;
	k *= 0xc4ceb9fe1a85ec53ULL;
	k ^= k >> 33;
	return k;
}
SPICE_HD void mix_block(u128& h, uint64_t k1, uint64_t k2) {
	k1 *= C1; k1 = rotl64(k1, 31); k1 *= C2; h.lo ^= k1;
	h.lo = rotl64(h.lo, 27); h.lo += h.hi; h.lo = h.lo * 5 + 0x52dce729;
	k2 *= C2; k2 = rotl64(k2, 33); k2 *= C1; h.hi ^= k2;
	h.hi = rotl64(h.hi, 31); h.hi += h.lo; h.hi = h.hi * 5 + 0x38495ab5;
}
SPICE_HD void finish(u128& h, uint64_t len) {
	h.lo ^= len; h.hi ^= len;
	h.lo += h.hi; h.hi += h.lo;
	h.lo = fmix64(h.lo); h.hi = fmix64(h.hi);
	h.lo += h.hi; h.hi += h.lo;
}
}  // namespace mm3

// The one-block hash that advances a seed_seq (random.h:108-139); host and device.
SPICE_HD u128 murmur3_u128(u128 k) {
	u128 h = {mm3::H0_LO, mm3::H0_HI};
	mm3::mix_block(h, k.lo, k.hi);
	mm3::finish(h, 16);
	return h;
}

// ---- host-side helpers (rng_host.cpp) ----
// MurmurHash3-x64-128 of bytes with the reference's fixed seed (random.h:32-107).
u128 murmur3_bytes(const void* data, uint64_t len);
// Characteristic polynomial of the xoroshiro128+ transition: x^128 + (hi:lo).
u128 xoro_charpoly();
// (a * b) mod P over GF(2); a, b of degree < 128.
u128 gf2_mulmod(u128 a, u128 b);
// x^n mod P.
u128 gf2_xpow(uint64_t n);
// Applies poly(T) to a state (host reference implementation of the jump).
void xoro_jump(uint64_t& s0, uint64_t& s1, u128 poly);

}  // namespace spice_gb300
