// rng_host.cpp -- host-side seed hashing and GF(2) jump-ahead for xoroshiro128+.
#include <string.h>

#include <vector>

#include "rng.h"

namespace spice_gb300 {

using mm3::C1;
using mm3::C2;
using mm3::finish;
using mm3::mix_block;

u128 murmur3_bytes(const void* ptr, uint64_t len) {
	const uint8_t* data = static_cast<const uint8_t*>(ptr);
	u128 h              = {mm3::H0_LO, mm3::H0_HI};
	uint64_t const nblocks = len / 16;
	for (uint64_t i = 0; i < nblocks; i++) {
		uint64_t k1, k2;
		memcpy(&k1, data + 16 * i, 8);
		memcpy(&k2, data + 16 * i + 8, 8);
		mix_block(h, k1, k2);
	}
	// tail: bytes 8..15 go to k2, bytes 0..7 to k1, little-endian (random.h:58-90)
	const uint8_t* tail = data + nblocks * 16;
	uint64_t const rem  = len & 15;
	uint64_t k1 = 0, k2 = 0;
	for (uint64_t b = rem; b > 8; b--) k2 ^= uint64_t(tail[b - 1]) << (8 * (b - 9));
	if (rem > 8) {
		k2 *= C2; k2 = rotl64(k2, 33); k2 *= C1; h.hi ^= k2;
	}
	for (uint64_t b = rem < 8 ? rem : 8; b > 0; b--) k1 ^= uint64_t(tail[b - 1]) << (8 * (b - 1));
	if (rem > 0) {
		k1 *= C1; k1 = rotl64(k1, 31); k1 *= C2; h.lo ^= k1;
	}
	finish(h, len);
	return h;
}


namespace {
// Berlekamp-Massey over GF(2): the shortest LFSR c_1..c_L with b[n] = sum c_i b[n-i].
std::vector<uint8_t> berlekamp_massey(std::vector<uint8_t> const& b, int& L) {
	size_t const N = b.size();
	std::vector<uint8_t> C(N + 1, 0), B(N + 1, 0), T;
	C[0] = B[0] = 1;
	L           = 0;
	int m       = 1;
	for (size_t n = 0; n < N; n++) {
		uint8_t d = b[n];
		for (int i = 1; i <= L; i++) d ^= C[i] & b[n - i];
		if (!d) {
			m++;
			continue;
		}
		T = C;
		for (size_t i = 0; i + m <= N; i++) C[i + m] ^= B[i];
		if (2 * L <= (int)n) {
			L = (int)n + 1 - L;
			B = T;
			m = 1;
		} else {
			m++;
		}
	}
	return C;
}

u128 compute_charpoly() {
	// 256 bits of a linear functional of the state (bit 0 of s0) along one trajectory.
	uint64_t s0 = 0x0123456789abcdefULL, s1 = 0xfedcba9876543210ULL;
	std::vector<uint8_t> bits(256);
	for (int n = 0; n < 256; n++) {
		bits[n] = s0 & 1;
		xoro_next(s0, s1);
	}
	int L  = 0;
	auto C = berlekamp_massey(bits, L);
	// P(x) = x^L C(1/x): the coefficient of x^k is c_{L-k}.
	u128 p = {0, 0};
	if (L != 128) return p;  // cannot happen for a full-period generator; callers check
	for (int k = 0; k < 128; k++)
		if (C[128 - k]) (k < 64 ? p.lo : p.hi) |= 1ULL << (k & 63);
	return p;
}
}  // namespace

u128 xoro_charpoly() {
	static u128 const P = compute_charpoly();
	return P;
}

u128 gf2_mulmod(u128 a, u128 b) {
	u128 const P = xoro_charpoly();
	u128 r       = {0, 0};
	for (int i = 127; i >= 0; i--) {
		uint64_t const carry = r.hi >> 63;
		r.hi                 = (r.hi << 1) | (r.lo >> 63);
		r.lo <<= 1;
		if (carry) {
			r.lo ^= P.lo;
			r.hi ^= P.hi;
		}
		if (((i < 64 ? b.lo : b.hi) >> (i & 63)) & 1) {
			r.lo ^= a.lo;
			r.hi ^= a.hi;
		}
	}
	return r;
}

u128 gf2_xpow(uint64_t n) {
	if (n < 128) {
		u128 r = {0, 0};
		(n < 64 ? r.lo : r.hi) = 1ULL << (n & 63);
		return r;
	}
	u128 result = {1, 0};
	u128 base   = {2, 0};  // x
	while (n) {
		if (n & 1) result = gf2_mulmod(result, base);
		base = gf2_mulmod(base, base);
		n >>= 1;
	}
	return result;
}

void xoro_jump(uint64_t& s0, uint64_t& s1, u128 poly) {
	uint64_t a0 = 0, a1 = 0;
	for (int i = 0; i < 128; i++) {
		if (((i < 64 ? poly.lo : poly.hi) >> (i & 63)) & 1) {
			a0 ^= s0;
			a1 ^= s1;
		}
		xoro_next(s0, s1);
	}
	s0 = a0;
	s1 = a1;
}

}  // namespace spice_gb300
