// (float)((double)a * f), bit-identical to __double2float_rn(__dmul_rn((double)a, f)), computed with
// integer arithmetic (the FP64 pipe of this GPU is slow): the exact product of a's 24-bit and f's
// 53-bit significands (at most 77 bits), rounded to nearest-even to 53 bits as the double multiply
// does, then to float precision (24 bits, or the fixed 2^-149 quantum of subnormal floats) as the
// conversion does, with overflow to +inf.  For finite a >= 0 and finite normal f > 0 whose double
// product is normal; f is given packed by pack_f64 below.
#pragma once
#include <stdint.h>

#ifndef SPICE_HD
#define SPICE_HD __host__ __device__
#endif

namespace spice_gb300 {

// significand (53 bits, leading bit set) | (binary exponent of its last bit + 1100) << 53
inline uint64_t pack_f64(double f) {
	int e          = 0;
	double const m = frexp(f, &e);  // f = m 2^e, m in [0.5, 1)
	uint64_t const mf = (uint64_t)ldexp(m, 53);
	return mf | ((uint64_t)(e - 53 + 1100) << 53);
}

__device__ __forceinline__ int bitlen64(uint64_t x) { return 64 - __clzll((long long)x); }

// The common case -- a normal, the result a normal float -- with 32 x 32 -> 64-bit products: f's
// significand split into its top 29 and low 24 bits, the exact product P = ma mf (76 or 77 bits) as
// U 2^24 + Ylo, the double's 53 bits d (U, or U with Ylo's top bit, rounded by the rest), then 24
// bits of d (rounded by its low 29).  Returns false (leaving *out alone) for the other cases.
__device__ __forceinline__ bool mul_f32_f64_rn_normal(uint32_t ab, uint64_t packed, float* out) {
	uint32_t const fa = ab >> 23;
	if (fa == 0u) return false;  // subnormal a
	uint32_t const ma = (ab & 0x7fffffu) | 0x800000u;
	uint64_t const mf = packed & ((1ull << 53) - 1);
	int const ef      = (int)(packed >> 53) - 1100;
	uint32_t const fh = (uint32_t)(mf >> 24);        // 29 bits
	uint32_t const fl = (uint32_t)mf & 0xffffffu;    // 24 bits
	uint64_t const y  = (uint64_t)ma * fl;           // < 2^48
	uint64_t const u  = (uint64_t)ma * fh + (y >> 24);  // floor(P / 2^24): 52 or 53 bits
	uint32_t const ylo = (uint32_t)y & 0xffffffu;
	uint64_t d;
	int e;  // the double product = d 2^e, d of 53 bits
	if (u >> 52) {  // P has 77 bits: d = U rounded by the 24 bits below
		d = u + ((ylo > 0x800000u || (ylo == 0x800000u && (u & 1))) ? 1 : 0);
		e = (int)fa - 150 + ef + 24;
	} else {  // 76 bits: d = U and Ylo's top bit, rounded by the 23 bits below
		uint64_t const k  = (u << 1) | (ylo >> 23);
		uint32_t const z  = ylo & 0x7fffffu;
		d = k + ((z > 0x400000u || (z == 0x400000u && (k & 1))) ? 1 : 0);
		e = (int)fa - 150 + ef + 23;
	}
	if (d >> 53) {  // rounded up to 2^53
		d >>= 1;
		e += 1;
	}
	// 24 bits of d, rounded by its low 29
	uint32_t const rem = (uint32_t)d & 0x1fffffffu;
	uint64_t m         = (d >> 29) + ((rem > 0x10000000u || (rem == 0x10000000u && ((d >> 29) & 1))) ? 1 : 0);
	int e2             = e + 29 + 23;  // the float's unbiased exponent
	if (m >> 24) {
		m >>= 1;
		e2 += 1;
	}
	if (e2 < -126 || e2 > 127) return false;  // subnormal, zero or infinite result
	*out = __uint_as_float(((uint32_t)(e2 + 127) << 23) | ((uint32_t)m & 0x7fffffu));
	return true;
}

__device__ __forceinline__ float mul_f32_f64_rn(float a, uint64_t packed) {
	uint32_t const ab = __float_as_uint(a);
	if (ab == 0u) return 0.0f;
	float fast;
	if (mul_f32_f64_rn_normal(ab, packed, &fast)) return fast;
	uint64_t const mf = packed & ((1ull << 53) - 1);
	int const ef      = (int)(packed >> 53) - 1100;  // f = mf 2^ef
	uint32_t const fa = ab >> 23;
	uint64_t const ma = fa ? (uint64_t)((ab & 0x7fffffu) | 0x800000u) : (uint64_t)ab;
	int E             = (fa ? (int)fa - 150 : -149) + ef;  // a f = P 2^E, P = ma mf < 2^77
	uint64_t const lo = ma * mf;
	uint64_t const hi = __umul64hi(ma, mf);
	int const L       = hi ? 64 + bitlen64(hi) : bitlen64(lo);
	uint64_t d        = lo;  // the double product's significand: d 2^E
	if (L > 53) {
		int const s         = L - 53;  // 1 .. 24
		uint64_t const keep = (lo >> s) | (hi << (64 - s));
		uint64_t const rem  = lo & ((1ull << s) - 1);
		uint64_t const half = 1ull << (s - 1);
		d = keep + ((rem > half || (rem == half && (keep & 1))) ? 1 : 0);
		E += s;
		if (d == (1ull << 53)) {
			d >>= 1;
			E += 1;
		}
	}
	int const Ld = bitlen64(d);
	if (E + Ld - 1 > 127) return __uint_as_float(0x7f800000u);
	// float rounding: keep 24 bits of a normal result, multiples of 2^-149 of a subnormal one
	int const s2 = (E + Ld - 1 >= -126) ? Ld - 24 : -149 - E;
	uint64_t m   = d;
	if (s2 > 0) {
		if (s2 > 60) return 0.0f;
		uint64_t const rem  = d & ((1ull << s2) - 1);
		uint64_t const half = 1ull << (s2 - 1);
		m = (d >> s2) + ((rem > half || (rem == half && ((d >> s2) & 1))) ? 1 : 0);
		E += s2;
	}
	if (m == 0) return 0.0f;
	int const Lm = bitlen64(m);
	int const e2 = E + Lm - 1;
	if (e2 > 127) return __uint_as_float(0x7f800000u);
	if (e2 >= -126) {
		uint32_t const mant = (uint32_t)(Lm >= 24 ? (m >> (Lm - 24)) : (m << (24 - Lm)));
		return __uint_as_float(((uint32_t)(e2 + 127) << 23) | (mant & 0x7fffffu));
	}
	return __uint_as_float((uint32_t)(m << (E + 149)));
}

}  // namespace spice_gb300
