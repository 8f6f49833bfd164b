// Host check of mul_f32_f64_rn (spice2_gb300/csrc/mulround.h): (float)((double)a * f) computed in
// integer arithmetic must equal the host's IEEE double multiply and float conversion bit for bit.
// Cases: random finite a >= 0 over every exponent (subnormals included) times random f in
// [2^-4, 2^5); the skip() factors (1 - dt/tau)^n of several traces; and constructed products whose
// double rounding lands on, or next to, a float rounding tie.  Prints "cases N mismatches M".
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#define __device__
#define __forceinline__ inline
static inline uint32_t __float_as_uint(float f) {
	uint32_t u;
	memcpy(&u, &f, 4);
	return u;
}
static inline float __uint_as_float(uint32_t u) {
	float f;
	memcpy(&f, &u, 4);
	return f;
}
static inline int __clzll(long long x) { return x ? __builtin_clzll((unsigned long long)x) : 64; }
static inline uint64_t __umul64hi(uint64_t a, uint64_t b) { return (uint64_t)(((unsigned __int128)a * b) >> 64); }
#include "mulround.h"

using namespace spice_gb300;

static long long cases = 0, bad = 0;

static void check(float a, double f) {
	volatile double p = (double)a * f;
	float const want  = (float)p;
	float const got   = mul_f32_f64_rn(a, pack_f64(f));
	cases++;
	if (__float_as_uint(want) != __float_as_uint(got)) {
		if (bad < 5) printf("mismatch a=%a f=%a want=%a got=%a\n", a, f, want, got);
		bad++;
	}
}

int main(int argc, char** argv) {
	long long const n = argc > 1 ? atoll(argv[1]) : 4000000;
	std::mt19937_64 g(12345);
	for (long long i = 0; i < n; i++) {  // random pairs
		uint64_t x  = g();
		uint32_t ab = (uint32_t)x & 0x7fffffffu;
		if ((ab >> 23) == 0xffu) ab &= 0x7f7fffffu;
		if ((i & 7) == 0) ab &= 0x007fffffu;
		double const f = ldexp(1.0 + (double)(g() >> 12) * 0x1p-52, (int)(g() % 9) - 4);
		check(__uint_as_float(ab), f);
	}
	double const taus[] = {0.02, 0.01, 0.005, 0.0137};
	for (double tau : taus) {  // the skip() factors of traces over every float a
		float const cdt = 1e-4f * (1.0f / (float)tau);
		for (int k = -64; k <= 64; k++) {
			double const f = pow((double)(1.0f - cdt), (double)k);
			for (long long i = 0; i < n / 200; i++) {
				uint32_t ab = (uint32_t)g() & 0x7fffffffu;
				if ((ab >> 23) == 0xffu) ab &= 0x7f7fffffu;
				check(__uint_as_float(ab), f);
			}
		}
	}
	for (long long i = 0; i < n; i++) {  // near float ties after the double rounding
		uint32_t const ma = 0x800000u | ((uint32_t)g() & 0x7fffffu);
		// a 53-bit double significand whose low 29 bits sit at (or next to) the float midpoint
		uint64_t d = (1ull << 52) | (g() & ((1ull << 52) - 1));
		d          = (d & ~0x1fffffffull) | 0x10000000ull;
		d += (int64_t)(g() % 5) - 2;
		// mf ~ d 2^24 / ma (53 bits), then small offsets around it
		unsigned __int128 num = (unsigned __int128)d << 24;
		uint64_t mf           = (uint64_t)(num / ma);
		mf += (int64_t)(g() % 7) - 3;
		if (mf >> 53) mf >>= 1;
		if (!(mf >> 52)) mf |= 1ull << 52;
		double const f = ldexp((double)mf, -52 + (int)(g() % 5) - 2);
		int const ea   = 1 + (int)(g() % 200);
		float const a  = __uint_as_float(((uint32_t)ea << 23) | (ma & 0x7fffffu));
		check(a, f);
	}
	printf("cases %lld mismatches %lld\n", cases, bad);
	return bad != 0;
}
