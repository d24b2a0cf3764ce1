// Exact fixed-point to FP64 conversion in integer arithmetic (host and device).
//
// The tensor-core projection accumulates each element of P exactly as two int64 sums: hi in units
// of 2^-32 and lo in units of 2^-64 of the tile scale, V = hi 2^32 + lo (|V| < 2^82).  This turns
// V 2^(k - 64) into the nearest double (ties to even) with integer operations only: a 128-bit
// two's-complement sum, the leading bit, a 53-bit mantissa with round-to-nearest-even on the 11
// dropped bits plus a sticky bit, and the scale 2^k folded into the exponent field.  GB300 issues
// integer operations at 32 times its FP64 rate, so this costs less than one FP64 operation.
// Results outside the normal range (and V = 0) take a slow path through ldexp.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define NLC_HD __host__ __device__ __forceinline__
#else
#define NLC_HD inline
#endif

namespace nlc {

NLC_HD int clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
	return __clzll((long long) x);
#else
	return __builtin_clzll(x);
#endif
}

NLC_HD double bits_to_double(unsigned long long b) {
#ifdef __CUDA_ARCH__
	return __longlong_as_double((long long) b);
#else
	double d;
	std::memcpy(&d, &b, sizeof d);
	return d;
#endif
}

// (hi 2^32 + lo) 2^(k - 64), rounded to nearest even
NLC_HD double fixed128_to_double(long long hi, long long lo, int k) {
	// V = hi 2^32 + lo as a 128-bit two's-complement number (vh, vl)
	const unsigned long long a_lo = (unsigned long long) hi << 32;
	unsigned long long vl = a_lo + (unsigned long long) lo;
	long long vh = (hi >> 32) + (lo >> 63) + (vl < a_lo ? 1 : 0);
	const bool neg = vh < 0;
	if (neg) {
		vl = ~vl + 1;
		vh = (long long) (~(unsigned long long) vh + (vl == 0 ? 1ull : 0ull));
	}
	const unsigned long long mh = (unsigned long long) vh;
	if (mh == 0 && vl == 0) return 0.;
	// the 64 leading bits m (leading one at bit 63), e = the leading bit's index in V, sticky = any
	// bit of V below m
	unsigned long long m;
	int e;
	bool sticky;
	if (mh) {
		const int lz = clz64(mh);
		m = lz ? (mh << lz) | (vl >> (64 - lz)) : mh;
		sticky = (lz ? vl << lz : vl) != 0;
		e = 127 - lz;
	} else {
		const int lz = clz64(vl);
		m = vl << lz;
		sticky = false;
		e = 63 - lz;
	}
	unsigned long long q = m >> 11;   // 53 bits, leading one at bit 52
	const unsigned long long r = m & 0x7ff;
	if (r > 0x400 || (r == 0x400 && (sticky || (q & 1)))) q++;
	if (q >> 53) q >>= 1, e++;
	// value = q 2^(e - 52) 2^(k - 64): unbiased exponent e + k - 64
	const int biased = e + k - 64 + 1023;
	if (biased >= 1 && biased <= 2046)
		return bits_to_double(((unsigned long long) neg << 63) | ((unsigned long long) biased << 52) |
		                      (q & 0xfffffffffffffull));
	const double v = std::ldexp((double) q, e - 52 + k - 64);
	return neg ? -v : v;
}

NLC_HD unsigned long long umulhi64(unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
	return __umul64hi(a, b);
#else
	return (unsigned long long) (((unsigned __int128) a * b) >> 64);
#endif
}

// ((hi 2^32 + lo) 2^(k - 64))^2 as a double, truncated toward zero to 53 bits (relative error below
// 2^-51): the square the mode energies need, without the sign, the rounding step or an FP64
// multiply.  |V| is normalised to its 64 leading bits m (the bits below are dropped), m^2 is taken
// to its high 64 bits, and those to a 53-bit mantissa.
NLC_HD double fixed128_square_to_double(long long hi, long long lo, int k) {
	const unsigned long long a_lo = (unsigned long long) hi << 32;
	unsigned long long vl = a_lo + (unsigned long long) lo;
	long long vh = (hi >> 32) + (lo >> 63) + (vl < a_lo ? 1 : 0);
	if (vh < 0) {
		vl = ~vl + 1;
		vh = (long long) (~(unsigned long long) vh + (vl == 0 ? 1ull : 0ull));
	}
	const unsigned long long mh = (unsigned long long) vh;
	if (mh == 0 && vl == 0) return 0.;
	unsigned long long m;
	int e;   // index of V's leading bit
	if (mh) {
		const int lz = clz64(mh);
		m = lz ? (mh << lz) | (vl >> (64 - lz)) : mh;
		e = 127 - lz;
	} else {
		const int lz = clz64(vl);
		m = vl << lz;
		e = 63 - lz;
	}
	// |V| ~ m 2^(e - 63); V^2 ~ sq 2^(2e - 62) with sq = (m^2) >> 64 in [2^62, 2^64)
	const unsigned long long sq = umulhi64(m, m);
	const int top = (int) (sq >> 63);
	const unsigned long long mant = sq >> (10 + top);   // leading one at bit 52
	// value = mant 2^(10 + top) 2^(2e - 62) 2^(2k - 128): unbiased exponent 52 + 10 + top + 2e - 190 + 2k
	const int biased = 52 + 10 + top + 2 * e - 190 + 2 * k + 1023;
	if (biased >= 1 && biased <= 2046)
		return bits_to_double(((unsigned long long) biased << 52) | (mant & 0xfffffffffffffull));
	return std::ldexp((double) mant, 10 + top + 2 * e - 190 + 2 * k);
}

}  // namespace nlc
