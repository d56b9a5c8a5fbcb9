// PCG32 (M. E. O'Neill, "PCG: A Family of Simple Fast Space-Efficient Statistically Good
// Algorithms for Random Number Generation", 2014): 64-bit LCG state, XSH-RR 32-bit output.
// The same generator runs on the device (device/pcg.cuh), so sampled rays are identical on the
// host and the GPU. It replaces the reference's curand XORWOW states (InitCurandKernel.cu:24-33).
#pragma once

#include <cstdint>

namespace phe_gb300 {

struct Pcg32 {
	uint64_t state = 0, inc = 1;
	Pcg32() = default;
	Pcg32(uint64_t initstate, uint64_t initseq) { seed(initstate, initseq); }
	void seed(uint64_t initstate, uint64_t initseq)
	{
		state = 0u;
		inc = (initseq << 1u) | 1u;
		next();
		state += initstate;
		next();
	}
	uint32_t next()
	{
		uint64_t old = state;
		state = old * 6364136223846793005ull + inc;
		uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
		uint32_t rot = (uint32_t)(old >> 59u);
		return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
	}
	// [0, 1) with 24 random bits.
	float uniform() { return (float)(next() >> 8) * 0x1.0p-24f; }
	// [0, 1) with 53 random bits.
	double uniform_d()
	{
		uint64_t hi = next() >> 5, lo = next() >> 6;
		return (double)((hi << 26) | lo) * 0x1.0p-53;
	}
};

} // namespace phe_gb300
