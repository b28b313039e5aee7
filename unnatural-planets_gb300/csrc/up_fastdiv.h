// Division of 32-bit unsigned integers by a divisor fixed ahead of time
// (a grid dimension): the round-up multiply-shift of Granlund and Montgomery,
// "Division by invariant integers using multiplication" (PLDI 1994), exact
// for every 32-bit dividend. Shared by the device kernels and the host tests.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define UP_FD_HD __host__ __device__ __forceinline__
#else
#define UP_FD_HD inline
#endif

namespace up {

struct FastDiv {
	uint32_t d, m, s;
	static FastDiv of(uint32_t d) {
		FastDiv f{d, 0, 0};
		uint32_t l = 0;
		while (l < 32 && (1ull << l) < d) l++; // ceil(log2 d)
		f.m = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
		f.s = l > 0 ? l - 1 : 0;
		return f;
	}
	UP_FD_HD uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
		const uint32_t t = __umulhi(m, n);
#else
		const uint32_t t = (uint32_t)(((uint64_t)m * n) >> 32);
#endif
		return d == 1 ? n : (t + ((n - t) >> 1)) >> s;
	}
};

} // namespace up
