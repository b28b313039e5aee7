// Device math for the planet SDF path: vectors, the integer lattice hash and
// the noise family (value, cubic, Perlin, simplex, simplex-reduced,
// cellular), each in a value-only and a fused value+gradient form.
//
// Definitions (shared with the CPU oracle, implemented independently):
//   mix32         "lowbias32" 32-bit finaliser (C. Wellons, hash-prospector)
//   lattice hash  mix32(x*73856093 ^ y*19349663 ^ z*83492791 ^ key), primes of
//                 Teschner et al. 2003 spatial hashing; key = mix32(seed + 0x9E3779B9)
//   value         hash -> [-1,1) lattice values, quintic-faded trilinear blend
//   cubic         tricubic Catmull-Rom of lattice values x 0.75
//   Perlin        K. Perlin, "Improving noise" (2002): 12 edge gradients from 4 bits
//   simplex       S. Gustavson, "Simplex noise demystified" (2005), kernel
//                 (0.5 - r^2)^4 x 76; simplex-reduced uses (0.5 - r^2)^3 x 31
//   cellular      Worley (1996), one jittered point per cell, 3x3x3 search
// Analytic derivatives of the lattice noises follow I. Quilez's closed forms
// for gradient/value noise derivatives (iquilezles.org, "gradient noise
// derivatives"); the simplex derivative differentiates each radial kernel.
//
// The header compiles for the device (nvcc) and, for CPU-side unit checks of
// the arithmetic only, as plain C++.
#pragma once
#include <stdint.h>
#include <math.h>
#include <string.h>

#ifdef __CUDACC__
#define UP_HD __host__ __device__ __forceinline__
#define UP_HD_OUTLINE static __host__ __device__ __noinline__
#else
#define UP_HD inline
#define UP_HD_OUTLINE static inline
#endif

namespace up {

// float <-> bits
UP_HD uint32_t f_bits(float x) {
#ifdef __CUDA_ARCH__
	return __float_as_uint(x);
#else
	uint32_t u;
	memcpy(&u, &x, 4);
	return u;
#endif
}
UP_HD float bits_f(uint32_t u) {
#ifdef __CUDA_ARCH__
	return __uint_as_float(u);
#else
	float x;
	memcpy(&x, &u, 4);
	return x;
#endif
}

// square root: the hardware approximation on the device (sqrt.approx, a
// few ulp; inputs below 2^-126 flush to 0), correctly rounded on the host
UP_HD float sqrt_hd(float x) {
#ifdef __CUDA_ARCH__
	float y;
	asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
#else
	return sqrtf(x);
#endif
}
// reciprocal square root: the hardware approximation on the device
// (rsqrt.approx, a few ulp; inputs below 2^-126 flush to 0 and give +inf, so
// callers guard their argument with a floor far above that), correctly rounded
// 1 / sqrt on the host; used for unit vectors only
UP_HD float rsqrt_hd(float x) {
#ifdef __CUDA_ARCH__
	float y;
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
#else
	return 1.f / sqrtf(x);
#endif
}

struct V3f { float x, y, z; };
UP_HD V3f v3(float x, float y, float z) { V3f r; r.x = x; r.y = y; r.z = z; return r; }
UP_HD V3f operator+(V3f a, V3f b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
UP_HD V3f operator-(V3f a, V3f b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
UP_HD V3f operator-(V3f a) { return v3(-a.x, -a.y, -a.z); }
UP_HD V3f operator*(V3f a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
UP_HD V3f operator*(float s, V3f a) { return v3(a.x * s, a.y * s, a.z * s); }
UP_HD V3f operator*(V3f a, V3f b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
UP_HD V3f &operator+=(V3f &a, V3f b) { a = a + b; return a; }
UP_HD V3f &operator-=(V3f &a, V3f b) { a = a - b; return a; }
UP_HD V3f &operator*=(V3f &a, float s) { a = a * s; return a; }
UP_HD float dot(V3f a, V3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
UP_HD float length(V3f a) { return sqrtf(dot(a, a)); }
UP_HD V3f cross(V3f a, V3f b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
UP_HD V3f zero3() { return v3(0.f, 0.f, 0.f); }

// value with gradient
struct NG { float v; V3f g; };
UP_HD NG ng(float v, V3f g) { NG r; r.v = v; r.g = g; return r; }
UP_HD NG ngc(float v) { return ng(v, zero3()); }

// Pairs of FP32 values for the packed FP32x2 instructions of sm_100+ (one
// issue slot for two independent FP32 operations, each rounded as its scalar
// form): fma2(a, b, c) = (fma(a.x, b.x, c.x), fma(a.y, b.y, c.y)), add2 and
// mul2 likewise. Host builds compute the same correctly rounded results one
// element at a time.
struct P2 { float x, y; };
UP_HD P2 p2(float x, float y) { P2 r; r.x = x; r.y = y; return r; }
UP_HD P2 p2s(float s) { return p2(s, s); }
UP_HD P2 fma2(P2 a, P2 b, P2 c) {
#ifdef __CUDA_ARCH__
	const float2 r = __ffma2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y), make_float2(c.x, c.y));
	return p2(r.x, r.y);
#else
	return p2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
#endif
}
UP_HD P2 add2(P2 a, P2 b) {
#ifdef __CUDA_ARCH__
	const float2 r = __fadd2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y));
	return p2(r.x, r.y);
#else
	volatile float x = a.x + b.x, y = a.y + b.y;
	return p2(x, y);
#endif
}
UP_HD P2 mul2(P2 a, P2 b) {
#ifdef __CUDA_ARCH__
	const float2 r = __fmul2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y));
	return p2(r.x, r.y);
#else
	volatile float x = a.x * b.x, y = a.y * b.y;
	return p2(x, y);
#endif
}

UP_HD float saturatef(float x) { return fminf(fmaxf(x, 0.f), 1.f); }
UP_HD float lerpf(float a, float b, float t) { return a + (b - a) * t; }

// ---------------------------------------------------------------- hash
UP_HD uint32_t mix32(uint32_t x) {
	x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
	return x;
}
// mix32 in two parts: its first step distributes over xor (a logical shift
// does), so mix32(a ^ b) == mix32_tail(mix32_head(a) ^ mix32_head(b)), and a
// caller that hashes many a ^ b with a shared b forms mix32_head(b) once
UP_HD uint32_t mix32_head(uint32_t x) { return x ^ (x >> 16); }
UP_HD uint32_t mix32_tail(uint32_t x) {
	x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
	return x;
}
UP_HD uint32_t seed_key(uint32_t seed) { return mix32(seed + 0x9E3779B9U); }
constexpr uint32_t HX = 73856093U, HY = 19349663U, HZ = 83492791U;
UP_HD uint32_t lattice_hash(int ix, int iy, int iz, uint32_t key) {
	return mix32(((uint32_t)ix * HX) ^ ((uint32_t)iy * HY) ^ ((uint32_t)iz * HZ) ^ key);
}
// top 24 bits -> [-1, 1) exactly
UP_HD float hash_signed(uint32_t h) { return (float)(h >> 8) * (1.0f / 8388608.0f) - 1.0f; }

// ---------------------------------------------------------------- lattice cell
struct Cell { int ix, iy, iz; float fx, fy, fz; };
UP_HD Cell cell_of(V3f p) {
	Cell c;
	const float x0 = floorf(p.x), y0 = floorf(p.y), z0 = floorf(p.z);
	c.ix = (int)x0; c.iy = (int)y0; c.iz = (int)z0;
	c.fx = p.x - x0; c.fy = p.y - y0; c.fz = p.z - z0;
	return c;
}
UP_HD float fade(float t) { return t * t * t * (t * (t * 6.f - 15.f) + 10.f); }
UP_HD float dfade(float t) { return 30.f * t * t * (t * (t - 2.f) + 1.f); }

// Perlin gradient index -> dot product and vector
UP_HD float grad_dot(uint32_t h, float x, float y, float z) {
	const uint32_t g = h & 15U;
	const float u = g < 8U ? x : y;
	const float v = g < 4U ? y : ((g == 12U || g == 14U) ? x : z);
	return ((g & 1U) ? -u : u) + ((g & 2U) ? -v : v);
}
UP_HD V3f grad_vec(uint32_t h) {
	const uint32_t g = h & 15U;
	const float su = (g & 1U) ? -1.f : 1.f, sv = (g & 2U) ? -1.f : 1.f;
	const int ua = g < 8U ? 0 : 1;
	const int va = g < 4U ? 1 : ((g == 12U || g == 14U) ? 0 : 2);
	return v3((ua == 0 ? su : 0.f) + (va == 0 ? sv : 0.f), (ua == 1 ? su : 0.f) + (va == 1 ? sv : 0.f), va == 2 ? sv : 0.f);
}

// Eight corner hashes of a lattice cell: the per-axis products are shared.
struct Corners { uint32_t h[8]; };
UP_HD Corners corner_hashes(const Cell &c, uint32_t key) {
	const uint32_t x0 = (uint32_t)c.ix * HX, x1 = x0 + HX;
	const uint32_t y0 = (uint32_t)c.iy * HY, y1 = y0 + HY;
	const uint32_t z0 = ((uint32_t)c.iz * HZ) ^ key, z1 = ((uint32_t)c.iz * HZ + HZ) ^ key;
	Corners r;
	r.h[0] = mix32(x0 ^ y0 ^ z0); r.h[1] = mix32(x1 ^ y0 ^ z0);
	r.h[2] = mix32(x0 ^ y1 ^ z0); r.h[3] = mix32(x1 ^ y1 ^ z0);
	r.h[4] = mix32(x0 ^ y0 ^ z1); r.h[5] = mix32(x1 ^ y0 ^ z1);
	r.h[6] = mix32(x0 ^ y1 ^ z1); r.h[7] = mix32(x1 ^ y1 ^ z1);
	return r;
}

// trilinear blend of 8 corner scalars with fades u,v,w; optional derivative of
// the blend with respect to the fades (the k-coefficient form)
UP_HD float tri(const float c[8], float u, float v, float w) {
	const float x00 = lerpf(c[0], c[1], u), x10 = lerpf(c[2], c[3], u);
	const float x01 = lerpf(c[4], c[5], u), x11 = lerpf(c[6], c[7], u);
	return lerpf(lerpf(x00, x10, v), lerpf(x01, x11, v), w);
}
UP_HD V3f tri_dfade(const float c[8], float u, float v, float w) {
	const float k1 = c[1] - c[0], k2 = c[2] - c[0], k3 = c[4] - c[0];
	const float k4 = c[0] - c[1] - c[2] + c[3];
	const float k5 = c[0] - c[2] - c[4] + c[6];
	const float k6 = c[0] - c[1] - c[4] + c[5];
	const float k7 = -c[0] + c[1] + c[2] - c[3] + c[4] - c[5] - c[6] + c[7];
	return v3(k1 + k4 * v + k6 * w + k7 * v * w, k2 + k5 * w + k4 * u + k7 * w * u, k3 + k6 * u + k5 * v + k7 * u * v);
}

// ---------------------------------------------------------------- value noise
UP_HD float value_v(V3f p, uint32_t key) {
	const Cell c = cell_of(p);
	const Corners h = corner_hashes(c, key);
	float cv[8];
	#pragma unroll
	for (int b = 0; b < 8; b++) cv[b] = hash_signed(h.h[b]);
	return tri(cv, fade(c.fx), fade(c.fy), fade(c.fz));
}
UP_HD NG value_g(V3f p, uint32_t key) {
	const Cell c = cell_of(p);
	const Corners h = corner_hashes(c, key);
	float cv[8];
	#pragma unroll
	for (int b = 0; b < 8; b++) cv[b] = hash_signed(h.h[b]);
	const float u = fade(c.fx), v = fade(c.fy), w = fade(c.fz);
	const V3f k = tri_dfade(cv, u, v, w);
	return ng(tri(cv, u, v, w), v3(k.x * dfade(c.fx), k.y * dfade(c.fy), k.z * dfade(c.fz)));
}

// ---------------------------------------------------------------- cubic value noise
UP_HD float catmull(float p0, float p1, float p2, float p3, float t) {
	return p1 + 0.5f * t * (p2 - p0 + t * (2.f * p0 - 5.f * p1 + 4.f * p2 - p3 + t * (3.f * (p1 - p2) + p3 - p0)));
}
UP_HD float dcatmull(float p0, float p1, float p2, float p3, float t) {
	return 0.5f * (p2 - p0 + t * (2.f * (2.f * p0 - 5.f * p1 + 4.f * p2 - p3) + t * 3.f * (3.f * (p1 - p2) + p3 - p0)));
}
template<bool GRAD>
UP_HD NG cubic_n(V3f p, uint32_t key) {
	const Cell c = cell_of(p);
	float Y[4], DYX[4], DY[4];
	#pragma unroll
	for (int k = 0; k < 4; k++) {
		float X[4], DX[4];
		const uint32_t zk = ((uint32_t)(c.iz + k - 1) * HZ) ^ key;
		#pragma unroll
		for (int j = 0; j < 4; j++) {
			const uint32_t yj = (uint32_t)(c.iy + j - 1) * HY;
			float v[4];
			#pragma unroll
			for (int i = 0; i < 4; i++) v[i] = hash_signed(mix32(((uint32_t)(c.ix + i - 1) * HX) ^ yj ^ zk));
			X[j] = catmull(v[0], v[1], v[2], v[3], c.fx);
			if (GRAD) DX[j] = dcatmull(v[0], v[1], v[2], v[3], c.fx);
		}
		Y[k] = catmull(X[0], X[1], X[2], X[3], c.fy);
		if (GRAD) {
			DYX[k] = catmull(DX[0], DX[1], DX[2], DX[3], c.fy);
			DY[k] = dcatmull(X[0], X[1], X[2], X[3], c.fy);
		}
	}
	const float s = 0.75f;
	if (!GRAD) return ngc(catmull(Y[0], Y[1], Y[2], Y[3], c.fz) * s);
	return ng(catmull(Y[0], Y[1], Y[2], Y[3], c.fz) * s,
		v3(catmull(DYX[0], DYX[1], DYX[2], DYX[3], c.fz) * s, catmull(DY[0], DY[1], DY[2], DY[3], c.fz) * s,
			dcatmull(Y[0], Y[1], Y[2], Y[3], c.fz) * s));
}

// ---------------------------------------------------------------- Perlin
UP_HD float perlin_v(V3f p, uint32_t key) {
	const Cell c = cell_of(p);
	const Corners h = corner_hashes(c, key);
	const float x1 = c.fx - 1.f, y1 = c.fy - 1.f, z1 = c.fz - 1.f;
	float cv[8];
	cv[0] = grad_dot(h.h[0], c.fx, c.fy, c.fz); cv[1] = grad_dot(h.h[1], x1, c.fy, c.fz);
	cv[2] = grad_dot(h.h[2], c.fx, y1, c.fz); cv[3] = grad_dot(h.h[3], x1, y1, c.fz);
	cv[4] = grad_dot(h.h[4], c.fx, c.fy, z1); cv[5] = grad_dot(h.h[5], x1, c.fy, z1);
	cv[6] = grad_dot(h.h[6], c.fx, y1, z1); cv[7] = grad_dot(h.h[7], x1, y1, z1);
	return tri(cv, fade(c.fx), fade(c.fy), fade(c.fz));
}
UP_HD NG perlin_g(V3f p, uint32_t key) {
	const Cell c = cell_of(p);
	const Corners h = corner_hashes(c, key);
	const float xs[2] = {c.fx, c.fx - 1.f}, ys[2] = {c.fy, c.fy - 1.f}, zs[2] = {c.fz, c.fz - 1.f};
	float cv[8];
	V3f gv[8];
	#pragma unroll
	for (int b = 0; b < 8; b++) {
		gv[b] = grad_vec(h.h[b]);
		cv[b] = gv[b].x * xs[b & 1] + gv[b].y * ys[(b >> 1) & 1] + gv[b].z * zs[b >> 2];
	}
	const float u = fade(c.fx), v = fade(c.fy), w = fade(c.fz);
	const V3f k = tri_dfade(cv, u, v, w);
	// gradient vectors blended with the same weights, plus the fade terms
	float gx[8], gy[8], gz[8];
	#pragma unroll
	for (int b = 0; b < 8; b++) { gx[b] = gv[b].x; gy[b] = gv[b].y; gz[b] = gv[b].z; }
	return ng(tri(cv, u, v, w),
		v3(tri(gx, u, v, w) + k.x * dfade(c.fx), tri(gy, u, v, w) + k.y * dfade(c.fy), tri(gz, u, v, w) + k.z * dfade(c.fz)));
}

// ---------------------------------------------------------------- simplex
template<bool GRAD, bool REDUCED>
UP_HD NG simplex_n(V3f p, uint32_t key) {
	const float F3 = 1.0f / 3.0f, G3 = 1.0f / 6.0f;
	const float s = (p.x + p.y + p.z) * F3;
	const float fi = floorf(p.x + s), fj = floorf(p.y + s), fk = floorf(p.z + s);
	const int i = (int)fi, j = (int)fj, k = (int)fk;
	const float t = (fi + fj + fk) * G3;
	const float x0 = p.x - (fi - t), y0 = p.y - (fj - t), z0 = p.z - (fk - t);
	int i1, j1, k1, i2, j2, k2;
	if (x0 >= y0) {
		if (y0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
		else if (x0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 0; k2 = 1; }
		else { i1 = 0; j1 = 0; k1 = 1; i2 = 1; j2 = 0; k2 = 1; }
	} else {
		if (y0 < z0) { i1 = 0; j1 = 0; k1 = 1; i2 = 0; j2 = 1; k2 = 1; }
		else if (x0 < z0) { i1 = 0; j1 = 1; k1 = 0; i2 = 0; j2 = 1; k2 = 1; }
		else { i1 = 0; j1 = 1; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
	}
	const int ci[4] = {0, i1, i2, 1}, cj[4] = {0, j1, j2, 1}, ck[4] = {0, k1, k2, 1};
	float n = 0.f;
	V3f g = zero3();
	#pragma unroll
	for (int c = 0; c < 4; c++) {
		const float off = G3 * (float)c;
		const float xc = x0 - (float)ci[c] + off, yc = y0 - (float)cj[c] + off, zc = z0 - (float)ck[c] + off;
		const float tt = 0.5f - xc * xc - yc * yc - zc * zc;
		if (tt > 0.f) {
			const uint32_t h = lattice_hash(i + ci[c], j + cj[c], k + ck[c], key);
			const float t2 = tt * tt;
			if (!GRAD) {
				n += (REDUCED ? t2 * tt : t2 * t2) * grad_dot(h, xc, yc, zc);
			} else {
				const V3f gv = grad_vec(h);
				const float gd = gv.x * xc + gv.y * yc + gv.z * zc;
				const float kern = REDUCED ? t2 * tt : t2 * t2;
				const float dk = REDUCED ? -6.f * t2 : -8.f * t2 * tt; // d kern / d x = dk * x
				n += kern * gd;
				g += gv * kern + v3(xc, yc, zc) * (dk * gd);
			}
		}
	}
	const float sc = REDUCED ? 31.0f : 76.0f;
	return ng(n * sc, g * sc);
}

// ---------------------------------------------------------------- cellular
// (m + 1/2) / 1024 for the 10-bit field m = (h >> s) & 1023: the float
// 1 + m / 1024 is assembled in the mantissa and 1 - 1/2048 subtracted, which
// is exact (both in [1, 2)), so this equals m * (1/1024) + 1/2048 without an
// integer-to-float conversion
UP_HD float jitter(uint32_t h, int s) { return bits_f(0x3F800000u | (((h >> s) & 1023U) << 13)) - 0.99951171875f; }

UP_HD float signf(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
// x with its sign flipped when s is negative: x sign(s) for s != 0, +-x for s = +-0
UP_HD float mul_sign(float x, float s) { return bits_f(f_bits(x) ^ (f_bits(s) & 0x80000000u)); }
// gradient with respect to p of the distance metric of v = q - p
// (Euclidean: F is the squared distance here; -v / |v| with the reciprocal
// square root of rsqrt_hd, 1 / sqrtf on the host)
UP_HD V3f cell_dist_grad(V3f v, float F, int dist) {
	if (dist == 0) return v * -(F > 1e-36f ? rsqrt_hd(F) : 0.f); // |v| <= 1e-18: no direction
	const V3f sg = v3(signf(v.x), signf(v.y), signf(v.z));
	if (dist == 1) return -sg;
	return -(v * 2.f + sg);
}

// DIST/OP >= 0 fix the metric/output at compile time; -1 reads them at run time.
// Candidates are ranked by an integer key: the distance (squared length for
// Euclidean; every metric is >= 0, so float bits order like values) with its
// low 6 mantissa bits replaced by the candidate id (dz, dy, dx order, the
// search order). The two smallest keys take three integer min/max per
// candidate; the winners' exact distances and difference vectors are then
// rebuilt from their ids. Exact ties keep the first candidate in search
// order; distances within 2^-17 relative of each other may be ranked by id.
template<int DIST>
UP_HD float cell_dist(float vx, float vy, float vz, int dist) {
	const int m = DIST >= 0 ? DIST : dist;
	const float e2 = vx * vx + vy * vy + vz * vz;
	if (m == 0) return e2;
	const float m1 = fabsf(vx) + fabsf(vy) + fabsf(vz);
	if (m == 1) return m1;
	return e2 + m1;
}
template<bool GRAD, int DIST = -1, int OP = -1>
UP_HD NG cellular_n(V3f p, uint32_t key, int dist_rt, int op_rt) {
	const int dist = DIST >= 0 ? DIST : dist_rt;
	const int op = OP >= 0 ? OP : op_rt;
	const Cell c = cell_of(p);
	uint32_t K1 = 0xFFFFFFFFu, K2 = 0xFFFFFFFFu;
	#pragma unroll 1
	for (int dz = -1; dz <= 1; dz++) {
		const uint32_t zh = ((uint32_t)(c.iz + dz) * HZ) ^ key;
		#pragma unroll 1
		for (int dy = -1; dy <= 1; dy++) {
			const uint32_t yzh = ((uint32_t)(c.iy + dy) * HY) ^ zh;
			const uint32_t id0 = (uint32_t)((dz + 1) * 9 + (dy + 1) * 3);
			#pragma unroll
			for (int dx = -1; dx <= 1; dx++) {
				const uint32_t h = mix32(((uint32_t)(c.ix + dx) * HX) ^ yzh);
				const float vx = ((float)dx + jitter(h, 0)) - c.fx;
				const float vy = ((float)dy + jitter(h, 10)) - c.fy;
				const float vz = ((float)dz + jitter(h, 20)) - c.fz;
				const uint32_t k = (f_bits(cell_dist<DIST>(vx, vy, vz, dist)) & ~63u) | (id0 + (uint32_t)(dx + 1));
				K2 = K2 < (K1 > k ? K1 : k) ? K2 : (K1 > k ? K1 : k);
				K1 = K1 < k ? K1 : k;
			}
		}
	}
	float F[2];
	V3f g[2];
	uint32_t cellh = 0;
	#pragma unroll
	for (int w = 0; w < 2; w++) {
		const uint32_t id = (w ? K2 : K1) & 63u;
		const int dz = (int)(id / 9u) - 1, dy = (int)((id / 3u) % 3u) - 1, dx = (int)(id % 3u) - 1;
		const uint32_t h = mix32(((uint32_t)(c.ix + dx) * HX) ^ ((uint32_t)(c.iy + dy) * HY) ^ (((uint32_t)(c.iz + dz) * HZ) ^ key));
		const float vx = ((float)dx + jitter(h, 0)) - c.fx;
		const float vy = ((float)dy + jitter(h, 10)) - c.fy;
		const float vz = ((float)dz + jitter(h, 20)) - c.fz;
		F[w] = cell_dist<DIST>(vx, vy, vz, dist);
		g[w] = v3(vx, vy, vz);
		if (w == 0) cellh = h;
	}
	// d F / d p for the stored difference vectors v = q - p (dv/dp = -I)
	V3f dF1 = zero3(), dF2 = zero3();
	if (GRAD) {
		dF1 = cell_dist_grad(g[0], F[0], dist);
		dF2 = cell_dist_grad(g[1], F[1], dist);
	}
	float F1 = F[0], F2 = F[1];
	if (dist == 0) { F1 = sqrt_hd(F1); F2 = sqrt_hd(F2); }
	switch (op) {
		case 0: return ngc(hash_signed(mix32(cellh)));
		case 1: return ng(F1 - 1.f, dF1);
		case 2: return ng(F2 - 1.f, dF2);
		case 3: return ng((F1 + F2) * 0.5f - 1.f, (dF1 + dF2) * 0.5f);
		case 4: return ng(F2 - F1 - 1.f, dF2 - dF1);
		case 5: return ng(F1 * F2 * 0.5f - 1.f, (dF1 * F2 + dF2 * F1) * 0.5f);
		default: return ng(F1 / F2 - 1.f, (dF1 * F2 - dF2 * F1) * (1.f / (F2 * F2)));
	}
}

// Warp-cooperative cellular_n for per-point kernels whose 32 lanes all call
// it together (device only). When the lanes' cells span at most two values
// per axis, the union of their 3x3x3 neighbourhoods fits a 4 x 4 x 4 block:
// the lanes hash it together (two cells each) into a per-warp shared table of
// jitters, and each lane reads its 27 candidates from it; otherwise every lane
// hashes its own, as cellular_n. The candidates, their ids and every
// arithmetic step are those of cellular_n, so the result is the same bit for
// bit. Spatially sorted points (neighbours in neighbouring lanes) take the
// table.
#ifdef __CUDACC__
constexpr int PT_WARPS = 8; // warps per block of the kernels that call it
__shared__ float4 g_pt_cells[PT_WARPS * 64];
template<bool GRAD, int DIST = -1, int OP = -1>
__device__ NG cellular_warp(V3f p, uint32_t key, int dist_rt, int op_rt) {
#ifdef __CUDA_ARCH__
	const Cell c = cell_of(p);
	const int x0 = __reduce_min_sync(0xFFFFFFFFu, c.ix), x1 = __reduce_max_sync(0xFFFFFFFFu, c.ix);
	const int y0 = __reduce_min_sync(0xFFFFFFFFu, c.iy), y1 = __reduce_max_sync(0xFFFFFFFFu, c.iy);
	const int z0 = __reduce_min_sync(0xFFFFFFFFu, c.iz), z1 = __reduce_max_sync(0xFFFFFFFFu, c.iz);
	if (x1 - x0 > 1 || y1 - y0 > 1 || z1 - z0 > 1) return cellular_n<GRAD, DIST, OP>(p, key, dist_rt, op_rt); // the same for every lane
	const int dist = DIST >= 0 ? DIST : dist_rt;
	const int op = OP >= 0 ? OP : op_rt;
	float4 *tab = g_pt_cells + (threadIdx.x >> 5) * 64;
	__syncwarp(); // the previous call's readers are done
	for (int e = (int)(threadIdx.x & 31); e < 64; e += 32) {
		const uint32_t h = mix32(((uint32_t)(x0 - 1 + (e >> 4)) * HX) ^ ((uint32_t)(y0 - 1 + ((e >> 2) & 3)) * HY) ^
			(((uint32_t)(z0 - 1 + (e & 3)) * HZ) ^ key));
		tab[e] = make_float4(jitter(h, 0), jitter(h, 10), jitter(h, 20), __uint_as_float(h));
	}
	__syncwarp();
	// entry of candidate (dx, dy, dz): ((ix + dx) - x0 + 1) * 16 + ((iy + dy) - y0 + 1) * 4 + (iz + dz) - z0 + 1
	const int o = (c.ix - x0) * 16 + (c.iy - y0) * 4 + (c.iz - z0);
	uint32_t K1 = 0xFFFFFFFFu, K2 = 0xFFFFFFFFu;
	#pragma unroll 1
	for (int dz = -1; dz <= 1; dz++) {
		#pragma unroll 1
		for (int dy = -1; dy <= 1; dy++) {
			const uint32_t id0 = (uint32_t)((dz + 1) * 9 + (dy + 1) * 3);
			const int row = o + (dy + 1) * 4 + (dz + 1);
			#pragma unroll
			for (int dx = -1; dx <= 1; dx++) {
				const float4 t = tab[row + (dx + 1) * 16];
				const float vx = ((float)dx + t.x) - c.fx;
				const float vy = ((float)dy + t.y) - c.fy;
				const float vz = ((float)dz + t.z) - c.fz;
				const uint32_t k = (f_bits(cell_dist<DIST>(vx, vy, vz, dist)) & ~63u) | (id0 + (uint32_t)(dx + 1));
				K2 = K2 < (K1 > k ? K1 : k) ? K2 : (K1 > k ? K1 : k);
				K1 = K1 < k ? K1 : k;
			}
		}
	}
	float F[2];
	V3f g[2];
	uint32_t cellh = 0;
	#pragma unroll
	for (int w = 0; w < 2; w++) {
		const uint32_t id = (w ? K2 : K1) & 63u;
		const int dz = (int)(id / 9u) - 1, dy = (int)((id / 3u) % 3u) - 1, dx = (int)(id % 3u) - 1;
		const float4 t = tab[o + (dx + 1) * 16 + (dy + 1) * 4 + (dz + 1)];
		const float vx = ((float)dx + t.x) - c.fx;
		const float vy = ((float)dy + t.y) - c.fy;
		const float vz = ((float)dz + t.z) - c.fz;
		F[w] = cell_dist<DIST>(vx, vy, vz, dist);
		g[w] = v3(vx, vy, vz);
		if (w == 0) cellh = __float_as_uint(t.w);
	}
	V3f dF1 = zero3(), dF2 = zero3();
	if (GRAD) {
		dF1 = cell_dist_grad(g[0], F[0], dist);
		dF2 = cell_dist_grad(g[1], F[1], dist);
	}
	float F1 = F[0], F2 = F[1];
	if (dist == 0) { F1 = sqrt_hd(F1); F2 = sqrt_hd(F2); }
	switch (op) {
		case 0: return ngc(hash_signed(mix32(cellh)));
		case 1: return ng(F1 - 1.f, dF1);
		case 2: return ng(F2 - 1.f, dF2);
		case 3: return ng((F1 + F2) * 0.5f - 1.f, (dF1 + dF2) * 0.5f);
		case 4: return ng(F2 - F1 - 1.f, dF2 - dF1);
		case 5: return ng(F1 * F2 * 0.5f - 1.f, (dF1 * F2 + dF2 * F1) * 0.5f);
		default: return ng(F1 / F2 - 1.f, (dF1 * F2 - dF2 * F1) * (1.f / (F2 * F2)));
	}
#else
	return cellular_n<GRAD, DIST, OP>(p, key, dist_rt, op_rt);
#endif
}
#endif

// ---------------------------------------------------------------- dispatch
// noise type codes follow up_noise_type in include/up_abi.h; the run-time
// dispatch is out of line (one copy per translation unit and GRAD)
template<bool GRAD>
UP_HD_OUTLINE NG noise_single(int type, V3f p, uint32_t key, int dist, int op) {
	switch (type) {
		case 0: if (GRAD) return value_g(p, key); return ngc(value_v(p, key));
		case 1: return cubic_n<GRAD>(p, key);
		case 2: if (GRAD) return perlin_g(p, key); return ngc(perlin_v(p, key));
		case 3: return simplex_n<GRAD, false>(p, key);
		case 4: return simplex_n<GRAD, true>(p, key);
		default: return cellular_n<GRAD>(p, key, dist, op);
	}
}

} // namespace up
