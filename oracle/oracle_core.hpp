// Oracle core: scalar types, the reference's math helpers, the integer hash
// and the noise family, restated on the CPU.
//
// THIS IS TEST INFRASTRUCTURE. Only tests/, the smoke check and the CPU
// baseline leg of the benchmark load it. The product (the CUDA library) never
// links, loads or calls it.
//
// PARITY UNPINNED. The reference evaluates its noise, SDF primitives and
// contouring inside the cage library (externals/cage), which is an empty git
// submodule with no recorded commit, so no reference-produced value exists to
// pin against. Where the reference's own sources define the arithmetic
// (sources/math.cpp, sources/sdf.cpp, sources/elevationModes.cpp,
// sources/coloringModes.cpp, sources/voronoi.cpp,
// sources/modesConfiguration.cpp) this file follows them line by line; the
// cage-side arithmetic (noise, hash, primitives, contouring) is the project's
// own definition built from the published methods named at each function.
//
// Every function is templated on the scalar T so one source serves:
//   double          FP64 oracle values
//   F32             FP32 restatement (the reference's precision)
//   Dual<N>         forward-mode derivatives (exact gradients, FP64)
//   Counted         FP32 with an operation counter (algorithmic FLOPs)
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <limits>

namespace orc {

// ---------------------------------------------------------------------------
// scalar adaptors
// ---------------------------------------------------------------------------
inline double val(double x) { return x; }
inline double val(float x) { return x; }

template<int N>
struct Dual {
	double v = 0;
	double d[N] = {};
	Dual() = default;
	Dual(double x) : v(x) {}
	static Dual var(double x, int i) { Dual r(x); r.d[i] = 1; return r; }
};
template<int N> inline double val(const Dual<N> &a) { return a.v; }
#define ORC_DUAL_BIN(OP, VEXPR, DEXPR) \
	template<int N> inline Dual<N> operator OP(const Dual<N> &a, const Dual<N> &b) { Dual<N> r; r.v = VEXPR; for (int i = 0; i < N; i++) r.d[i] = DEXPR; return r; } \
	template<int N> inline Dual<N> operator OP(const Dual<N> &a, double bb) { return a OP Dual<N>(bb); } \
	template<int N> inline Dual<N> operator OP(double aa, const Dual<N> &b) { return Dual<N>(aa) OP b; }
ORC_DUAL_BIN(+, a.v + b.v, a.d[i] + b.d[i])
ORC_DUAL_BIN(-, a.v - b.v, a.d[i] - b.d[i])
ORC_DUAL_BIN(*, a.v * b.v, a.d[i] * b.v + a.v * b.d[i])
ORC_DUAL_BIN(/, a.v / b.v, (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v))
#undef ORC_DUAL_BIN
template<int N> inline Dual<N> operator-(const Dual<N> &a) { Dual<N> r; r.v = -a.v; for (int i = 0; i < N; i++) r.d[i] = -a.d[i]; return r; }
template<int N> inline Dual<N> &operator+=(Dual<N> &a, const Dual<N> &b) { a = a + b; return a; }
template<int N> inline Dual<N> &operator-=(Dual<N> &a, const Dual<N> &b) { a = a - b; return a; }
template<int N> inline Dual<N> &operator*=(Dual<N> &a, const Dual<N> &b) { a = a * b; return a; }
template<int N> inline Dual<N> &operator/=(Dual<N> &a, const Dual<N> &b) { a = a / b; return a; }
template<int N> inline Dual<N> chain(const Dual<N> &a, double v, double dv) { Dual<N> r; r.v = v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] * dv; return r; }
template<int N> inline Dual<N> sqrt(const Dual<N> &a) { double s = std::sqrt(a.v); return chain(a, s, s > 0 ? 0.5 / s : 0.0); }
template<int N> inline Dual<N> abs(const Dual<N> &a) { return chain(a, std::fabs(a.v), a.v > 0 ? 1.0 : (a.v < 0 ? -1.0 : 0.0)); }
template<int N> inline Dual<N> floor(const Dual<N> &a) { return chain(a, std::floor(a.v), 0.0); }
template<int N> inline Dual<N> sin(const Dual<N> &a) { return chain(a, std::sin(a.v), std::cos(a.v)); }
template<int N> inline Dual<N> cos(const Dual<N> &a) { return chain(a, std::cos(a.v), -std::sin(a.v)); }
template<int N> inline Dual<N> atan(const Dual<N> &a) { return chain(a, std::atan(a.v), 1.0 / (1.0 + a.v * a.v)); }
template<int N> inline Dual<N> acos(const Dual<N> &a) { double t = 1 - a.v * a.v; return chain(a, std::acos(a.v), t > 0 ? -1.0 / std::sqrt(t) : 0.0); }
template<int N> inline Dual<N> log(const Dual<N> &a) { return chain(a, std::log(a.v), 1.0 / a.v); }
template<int N> inline Dual<N> exp(const Dual<N> &a) { double e = std::exp(a.v); return chain(a, e, e); }
template<int N> inline Dual<N> pow(const Dual<N> &a, double p) { double v = std::pow(a.v, p); return chain(a, v, a.v != 0 ? p * std::pow(a.v, p - 1) : 0.0); }
template<int N> inline Dual<N> atan2(const Dual<N> &y, const Dual<N> &x) {
	Dual<N> r; r.v = std::atan2(y.v, x.v); double den = x.v * x.v + y.v * y.v;
	for (int i = 0; i < N; i++) r.d[i] = den > 0 ? (x.v * y.d[i] - y.v * x.d[i]) / den : 0.0;
	return r;
}

// FP32 scalar: every operation rounds to float, constants are converted to
// float first. Fl<true> also counts operations: add/sub/mul/neg/min/max/abs/
// compare-select = 1 "flop" each (an FMA is one mul + one add = 2); div,
// sqrt, floor and transcendental calls are counted in separate bins.
struct OpCounts { uint64_t flop = 0, div = 0, sqrt = 0, floor = 0, transc = 0; };
inline OpCounts &opcounts() { static thread_local OpCounts c; return c; }
template<bool CNT>
struct Fl {
	float v = 0;
	Fl() = default;
	Fl(double x) : v((float)x) {}
};
using F32 = Fl<false>;
using Counted = Fl<true>;
template<bool C> inline double val(const Fl<C> &a) { return a.v; }
template<bool C> inline void cnt(uint64_t OpCounts::*f) { if (C) opcounts().*f += 1; }
#define ORC_FL_BIN(OP) \
	template<bool C> inline Fl<C> operator OP(const Fl<C> &a, const Fl<C> &b) { cnt<C>(&OpCounts::flop); Fl<C> r; r.v = a.v OP b.v; return r; } \
	template<bool C> inline Fl<C> operator OP(const Fl<C> &a, double b) { return a OP Fl<C>(b); } \
	template<bool C> inline Fl<C> operator OP(double a, const Fl<C> &b) { return Fl<C>(a) OP b; }
ORC_FL_BIN(+) ORC_FL_BIN(-) ORC_FL_BIN(*)
#undef ORC_FL_BIN
template<bool C> inline Fl<C> operator/(const Fl<C> &a, const Fl<C> &b) { cnt<C>(&OpCounts::div); Fl<C> r; r.v = a.v / b.v; return r; }
template<bool C> inline Fl<C> operator/(const Fl<C> &a, double b) { return a / Fl<C>(b); }
template<bool C> inline Fl<C> operator/(double a, const Fl<C> &b) { return Fl<C>(a) / b; }
template<bool C> inline Fl<C> operator-(const Fl<C> &a) { cnt<C>(&OpCounts::flop); Fl<C> r; r.v = -a.v; return r; }
template<bool C> inline Fl<C> &operator+=(Fl<C> &a, const Fl<C> &b) { a = a + b; return a; }
template<bool C> inline Fl<C> &operator-=(Fl<C> &a, const Fl<C> &b) { a = a - b; return a; }
template<bool C> inline Fl<C> &operator*=(Fl<C> &a, const Fl<C> &b) { a = a * b; return a; }
template<bool C> inline Fl<C> &operator/=(Fl<C> &a, const Fl<C> &b) { a = a / b; return a; }
template<bool C> inline Fl<C> sqrt(const Fl<C> &a) { cnt<C>(&OpCounts::sqrt); Fl<C> r; r.v = std::sqrt(a.v); return r; }
template<bool C> inline Fl<C> abs(const Fl<C> &a) { cnt<C>(&OpCounts::flop); Fl<C> r; r.v = std::fabs(a.v); return r; }
template<bool C> inline Fl<C> floor(const Fl<C> &a) { cnt<C>(&OpCounts::floor); Fl<C> r; r.v = std::floor(a.v); return r; }
#define ORC_FL_T(F) template<bool C> inline Fl<C> F(const Fl<C> &a) { cnt<C>(&OpCounts::transc); Fl<C> r; r.v = std::F(a.v); return r; }
ORC_FL_T(sin) ORC_FL_T(cos) ORC_FL_T(atan) ORC_FL_T(acos) ORC_FL_T(log) ORC_FL_T(exp)
#undef ORC_FL_T
template<bool C> inline Fl<C> pow(const Fl<C> &a, double p) { cnt<C>(&OpCounts::transc); Fl<C> r; r.v = std::pow(a.v, (float)p); return r; }
template<bool C> inline Fl<C> atan2(const Fl<C> &y, const Fl<C> &x) { cnt<C>(&OpCounts::transc); Fl<C> r; r.v = std::atan2(y.v, x.v); return r; }

// Forward-mode value + gradient over the counting FP32 scalar: the
// algorithmic operation count of evaluating d and dd/dp together. A quantity
// with a zero derivative (a constant, or anything computed only from
// constants or from floor) carries no derivative lanes and costs nothing
// extra, so the count is that of sparse forward-mode differentiation.
struct CDual {
	Counted v;
	Counted d[3];
	bool live = false;
	CDual() = default;
	CDual(double x) : v(x) {}
	static CDual var(double x, int i) { CDual r(x); r.d[i] = Counted(1.0); r.live = true; return r; }
};
inline double val(const CDual &a) { return a.v.v; }
inline CDual operator+(const CDual &a, const CDual &b) {
	CDual r; r.v = a.v + b.v; r.live = a.live || b.live;
	for (int i = 0; i < 3; i++) r.d[i] = a.live && b.live ? a.d[i] + b.d[i] : (a.live ? a.d[i] : b.d[i]);
	return r;
}
inline CDual operator-(const CDual &a) {
	CDual r; r.v = -a.v; r.live = a.live;
	for (int i = 0; a.live && i < 3; i++) r.d[i] = -a.d[i];
	return r;
}
inline CDual operator-(const CDual &a, const CDual &b) {
	CDual r; r.v = a.v - b.v; r.live = a.live || b.live;
	for (int i = 0; i < 3; i++) r.d[i] = a.live && b.live ? a.d[i] - b.d[i] : (a.live ? a.d[i] : (b.live ? -b.d[i] : Counted()));
	return r;
}
inline CDual operator*(const CDual &a, const CDual &b) {
	CDual r; r.v = a.v * b.v; r.live = a.live || b.live;
	for (int i = 0; i < 3; i++)
		r.d[i] = a.live && b.live ? a.d[i] * b.v + a.v * b.d[i] : (a.live ? a.d[i] * b.v : (b.live ? a.v * b.d[i] : Counted()));
	return r;
}
inline CDual cd_chain(const CDual &a, Counted v, Counted dv) {
	CDual r; r.v = v; r.live = a.live;
	for (int i = 0; a.live && i < 3; i++) r.d[i] = a.d[i] * dv;
	return r;
}
inline CDual operator/(const CDual &a, const CDual &b) {
	CDual r; r.v = a.v / b.v; r.live = a.live || b.live;
	if (!r.live) return r;
	const Counted inv = Counted(1.0) / b.v;
	for (int i = 0; i < 3; i++) {
		if (a.live && b.live) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
		else if (a.live) r.d[i] = a.d[i] * inv;
		else r.d[i] = -(r.v * b.d[i]) * inv;
	}
	return r;
}
#define ORC_CD_MIX(OP) \
	inline CDual operator OP(const CDual &a, double b) { return a OP CDual(b); } \
	inline CDual operator OP(double a, const CDual &b) { return CDual(a) OP b; }
ORC_CD_MIX(+) ORC_CD_MIX(-) ORC_CD_MIX(*) ORC_CD_MIX(/)
#undef ORC_CD_MIX
inline CDual &operator+=(CDual &a, const CDual &b) { a = a + b; return a; }
inline CDual &operator-=(CDual &a, const CDual &b) { a = a - b; return a; }
inline CDual &operator*=(CDual &a, const CDual &b) { a = a * b; return a; }
inline CDual &operator/=(CDual &a, const CDual &b) { a = a / b; return a; }
inline CDual sqrt(const CDual &a) { const Counted s = sqrt(a.v); return cd_chain(a, s, a.live ? Counted(0.5) / s : Counted()); }
inline CDual abs(const CDual &a) {
	CDual r; r.v = abs(a.v); r.live = a.live;
	for (int i = 0; a.live && i < 3; i++) r.d[i] = val(a) < 0 ? -a.d[i] : a.d[i];
	return r;
}
inline CDual floor(const CDual &a) { CDual r; r.v = floor(a.v); return r; }
inline void count_sel(const CDual &) { cnt<true>(&OpCounts::flop); }

using std::sqrt; using std::floor; using std::sin; using std::cos; using std::atan; using std::acos;
using std::log; using std::exp; using std::atan2; using std::pow;
inline double abs(double x) { return std::fabs(x); }

// comparison-based helpers; for Counted each select counts one op
template<class T> inline void count_sel(const T &) {}
template<bool C> inline void count_sel(const Fl<C> &) { cnt<C>(&OpCounts::flop); }
template<class T> inline T tmin(const T &a, const T &b) { count_sel(a); return val(b) < val(a) ? b : a; }
template<class T> inline T tmax(const T &a, const T &b) { count_sel(a); return val(b) > val(a) ? b : a; }
template<class T> inline T tclamp(const T &x, double lo, double hi) { return tmin(tmax(x, T(lo)), T(hi)); }
template<class T> inline T saturate(const T &x) { return tclamp(x, 0.0, 1.0); }
template<class T> inline T sqr(const T &x) { return x * x; }
template<class T> inline T tsign(const T &x) { return T(val(x) > 0 ? 1.0 : (val(x) < 0 ? -1.0 : 0.0)); }

// ---------------------------------------------------------------------------
// vectors
// ---------------------------------------------------------------------------
template<class T>
struct V3 {
	T x, y, z;
	V3() : x(0.0), y(0.0), z(0.0) {}
	V3(const T &a, const T &b, const T &c) : x(a), y(b), z(c) {}
	explicit V3(double s) : x(s), y(s), z(s) {}
	T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
	const T &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template<class T> inline V3<T> operator+(const V3<T> &a, const V3<T> &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template<class T> inline V3<T> operator-(const V3<T> &a, const V3<T> &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template<class T> inline V3<T> operator-(const V3<T> &a) { return {-a.x, -a.y, -a.z}; }
template<class T, class S> inline V3<T> operator*(const V3<T> &a, const S &s) { return {a.x * s, a.y * s, a.z * s}; }
template<class T, class S> inline V3<T> operator*(const S &s, const V3<T> &a) { return {a.x * s, a.y * s, a.z * s}; }
template<class T> inline V3<T> operator*(const V3<T> &a, const V3<T> &b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template<class T, class S> inline V3<T> operator/(const V3<T> &a, const S &s) { return {a.x / s, a.y / s, a.z / s}; }
template<class T> inline T dot(const V3<T> &a, const V3<T> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template<class T> inline T length(const V3<T> &a) { return sqrt(dot(a, a)); }
template<class T> inline V3<T> normalize(const V3<T> &a) { return a / length(a); }
template<class T> inline V3<T> cross(const V3<T> &a, const V3<T> &b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
template<class T> inline V3<T> vabs(const V3<T> &a) { return {abs(a.x), abs(a.y), abs(a.z)}; }
template<class T> inline V3<T> vmax(const V3<T> &a, double s) { return {tmax(a.x, T(s)), tmax(a.y, T(s)), tmax(a.z, T(s))}; }
template<class T> inline V3<T> vsat(const V3<T> &a) { return {saturate(a.x), saturate(a.y), saturate(a.z)}; }
template<class T> inline T len2(const T &x, const T &y) { return sqrt(x * x + y * y); }

// ---------------------------------------------------------------------------
// reference math helpers (sources/math.cpp)
// ---------------------------------------------------------------------------
// linear interpolation a + (b - a) * f
template<class T> inline T interpolate(const T &a, const T &b, const T &f) { return a + (b - a) * f; }
template<class T> inline V3<T> interpolate(const V3<T> &a, const V3<T> &b, const T &f) { return {interpolate(a.x, b.x, f), interpolate(a.y, b.y, f), interpolate(a.z, b.z, f)}; }
// smoothstep(x) = x^2 (3 - 2x), smootherstep(x) = x^3 (x (6x - 15) + 10)
template<class T> inline T smoothstep(const T &x) { return x * x * (3.0 - 2.0 * x); }
template<class T> inline T smootherstep(const T &x) { return x * x * x * (x * (x * 6.0 - 15.0) + 10.0); }
// sources/math.cpp:8-11
template<class T> inline T rescale(const T &v, double ia, double ib, double oa, double ob) { return (v - ia) / (ib - ia) * (ob - oa) + oa; }
// sources/math.cpp:13-16
template<class T> inline T sharpEdge(const T &v, double p = 0.05) { return rescale(tclamp(v, 0.5 - p, 0.5 + p), 0.5 - p, 0.5 + p, 0.0, 1.0); }
// sources/math.cpp:18-26
template<class T> inline T terrace(const T &x, double steepness) {
	const T f = floor(x);
	const T t = smootherstep(saturate((x - f) * std::max(steepness, 1.0))) + f;
	return interpolate(x, t, T(std::min(std::max(steepness, 0.0), 1.0)));
}
// sources/math.cpp:28-33 (polynomial smooth minimum)
template<class T> inline T smoothMin(const T &a, const T &b, const T &k) {
	const T h = saturate((b - a) / k * 0.5 + 0.5);
	return interpolate(b, a, h) - k * h * (1.0 - h);
}
// sources/math.cpp:35-38
template<class T> inline T smoothMax(const T &a, const T &b, const T &k) { return -smoothMin(-a, -b, k); }

// ---------------------------------------------------------------------------
// integer hash (project definition; cage's hash() is absent)
// ---------------------------------------------------------------------------
// mix32: the "lowbias32" 32-bit finaliser published by C. Wellons
// (hash-prospector, public domain).
inline uint32_t mix32(uint32_t x) {
	x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
	return x;
}
// per-instance seed key
inline uint32_t seed_key(uint32_t seed) { return mix32(seed + 0x9E3779B9U); }
// lattice hash: spatial-hash primes of Teschner et al. 2003 ("Optimized
// spatial hashing for collision detection of deformable objects") combined
// with XOR, then mix32.
inline uint32_t lattice_hash(int32_t ix, int32_t iy, int32_t iz, uint32_t key) {
	return mix32(((uint32_t)ix * 73856093U) ^ ((uint32_t)iy * 19349663U) ^ ((uint32_t)iz * 83492791U) ^ key);
}
// top 24 bits -> [-1, 1), exact in FP32
inline double hash_signed(uint32_t h) { return (double)(float)((float)(h >> 8) * (1.0f / 8388608.0f) - 1.0f); }

// ---------------------------------------------------------------------------
// noise family (project definition from published methods)
// ---------------------------------------------------------------------------
enum NoiseType { NT_VALUE = 0, NT_CUBIC = 1, NT_PERLIN = 2, NT_SIMPLEX = 3, NT_SIMPLEX_REDUCED = 4, NT_CELLULAR = 5 };
enum FractalType { FR_NONE = 0, FR_FBM = 1, FR_RIDGED = 2 };
enum DistanceType { DI_EUCLID = 0, DI_MANHATTAN = 1, DI_HYBRID = 2 };
enum CellOp { OP_CELL = 0, OP_DIST = 1, OP_DIST2 = 2, OP_ADD = 3, OP_SUB = 4, OP_MUL = 5, OP_DIV = 6 };

// Perlin's improved-noise gradient selection (K. Perlin, "Improving noise",
// SIGGRAPH 2002): 12 cube-edge directions, 4 of them repeated, from 4 bits.
template<class T> inline T grad3(uint32_t h, const T &x, const T &y, const T &z) {
	const uint32_t g = h & 15;
	const T &u = g < 8 ? x : y;
	const T &v = g < 4 ? y : ((g == 12 || g == 14) ? x : z);
	return ((g & 1) ? -u : u) + ((g & 2) ? -v : v);
}
template<class T> inline T fade5(const T &t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }

// value noise: lattice values from the hash, quintic-faded trilinear blend.
template<class T> T noise_value(const V3<T> &p, uint32_t key) {
	const T fx0 = floor(p.x), fy0 = floor(p.y), fz0 = floor(p.z);
	const int ix = (int)val(fx0), iy = (int)val(fy0), iz = (int)val(fz0);
	const T fx = p.x - fx0, fy = p.y - fy0, fz = p.z - fz0;
	const T u = fade5(fx), v = fade5(fy), w = fade5(fz);
	T c[8];
	for (int b = 0; b < 8; b++)
		c[b] = T(hash_signed(lattice_hash(ix + (b & 1), iy + ((b >> 1) & 1), iz + (b >> 2), key)));
	const T x00 = interpolate(c[0], c[1], u), x10 = interpolate(c[2], c[3], u);
	const T x01 = interpolate(c[4], c[5], u), x11 = interpolate(c[6], c[7], u);
	return interpolate(interpolate(x00, x10, v), interpolate(x01, x11, v), w);
}

// Catmull-Rom spline through p0..p3 at t in [0,1]
template<class T> inline T catmull(const T &p0, const T &p1, const T &p2, const T &p3, const T &t) {
	return p1 + 0.5 * t * (p2 - p0 + t * (2.0 * p0 - 5.0 * p1 + 4.0 * p2 - p3 + t * (3.0 * (p1 - p2) + p3 - p0)));
}
// cubic value noise: tricubic Catmull-Rom over the 4x4x4 lattice values,
// scaled by 0.75 (the spline overshoots the lattice range by up to 1.25 per
// axis; with the scale the observed range is about [-1, 1]).
template<class T> T noise_cubic(const V3<T> &p, uint32_t key) {
	const T fx0 = floor(p.x), fy0 = floor(p.y), fz0 = floor(p.z);
	const int ix = (int)val(fx0), iy = (int)val(fy0), iz = (int)val(fz0);
	const T fx = p.x - fx0, fy = p.y - fy0, fz = p.z - fz0;
	T zs[4];
	for (int k = 0; k < 4; k++) {
		T ys[4];
		for (int j = 0; j < 4; j++) {
			T xs[4];
			for (int i = 0; i < 4; i++)
				xs[i] = T(hash_signed(lattice_hash(ix + i - 1, iy + j - 1, iz + k - 1, key)));
			ys[j] = catmull(xs[0], xs[1], xs[2], xs[3], fx);
		}
		zs[k] = catmull(ys[0], ys[1], ys[2], ys[3], fy);
	}
	return catmull(zs[0], zs[1], zs[2], zs[3], fz) * 0.75;
}

// improved Perlin gradient noise (Perlin 2002), gradients from grad3.
template<class T> T noise_perlin(const V3<T> &p, uint32_t key) {
	const T fx0 = floor(p.x), fy0 = floor(p.y), fz0 = floor(p.z);
	const int ix = (int)val(fx0), iy = (int)val(fy0), iz = (int)val(fz0);
	const T fx = p.x - fx0, fy = p.y - fy0, fz = p.z - fz0;
	const T u = fade5(fx), v = fade5(fy), w = fade5(fz);
	T c[8];
	for (int b = 0; b < 8; b++) {
		const int dx = b & 1, dy = (b >> 1) & 1, dz = b >> 2;
		c[b] = grad3(lattice_hash(ix + dx, iy + dy, iz + dz, key), fx - (double)dx, fy - (double)dy, fz - (double)dz);
	}
	const T x00 = interpolate(c[0], c[1], u), x10 = interpolate(c[2], c[3], u);
	const T x01 = interpolate(c[4], c[5], u), x11 = interpolate(c[6], c[7], u);
	return interpolate(interpolate(x00, x10, v), interpolate(x01, x11, v), w);
}

// 3-D simplex noise after S. Gustavson, "Simplex noise demystified" (2005):
// skew 1/3, unskew 1/6, four corners, radial kernel (0.5 - r^2)^4 (a radius
// of 0.5 keeps the sum continuous), gradients from grad3. SimplexReduced uses
// the cubic kernel (0.5 - r^2)^3. The scales (76, 31) map the range to
// about [-1, 1].
constexpr double SIMPLEX_SCALE = 76.0;
constexpr double SIMPLEX_REDUCED_SCALE = 31.0;
template<class T> T noise_simplex(const V3<T> &p, uint32_t key, bool reduced) {
	const double F3 = 1.0 / 3.0, G3 = 1.0 / 6.0;
	const T s = (p.x + p.y + p.z) * F3;
	const T fi = floor(p.x + s), fj = floor(p.y + s), fk = floor(p.z + s);
	const int i = (int)val(fi), j = (int)val(fj), k = (int)val(fk);
	const T t = (fi + fj + fk) * G3;
	const T x0 = p.x - (fi - t), y0 = p.y - (fj - t), z0 = p.z - (fk - t);
	int i1, j1, k1, i2, j2, k2;
	const double X = val(x0), Y = val(y0), Z = val(z0);
	if (X >= Y) {
		if (Y >= Z) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
		else if (X >= Z) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 0; k2 = 1; }
		else { i1 = 0; j1 = 0; k1 = 1; i2 = 1; j2 = 0; k2 = 1; }
	} else {
		if (Y < Z) { i1 = 0; j1 = 0; k1 = 1; i2 = 0; j2 = 1; k2 = 1; }
		else if (X < Z) { i1 = 0; j1 = 1; k1 = 0; i2 = 0; j2 = 1; k2 = 1; }
		else { i1 = 0; j1 = 1; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
	}
	const int ci[4][3] = {{0, 0, 0}, {i1, j1, k1}, {i2, j2, k2}, {1, 1, 1}};
	T n = T(0.0);
	for (int c = 0; c < 4; c++) {
		const double off = G3 * c;
		const T xc = x0 - (double)ci[c][0] + off, yc = y0 - (double)ci[c][1] + off, zc = z0 - (double)ci[c][2] + off;
		T tt = 0.5 - xc * xc - yc * yc - zc * zc;
		if (val(tt) > 0) {
			T t2 = tt * tt;
			T kern = reduced ? t2 * tt : t2 * t2;
			n += kern * grad3(lattice_hash(i + ci[c][0], j + ci[c][1], k + ci[c][2], key), xc, yc, zc);
		}
	}
	return n * (reduced ? SIMPLEX_REDUCED_SCALE : SIMPLEX_SCALE);
}

// cellular (Worley 1996) noise: one feature point per lattice cell at
// cell + jitter, jitter from three 10-bit fields of the cell hash; the 3x3x3
// neighbourhood is searched (z outer, x inner; strict < keeps the first on
// ties). Outputs, each offset into about [-1, 1]:
//   Cell: value of the nearest cell; Distance: F1-1; Distance2: F2-1;
//   Add: (F1+F2)/2-1; Subtract: F2-F1-1; Multiply: F1*F2/2-1; Divide: F1/F2-1
// Distances: Euclidean |v|, Manhattan sum|v_i|, Hybrid |v|^2 + sum|v_i|.
inline double jitter_of(uint32_t h, int s) { return (double)(((h >> s) & 1023U) * (1.0f / 1024.0f) + (1.0f / 2048.0f)); }
template<class T> T noise_cellular(const V3<T> &p, uint32_t key, int dist, int op) {
	const T fx0 = floor(p.x), fy0 = floor(p.y), fz0 = floor(p.z);
	const int ix = (int)val(fx0), iy = (int)val(fy0), iz = (int)val(fz0);
	const T fx = p.x - fx0, fy = p.y - fy0, fz = p.z - fz0;
	T F1 = T(1e10), F2 = T(1e10);
	uint32_t cellh = 0;
	for (int dz = -1; dz <= 1; dz++)
		for (int dy = -1; dy <= 1; dy++)
			for (int dx = -1; dx <= 1; dx++) {
				const uint32_t h = lattice_hash(ix + dx, iy + dy, iz + dz, key);
				const T vx = (dx + jitter_of(h, 0)) - fx;
				const T vy = (dy + jitter_of(h, 10)) - fy;
				const T vz = (dz + jitter_of(h, 20)) - fz;
				T d;
				if (dist == DI_EUCLID) d = sqrt(vx * vx + vy * vy + vz * vz);
				else if (dist == DI_MANHATTAN) d = abs(vx) + abs(vy) + abs(vz);
				else d = (vx * vx + vy * vy + vz * vz) + (abs(vx) + abs(vy) + abs(vz));
				if (val(d) < val(F1)) { F2 = F1; F1 = d; cellh = h; }
				else if (val(d) < val(F2)) F2 = d;
			}
	switch (op) {
		case OP_CELL: return T(hash_signed(mix32(cellh)));
		case OP_DIST: return F1 - 1.0;
		case OP_DIST2: return F2 - 1.0;
		case OP_ADD: return (F1 + F2) * 0.5 - 1.0;
		case OP_SUB: return F2 - F1 - 1.0;
		case OP_MUL: return F1 * F2 * 0.5 - 1.0;
		default: return F1 / F2 - 1.0;
	}
}

template<class T> T noise_single(int type, const V3<T> &p, uint32_t key, int dist, int op) {
	switch (type) {
		case NT_VALUE: return noise_value(p, key);
		case NT_CUBIC: return noise_cubic(p, key);
		case NT_PERLIN: return noise_perlin(p, key);
		case NT_SIMPLEX: return noise_simplex(p, key, false);
		case NT_SIMPLEX_REDUCED: return noise_simplex(p, key, true);
		default: return noise_cellular(p, key, dist, op);
	}
}

// A configured noise function with its fractal expanded into per-octave
// (frequency, amplitude, seed). Fractal definitions:
//   None:   n(f p)
//   Fbm:    sum_i a_i n(f_i p, seed+i)
//   Ridged: sum_i a_i (1 - 2 |n(f_i p, seed+i)|)
// with f_i = f lacunarity^i and a_i = gain^i / sum_j |gain|^j.
struct NoiseCfg {
	int type = NT_SIMPLEX, fractal = FR_NONE, octaves = 3, dist = DI_EUCLID, op = OP_DIST;
	double frequency = 1, lacunarity = 2, gain = 0.5;
	uint32_t seed = 0;
};
struct NoiseFn {
	int type = NT_SIMPLEX, fractal = FR_NONE, dist = DI_EUCLID, op = OP_DIST, octaves = 1;
	double freq[8] = {}, amp[8] = {};
	uint32_t key[8] = {};
};
inline NoiseFn make_noise(const NoiseCfg &c) {
	NoiseFn n;
	n.type = c.type; n.fractal = c.fractal; n.dist = c.dist; n.op = c.op;
	n.octaves = c.fractal == FR_NONE ? 1 : std::min(std::max(c.octaves, 1), 8);
	double bound = 0, g = 1;
	for (int i = 0; i < n.octaves; i++) { bound += std::fabs(g); g *= c.gain; }
	double f = c.frequency; g = 1;
	for (int i = 0; i < n.octaves; i++) {
		n.freq[i] = (double)(float)f;
		n.amp[i] = n.fractal == FR_NONE ? 1.0 : (double)(float)(g / bound);
		n.key[i] = seed_key(c.seed + (uint32_t)i);
		f *= c.lacunarity; g *= c.gain;
	}
	return n;
}
template<class T> T noise_eval(const NoiseFn &n, const V3<T> &p) {
	T acc = T(0.0);
	for (int i = 0; i < n.octaves; i++) {
		const T f = T(n.freq[i]);
		const V3<T> q(p.x * f, p.y * f, p.z * f);
		T v = noise_single(n.type, q, n.key[i], n.dist, n.op);
		if (n.fractal == FR_RIDGED) v = 1.0 - 2.0 * abs(v);
		acc += v * T(n.amp[i]);
	}
	return acc;
}

} // namespace orc
