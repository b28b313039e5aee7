// Oracle: the reference modes -- 34 base shapes (sources/sdf.cpp), 6
// elevation modes (sources/elevationModes.cpp), Voronoi
// (sources/voronoi.cpp), the SDF fields (sources/modesConfiguration.cpp:
// 230-279) and the per-texel coloring pipelines (sources/coloringModes.cpp).
// TEST INFRASTRUCTURE, parity unpinned (see oracle_core.hpp). The cage
// primitives the reference calls (sdfSphere/Box/Torus/..., Triangle distance,
// Quat, colour conversions) are restated from published closed forms named at
// each one; everything else follows the reference line by line.
#pragma once
#include "oracle_core.hpp"
#include "../unnatural-planets_gb300/csrc/up_sinnet_data.h"
#include <cstring>
#include <string>

namespace orc {

// ---------------------------------------------------------------------------
// cage-side primitives (I. Quilez's distance functions; axis conventions:
// torus/capsule/cylinder/hexagonal prism around z)
// ---------------------------------------------------------------------------
template<class T> T prim_sphere(const V3<T> &p, double r) { return length(p) - r; }
template<class T> T prim_plane(const V3<T> &p, const V3<T> &n) { return dot(p, n); }
template<class T> T prim_capsule(V3<T> p, double height, double radius) {
	p.z = p.z - tclamp(p.z, -0.5 * height, 0.5 * height);
	return length(p) - radius;
}
template<class T> T prim_cylinder(const V3<T> &p, double height, double radius) {
	const T dx = len2(p.x, p.y) - radius, dy = abs(p.z) - 0.5 * height;
	return tmin(tmax(dx, dy), T(0.0)) + len2(tmax(dx, T(0.0)), tmax(dy, T(0.0)));
}
template<class T> T prim_box(const V3<T> &p, const V3<double> &h) {
	const V3<T> q(abs(p.x) - h.x, abs(p.y) - h.y, abs(p.z) - h.z);
	return length(vmax(q, 0.0)) + tmin(tmax(q.x, tmax(q.y, q.z)), T(0.0));
}
template<class T> T prim_tetrahedron(const V3<T> &p, double r) {
	return (tmax(abs(p.x + p.y) - p.z, abs(p.x - p.y) + p.z) - r) * (1.0 / std::sqrt(3.0));
}
template<class T> T prim_octahedron(const V3<T> &p, double r) { return (abs(p.x) + abs(p.y) + abs(p.z) - r) * 0.57735026918962576; }
template<class T> T prim_hexprism(const V3<T> &p_, double height, double radius) {
	const double kx = -0.86602540378443865, ky = 0.5, kz = 0.57735026918962576;
	V3<T> p = vabs(p_);
	const T t = 2.0 * tmin(kx * p.x + ky * p.y, T(0.0));
	p.x = p.x - t * kx;
	p.y = p.y - t * ky;
	const T cx = tclamp(p.x, -kz * radius, kz * radius);
	const T ex = p.x - cx, ey = p.y - radius;
	const T dx = len2(ex, ey) * tsign(ey), dy = p.z - 0.5 * height;
	return tmin(tmax(dx, dy), T(0.0)) + len2(tmax(dx, T(0.0)), tmax(dy, T(0.0)));
}
template<class T> T prim_torus(const V3<T> &p, double major, double minor) { return len2(len2(p.x, p.y) - major, p.z) - minor; }
// torus knot: a torus of radius R = size/2 around z whose cross-section is two
// discs (offset 0.35R, radius 0.15R) rotated by twist * azimuth; twist 1.5
// joins the two discs into one closed knotted tube
template<class T> T prim_knot(const V3<T> &p, double size, double twist) {
	const double R = 0.5 * size;
	const T r = len2(p.x, p.y);
	const T a = atan2(p.y, p.x);
	const T ang = a * twist;
	const T c = cos(ang), s = sin(ang);
	const T u0 = r - R, v0 = p.z;
	const T u = c * u0 - s * v0, v = s * u0 + c * v0;
	return len2(abs(u) - 0.35 * R, v) - 0.15 * R;
}
// rotation about z by a (radians)
template<class T> V3<T> rot_z(const V3<T> &p, const T &a) {
	const T c = cos(a), s = sin(a);
	return V3<T>(c * p.x - s * p.y, s * p.x + c * p.y, p.z);
}
// point-triangle distance (C. Ericson, Real-Time Collision Detection, 5.1.5)
template<class T> T tri_distance(const V3<T> &p, const V3<double> &A, const V3<double> &B, const V3<double> &C) {
	const V3<T> a(T(A.x), T(A.y), T(A.z)), b(T(B.x), T(B.y), T(B.z)), c(T(C.x), T(C.y), T(C.z));
	const V3<T> ab = b - a, ac = c - a, ap = p - a;
	const T d1 = dot(ab, ap), d2 = dot(ac, ap);
	if (val(d1) <= 0 && val(d2) <= 0) return length(p - a);
	const V3<T> bp = p - b;
	const T d3 = dot(ab, bp), d4 = dot(ac, bp);
	if (val(d3) >= 0 && val(d4) <= val(d3)) return length(p - b);
	const T vc = d1 * d4 - d3 * d2;
	if (val(vc) <= 0 && val(d1) >= 0 && val(d3) <= 0) { const T v = d1 / (d1 - d3); return length(p - (a + ab * v)); }
	const V3<T> cp = p - c;
	const T d5 = dot(ab, cp), d6 = dot(ac, cp);
	if (val(d6) >= 0 && val(d5) <= val(d6)) return length(p - c);
	const T vb = d5 * d2 - d1 * d6;
	if (val(vb) <= 0 && val(d2) >= 0 && val(d6) <= 0) { const T w = d2 / (d2 - d6); return length(p - (a + ac * w)); }
	const T va = d3 * d6 - d5 * d4;
	if (val(va) <= 0 && val(d4 - d3) >= 0 && val(d5 - d6) >= 0) {
		const T w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
		return length(p - (b + (c - b) * w));
	}
	const T denom = 1.0 / (va + vb + vc);
	const T v = vb * denom, w = vc * denom;
	return length(p - (a + ab * v + ac * w));
}

// ---------------------------------------------------------------------------
// planet description (the oracle's own expansion of the mode names)
// ---------------------------------------------------------------------------
struct VoronoiCfg {
	int32_t seed_hash[3];
	double cell_size, frequency;
	int ppc;
};

enum { N_SLOTS = 64 };
struct Planet {
	int shape = 0, elevation = 0, coloring = 0;
	bool poles = false, flowers = false;
	double fibers_offset[3] = {0, 0, 0};
	uint32_t deviation_key = 0;
	NoiseFn noise[N_SLOTS];
	VoronoiCfg craters, boulders, flower_cluster, flower_center;
};

static const char *const kShapes[34] = {"asteroid", "belt", "bowl", "box", "bunny", "capsule", "cube", "disk", "doubletorus", "fibers",
	"gear", "h2o", "h3o", "h4o", "hemispheres", "hexagon", "hexagonalprism", "insidecube", "knot", "mandelbulb", "mobiusstrip",
	"monkeyhead", "octahedron", "pipe", "sphere", "square", "tetrahedron", "torus", "toruscross", "triangularprism", "tube",
	"twistedhexagonalprism", "twistedplane", "wormhole"};
static const char *const kElevations[6] = {"none", "simple", "legacy", "lakes", "islands", "craters"};
static const char *const kColorings[3] = {"default", "barren", "debug"};

// slot numbers of the noise instances (the seed derivation is part of the
// planet definition: slot s of planet seed S has seed mix32(S + 0x9E3779B9 (s+1)))
enum Slot {
	S_ASTEROID = 0, S_SIMPLE, S_LEGACY_SCALE, S_LEGACY_ELEV, S_MTN_MASK, S_MTN_RIDGE, S_MTN_TERRACE, S_LAKES_LAND, S_ISLANDS_LAND,
	S_CRATERS_SCALE, S_BEACH, S_PRECIP, S_TEMP, S_POLAR, S_BED_DEPTH, S_BED_FREQ, S_BED_CRACKS, S_BED_VALUE, S_BED_SAT,
	S_CLIFF_CRACKS, S_MICA_MASK, S_MICA_CRACKS, S_DIRT_HEIGHT, S_DIRT_CRACKS, S_DIRT_CMASK, S_SAND_HSCALE, S_SAND_HEIGHT,
	S_SAND_COLOR, S_SAND_HUE, S_GRASS_HUE, S_GRASS_PCELLS, S_GRASS_PDIST, S_GRASS_SCRATCH, S_BOUL_THRESH, S_BOUL_SIZE,
	S_BOUL_HUE, S_BOUL_VALUE, S_BOUL_SCRATCH, S_WATER_SWITCH, S_WATER_HUE, S_FLOW_SIZE, S_FLOW_COLOR, S_FLOW_HUE1, S_FLOW_HUE2,
	S_ICE_TEMPOFF, S_ICE_FREQ, S_ICE_THICK, S_ICE_CRACKS, S_SNOW_ELEVOFF, S_SNOW_THICK,
	X_CRATERS_VORONOI = 64, X_BOUL_VORONOI, X_FLOW_CLUSTER, X_FLOW_CENTER, X_FIBERS_OFFSET, X_ASTEROID_FREQ, X_COLOR_DEVIATION,
	X_SHARED_BEDROCK, X_SHARED_GRASS, X_SHARED_ICE, X_RANDOM_SHAPE = 90
};

inline uint32_t slot_seed(uint32_t seed, uint32_t slot) { return mix32(seed + 0x9E3779B9U * (slot + 1U)); }
inline double slot_draw(uint32_t seed, uint32_t i) { return (mix32(seed ^ (0x85EBCA6BU * (i + 1U))) >> 8) * (1.0 / 16777216.0); }

inline VoronoiCfg make_voronoi(uint32_t seed, double cell, int ppc) {
	VoronoiCfg v;
	const uint32_t h1 = mix32(seed), h2 = mix32(h1), h3 = mix32(h2); // voronoi.cpp:17
	v.seed_hash[0] = (int32_t)h1; v.seed_hash[1] = (int32_t)h2; v.seed_hash[2] = (int32_t)h3;
	v.cell_size = (double)(float)cell;
	v.frequency = (double)(float)(1.0 / cell);
	v.ppc = ppc;
	return v;
}

// returns "" or an error message
inline std::string make_planet(const char *shape, const char *elevation, const char *coloring, bool poles, bool flowers, uint32_t seed, Planet &P) {
	P = Planet();
	auto S = [&](uint32_t s) { return slot_seed(seed, s); };
	const std::string sh = shape ? shape : "", el = elevation ? elevation : "", co = coloring ? coloring : "";
	P.shape = -1;
	if (sh == "random") P.shape = std::min(33, (int)(slot_draw(S(X_RANDOM_SHAPE), 0) * 34.0)); // modesConfiguration.cpp:119-125
	for (int i = 0; i < 34; i++) if (sh == kShapes[i]) P.shape = i;
	if (P.shape < 0) return "unknown shape mode configuration";
	P.elevation = -1;
	for (int i = 0; i < 6; i++) if (el == kElevations[i]) P.elevation = i;
	if (P.elevation < 0) return "unknown elevation mode configuration";
	P.coloring = -1;
	for (int i = 0; i < 3; i++) if (co == kColorings[i]) P.coloring = i;
	if (P.coloring < 0) return "unknown coloring mode configuration";
	P.poles = poles; P.flowers = flowers;
	for (int a = 0; a < 3; a++) P.fibers_offset[a] = (double)(float)(slot_draw(S(X_FIBERS_OFFSET), a) * 200.0 - 100.0);
	P.deviation_key = S(X_COLOR_DEVIATION);
	auto mk = [&](int slot, int type, double freq, uint32_t sd, int fractal = FR_NONE, int oct = 3, double gain = 0.5, double lac = 2.0) {
		NoiseCfg c; c.type = type; c.frequency = freq; c.seed = sd; c.fractal = fractal; c.octaves = oct; c.gain = gain; c.lacunarity = lac;
		P.noise[slot] = make_noise(c);
	};
	auto mkc = [&](int slot, double freq, uint32_t sd, int dist, int op, int fractal = FR_NONE, int oct = 3) {
		NoiseCfg c; c.type = NT_CELLULAR; c.frequency = freq; c.seed = sd; c.dist = dist; c.op = op; c.fractal = fractal; c.octaves = oct;
		P.noise[slot] = make_noise(c);
	};
	mk(S_ASTEROID, NT_SIMPLEX, 0.65 + 0.1 * slot_draw(S(X_ASTEROID_FREQ), 0), S(S_ASTEROID), FR_FBM, 2, 0.3); // sdf.cpp:335-345
	mk(S_SIMPLE, NT_SIMPLEX, 0.0005, S(S_SIMPLE), FR_RIDGED, 6, 0.4);          // elevationModes.cpp:16-26
	mk(S_LEGACY_SCALE, NT_VALUE, 0.0005, S(S_LEGACY_SCALE), FR_FBM, 4);         // :36-45
	mk(S_LEGACY_ELEV, NT_VALUE, 1.0, S(S_LEGACY_ELEV), FR_FBM, 4);              // :46-54
	mk(S_MTN_MASK, NT_PERLIN, 0.0015, S(S_MTN_MASK));                           // :70-77
	mk(S_MTN_RIDGE, NT_SIMPLEX, 0.001, S(S_MTN_RIDGE), FR_RIDGED, 4, -0.4, 1.5); // :78-89
	mk(S_MTN_TERRACE, NT_PERLIN, 0.002, S(S_MTN_TERRACE), FR_FBM, 3, 0.3);      // :90-100
	mk(S_LAKES_LAND, NT_VALUE, 0.0013, S(S_LAKES_LAND), FR_FBM, 4);             // :131-140
	mk(S_ISLANDS_LAND, NT_VALUE, 0.0013, S(S_ISLANDS_LAND), FR_FBM, 4);         // :153-162
	mk(S_CRATERS_SCALE, NT_VALUE, 1.0, S(S_CRATERS_SCALE));                     // :183-190
	P.craters = make_voronoi(S(X_CRATERS_VORONOI), 300, 2);                     // :175-182
	const uint32_t bed = S(X_SHARED_BEDROCK), grass = S(X_SHARED_GRASS), ice = S(X_SHARED_ICE);
	// coloringModes.cpp
	mk(S_BEACH, NT_VALUE, 0.035, S(S_BEACH));                                   // :36-43
	mk(S_PRECIP, NT_CUBIC, 0.001, S(S_PRECIP), FR_FBM, 2);                      // :61-70
	mk(S_TEMP, NT_SIMPLEX, 0.0003, S(S_TEMP), FR_FBM, 2, 0.4);                  // :84-94
	mk(S_POLAR, NT_VALUE, 0.007, S(S_POLAR), FR_FBM, 3);                        // :95-104
	mk(S_BED_DEPTH, NT_CUBIC, 0.0031, S(S_BED_DEPTH));                          // :205-212
	mk(S_BED_FREQ, NT_CUBIC, 0.013, S(S_BED_FREQ));                             // :213-220
	mkc(S_BED_CRACKS, 0.017, bed, DI_HYBRID, OP_SUB);                           // :221-230
	mkc(S_BED_VALUE, 0.017, bed, DI_HYBRID, OP_CELL);                           // :231-240
	mk(S_BED_SAT, NT_CUBIC, 0.0022, S(S_BED_SAT), FR_FBM, 2);                   // :241-250
	mk(S_CLIFF_CRACKS, NT_SIMPLEX_REDUCED, 0.047, S(S_CLIFF_CRACKS), FR_RIDGED, 2); // :265-274
	mkc(S_MICA_MASK, 0.02, S(S_MICA_MASK), DI_HYBRID, OP_MUL);                  // :297-306
	mkc(S_MICA_CRACKS, 0.05, S(S_MICA_CRACKS), DI_MANHATTAN, OP_DIV);           // :307-317
	mk(S_DIRT_HEIGHT, NT_PERLIN, 0.05, S(S_DIRT_HEIGHT), FR_FBM, 3, 0.4, 2.3);  // :340-351
	mk(S_DIRT_CRACKS, NT_SIMPLEX_REDUCED, 0.07, S(S_DIRT_CRACKS), FR_RIDGED, 2); // :352-361
	mk(S_DIRT_CMASK, NT_CUBIC, 0.02, S(S_DIRT_CMASK), FR_FBM, 4);               // :362-371
	mk(S_SAND_HSCALE, NT_SIMPLEX, 0.001, S(S_SAND_HSCALE), FR_FBM, 3);          // :406-415
	mk(S_SAND_HEIGHT, NT_SIMPLEX, 0.01, S(S_SAND_HEIGHT), FR_RIDGED, 3, 0.7);   // :416-426
	mk(S_SAND_COLOR, NT_PERLIN, 0.0008, S(S_SAND_COLOR));                       // :427-433
	mk(S_SAND_HUE, NT_CUBIC, 0.02, S(S_SAND_HUE), FR_FBM, 2);                   // :435-444
	mk(S_GRASS_HUE, NT_PERLIN, 0.01, S(S_GRASS_HUE), FR_FBM, 2);                // :470-479
	mkc(S_GRASS_PCELLS, 0.1, grass, DI_HYBRID, OP_CELL);                        // :480-489
	mkc(S_GRASS_PDIST, 0.1, grass, DI_HYBRID, OP_SUB);                          // :490-499
	mkc(S_GRASS_SCRATCH, 0.3, S(S_GRASS_SCRATCH), DI_HYBRID, OP_MUL);           // :500-509
	mk(S_BOUL_THRESH, NT_PERLIN, 0.01, S(S_BOUL_THRESH));                       // :537-544
	mk(S_BOUL_SIZE, NT_PERLIN, 0.09, S(S_BOUL_SIZE));                           // :553-560
	mk(S_BOUL_HUE, NT_PERLIN, 0.3, S(S_BOUL_HUE));                              // :561-567
	mk(S_BOUL_VALUE, NT_PERLIN, 0.5, S(S_BOUL_VALUE));                          // :569-576
	mk(S_BOUL_SCRATCH, NT_PERLIN, 0.5, S(S_BOUL_SCRATCH));                      // :577-584
	mk(S_WATER_SWITCH, NT_PERLIN, 0.0015, S(S_WATER_SWITCH), FR_FBM, 2);        // :619-628
	mk(S_WATER_HUE, NT_CUBIC, 0.004, S(S_WATER_HUE), FR_FBM, 3);                // :629-638
	mk(S_FLOW_SIZE, NT_PERLIN, 0.35, S(S_FLOW_SIZE));                           // :674-681
	mk(S_FLOW_COLOR, NT_PERLIN, 0.02, S(S_FLOW_COLOR));                         // :682-689
	mk(S_FLOW_HUE1, NT_PERLIN, 0.005, S(S_FLOW_HUE1));                          // :690-697
	mk(S_FLOW_HUE2, NT_PERLIN, 0.4, S(S_FLOW_HUE2));                            // :698-705
	mk(S_ICE_TEMPOFF, NT_VALUE, 0.035, S(S_ICE_TEMPOFF));                       // :749-756
	mk(S_ICE_FREQ, NT_VALUE, 0.01, S(S_ICE_FREQ), FR_FBM, 3);                   // :757-766
	mkc(S_ICE_THICK, 0.05, ice, DI_HYBRID, OP_CELL, FR_FBM, 2);                 // :767-778
	mkc(S_ICE_CRACKS, 0.05, ice, DI_HYBRID, OP_SUB, FR_FBM, 2);                 // :779-790
	mk(S_SNOW_ELEVOFF, NT_VALUE, 0.055, S(S_SNOW_ELEVOFF));                     // :821-828
	mk(S_SNOW_THICK, NT_CUBIC, 0.05, S(S_SNOW_THICK), FR_FBM, 3);               // :829-838
	P.boulders = make_voronoi(S(X_BOUL_VORONOI), 200, 2);                       // :545-552
	P.flower_cluster = make_voronoi(S(X_FLOW_CLUSTER), 200, 1);                 // :660-666
	P.flower_center = make_voronoi(S(X_FLOW_CENTER), 35, 1);                    // :667-673
	return "";
}

// ---------------------------------------------------------------------------
// Voronoi (sources/voronoi.cpp:10-91); cage's hash() is the project mix32.
// Only the nearest point is needed by every caller (points[0]); ties keep the
// first point in generation order.
// ---------------------------------------------------------------------------
inline void vor_mix(const VoronoiCfg &v, const int32_t s[3], int32_t o[3]) {
	// voronoi.cpp:19-24: seedHashes + s + (s1, s2, s0) + (h(s0), h(s1), h(s2)), int32 wrap-around
	const uint32_t a[3] = {(uint32_t)s[1], (uint32_t)s[2], (uint32_t)s[0]};
	for (int i = 0; i < 3; i++) o[i] = (int32_t)((uint32_t)v.seed_hash[i] + (uint32_t)s[i] + a[i] + mix32((uint32_t)s[i]));
}
template<class T>
V3<T> voronoi_nearest(const VoronoiCfg &v, const V3<T> &pos, const V3<T> *normal) {
	// voronoi.cpp:351: cell = Vec3i(position * frequency), FP32 product, truncation
	const float fr = (float)v.frequency;
	const int32_t cell[3] = {(int32_t)((float)val(pos.x) * fr), (int32_t)((float)val(pos.y) * fr), (int32_t)((float)val(pos.z) * fr)};
	V3<T> best;
	double bestd = 1e300;
	for (int z = -1; z < 2; z++)
		for (int y = -1; y < 2; y++)
			for (int x = -1; x < 2; x++) {
				const int32_t c[3] = {cell[0] + x, cell[1] + y, cell[2] + z};
				int32_t s[3];
				vor_mix(v, c, s);
				for (int i = 0; i < v.ppc; i++) {
					int32_t s2[3];
					vor_mix(v, s, s2);
					for (int k = 0; k < 3; k++) s[k] = s2[k];
					// genPoint: Vec3(s % 65536) / 65535 (signed remainder), then (point + cell) * cellSize
					V3<T> p(T((double)(float)((float)(s[0] % 65536) / 65535.0f)) + (double)c[0],
						T((double)(float)((float)(s[1] % 65536) / 65535.0f)) + (double)c[1],
						T((double)(float)((float)(s[2] % 65536) / 65535.0f)) + (double)c[2]);
					p = p * v.cell_size;
					if (normal) { // voronoi.cpp:61-66: project onto the tangent plane at position
						const T dd = dot(*normal, p - pos);
						p = p - (*normal) * dd;
					}
					const V3<T> dp = p - pos;
					const double d = val(dot(dp, dp));
					if (d < bestd) { bestd = d; best = p; }
				}
			}
	return best;
}

// ---------------------------------------------------------------------------
// sine-network shapes (sdf.cpp:252-290)
// ---------------------------------------------------------------------------
template<class T> T sinnet(const SinNetWeights &W, const V3<T> &p) {
	if (val(length(p)) > 1) return length(p) - 0.8;
	T f0[4][4], f1[4][4], f2[4][4];
	for (int j = 0; j < 4; j++)
		for (int r = 0; r < 4; r++)
			f0[j][r] = sin(p.y * (double)W.in_y[j][r] + p.z * (double)W.in_z[j][r] + p.x * ((double)W.x_sign * W.in_x[j][r]) + (double)W.in_b[j][r]);
	auto layer = [&](T in[4][4], T out[4][4], int base) {
		for (int j = 0; j < 4; j++)
			for (int r = 0; r < 4; r++) {
				T acc = T((double)W.b[base + j][r]);
				for (int m = 0; m < 4; m++)
					for (int c = 0; c < 4; c++) acc = acc + in[m][c] * (double)W.M[base + j][m][4 * c + r];
				out[j][r] = sin(acc) / (double)W.div[base + j] + in[j][r];
			}
	};
	layer(f0, f1, 0);
	layer(f1, f2, 4);
	T d = T((double)W.out_b);
	for (int j = 0; j < 4; j++)
		for (int r = 0; r < 4; r++) d = d + f2[j][r] * (double)W.out_w[j][r];
	return d;
}

// ---------------------------------------------------------------------------
// the 34 shapes (sources/sdf.cpp), in name order
// ---------------------------------------------------------------------------
template<class T> T shape_eval(const Planet &P, const V3<T> &pos) {
	using V = V3<T>;
	switch (P.shape) {
		case 0: { // asteroid, sdf.cpp:333-353
			const T l = length(pos);
			if (val(l) < 1) return T(-100.0);
			const V d = pos / l;
			return l + noise_eval(P.noise[S_ASTEROID], d) * 600.0 - 1300.0;
		}
		case 1: // belt, :375-381
			if (val(pos.x) > 0) return prim_cylinder(V(pos.x, pos.z, pos.y), 10000, 1800) * -1.0;
			return 1800.0 - abs(pos.z);
		case 2: // bowl, :323-326
			return 2000.0 - length(pos - V(T(0.0), T(0.0), T(-3000.0)));
		case 3: return prim_box(pos, V3<double>(550, 1000, 550)) - 200.0;          // box, :40-43
		case 4: { // bunny, :293-297
			const double sc = 0.0005;
			return sinnet(kSinNet_bunny, V(pos.x, pos.z, pos.y) * sc) / sc;
		}
		case 5: return prim_capsule(V(pos.x, pos.z, pos.y), 2500, 600);            // capsule, :25-28
		case 6: return prim_box(pos, V3<double>(450, 450, 450)) - 100.0;          // cube, :45-48
		case 7: return prim_cylinder(pos, 200, 600) - 100.0;                      // disk, :35-38
		case 8: { // doubletorus, :305-312
			const V p1(pos.y, pos.z, pos.x), p2(pos.y, pos.x, pos.z);
			return smoothMin(prim_torus(p1, 900, 400), prim_torus(p2, 900, 400), T(200.0));
		}
		case 9: { // fibers, :122-139
			const double scale = 0.0007;
			const V p = pos * scale + V(T(P.fibers_offset[0]), T(P.fibers_offset[1]), T(P.fibers_offset[2]));
			const double gs = 3.23;
			const V q = p * gs;
			const T g = abs(sin(q.x) * cos(q.z) + sin(q.y) * cos(q.x) + sin(q.z) * cos(q.y) + 1.6) / gs - 0.2;
			const T v = g * 0.7 / scale;
			const T d = tmax(length(pos) - 1500.0, T(0.0)) * 0.5;
			return v + d;
		}
		case 10: { // gear, :180-204
			const double scale = 2;
			const V p3 = V(pos.x, pos.z, pos.y) / scale;
			const T px = p3.x, py = p3.z;
			const double angle = 2.0 * M_PI / 9.0;
			const double at = val(atan2(px, py)) / angle + 9 + 0.5;
			const uint32_t sector = (uint32_t)at % 9u;
			const double a = -(double)sector * angle;
			const double s = std::sin(a), c = std::cos(a);
			const T qx = px * c - py * s, qy = px * s + py * c;
			const T bx = tmax(abs(qx - 700.0) - 150.0, T(0.0)), by = tmax(abs(qy) - 70.0, T(0.0));
			const T b = len2(bx, by);
			const T cc = abs(len2(px, py) - 450.0) - 150.0;
			const T h = abs(p3.y) - 30.0;
			return (smoothMax(tmin(b, cc), h, T(50.0)) - 50.0) * scale;
		}
		case 11: { // h2o, :141-149
			const double sc = 0.75;
			const V p = pos * sc;
			const T h1 = prim_sphere(p - V(T(-550.0), T(300.0), T(0.0)), 450);
			const T h2 = prim_sphere(p - V(T(550.0), T(300.0), T(0.0)), 450);
			const T o = prim_sphere(p - V(T(0.0), T(-100.0), T(0.0)), 650);
			return smoothMin(o, tmin(h1, h2), T(150.0)) / sc;
		}
		case 12: { // h3o, :151-163
			const double sc = 0.75;
			const V p = pos * sc;
			T h = T(1e30);
			for (int i = 0; i < 3; i++) {
				const double a = i * 2.0 * M_PI / 3.0;
				const V c(T(680.0 * std::cos(a)), T(680.0 * std::sin(a)), T(0.0));
				h = tmin(h, prim_sphere(p - c, 450));
			}
			return smoothMin(prim_sphere(p, 650), h, T(150.0)) / sc;
		}
		case 13: { // h4o, :165-178
			const double sc = 0.75;
			const V p = pos * sc;
			const T a = prim_sphere(p - V(T(-550.0), T(400.0), T(0.0)), 450), b = prim_sphere(p - V(T(550.0), T(400.0), T(0.0)), 450);
			const T c = prim_sphere(p - V(T(0.0), T(-400.0), T(-550.0)), 450), d = prim_sphere(p - V(T(0.0), T(-400.0), T(550.0)), 450);
			return smoothMin(prim_sphere(p, 650), tmin(tmin(a, b), tmin(c, d)), T(150.0)) / sc;
		}
		case 14: { // hemispheres, :383-397
			const V p(abs(pos.x), abs(pos.y), pos.z);
			const double s = 0.707106781186547524400844362104;
			auto rot = [&](const V &q) { return V((q.x - q.y) * s, (q.x + q.y) * s, q.z); };
			const V q = rot(p + V(T(-2000.0), T(0.0), T(0.0)));
			const T c = prim_cylinder(V(q.y, q.z, q.x), 10000, 200);
			const T s1 = prim_sphere(q, 1000);
			const T s2 = prim_sphere(rot(p + V(T(0.0), T(-2000.0), T(0.0))), 1000);
			return smoothMin(c, tmin(s1, s2), T(100.0));
		}
		case 15: { // hexagon, :10-13
			const double k = 1.0 / std::sqrt(3.0);
			return prim_plane(pos, V(T(k), T(k), T(-k)));
		}
		case 16: return prim_hexprism(V(pos.x, pos.z, pos.y), 300, 400) - 100.0;  // hexagonalprism, :76-79
		case 17: return -(prim_box(pos, V3<double>(1300, 1300, 1300)) - 200.0);    // insidecube, :328-331
		case 18: { // knot, :86-90
			const V p(pos.x, pos.y, pos.z * 0.3);
			return prim_knot(p, 1600, 1.5) / std::sqrt(1.0 + 1.0 + 0.09);
		}
		case 19: { // mandelbulb, :206-232
			if (val(dot(pos, pos)) < 1e-3) return T(0.0);
			const V p = pos * 0.0004;
			V z = p;
			T dr = T(1.0), r = T(0.0);
			for (int i = 0; i < 20; i++) {
				r = length(z);
				if (val(r) > 4.0) break;
				T theta = acos(z.z / r);
				T phi = atan2(z.y, z.x);
				dr = pow(r, 2.0) * 3.0 * dr + 1.0;
				const T zr = pow(r, 3.0);
				theta = theta * 3.0;
				phi = phi * 3.0;
				z = V(sin(theta) * cos(phi), sin(phi) * sin(theta), cos(theta)) * zr;
				z = z + p;
			}
			const T value = 0.5 * log(r) * r / dr;
			return (value + 0.1) * 150.0;
		}
		case 20: { // mobiusstrip, :92-120
			const V pp(pos.x, pos.z, pos.y);
			const T planeRot = atan2(pp.x, pp.z);
			const T lxz = len2(pp.x, pp.z);
			const T projx = (pp.x * pp.x + pp.z * pp.z) / lxz - 1000.0; // dot((x,z), normalize(x,z)) + (-radius)
			const T projy = pp.y;
			T a = atan2(projx, projy) + planeRot * 0.5;
			const T l = len2(projx, projy);
			const T rx = abs(cos(a) * l) - 400.0, ry = abs(sin(a) * l) - 40.0;
			const T rect = len2(tmax(rx, T(0.0)), tmax(ry, T(0.0))) + tmin(tmax(rx, ry), T(0.0));
			return rect - 200.0;
		}
		case 21: { // monkeyhead, :299-303
			const double sc = 0.0005;
			return sinnet(kSinNet_monkey, V(pos.x, pos.z, pos.y) * sc) / sc;
		}
		case 22: return prim_octahedron(pos, 800) - 100.0;                        // octahedron, :55-58
		case 23: { // pipe, :355-366
			V p = pos;
			if (val(p.x) < 0) { p.x = -p.x; std::swap(p.y, p.z); }
			p.y = abs(p.y) - 800.0;
			std::swap(p.y, p.z);
			return prim_torus(p, 800, 400);
		}
		case 24: return prim_sphere(pos, 1100);                                   // sphere, :20-23
		case 25: return prim_plane(pos, V(T(0.0), T(0.0), T(-1.0)));              // square, :15-18
		case 26: return prim_tetrahedron(pos, 600) - 100.0;                       // tetrahedron, :50-53
		case 27: return prim_torus(pos, 950, 530);                                // torus, :81-84
		case 28: { // toruscross, :314-321
			const V p1(pos.y - 750.0, pos.z, pos.x), p2(pos.y + 750.0, pos.x, pos.z);
			return smoothMin(prim_torus(p1, 750, 400), prim_torus(p2, 750, 400), T(200.0));
		}
		case 29: { // triangularprism, :60-74
			V p(pos.x, pos.z, pos.y);
			p.z = tmax(abs(p.z) - 150.0, T(0.0));
			const double r = 900, c = std::cos(2.0 * M_PI / 3.0), s = std::sin(2.0 * M_PI / 3.0);
			const V3<double> A(0, r, 0), B(-s * r, c * r, 0), Cc(s * r, c * r, 0);
			return tri_distance(p, A, B, Cc) - 100.0;
		}
		case 30: return prim_cylinder(V(pos.x, pos.z, pos.y), 10000, 800);        // tube, :30-33
		case 31: { // twistedhexagonalprism, :234-241
			const T ang = pos.y * 0.001;
			const V r = rot_z(V(pos.x, pos.z, T(0.0)), ang);
			const V p(r.x, pos.y, r.y);
			return prim_hexprism(V(p.x, p.z, p.y), 900, 650) - 200.0;
		}
		case 32: { // twistedplane, :368-373
			const T rot = 1.0 - sqr(1.0 - tmin(T(1.0), abs(pos.z) / 1000.0));
			const T angle = tsign(pos.z) * rot * (35.0 * M_PI / 180.0);
			return pos.y * cos(angle) + pos.x * sin(angle);
		}
		default: { // wormhole, :399-404
			const T x = tmin(len2(pos.x, pos.z) - 1400.0, T(0.0));
			return 700.0 - len2(x, pos.y);
		}
	}
}

// ---------------------------------------------------------------------------
// elevation modes (sources/elevationModes.cpp)
// ---------------------------------------------------------------------------
template<class T> T mountains(const Planet &P, const V3<T> &pos, const T &land) { // :68-123
	const T cover = 1.0 - saturate(land * -0.1);
	if (val(cover) < 1e-7) return land;
	const T mask = noise_eval(P.noise[S_MTN_MASK], pos);
	const T rm = smoothstep(saturate(mask * 7.0 - 0.3));
	const T tm = smoothstep(saturate(mask * -7.0 - 1.5));
	T ridge = noise_eval(P.noise[S_MTN_RIDGE], pos);
	ridge = tmax(ridge - 0.1, T(0.0));
	ridge = pow(ridge, 1.6);
	ridge = ridge * rm * cover;
	ridge = ridge * 1000.0;
	T terraces = noise_eval(P.noise[S_MTN_TERRACE], pos);
	terraces = tmax(terraces + 0.1, T(0.0)) * 2.5;
	terraces = terrace(terraces, 4.0);
	terraces = terraces * tm * cover;
	terraces = terraces * 250.0;
	return land + smoothMax(T(0.0), tmax(ridge, terraces), T(50.0));
}
template<class T> T lakes_islands(const Planet &P, const V3<T> &pos, int slot, double ex) { // :129-171
	T land = noise_eval(P.noise[slot], pos) * 0.5 + 0.5;
	land = saturate(land);
	land = 1.0 - pow(land, ex);
	land = land * 2.0 - 1.0;
	land = land / (abs(land) + 0.17) + 0.15;
	land = land * 150.0;
	return mountains(P, pos, land);
}
template<class T> T elevation_eval(const Planet &P, const V3<T> &pos) {
	switch (P.elevation) {
		case 0: return T(100.0); // :9-12
		case 1: { // :14-32
			T a = noise_eval(P.noise[S_SIMPLE], pos);
			a = -a + 0.3;
			a = pow(a * 1.3 - 0.35, 3.0) + 0.1;
			return 100.0 - a * 1000.0;
		}
		case 2: { // :34-64
			const T scale = noise_eval(P.noise[S_LEGACY_SCALE], pos) * 0.0005 + 0.0015;
			T a = noise_eval(P.noise[S_LEGACY_ELEV], pos * scale);
			a = a + 0.11;
			if (val(a) < 0) a = -pow(-a, 0.85);
			else a = pow(a, 1.7);
			return a * 2500.0;
		}
		case 3: return lakes_islands(P, pos, S_LAKES_LAND, 1.24);
		case 4: return lakes_islands(P, pos, S_ISLANDS_LAND, 0.83);
		default: { // :173-198
			const V3<T> c = voronoi_nearest(P.craters, pos, (const V3<T> *)nullptr);
			const T s = 100.0 + noise_eval(P.noise[S_CRATERS_SCALE], c) * 50.0;
			const T d = length(pos - c);
			const T x = saturate(d / s);
			const T h = (pow(x, 4.0) - 0.9 * pow(x, 5.0) - 0.1) * 10.0;
			return 200.0 + h * 190.0;
		}
	}
}

// fields (modesConfiguration.cpp:230-279)
template<class T> T field_eval(const Planet &P, int field, const V3<T> &pos) {
	switch (field) {
		case 0: return shape_eval(P, pos) - elevation_eval(P, pos) / 10.0;                     // land
		case 1: return shape_eval(P, pos);                                                      // water
		case 2: return shape_eval(P, pos) - tmax(elevation_eval(P, pos) / 10.0, T(0.0));        // navigation
		case 3: return shape_eval(P, pos) * 10.0;                                               // elevation
		default: return elevation_eval(P, pos);                                                 // elevation raw
	}
}

} // namespace orc
