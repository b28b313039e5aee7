// Synthetic unit-scale planet programs (include/up_abi.h, up_synth_program):
// fused value + analytic gradient, and the per-point parameter adjoint.
//
// d(p) = base(p) - sum_layers sum_i amp_i s(n_i(freq_i p)), s = n or 1 - 2|n|
// The smooth union is the reference's polynomial smoothMin
// (sources/math.cpp:28-33); the composition "shape minus elevation" follows
// terrainSdfLand (sources/modesConfiguration.cpp:248-258) at unit scale.
#pragma once
#include "up_noise.cuh"
#include "../../include/up_abi.h"

namespace up {

// Layer noise spec for kernel specialisation: -1 = everything at run time;
// 0..4 = that noise type; cellular = 5 | (distance + 1) << 4 | (operation + 1) << 8
constexpr int cell_spec(int dist, int op) { return 5 | ((dist + 1) << 4) | ((op + 1) << 8); }

// COOP: the caller's 32 lanes call together (cellular_warp for a
// compile-time cellular layer; the same results)
template<bool GRAD, int TYPE, bool COOP = false>
UP_HD NG noise_t(const up_noise_layer &L, V3f q, uint32_t key) {
#ifdef __CUDA_ARCH__
	if (COOP && TYPE >= 0 && (TYPE & 15) == 5) return cellular_warp<GRAD, ((TYPE >> 4) & 15) - 1, ((TYPE >> 8) & 15) - 1>(q, key, L.distance, L.operation);
#endif
	if (TYPE >= 0 && (TYPE & 15) == 5) return cellular_n<GRAD, ((TYPE >> 4) & 15) - 1, ((TYPE >> 8) & 15) - 1>(q, key, L.distance, L.operation);
	const int t = TYPE >= 0 ? TYPE : L.type;
	if (TYPE == 2 || (TYPE < 0 && t == 2)) { if (GRAD) return perlin_g(q, key); return ngc(perlin_v(q, key)); }
	if (TYPE == 3 || (TYPE < 0 && t == 3)) return simplex_n<GRAD, false>(q, key);
	if (TYPE < 0 && t == 5) return cellular_n<GRAD>(q, key, L.distance, L.operation);
	return noise_single<GRAD>(t, q, key, L.distance, L.operation);
}

// Specialisations: the two benchmark programs get compile-time noise types;
// everything else dispatches on the layer type at run time.
enum Spec { SPEC_PERLIN_CELL = 0, SPEC_SIMPLEX = 1, SPEC_GENERIC = 2 };
constexpr int CELL_EU_SUB = cell_spec(UP_DIST_EUCLIDEAN, UP_OP_SUBTRACT);
inline Spec spec_of(const up_synth_program &P) {
	if (P.n_layers == 2 && P.layer[0].type == UP_NOISE_PERLIN && P.layer[1].type == UP_NOISE_CELLULAR &&
		P.layer[1].distance == UP_DIST_EUCLIDEAN && P.layer[1].operation == UP_OP_SUBTRACT)
		return SPEC_PERLIN_CELL;
	if (P.n_layers == 1 && P.layer[0].type == UP_NOISE_SIMPLEX) return SPEC_SIMPLEX;
	return SPEC_GENERIC;
}

// one layer: value and gradient with respect to p
template<bool GRAD, int TYPE, bool COOP = false>
UP_HD NG layer_eval(const up_noise_layer &L, V3f p) {
	float v = 0.f;
	V3f g = zero3();
	const bool ridged = L.fractal == UP_FRACTAL_RIDGED;
	#pragma unroll 1
	for (int i = 0; i < L.octaves; i++) {
		const float f = L.freq[i];
		const NG n = noise_t<GRAD, TYPE, COOP>(L, p * f, seed_key(L.seed + (uint32_t)i));
		float s = n.v, ds = 1.f;
		if (ridged) { s = 1.f - 2.f * fabsf(n.v); ds = n.v > 0.f ? -2.f : (n.v < 0.f ? 2.f : 0.f); }
		v += L.amp[i] * s;
		if (GRAD) g += n.g * (L.amp[i] * ds * f);
	}
	return ng(v, g);
}

// polynomial smooth minimum with partials (sources/math.cpp:28-33)
struct SMin { float s, da, db, dk; };
// ik = 1 / k, hoisted by the callers
UP_HD SMin smooth_min_d(float a, float b, float k, float ik) {
	const float u = (b - a) * ik * 0.5f + 0.5f;
	const float h = saturatef(u);
	SMin r;
	r.s = b + (a - b) * h - k * h * (1.f - h);
	const float S = (a - b) - k * (1.f - 2.f * h);
	const bool in = u > 0.f && u < 1.f;
	const float dha = in ? -0.5f * ik : 0.f;
	const float dhk = in ? -(b - a) * 0.5f * ik * ik : 0.f;
	r.da = h + S * dha;
	r.db = (1.f - h) - S * dha;
	r.dk = -h * (1.f - h) + S * dhk;
	return r;
}

// Lengths and their reciprocals through sqrt_hd and rsqrt_hd: the hardware
// approximations on the device (a few ulp), and on the host sqrtf and
// 1 / sqrtf, the correctly rounded forms the oracle's FP32 path takes.
// s = squared length; lengths of 1e-18 or less have no direction (0)
UP_HD float inv_len_hd(float s) { return s > 1e-36f ? rsqrt_hd(s) : 0.f; }
UP_HD NG torus_d(V3f p, float R, float r) {
	const float sa = p.x * p.x + p.y * p.y;
	const float a = sqrt_hd(sa);
	const float qx = a - R, qz = p.z;
	const float sq = qx * qx + qz * qz;
	const float ql = sqrt_hd(sq);
	const float ia = inv_len_hd(sa), iq = inv_len_hd(sq);
	return ng(ql - r, v3(qx * iq * p.x * ia, qx * iq * p.y * ia, qz * iq));
}
UP_HD NG sphere_d(V3f p, V3f c, float r) {
	const V3f d = p - c;
	const float s = dot(d, d);
	return ng(sqrt_hd(s) - r, d * inv_len_hd(s));
}
UP_HD NG box_d(V3f p, float h, float rr) {
	const V3f q = v3(fabsf(p.x) - h, fabsf(p.y) - h, fabsf(p.z) - h);
	const V3f m = v3(fmaxf(q.x, 0.f), fmaxf(q.y, 0.f), fmaxf(q.z, 0.f));
	const float ml = sqrt_hd(dot(m, m));
	const float mx = fmaxf(q.x, fmaxf(q.y, q.z));
	const V3f sg = v3(p.x >= 0.f ? 1.f : -1.f, p.y >= 0.f ? 1.f : -1.f, p.z >= 0.f ? 1.f : -1.f);
	V3f g;
	if (ml > 0.f) g = v3(sg.x * m.x, sg.y * m.y, sg.z * m.z) * inv_len_hd(dot(m, m));
	else if (q.x >= q.y && q.x >= q.z) g = v3(sg.x, 0.f, 0.f);
	else if (q.y >= q.z) g = v3(0.f, sg.y, 0.f);
	else g = v3(0.f, 0.f, sg.z);
	return ng(ml + fminf(mx, 0.f) - rr, g);
}

UP_HD int lowest_bit(uint32_t m) {
#ifdef __CUDA_ARCH__
	return __ffs(m) - 1;
#else
	return __builtin_ctz(m);
#endif
}

// spheres: bit s clear = sphere s is known to be skipped at p (the test
// below would skip it; synth_segment_spheres); the others are tested
// BASE >= 0: the base shape fixed at compile time (no per-sample switch);
// BASE < 0: dispatched on P.base at run time
template<bool GRAD, int BASE = -1>
UP_HD NG synth_base(const up_synth_program &P, V3f p, uint32_t spheres = 0xFFFFFFFFu) {
	const int base = BASE >= 0 ? BASE : P.base;
	switch (base) {		case UP_BASE_SPHERE: return sphere_d(p, zero3(), P.param[0]);
		case UP_BASE_TORUS: return torus_d(p, P.param[0], P.param[1]);
		case UP_BASE_ROUNDED_BOX: return box_d(p, P.param[0], P.param[1]);
		default: {
			NG b = torus_d(p, P.param[0], P.param[1]);
			const float ik = 1.f / P.k;
			// in increasing s, as the union is defined
			#pragma unroll 1
			for (uint32_t live = spheres & ((1u << P.n_spheres) - 1u); live != 0u; live &= live - 1u) {
				const int s = lowest_bit(live);
				const V3f c = v3(P.sphere[s][0], P.sphere[s][1], P.sphere[s][2]);
				// A sphere at distance l >= radius + b + k leaves the blend
				// weight saturated (h = 1): the smooth minimum returns b and
				// its gradient unchanged, so such spheres are skipped (the
				// margin keeps h exactly 1 under FP32 rounding).
				const V3f dc = p - c;
				const float lim = P.sphere[s][3] + b.v + P.k * 1.001f + 1e-6f;
				if (lim <= 0.f || dot(dc, dc) >= lim * lim) continue;
				const NG sd = sphere_d(p, c, P.sphere[s][3]);
				const SMin m = smooth_min_d(b.v, sd.v, P.k, ik);
				b = ng(m.s, b.g * m.da + sd.g * m.db);
			}
			return b;
		}
	}
}

// Spheres of a torus-spheres union that can change it somewhere on the
// segment of samples (x, y, z), x in [x0, x1]: every sphere whose bit is
// clear is skipped by synth_base's own test at every sample of the segment.
// That test skips sphere s at p when |p - c_s|^2 >= lim^2 (or lim <= 0),
// lim = r_s + b + 1.001 k + 1e-6, with b the union so far. b never exceeds
// the torus (the smooth minimum is below both arguments), and the torus is
// 1-Lipschitz, so b <= torus(midpoint) + half the segment; with that bound
// in lim and the segment's nearest point to c_s in |p - c_s|, the margins
// (relative 1e-5 on the bound, 1e-4 on the squares) cover FP32 rounding.
UP_HD uint32_t synth_segment_spheres(const up_synth_program &P, float x0, float x1, float y, float z) {
	if (P.base != UP_BASE_TORUS_SPHERES) return 0xFFFFFFFFu;
	const float xm = 0.5f * (x0 + x1), half = 0.5f * (x1 - x0);
	const float tm = torus_d(v3(xm, y, z), P.param[0], P.param[1]).v;
	const float bmax = tm + half + 1e-5f * (1.f + fabsf(tm) + fabsf(xm) + fabsf(y) + fabsf(z) + half);
	uint32_t live = 0u;
	#pragma unroll 1
	for (int s = 0; s < P.n_spheres; s++) {
		const float L = P.sphere[s][3] + bmax + P.k * 1.001f + 1e-6f;
		if (L <= 0.f) continue;
		const float cx = P.sphere[s][0];
		const float dx = fmaxf(fmaxf(x0 - cx, cx - x1), 0.f), dy = y - P.sphere[s][1], dz = z - P.sphere[s][2];
		const float d2 = dx * dx + dy * dy + dz * dz;
		if (d2 >= L * L * 1.0001f + 1e-9f) continue;
		live |= 1u << s;
	}
	return live;
}

// Upper bounds of |n| per noise type, from the definitions in up_noise.cuh:
//  value: a convex combination of lattice values in [-1, 1) -> 1;
//  cubic: 0.75 x (sum of |Catmull-Rom weights| <= 1 + t(1 - t) <= 1.25)^3;
//  Perlin, simplex, simplex-reduced: |g.d| <= max over axis pairs of
//    |d_a| + |d_b| for a 12-edge gradient g, so |n| <= M(p) = sum over the
//    corners of weight x that maximum; M's maximum over the cell (Perlin:
//    trilinear quintic weights, 1.037; simplex: 76 (0.5 - r^2)^4, 0.989;
//    reduced: 31 (0.5 - r^2)^3, 0.992, found on dense grids of the cell with
//    a Lipschitz margin, recomputed by tests/test_noise_bounds.py) is below
//    1.1 for all three;
//  cellular: F1 <= the distance to the own cell's point (|v_a| < 1) and
//    F2 <= the larger of that and the distance to a face neighbour's point
//    (|v_a| < 2 on one axis, < 1 on the others): Euclidean sqrt(3) / sqrt(6),
//    Manhattan 3 / 4, Hybrid 6 / 10; then the operation.
UP_HD float noise_abs_bound(int type, int dist, int op) {
	switch (type) {
		case UP_NOISE_VALUE: return 1.f;
		case UP_NOISE_CUBIC: return 0.75f * 1.953125f;
		case UP_NOISE_PERLIN: return 1.1f;
		case UP_NOISE_SIMPLEX: return 1.1f;
		case UP_NOISE_SIMPLEX_REDUCED: return 1.1f;
		default: {
			const float f1 = dist == UP_DIST_EUCLIDEAN ? 1.7320509f : (dist == UP_DIST_MANHATTAN ? 3.f : 6.f);
			const float f2 = dist == UP_DIST_EUCLIDEAN ? 2.4494898f : (dist == UP_DIST_MANHATTAN ? 4.f : 10.f);
			float m = 1.f;
			switch (op) {
				case UP_OP_DISTANCE: m = f1 - 1.f; break;
				case UP_OP_DISTANCE2: case UP_OP_SUBTRACT: m = f2 - 1.f; break;
				case UP_OP_ADD: m = 0.5f * (f1 + f2) - 1.f; break;
				case UP_OP_MULTIPLY: m = 0.5f * f1 * f2 - 1.f; break;
				default: m = 1.f; break; // cell value, F1 / F2 - 1
			}
			return m > 1.f ? m : 1.f;
		}
	}
}
// |sum of the layers| <= this everywhere; NaN when a parameter is not finite
UP_HD float synth_noise_bound(const up_synth_program &P) {
	float b = 0.f;
	for (int l = 0; l < P.n_layers; l++) {
		const up_noise_layer &L = P.layer[l];
		const float nm = noise_abs_bound(L.type, L.distance, L.operation);
		const float sm = L.fractal == UP_FRACTAL_RIDGED ? (2.f * nm - 1.f > 1.f ? 2.f * nm - 1.f : 1.f) : nm;
		for (int i = 0; i < L.octaves; i++) b += fabsf(L.amp[i]) * sm;
	}
	return b;
}

// full program; T0/T1 = compile-time noise type of layer 0/1 (-1 = runtime)
template<bool GRAD, int T0, int T1, bool COOP = false>
UP_HD NG synth_eval(const up_synth_program &P, V3f p) {
	NG d = synth_base<GRAD>(P, p);
	if (P.n_layers > 0) {
		const NG e = layer_eval<GRAD, T0, COOP>(P.layer[0], p);
		d.v -= e.v;
		if (GRAD) d.g -= e.g;
	}
	if (P.n_layers > 1) {
		const NG e = layer_eval<GRAD, T1, COOP>(P.layer[1], p);
		d.v -= e.v;
		if (GRAD) d.g -= e.g;
	}
	return d;
}

// ---------------------------------------------------------------- adjoint
// Fixed accumulator layout (compile-time register indices):
//   [0,8)  layer0 amp   [8,16)  layer0 freq
//   [16,24) layer1 amp  [24,32) layer1 freq
//   [32]   R or h, [33] r or rr, [34,42) sphere radii, [42] k
constexpr int ACC_N = 43;

template<int TYPE, int SLOT, bool COOP = false>
UP_HD void layer_bwd(const up_noise_layer &L, V3f p, float w, float acc[ACC_N]) {
	const bool ridged = L.fractal == UP_FRACTAL_RIDGED;
	#pragma unroll
	for (int i = 0; i < 8; i++) {
		if (i < L.octaves) {
			const float f = L.freq[i];
			const NG n = noise_t<true, TYPE, COOP>(L, p * f, seed_key(L.seed + (uint32_t)i));
			float s = n.v, ds = 1.f;
			if (ridged) { s = 1.f - 2.f * fabsf(n.v); ds = n.v > 0.f ? -2.f : (n.v < 0.f ? 2.f : 0.f); }
			acc[SLOT * 16 + i] -= w * s;
			acc[SLOT * 16 + 8 + i] -= w * L.amp[i] * ds * dot(n.g, p);
		}
	}
}

template<int T0, int T1, bool COOP = false>
UP_HD void synth_bwd(const up_synth_program &P, V3f p, float w, float acc[ACC_N]) {
	if (P.n_layers > 0) layer_bwd<T0, 0, COOP>(P.layer[0], p, w, acc);
	if (P.n_layers > 1) layer_bwd<T1, 1, COOP>(P.layer[1], p, w, acc);
	switch (P.base) {
		case UP_BASE_SPHERE: acc[32] -= w; break;
		case UP_BASE_TORUS: {
			const float a = sqrtf(p.x * p.x + p.y * p.y), qx = a - P.param[0];
			const float ql = sqrtf(qx * qx + p.z * p.z);
			acc[32] -= w * (ql > 0.f ? qx / ql : 0.f);
			acc[33] -= w;
			break;
		}
		case UP_BASE_ROUNDED_BOX: {
			const float h = P.param[0];
			const V3f q = v3(fabsf(p.x) - h, fabsf(p.y) - h, fabsf(p.z) - h);
			const V3f m = v3(fmaxf(q.x, 0.f), fmaxf(q.y, 0.f), fmaxf(q.z, 0.f));
			const float ml = length(m);
			acc[32] -= w * (ml > 0.f ? (m.x + m.y + m.z) / ml : 1.f);
			acc[33] -= w;
			break;
		}
		default: {
			// forward: keep every intermediate union value, then sweep back
			float bv[9];
			const float R = P.param[0];
			const float a = sqrtf(p.x * p.x + p.y * p.y), qx = a - R;
			const float ql = sqrtf(qx * qx + p.z * p.z);
			bv[0] = ql - P.param[1];
			float sdv[8];
			const float ik = 1.f / P.k;
			#pragma unroll
			for (int s = 0; s < 8; s++) {
				if (s < P.n_spheres) {
					const V3f d = p - v3(P.sphere[s][0], P.sphere[s][1], P.sphere[s][2]);
					sdv[s] = length(d) - P.sphere[s][3];
					bv[s + 1] = smooth_min_d(bv[s], sdv[s], P.k, ik).s;
				}
			}
			float gb = w; // dL/d(current union value)
			#pragma unroll
			for (int s = 7; s >= 0; s--) {
				if (s < P.n_spheres) {
					const SMin m = smooth_min_d(bv[s], sdv[s], P.k, ik);
					acc[34 + s] -= gb * m.db; // d sd / d radius = -1
					acc[42] += gb * m.dk;
					gb *= m.da;
				}
			}
			acc[32] -= gb * (ql > 0.f ? qx / ql : 0.f);
			acc[33] -= gb;
		}
	}
}

// compact theta index -> accumulator slot (host helper, same order as
// up_synth_theta_count's layout)
inline int theta_slots(const up_synth_program &P, int *slots) {
	int n = 0;
	for (int l = 0; l < P.n_layers; l++) {
		for (int i = 0; i < P.layer[l].octaves; i++) slots[n++] = l * 16 + i;
		for (int i = 0; i < P.layer[l].octaves; i++) slots[n++] = l * 16 + 8 + i;
	}
	switch (P.base) {
		case UP_BASE_SPHERE: slots[n++] = 32; break;
		case UP_BASE_TORUS: case UP_BASE_ROUNDED_BOX: slots[n++] = 32; slots[n++] = 33; break;
		default:
			slots[n++] = 32; slots[n++] = 33;
			for (int s = 0; s < P.n_spheres; s++) slots[n++] = 34 + s;
			slots[n++] = 42;
	}
	return n;
}

} // namespace up
