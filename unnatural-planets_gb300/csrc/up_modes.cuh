// Device evaluation of the reference modes: the 34 base shapes
// (sources/sdf.cpp), the 6 elevation modes (sources/elevationModes.cpp),
// Voronoi (sources/voronoi.cpp) and the SDF fields
// (sources/modesConfiguration.cpp:230-279).
//
// Every function is templated on the scalar S: float (values) or Df (value
// plus gradient with respect to the sample position, forward mode), so the
// analytic dd/dp of any shape/elevation pair comes from the same source.
// Noise inside Df code uses the analytic value+gradient noise of
// up_noise.cuh and the chain rule.
#pragma once
#include "up_noise.cuh"
#include "up_modes_desc.h"
#include "up_sinnet_data.h"

// out-of-line functions: compiled once per translation unit (and per scalar
// type) instead of being expanded at every call site
#define UP_HD_NOINLINE UP_HD_OUTLINE

namespace up {

// ---------------------------------------------------------------- forward-mode scalar
struct Df { float v; V3f d; };
UP_HD Df dconst(float v) { Df r; r.v = v; r.d = zero3(); return r; }
UP_HD Df operator+(Df a, Df b) { Df r; r.v = a.v + b.v; r.d = a.d + b.d; return r; }
UP_HD Df operator-(Df a, Df b) { Df r; r.v = a.v - b.v; r.d = a.d - b.d; return r; }
UP_HD Df operator*(Df a, Df b) { Df r; r.v = a.v * b.v; r.d = a.d * b.v + b.d * a.v; return r; }
UP_HD Df operator/(Df a, Df b) { Df r; r.v = a.v / b.v; r.d = (a.d * b.v - b.d * a.v) * (1.f / (b.v * b.v)); return r; }
UP_HD Df operator+(Df a, float b) { a.v += b; return a; }
UP_HD Df operator+(float b, Df a) { a.v += b; return a; }
UP_HD Df operator-(Df a, float b) { a.v -= b; return a; }
UP_HD Df operator-(float b, Df a) { Df r; r.v = b - a.v; r.d = -a.d; return r; }
UP_HD Df operator*(Df a, float b) { a.v *= b; a.d *= b; return a; }
UP_HD Df operator*(float b, Df a) { a.v *= b; a.d *= b; return a; }
UP_HD Df operator/(Df a, float b) { const float i = 1.f / b; a.v *= i; a.d *= i; return a; }
UP_HD Df operator/(float b, Df a) { Df r; r.v = b / a.v; r.d = a.d * (-b / (a.v * a.v)); return r; }
UP_HD Df operator-(Df a) { a.v = -a.v; a.d = -a.d; return a; }
UP_HD Df chainf(Df a, float v, float dv) { Df r; r.v = v; r.d = a.d * dv; return r; }

UP_HD float val(float x) { return x; }
UP_HD float val(Df x) { return x.v; }
UP_HD float sq_(float x) { return x * x; }
template<class S> UP_HD S mk(float v) { return S(v); }
template<> UP_HD Df mk<Df>(float v) { return dconst(v); }

UP_HD float s_sqrt(float x) { return sqrtf(x); }
UP_HD Df s_sqrt(Df a) { const float s = sqrtf(a.v); return chainf(a, s, s > 0.f ? 0.5f / s : 0.f); }
UP_HD float s_abs(float x) { return fabsf(x); }
UP_HD Df s_abs(Df a) { return chainf(a, fabsf(a.v), a.v > 0.f ? 1.f : (a.v < 0.f ? -1.f : 0.f)); }
UP_HD float s_sin(float x) { return sinf(x); }
UP_HD Df s_sin(Df a) { return chainf(a, sinf(a.v), cosf(a.v)); }
UP_HD float s_cos(float x) { return cosf(x); }
UP_HD Df s_cos(Df a) { return chainf(a, cosf(a.v), -sinf(a.v)); }
UP_HD float s_atan(float x) { return atanf(x); }
UP_HD Df s_atan(Df a) { return chainf(a, atanf(a.v), 1.f / (1.f + a.v * a.v)); }
UP_HD float s_acos(float x) { return acosf(x); }
UP_HD Df s_acos(Df a) { const float t = 1.f - a.v * a.v; return chainf(a, acosf(a.v), t > 0.f ? -1.f / sqrtf(t) : 0.f); }
UP_HD float s_log(float x) { return logf(x); }
UP_HD Df s_log(Df a) { return chainf(a, logf(a.v), 1.f / a.v); }
UP_HD float s_pow(float x, float p) { return powf(x, p); }
UP_HD Df s_pow(Df a, float p) { return chainf(a, powf(a.v, p), a.v != 0.f ? p * powf(a.v, p - 1.f) : 0.f); }
UP_HD float s_atan2(float y, float x) { return atan2f(y, x); }
UP_HD Df s_atan2(Df y, Df x) {
	Df r;
	r.v = atan2f(y.v, x.v);
	const float den = x.v * x.v + y.v * y.v;
	r.d = den > 0.f ? (y.d * x.v - x.d * y.v) * (1.f / den) : zero3();
	return r;
}
template<class S> UP_HD S s_min(S a, S b) { return val(b) < val(a) ? b : a; }
template<class S> UP_HD S s_max(S a, S b) { return val(b) > val(a) ? b : a; }
template<class S> UP_HD S s_clamp(S x, float lo, float hi) { return s_min(s_max(x, mk<S>(lo)), mk<S>(hi)); }
template<class S> UP_HD S s_sat(S x) { return s_clamp(x, 0.f, 1.f); }
template<class S> UP_HD S s_sign(S x) { return mk<S>(val(x) > 0.f ? 1.f : (val(x) < 0.f ? -1.f : 0.f)); }
template<class S> UP_HD S s_floor(S x) { return mk<S>(floorf(val(x))); }
template<class S> UP_HD S s_lerp(S a, S b, S f) { return a + (b - a) * f; }
template<class S> UP_HD S s_smoothstep(S x) { return x * x * (3.f - 2.f * x); }
template<class S> UP_HD S s_smootherstep(S x) { return x * x * x * (x * (x * 6.f - 15.f) + 10.f); }

template<class S> struct V3S { S x, y, z; };
template<class S> UP_HD V3S<S> vs(S x, S y, S z) { V3S<S> r; r.x = x; r.y = y; r.z = z; return r; }
template<class S> UP_HD V3S<S> operator+(V3S<S> a, V3S<S> b) { return vs(a.x + b.x, a.y + b.y, a.z + b.z); }
template<class S> UP_HD V3S<S> operator-(V3S<S> a, V3S<S> b) { return vs(a.x - b.x, a.y - b.y, a.z - b.z); }
template<class S> UP_HD V3S<S> operator*(V3S<S> a, float s) { return vs(a.x * s, a.y * s, a.z * s); }
UP_HD V3S<Df> operator*(V3S<Df> a, Df s) { return vs(a.x * s, a.y * s, a.z * s); }
template<class S> UP_HD V3S<S> vsc(float x, float y, float z) { return vs(mk<S>(x), mk<S>(y), mk<S>(z)); }
template<class S> UP_HD S s_dot(V3S<S> a, V3S<S> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template<class S> UP_HD S s_len(V3S<S> a) { return s_sqrt(s_dot(a, a)); }
template<class S> UP_HD S s_len2(S a, S b) { return s_sqrt(a * a + b * b); }
template<class S> UP_HD V3S<S> s_vabs(V3S<S> a) { return vs(s_abs(a.x), s_abs(a.y), s_abs(a.z)); }
UP_HD V3f vval(V3S<float> p) { return v3(p.x, p.y, p.z); }
UP_HD V3f vval(V3S<Df> p) { return v3(p.x.v, p.y.v, p.z.v); }

// polynomial smooth minimum, sources/math.cpp:28-38
template<class S> UP_HD S s_smin(S a, S b, float k) {
	const S h = s_sat((b - a) * (0.5f / k) + 0.5f);
	return b + (a - b) * h - k * h * (1.f - h);
}
template<class S> UP_HD S s_smax(S a, S b, float k) { return -s_smin(-a, -b, k); }
// sources/math.cpp:8-26
template<class S> UP_HD S s_rescale(S v, float ia, float ib, float oa, float ob) { return (v - ia) / (ib - ia) * (ob - oa) + oa; }
template<class S> UP_HD S s_sharp(S v, float p = 0.05f) { return s_rescale(s_clamp(v, 0.5f - p, 0.5f + p), 0.5f - p, 0.5f + p, 0.f, 1.f); }
template<class S> UP_HD S s_terrace(S x, float steep) {
	const S f = s_floor(x);
	const S t = s_smootherstep(s_sat((x - f) * fmaxf(steep, 1.f))) + f;
	return s_lerp(x, t, mk<S>(fminf(fmaxf(steep, 0.f), 1.f)));
}

// ---------------------------------------------------------------- noise on S
// a configured noise function (NoiseDev) at point p
UP_HD_NOINLINE float noise_dev(const NoiseDev &n, V3S<float> p) {
	float acc = 0.f;
	for (int i = 0; i < n.octaves; i++) {
		const float f = n.freq[i];
		float v = noise_single<false>(n.type, v3(p.x * f, p.y * f, p.z * f), seed_key(n.seed + (uint32_t)i), n.dist, n.op).v;
		if (n.fractal == 2) v = 1.f - 2.f * fabsf(v);
		acc += v * n.amp[i];
	}
	return acc;
}
UP_HD_NOINLINE Df noise_dev(const NoiseDev &n, V3S<Df> p) {
	float acc = 0.f;
	V3f g = zero3(); // gradient with respect to the argument
	for (int i = 0; i < n.octaves; i++) {
		const float f = n.freq[i];
		const NG r = noise_single<true>(n.type, v3(p.x.v * f, p.y.v * f, p.z.v * f), seed_key(n.seed + (uint32_t)i), n.dist, n.op);
		float v = r.v, dv = 1.f;
		if (n.fractal == 2) { v = 1.f - 2.f * fabsf(r.v); dv = r.v > 0.f ? -2.f : (r.v < 0.f ? 2.f : 0.f); }
		acc += v * n.amp[i];
		g += r.g * (dv * n.amp[i] * f);
	}
	Df o;
	o.v = acc;
	o.d = p.x.d * g.x + p.y.d * g.y + p.z.d * g.z;
	return o;
}

// ---------------------------------------------------------------- primitives (axis z)
template<class S> UP_HD S p_sphere(V3S<S> p, float r) { return s_len(p) - r; }
template<class S> UP_HD S p_capsule(V3S<S> p, float h, float r) { p.z = p.z - s_clamp(p.z, -0.5f * h, 0.5f * h); return s_len(p) - r; }
template<class S> UP_HD S p_cylinder(V3S<S> p, float h, float r) {
	const S dx = s_len2(p.x, p.y) - r, dy = s_abs(p.z) - 0.5f * h;
	return s_min(s_max(dx, dy), mk<S>(0.f)) + s_len2(s_max(dx, mk<S>(0.f)), s_max(dy, mk<S>(0.f)));
}
template<class S> UP_HD S p_box(V3S<S> p, float hx, float hy, float hz) {
	const S qx = s_abs(p.x) - hx, qy = s_abs(p.y) - hy, qz = s_abs(p.z) - hz;
	const S z = mk<S>(0.f);
	return s_len(vs(s_max(qx, z), s_max(qy, z), s_max(qz, z))) + s_min(s_max(qx, s_max(qy, qz)), z);
}
template<class S> UP_HD S p_tetra(V3S<S> p, float r) { return (s_max(s_abs(p.x + p.y) - p.z, s_abs(p.x - p.y) + p.z) - r) * 0.57735026918962576f; }
template<class S> UP_HD S p_octa(V3S<S> p, float r) { return (s_abs(p.x) + s_abs(p.y) + s_abs(p.z) - r) * 0.57735026918962576f; }
template<class S> UP_HD S p_hexprism(V3S<S> p, float h, float r) {
	const float kx = -0.86602540378443865f, ky = 0.5f, kz = 0.57735026918962576f;
	p = s_vabs(p);
	const S t = 2.f * s_min(kx * p.x + ky * p.y, mk<S>(0.f));
	p.x = p.x - t * kx;
	p.y = p.y - t * ky;
	const S cx = s_clamp(p.x, -kz * r, kz * r);
	const S ey = p.y - r;
	const S dx = s_len2(p.x - cx, ey) * s_sign(ey), dy = p.z - 0.5f * h;
	return s_min(s_max(dx, dy), mk<S>(0.f)) + s_len2(s_max(dx, mk<S>(0.f)), s_max(dy, mk<S>(0.f)));
}
template<class S> UP_HD S p_torus(V3S<S> p, float R, float r) { return s_len2(s_len2(p.x, p.y) - R, p.z) - r; }
// torus knot: radius size/2 around z, two discs (offset 0.35R, radius 0.15R)
// of the cross-section rotated by twist * azimuth
template<class S> UP_HD S p_knot(V3S<S> p, float size, float twist) {
	const float R = 0.5f * size;
	const S r = s_len2(p.x, p.y);
	const S ang = s_atan2(p.y, p.x) * twist;
	const S c = s_cos(ang), s = s_sin(ang);
	const S u0 = r - R, v0 = p.z;
	const S u = c * u0 - s * v0, v = s * u0 + c * v0;
	return s_len2(s_abs(u) - 0.35f * R, v) - 0.15f * R;
}
// point-triangle distance (C. Ericson, Real-Time Collision Detection 5.1.5), triangle in the z = 0 plane
template<class S> UP_HD S p_tri(V3S<S> p, V3f A, V3f B, V3f C) {
	const V3S<S> a = vsc<S>(A.x, A.y, A.z), b = vsc<S>(B.x, B.y, B.z), c = vsc<S>(C.x, C.y, C.z);
	const V3S<S> ab = b - a, ac = c - a, ap = p - a;
	const S d1 = s_dot(ab, ap), d2 = s_dot(ac, ap);
	if (val(d1) <= 0.f && val(d2) <= 0.f) return s_len(p - a);
	const V3S<S> bp = p - b;
	const S d3 = s_dot(ab, bp), d4 = s_dot(ac, bp);
	if (val(d3) >= 0.f && val(d4) <= val(d3)) return s_len(p - b);
	const S vc = d1 * d4 - d3 * d2;
	if (val(vc) <= 0.f && val(d1) >= 0.f && val(d3) <= 0.f) return s_len(p - (a + ab * (d1 / (d1 - d3))));
	const V3S<S> cp = p - c;
	const S d5 = s_dot(ab, cp), d6 = s_dot(ac, cp);
	if (val(d6) >= 0.f && val(d5) <= val(d6)) return s_len(p - c);
	const S vb = d5 * d2 - d1 * d6;
	if (val(vb) <= 0.f && val(d2) >= 0.f && val(d6) <= 0.f) return s_len(p - (a + ac * (d2 / (d2 - d6))));
	const S va = d3 * d6 - d5 * d4;
	if (val(va) <= 0.f && val(d4 - d3) >= 0.f && val(d5 - d6) >= 0.f) return s_len(p - (b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)))));
	const S den = 1.f / (va + vb + vc);
	return s_len(p - (a + ab * (vb * den) + ac * (vc * den)));
}

// ---------------------------------------------------------------- Voronoi (voronoi.cpp:10-91)
UP_HD void vor_mix(const VoronoiDev &v, const int32_t s[3], int32_t o[3]) {
	const uint32_t a[3] = {(uint32_t)s[1], (uint32_t)s[2], (uint32_t)s[0]};
	#pragma unroll
	for (int i = 0; i < 3; i++) o[i] = (int32_t)((uint32_t)v.seed_hash[i] + (uint32_t)s[i] + a[i] + mix32((uint32_t)s[i]));
}
// nearest generated point (points[0]); normal (optional) projects onto the tangent plane at pos
template<class S> UP_HD_NOINLINE V3S<S> voronoi_nearest(const VoronoiDev &v, V3S<S> pos, const V3f *normal) {
	const V3f pf = vval(pos);
	const int32_t cell[3] = {(int32_t)(pf.x * v.frequency), (int32_t)(pf.y * v.frequency), (int32_t)(pf.z * v.frequency)};
	float bestd = 3.4e38f;
	V3f best = zero3();
	for (int z = -1; z < 2; z++)
		for (int y = -1; y < 2; y++)
			for (int x = -1; x < 2; x++) {
				const int32_t c[3] = {cell[0] + x, cell[1] + y, cell[2] + z};
				int32_t s[3];
				vor_mix(v, c, s);
				for (int i = 0; i < v.points_per_cell; i++) {
					int32_t s2[3];
					vor_mix(v, s, s2);
					s[0] = s2[0]; s[1] = s2[1]; s[2] = s2[2];
					V3f q = v3(((float)(s[0] % 65536) / 65535.0f + (float)c[0]) * v.cell_size,
						((float)(s[1] % 65536) / 65535.0f + (float)c[1]) * v.cell_size,
						((float)(s[2] % 65536) / 65535.0f + (float)c[2]) * v.cell_size);
					if (normal) q -= (*normal) * dot(*normal, q - pf);
					const V3f d = q - pf;
					const float dd = dot(d, d);
					if (dd < bestd) { bestd = dd; best = q; }
				}
			}
	return vsc<S>(best.x, best.y, best.z); // the nearest point is piecewise constant in pos
}

// ---------------------------------------------------------------- shapes
template<class S> UP_HD S sinnet_eval(const SinNetWeights &W, V3S<S> p) {
	if (val(s_len(p)) > 1.f) return s_len(p) - 0.8f;
	S f0[16], f1[16]; // [4 * j + r]
	#pragma unroll 1
	for (int q = 0; q < 16; q++) {
		const int j = q >> 2, r = q & 3;
		f0[q] = s_sin(p.y * W.in_y[j][r] + p.z * W.in_z[j][r] + p.x * (W.x_sign * W.in_x[j][r]) + W.in_b[j][r]);
	}
	#pragma unroll 1
	for (int L = 0; L < 2; L++) {
		#pragma unroll 1
		for (int q = 0; q < 16; q++) {
			const int j = q >> 2, r = q & 3;
			S acc = mk<S>(W.b[4 * L + j][r]);
			#pragma unroll 1
			for (int m = 0; m < 16; m++) acc = acc + f0[m] * W.M[4 * L + j][m >> 2][4 * (m & 3) + r];
			f1[q] = s_sin(acc) / W.div[4 * L + j] + f0[q];
		}
		#pragma unroll 1
		for (int q = 0; q < 16; q++) f0[q] = f1[q];
	}
	S d = mk<S>(W.out_b);
	#pragma unroll 1
	for (int q = 0; q < 16; q++) d = d + f0[q] * W.out_w[q >> 2][q & 3];
	return d;
}

template<class S> UP_HD S mandelbulb_eval(V3S<S> pos) {
	if (val(s_dot(pos, pos)) < 1e-3f) return mk<S>(0.f);
	const V3S<S> p = pos * 0.0004f;
	V3S<S> z = p;
	S dr = mk<S>(1.f), r = mk<S>(0.f);
	for (int i = 0; i < 20; i++) {
		r = s_len(z);
		if (val(r) > 4.f) break;
		S theta = s_acos(z.z / r);
		S phi = s_atan2(z.y, z.x);
		dr = s_pow(r, 2.f) * 3.f * dr + 1.f;
		const S zr = s_pow(r, 3.f);
		theta = theta * 3.f;
		phi = phi * 3.f;
		z = vs(s_sin(theta) * s_cos(phi), s_sin(phi) * s_sin(theta), s_cos(theta)) * zr;
		z = z + p;
	}
	return (0.5f * s_log(r) * r / dr + 0.1f) * 150.f;
}

// out of line: compiled once per scalar type, shared by every kernel
template<class S> UP_HD_NOINLINE S shape_eval(const ModesDesc &M, V3S<S> pos) {
	const S zero = mk<S>(0.f);
	switch (M.shape) {
		case 0: { // asteroid, sdf.cpp:333-353
			const S l = s_len(pos);
			if (val(l) < 1.f) return mk<S>(-100.f);
			const S il = 1.f / l;
			return l + noise_dev(M.elev[NS_ASTEROID], pos * il) * 600.f - 1300.f;
		}
		case 1: // belt, :375-381
			if (val(pos.x) > 0.f) return p_cylinder(vs(pos.x, pos.z, pos.y), 10000.f, 1800.f) * -1.f;
			return 1800.f - s_abs(pos.z);
		case 2: return 2000.f - s_len(vs(pos.x, pos.y, pos.z + 3000.f));                 // bowl, :323-326
		case 3: return p_box(pos, 550.f, 1000.f, 550.f) - 200.f;                          // box, :40-43
		case 4: return sinnet_eval(kSinNet_bunny, vs(pos.x, pos.z, pos.y) * 0.0005f) / 0.0005f; // bunny, :293-297
		case 5: return p_capsule(vs(pos.x, pos.z, pos.y), 2500.f, 600.f);                 // capsule, :25-28
		case 6: return p_box(pos, 450.f, 450.f, 450.f) - 100.f;                           // cube, :45-48
		case 7: return p_cylinder(pos, 200.f, 600.f) - 100.f;                             // disk, :35-38
		case 8: return s_smin(p_torus(vs(pos.y, pos.z, pos.x), 900.f, 400.f), p_torus(vs(pos.y, pos.x, pos.z), 900.f, 400.f), 200.f); // doubletorus :305-312
		case 9: { // fibers, :122-139
			const float sc = 0.0007f, gs = 3.23f;
			const V3S<S> q = vs(pos.x * sc + M.fibers_offset[0], pos.y * sc + M.fibers_offset[1], pos.z * sc + M.fibers_offset[2]) * gs;
			const S g = s_abs(s_sin(q.x) * s_cos(q.z) + s_sin(q.y) * s_cos(q.x) + s_sin(q.z) * s_cos(q.y) + 1.6f) / gs - 0.2f;
			return g * 0.7f / sc + s_max(s_len(pos) - 1500.f, zero) * 0.5f;
		}
		case 10: { // gear, :180-204
			const float scale = 2.f;
			const V3S<S> p3 = vs(pos.x, pos.z, pos.y) * (1.f / scale);
			const S px = p3.x, py = p3.z;
			const float angle = 6.28318530717958647f / 9.f;
			const uint32_t sector = (uint32_t)(atan2f(val(px), val(py)) / angle + 9.f + 0.5f) % 9u;
			float sa, ca;
			sincosf(-(float)sector * angle, &sa, &ca);
			const S qx = px * ca - py * sa, qy = px * sa + py * ca;
			const S b = s_len2(s_max(s_abs(qx - 700.f) - 150.f, zero), s_max(s_abs(qy) - 70.f, zero));
			const S c = s_abs(s_len2(px, py) - 450.f) - 150.f;
			const S h = s_abs(p3.y) - 30.f;
			return (s_smax(s_min(b, c), h, 50.f) - 50.f) * scale;
		}
		case 11: { // h2o, :141-149
			const V3S<S> p = pos * 0.75f;
			const S h1 = p_sphere(p - vsc<S>(-550.f, 300.f, 0.f), 450.f), h2 = p_sphere(p - vsc<S>(550.f, 300.f, 0.f), 450.f);
			return s_smin(p_sphere(p - vsc<S>(0.f, -100.f, 0.f), 650.f), s_min(h1, h2), 150.f) / 0.75f;
		}
		case 12: { // h3o, :151-163
			const V3S<S> p = pos * 0.75f;
			S h = mk<S>(3.4e38f);
			for (int i = 0; i < 3; i++) {
				float sa, ca;
				sincosf((float)i * 2.0943951023931955f, &sa, &ca);
				h = s_min(h, p_sphere(p - vsc<S>(680.f * ca, 680.f * sa, 0.f), 450.f));
			}
			return s_smin(p_sphere(p, 650.f), h, 150.f) / 0.75f;
		}
		case 13: { // h4o, :165-178
			const V3S<S> p = pos * 0.75f;
			const S a = p_sphere(p - vsc<S>(-550.f, 400.f, 0.f), 450.f), b = p_sphere(p - vsc<S>(550.f, 400.f, 0.f), 450.f);
			const S c = p_sphere(p - vsc<S>(0.f, -400.f, -550.f), 450.f), d = p_sphere(p - vsc<S>(0.f, -400.f, 550.f), 450.f);
			return s_smin(p_sphere(p, 650.f), s_min(s_min(a, b), s_min(c, d)), 150.f) / 0.75f;
		}
		case 14: { // hemispheres, :383-397
			const V3S<S> p = vs(s_abs(pos.x), s_abs(pos.y), pos.z);
			const float s = 0.707106781186547524f;
			const V3S<S> a = p + vsc<S>(-2000.f, 0.f, 0.f), b2 = p + vsc<S>(0.f, -2000.f, 0.f);
			const V3S<S> q = vs((a.x - a.y) * s, (a.x + a.y) * s, a.z);
			const V3S<S> r = vs((b2.x - b2.y) * s, (b2.x + b2.y) * s, b2.z);
			return s_smin(p_cylinder(vs(q.y, q.z, q.x), 10000.f, 200.f), s_min(p_sphere(q, 1000.f), p_sphere(r, 1000.f)), 100.f);
		}
		case 15: { const float k = 0.57735026918962576f; return pos.x * k + pos.y * k - pos.z * k; } // hexagon, :10-13
		case 16: return p_hexprism(vs(pos.x, pos.z, pos.y), 300.f, 400.f) - 100.f;        // hexagonalprism, :76-79
		case 17: return -(p_box(pos, 1300.f, 1300.f, 1300.f) - 200.f);                   // insidecube, :328-331
		case 18: return p_knot(vs(pos.x, pos.y, pos.z * 0.3f), 1600.f, 1.5f) * 0.69171446f; // knot, :86-90 (1/|(1,1,0.3)|)
		case 19: return mandelbulb_eval(pos);                                             // mandelbulb, :206-232
		case 20: { // mobiusstrip, :92-120
			const V3S<S> pp = vs(pos.x, pos.z, pos.y);
			const S rot = s_atan2(pp.x, pp.z) * 0.5f;
			const S lxz = s_len2(pp.x, pp.z);
			const S px = (pp.x * pp.x + pp.z * pp.z) / lxz - 1000.f, py = pp.y;
			const S a = s_atan2(px, py) + rot;
			const S l = s_len2(px, py);
			const S rx = s_abs(s_cos(a) * l) - 400.f, ry = s_abs(s_sin(a) * l) - 40.f;
			return s_len2(s_max(rx, zero), s_max(ry, zero)) + s_min(s_max(rx, ry), zero) - 200.f;
		}
		case 21: return sinnet_eval(kSinNet_monkey, vs(pos.x, pos.z, pos.y) * 0.0005f) / 0.0005f; // monkeyhead, :299-303
		case 22: return p_octa(pos, 800.f) - 100.f;                                       // octahedron, :55-58
		case 23: { // pipe, :355-366
			V3S<S> p = pos;
			if (val(p.x) < 0.f) { p.x = -p.x; const S t = p.y; p.y = p.z; p.z = t; }
			p.y = s_abs(p.y) - 800.f;
			const S t = p.y; p.y = p.z; p.z = t;
			return p_torus(p, 800.f, 400.f);
		}
		case 24: return p_sphere(pos, 1100.f);                                            // sphere, :20-23
		case 25: return -pos.z;                                                           // square, :15-18
		case 26: return p_tetra(pos, 600.f) - 100.f;                                      // tetrahedron, :50-53
		case 27: return p_torus(pos, 950.f, 530.f);                                       // torus, :81-84
		case 28: return s_smin(p_torus(vs(pos.y - 750.f, pos.z, pos.x), 750.f, 400.f), p_torus(vs(pos.y + 750.f, pos.x, pos.z), 750.f, 400.f), 200.f); // toruscross :314-321
		case 29: { // triangularprism, :60-74
			V3S<S> p = vs(pos.x, pos.z, pos.y);
			p.z = s_max(s_abs(p.z) - 150.f, zero);
			const float r = 900.f, c = -0.5f, s = 0.86602540378443865f;
			return p_tri(p, v3(0.f, r, 0.f), v3(-s * r, c * r, 0.f), v3(s * r, c * r, 0.f)) - 100.f;
		}
		case 30: return p_cylinder(vs(pos.x, pos.z, pos.y), 10000.f, 800.f);              // tube, :30-33
		case 31: { // twistedhexagonalprism, :234-241
			const S ang = pos.y * 0.001f;
			const S c = s_cos(ang), s = s_sin(ang);
			const S rx = c * pos.x - s * pos.z, ry = s * pos.x + c * pos.z;
			return p_hexprism(vs(rx, ry, pos.y), 900.f, 650.f) - 200.f;
		}
		case 32: { // twistedplane, :368-373
			const S rot = 1.f - s_min(mk<S>(1.f), s_abs(pos.z) * 0.001f);
			const S angle = s_sign(pos.z) * (1.f - rot * rot) * 0.610865238198015f;
			return pos.y * s_cos(angle) + pos.x * s_sin(angle);
		}
		default: { // wormhole, :399-404
			const S x = s_min(s_len2(pos.x, pos.z) - 1400.f, zero);
			return 700.f - s_len2(x, pos.y);
		}
	}
}

// ---------------------------------------------------------------- elevation modes
// The elevation noise instances are read through a source NZ: nz(M, slot, pos)
// returns noise_dev(M.elev[slot], pos) (NoiseDirect), or the same quantity
// taken from a table that a grid kernel filled for a run of samples along x.
struct NoiseDirect {
	template<class S> UP_HD S operator()(const ModesDesc &M, int slot, V3S<S> pos) const { return noise_dev(M.elev[slot], pos); }
};
template<class S, class NZ> UP_HD S mountains(const ModesDesc &M, V3S<S> pos, S land, const NZ &nz) { // elevationModes.cpp:68-123
	const S cover = 1.f - s_sat(land * -0.1f);
	if (val(cover) < 1e-7f) return land;
	const S mask = nz(M, NS_MTN_MASK, pos);
	const S rm = s_smoothstep(s_sat(mask * 7.f - 0.3f));
	const S tm = s_smoothstep(s_sat(mask * -7.f - 1.5f));
	S ridge = nz(M, NS_MTN_RIDGE, pos);
	ridge = s_max(ridge - 0.1f, mk<S>(0.f));
	ridge = s_pow(ridge, 1.6f) * rm * cover * 1000.f;
	S terraces = s_max(nz(M, NS_MTN_TERRACE, pos) + 0.1f, mk<S>(0.f)) * 2.5f;
	terraces = s_terrace(terraces, 4.f) * tm * cover * 250.f;
	return land + s_smax(mk<S>(0.f), s_max(ridge, terraces), 50.f);
}
// EM >= 0: the elevation mode is known at compile time (M.elevation == EM)
template<class S, class NZ, int EM = -1> UP_HD S elevation_nz(const ModesDesc &M, V3S<S> pos, const NZ &nz) {
	const int em = EM >= 0 ? EM : M.elevation;
	switch (em) {
		case 0: return mk<S>(100.f); // :9-12
		case 1: { // :14-32
			S a = -nz(M, NS_SIMPLE, pos) + 0.3f;
			a = s_pow(a * 1.3f - 0.35f, 3.f) + 0.1f;
			return 100.f - a * 1000.f;
		}
		case 2: { // :34-64
			const S scale = nz(M, NS_LEGACY_SCALE, pos) * 0.0005f + 0.0015f;
			S a = noise_dev(M.elev[NS_LEGACY_ELEV], pos * scale) + 0.11f;
			if (val(a) < 0.f) a = -s_pow(-a, 0.85f);
			else a = s_pow(a, 1.7f);
			return a * 2500.f;
		}
		case 3: case 4: { // lakes :129-149, islands :151-171
			S land = s_sat(nz(M, em == 3 ? NS_LAKES_LAND : NS_ISLANDS_LAND, pos) * 0.5f + 0.5f);
			land = 1.f - s_pow(land, em == 3 ? 1.24f : 0.83f);
			land = land * 2.f - 1.f;
			land = (land / (s_abs(land) + 0.17f) + 0.15f) * 150.f;
			return mountains(M, pos, land, nz);
		}
		default: { // craters :173-198
			const V3S<S> c = voronoi_nearest(M.craters, pos, (const V3f *)nullptr);
			const S s = 100.f + noise_dev(M.elev[NS_CRATERS_SCALE], c) * 50.f;
			const S x = s_sat(s_len(pos - c) / s);
			const S h = (s_pow(x, 4.f) - 0.9f * s_pow(x, 5.f) - 0.1f) * 10.f;
			return 200.f + h * 190.f;
		}
	}
}
template<class S> UP_HD_NOINLINE S elevation_eval(const ModesDesc &M, V3S<S> pos) { return elevation_nz(M, pos, NoiseDirect{}); }

// the five fields (modesConfiguration.cpp:230-279)
template<class S> UP_HD S field_eval(const ModesDesc &M, int field, V3S<S> p) {
	switch (field) {
		case 0: return shape_eval(M, p) - elevation_eval(M, p) * 0.1f;
		case 1: return shape_eval(M, p);
		case 2: return shape_eval(M, p) - s_max(elevation_eval(M, p) * 0.1f, mk<S>(0.f));
		case 3: return shape_eval(M, p) * 10.f;
		default: return elevation_eval(M, p);
	}
}
UP_HD V3S<Df> dual_point(V3f p) { return vs(Df{p.x, v3(1.f, 0.f, 0.f)}, Df{p.y, v3(0.f, 1.f, 0.f)}, Df{p.z, v3(0.f, 0.f, 1.f)}); }

} // namespace up
