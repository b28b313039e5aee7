// Oracle: per-texel coloring (sources/coloringModes.cpp), colour helpers
// (sources/math.cpp:40-57 plus the cage colour conversions), the synthetic
// texel program, UV rasterisation, dilation and 8-bit quantisation
// (sources/textures.cpp:24-82). TEST INFRASTRUCTURE, parity unpinned (see
// oracle_core.hpp). Evaluated in FP64 (T = double) or FP32 (T = F32).
#pragma once
#include "oracle_modes.hpp"
#include "oracle_synth.hpp"
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------
// colour conversions (published formulas; components in [0,1], hue in [0,1))
// ---------------------------------------------------------------------------
// RGB <-> HSV: A. R. Smith, "Color gamut transform pairs" (1978)
template<class T> V3<T> rgb_to_hsv(const V3<T> &c) {
	const T mx = tmax(c.x, tmax(c.y, c.z)), mn = tmin(c.x, tmin(c.y, c.z));
	const T d = mx - mn;
	T h = T(0.0);
	if (val(d) > 0) {
		if (val(mx) == val(c.x)) h = (c.y - c.z) / d;
		else if (val(mx) == val(c.y)) h = (c.z - c.x) / d + 2.0;
		else h = (c.x - c.y) / d + 4.0;
		h = h / 6.0;
		if (val(h) < 0) h = h + 1.0;
	}
	const T s = val(mx) > 0 ? d / mx : T(0.0);
	return V3<T>(h, s, mx);
}
template<class T> V3<T> hsv_to_rgb(const V3<T> &hsv) {
	const T h6 = (hsv.x - floor(hsv.x)) * 6.0;
	const T s = hsv.y, v = hsv.z;
	const int i = std::min(5, std::max(0, (int)val(floor(h6))));
	const T f = h6 - (double)i;
	const T p = v * (1.0 - s), q = v * (1.0 - s * f), t = v * (1.0 - s * (1.0 - f));
	switch (i) {
		case 0: return V3<T>(v, t, p);
		case 1: return V3<T>(q, v, p);
		case 2: return V3<T>(p, v, t);
		case 3: return V3<T>(p, q, v);
		case 4: return V3<T>(t, p, v);
		default: return V3<T>(v, p, q);
	}
}

// HSLuv (A. Boronine, hsluv.org): sRGB (D65) -> CIE XYZ -> CIELUV -> LCh ->
// saturation relative to the sRGB gamut boundary. Here h, s, l are in [0,1].
namespace hsluv {
static const double M[3][3] = {{3.240969941904521, -1.537383177570093, -0.498610760293},
	{-0.96924363628087, 1.87596750150772, 0.041555057407175}, {0.055630079696993, -0.20397695888897, 1.056971514242878}};
static const double MI[3][3] = {{0.41239079926595, 0.35758433938387, 0.18048078840183},
	{0.21263900587151, 0.71516867876775, 0.072192315360733}, {0.019330818715591, 0.11919477979462, 0.95053215224966}};
constexpr double REF_U = 0.19783000664283, REF_V = 0.46831999493879, KAPPA = 903.2962962, EPS = 0.0088564516;
template<class T> T to_linear(const T &c) { return val(c) > 0.04045 ? pow((c + 0.055) / 1.055, 2.4) : c / 12.92; }
template<class T> T from_linear(const T &c) { return val(c) <= 0.0031308 ? 12.92 * c : 1.055 * pow(c, 1.0 / 2.4) - 0.055; }
template<class T> T max_chroma(const T &L, const T &H) { // H in radians
	const T sub1 = (L + 16.0) * (L + 16.0) * (L + 16.0) / 1560896.0;
	const T sub2 = val(sub1) > EPS ? sub1 : L / KAPPA;
	T best = T(1e30);
	for (int c = 0; c < 3; c++) {
		const double m1 = M[c][0], m2 = M[c][1], m3 = M[c][2];
		for (int t = 0; t < 2; t++) {
			const T top1 = (284517.0 * m1 - 94839.0 * m3) * sub2;
			const T top2 = (838422.0 * m3 + 769860.0 * m2 + 731718.0 * m1) * L * sub2 - 769860.0 * t * L;
			const T bottom = (632260.0 * m3 - 126452.0 * m2) * sub2 + 126452.0 * t;
			const T slope = top1 / bottom, icpt = top2 / bottom;
			const T len = icpt / (sin(H) - slope * cos(H));
			if (val(len) >= 0 && val(len) < val(best)) best = len;
		}
	}
	return best;
}
} // namespace hsluv

template<class T> V3<T> rgb_to_hsluv(const V3<T> &c) {
	using namespace hsluv;
	const T r = to_linear(c.x), g = to_linear(c.y), b = to_linear(c.z);
	const T X = MI[0][0] * r + MI[0][1] * g + MI[0][2] * b;
	const T Y = MI[1][0] * r + MI[1][1] * g + MI[1][2] * b;
	const T Z = MI[2][0] * r + MI[2][1] * g + MI[2][2] * b;
	const T L = val(Y) <= EPS ? Y * KAPPA : 116.0 * pow(Y, 1.0 / 3.0) - 16.0;
	if (val(L) < 1e-8) return V3<T>(T(0.0), T(0.0), T(0.0));
	const T den = X + 15.0 * Y + 3.0 * Z;
	const T U = 13.0 * L * (4.0 * X / den - REF_U), V = 13.0 * L * (9.0 * Y / den - REF_V);
	const T C = len2(U, V);
	T H = atan2(V, U);
	if (val(H) < 0) H = H + 2.0 * M_PI;
	if (val(L) > 99.9999999) return V3<T>(H / (2.0 * M_PI), T(0.0), T(1.0));
	return V3<T>(H / (2.0 * M_PI), C / max_chroma(L, H), L / 100.0);
}
template<class T> V3<T> hsluv_to_rgb(const V3<T> &hsl) {
	using namespace hsluv;
	const T L = hsl.z * 100.0;
	if (val(L) > 99.9999999) return V3<T>(T(1.0), T(1.0), T(1.0));
	if (val(L) < 1e-8) return V3<T>(T(0.0), T(0.0), T(0.0));
	const T H = hsl.x * (2.0 * M_PI);
	const T C = max_chroma(L, H) * hsl.y;
	const T U = cos(H) * C, V = sin(H) * C;
	const T vu = U / (13.0 * L) + REF_U, vv = V / (13.0 * L) + REF_V;
	const T Y = val(L) <= 8.0 ? L / KAPPA : (L + 16.0) * (L + 16.0) * (L + 16.0) / 1560896.0;
	const T X = -(9.0 * Y * vu) / ((vu - 4.0) * vv - vu * vv);
	const T Z = (9.0 * Y - 15.0 * vv * Y - vv * X) / (3.0 * vv);
	return V3<T>(from_linear(M[0][0] * X + M[0][1] * Y + M[0][2] * Z), from_linear(M[1][0] * X + M[1][1] * Y + M[1][2] * Z),
		from_linear(M[2][0] * X + M[2][1] * Y + M[2][2] * Z));
}
template<class T> T fmod1(const T &x) { return x - floor(x); }
// interpolateColor: interpolation in HSLuv with the hue along the shorter arc
template<class T> V3<T> interpolate_color(const V3<T> &a, const V3<T> &b, const T &f) {
	const V3<T> ha = rgb_to_hsluv(a), hb = rgb_to_hsluv(b);
	T dh = hb.x - ha.x;
	if (val(dh) > 0.5) dh = dh - 1.0;
	if (val(dh) < -0.5) dh = dh + 1.0;
	return hsluv_to_rgb(V3<T>(fmod1(ha.x + dh * f), interpolate(ha.y, hb.y, f), interpolate(ha.z, hb.z, f)));
}
// sources/math.cpp:47-52
template<class T> V3<T> color_hue_shift(const V3<T> &rgb, const T &shift) {
	V3<T> hsv = rgb_to_hsv(rgb);
	hsv.x = fmod1(hsv.x + shift + 1.0);
	return hsv_to_rgb(hsv);
}
// sources/math.cpp:40-45; the random triple comes from the texel's position
// (0.25 m cells hashed with the planet's deviation key) instead of a global RNG
template<class T> V3<T> color_deviation(const Planet &P, const V3<T> &color, double dev, const V3<T> &pos) {
	const uint32_t h = lattice_hash((int)std::floor(val(pos.x) * 4.0), (int)std::floor(val(pos.y) * 4.0), (int)std::floor(val(pos.z) * 4.0), P.deviation_key);
	V3<T> hsl = rgb_to_hsluv(color);
	hsl.x = hsl.x + (jitter_of(h, 0) - 0.5) * dev;
	hsl.y = hsl.y + (jitter_of(h, 10) - 0.5) * dev;
	hsl.z = hsl.z + (jitter_of(h, 20) - 0.5) * dev;
	hsl.x = fmod1(hsl.x + 1.0);
	return hsluv_to_rgb(vsat(hsl));
}
// sources/math.cpp:64-71
template<class T> V3<T> any_perpendicular(const V3<T> &a) {
	V3<T> b(T(1.0), T(0.0), T(0.0));
	if (std::fabs(val(a.x)) > 0.9) b = V3<T>(T(0.0), T(1.0), T(0.0));
	return normalize(cross(a, b));
}

// ---------------------------------------------------------------------------
// Tile (planets.h:63-83) and the coloring stages (coloringModes.cpp)
// ---------------------------------------------------------------------------
enum Biome { B_BARE, B_TUNDRA, B_TAIGA, B_SHRUB, B_GRASS, B_TEMP_SEASONAL, B_TEMP_RAIN, B_DESERT, B_SAVANNA, B_TROP_SEASONAL, B_TROP_RAIN,
	B_WATER, B_TOTAL };
enum TType { TT_ROAD, TT_FLAT, TT_ROUGH, TT_CLIFFS, TT_WATER, TT_TOTAL };
enum Purpose { PU_UNDEFINED, PU_LAND, PU_WATER, PU_NAVIGATION };

template<class T> struct Tile {
	V3<T> position, normal, albedo;
	T roughness = T(0.0), metallic = T(0.0), height = T(0.0), elevation = T(0.0), slope = T(0.0), temperature = T(0.0),
	  precipitation = T(0.0), opacity = T(1.0);
	int biome = B_TOTAL, type = TT_TOTAL, purpose = PU_UNDEFINED;
};

template<class T> struct Col {
	const Planet &P;
	explicit Col(const Planet &p) : P(p) {}
	T n(int slot, const V3<T> &p) const { return noise_eval(P.noise[slot], p); }
	T n1(int slot, const T &x) const { return noise_eval(P.noise[slot], V3<T>(x, T(0.0), T(0.0))); } // 1-D evaluate -> (x, 0, 0)
	T sdf_elev(const V3<T> &p) const { return shape_eval(P, p) * 10.0; }        // terrainSdfElevation
	// steepnessMask :23-27, slope in radians, threshold and smoothing in degrees
	T steep(const T &slope, double thr, double sm) const { return saturate((T(thr * M_PI / 180.0) + sm * M_PI / 180.0 - slope) / (2.0 * sm * M_PI / 180.0)); }
	static T range_mask(const T &v, double z, double o) { return saturate((v - z) / (o - z)); } // :29-32
	T beach_mask(const Tile<T> &t) const { // :34-49
		if (t.biome == B_WATER) return T(0.0);
		return range_mask(t.elevation + n1(S_BEACH, t.elevation) * 20.0, 10, 15);
	}
	void elevation(Tile<T> &t) const { t.elevation = t.purpose == PU_LAND ? sdf_elev(t.position) : elevation_eval(P, t.position); } // :51-57
	void precipitation(Tile<T> &t) const { // :59-80
		T p = n(S_PRECIP, t.position) * 0.5 + 0.5;
		p = saturate(p);
		p = smootherstep(p);
		p = smootherstep(p);
		p = pow(tmax(p + 0.2, T(0.0)), 3.0) * 0.6;
		p = p * 400.0;
		p = p + tmax(120.0 - abs(t.elevation), T(0.0)) * 0.2;
		t.precipitation = tmax(p, T(0.0));
	}
	void temperature(Tile<T> &t) const { // :82-120
		T x = n(S_TEMP, t.position) * 0.5 + 0.5;
		x = saturate(x);
		x = smoothstep(x);
		x = x * 2.0 - 1.0;
		if (P.poles) {
			T polar = abs(atan(t.position.y / len2(t.position.x, t.position.z))) / M_PI * 2.0;
			polar = pow(polar, 1.7);
			polar = polar + n(S_POLAR, t.position) * 0.1;
			x = x + (0.6 - polar * 3.2);
		}
		t.temperature = 15.0 + x * 30.0 - tmax(t.elevation, T(0.0)) * 0.02;
	}
	void slope(Tile<T> &t) const { // :122-151
		const double radius = 0.5;
		V3<T> a = any_perpendicular(t.normal);
		V3<T> b = cross(t.normal, a);
		a = a * radius;
		b = b * radius;
		const double div = 1.0 / std::sqrt(2.0);
		const V3<T> c = (a + b) * div, d = (a - b) * div;
		const V3<T> taps[8] = {t.position + a, t.position + b, t.position - a, t.position - b, t.position + c, t.position + d, t.position - c, t.position - d};
		T e1 = sdf_elev(taps[0]), e2 = e1;
		for (int i = 1; i < 8; i++) {
			const T e = sdf_elev(taps[i]);
			e1 = tmin(e1, e);
			e2 = tmax(e2, e);
		}
		const T md = (e2 - e1) * 0.1;
		t.slope = atan(md / radius);
	}
	static void biome(Tile<T> &t) { // :153-190
		const double e = val(t.elevation), tp = val(t.temperature), pr = val(t.precipitation);
		if (e < 0) t.biome = B_WATER;
		else if (tp > 20) t.biome = pr < 40 ? B_DESERT : (pr < 130 ? B_SAVANNA : (pr < 230 ? B_TROP_SEASONAL : B_TROP_RAIN));
		else if (tp > 5) t.biome = pr < 30 ? B_SHRUB : (pr < 100 ? B_GRASS : (pr < 200 ? B_TEMP_SEASONAL : B_TEMP_RAIN));
		else if (tp > -5) t.biome = pr < 30 ? B_BARE : B_TAIGA;
		else if (pr < 10) t.biome = B_BARE;
		else t.biome = B_TUNDRA;
	}
	static void type(Tile<T> &t) { // :192-200
		if (val(t.elevation) < 0) t.type = TT_WATER;
		else if (val(t.slope) > 20.0 * M_PI / 180.0) t.type = TT_CLIFFS;
		else t.type = TT_FLAT;
	}
	void bedrock(Tile<T> &t) const { // :202-261
		const T depth = sqr(n(S_BED_DEPTH, t.position) * 0.5 + 0.501) * 2.0;
		const T freq = n(S_BED_FREQ, t.position) * 0.15 + 1.0;
		const T cracks = saturate(pow(n(S_BED_CRACKS, t.position * freq) * 0.5 + 0.5, 0.7));
		const T value = n(S_BED_VALUE, t.position * freq);
		const T saturation = saturate(n(S_BED_SAT, t.position) * 0.35 + 0.3);
		t.albedo = hsv_to_rgb(V3<T>(T(0.07), saturation, saturate(value * 0.1 + 0.7) * (cracks * 0.4 + 0.6)));
		t.roughness = interpolate(T(0.9), value * -0.15 + 0.65, cracks);
		t.height = cracks * depth;
	}
	void cliffs(Tile<T> &t) const { // :263-293
		const T bf = steep(t.slope, 19, 4);
		if (val(bf) > 0.99999) return;
		V3<T> hsv = rgb_to_hsv(t.albedo);
		hsv.x = interpolate(T(155.0 / 255.0), hsv.x, sharpEdge(bf, 0.005));
		hsv.y = hsv.y * (bf * 0.4 + 0.6);
		hsv.z = interpolate(T(0.7), hsv.y, bf * 0.8 + 0.2);
		t.albedo = hsv_to_rgb(hsv);
		t.roughness = t.roughness * (bf * 0.2 + 0.8);
		const T cr = sharpEdge(saturate(n(S_CLIFF_CRACKS, t.position) * 2.0 - 1.1), 0.2);
		t.height = t.height * interpolate(T(1.0), T(0.8), cr);
		t.albedo = t.albedo * interpolate(T(1.0), T(0.9), cr);
		t.roughness = interpolate(t.roughness, T(0.9), cr);
	}
	void mica(Tile<T> &t) const { // :295-336
		if (!P.flowers) return;
		const T bf = saturate((n(S_MICA_MASK, t.position) - 0.98) * 10.0);
		if (val(bf) < 1e-7) return;
		const T cr = sharpEdge(saturate(n(S_MICA_CRACKS, t.position) + 0.6));
		const V3<T> color = interpolate(V3<T>(T(122 / 255.0), T(90 / 255.0), T(88 / 255.0)), V3<T>(T(184 / 255.0), T(209 / 255.0), T(187 / 255.0)), cr);
		const T roughness = cr * 0.3 + 0.4, metallic = T(1.0), height = t.height * 0.5;
		t.albedo = interpolate(t.albedo, color, bf);
		t.roughness = interpolate(t.roughness, roughness, bf);
		t.metallic = interpolate(t.metallic, metallic, bf);
		t.height = interpolate(t.height, height, bf);
	}
	void dirt(Tile<T> &t) const { // :338-402
		T height = n(S_DIRT_HEIGHT, t.position) * 0.2 + 0.5;
		const T bf = sharpEdge(saturate(height - t.height + 0.4)) * steep(t.slope, 20, 5);
		if (val(bf) < 1e-7) return;
		V3<T> color(T(168 / 255.0), T(94 / 255.0), T(28 / 255.0));
		{
			const T sat = range_mask(t.precipitation, 0, 50);
			V3<T> hsv = rgb_to_hsv(color);
			hsv.y = hsv.y * (sat * 0.7);
			hsv.z = hsv.z * 0.8;
			color = hsv_to_rgb(hsv);
		}
		T roughness = T(0.8);
		const T metallic = T(0.0);
		{
			T cr = sharpEdge(saturate(n(S_DIRT_CRACKS, t.position) * 2.0 - 1.2), 0.15);
			cr = cr * (sqr(smoothstep(saturate(n(S_DIRT_CMASK, t.position) * 0.5 + 0.5))) * 0.9 + 0.1);
			cr = cr * (range_mask(t.precipitation, 70, 20) * 0.9 + 0.1);
			height = interpolate(height, height * 0.5, cr);
			color = interpolate(color, V3<T>(T(0.1), T(0.1), T(0.1)), cr);
			roughness = interpolate(roughness, T(0.9), cr);
		}
		t.albedo = interpolate(t.albedo, color, bf);
		t.roughness = interpolate(t.roughness, roughness, bf);
		t.metallic = interpolate(t.metallic, metallic, bf);
		t.height = interpolate(t.height, height, bf);
	}
	void sand(Tile<T> &t) const { // :404-465
		const T bf = range_mask(t.temperature, 24, 28) * steep(t.slope, 19, 10);
		if (val(bf) < 1e-7) return;
		const T hs = n(S_SAND_HSCALE, t.position) * 0.3 + 1.0;
		const T height = (n(S_SAND_HEIGHT, t.position * hs) * 0.2) * (range_mask(t.precipitation, 100, 50) * 0.4 + 0.6) + 0.5;
		const T cs = smootherstep(smootherstep(n(S_SAND_COLOR, t.position) * 0.5 + 0.5));
		const T hue = n(S_SAND_HUE, t.position) * 0.1;
		V3<T> color = color_hue_shift(V3<T>(T(189 / 255.0), T(174 / 255.0), T(152 / 255.0)), hue);
		color = interpolate_color(color, V3<T>(T(187 / 255.0), T(104 / 255.0), T(50 / 255.0)), cs);
		color = color_deviation(P, color, 0.08, t.position);
		V3<T> hsv = rgb_to_hsv(color);
		color = hsv_to_rgb(V3<T>(hsv.x, hsv.y * 0.7, hsv.z * 0.8));
		const T roughness = (hs - 1.0) * 0.7 + 0.55 + hue;
		t.albedo = interpolate(t.albedo, color, bf);
		t.roughness = interpolate(t.roughness, roughness, bf);
		t.metallic = interpolate(t.metallic, T(0.0), bf);
		t.height = interpolate(t.height, height, bf);
	}
	void grass(Tile<T> &t) const { // :467-533
		const T bf = range_mask(t.temperature, 35, 25) * range_mask(t.precipitation, 15, 35) * steep(t.slope, 22, 3) * beach_mask(t);
		if (val(bf) < 1e-7) return;
		const T dryness = tclamp(t.temperature - (t.precipitation + 100.0) * 30.0 / 400.0, 0.0, 5.0) / 5.0;
		const T hb = n(S_GRASS_HUE, t.position);
		const T hue = hb * 0.09 - dryness * 0.1;
		V3<T> color = color_hue_shift(V3<T>(T(114 / 255.0), T(187 / 255.0), T(77 / 255.0)), hue);
		const T pm = sharpEdge(n(S_GRASS_PCELLS, t.position) * 0.5 + 0.2);
		const T patches = pow(n(S_GRASS_PDIST, t.position) * 0.5 + 0.5, 0.5) * pm * (1.0 - dryness * 0.8);
		color = color * (1.0 - patches * 0.09);
		const T scratches = saturate(n(S_GRASS_SCRATCH, t.position) - 0.2) * (1.0 - dryness * 0.5);
		color = color * (1.0 - scratches * 0.1);
		const T roughness = 0.6 + dryness * 0.1 + patches * 0.1 + scratches * 0.1 - hb * 0.1;
		const T height = interpolate(t.height, T(0.5), T(0.7)) + (0.5 - dryness) * 0.2 + patches * 0.05 - scratches * 0.02 + hb * 0.1 + 0.1;
		t.albedo = interpolate(t.albedo, color, bf);
		t.roughness = interpolate(t.roughness, roughness, bf);
		t.metallic = interpolate(t.metallic, T(0.0), bf);
		t.height = interpolate(t.height, height, bf);
	}
	void boulders(Tile<T> &t) const { // :535-615
		if (!P.flowers) return;
		if (val(n(S_BOUL_THRESH, t.position)) < 0.15) return;
		const V3<T> center = voronoi_nearest(P.boulders, t.position, &t.normal);
		const T dist = length(center - t.position);
		const T size = smootherstep(smootherstep(saturate(n(S_BOUL_SIZE, t.position) * 0.5 + 0.5))) * 3.0 + 3.0;
		const T bf = range_mask(size - dist, 0, 0.5);
		if (val(bf) < 1e-7) return;
		const T hs = n(S_BOUL_HUE, t.position) * 0.12;
		const T vs = n(S_BOUL_VALUE, t.position) * 0.18;
		V3<T> color = rgb_to_hsv(V3<T>(T(154 / 255.0), T(154 / 255.0), T(154 / 255.0)));
		color.x = fmod1(color.x + hs + 1.0);
		color.z = saturate(color.z + vs);
		color = hsv_to_rgb(color);
		const T roughness = n(S_BOUL_SCRATCH, t.position) * 0.1 + 0.4;
		const T height = 1.0 - sqr(dist / size) * 0.5;
		t.albedo = interpolate(t.albedo, color, bf);
		t.roughness = interpolate(t.roughness, roughness, bf);
		t.metallic = interpolate(t.metallic, T(0.0), bf);
		t.height = interpolate(t.height, height, bf);
	}
	void water(Tile<T> &t) const { // :617-656
		const T sw = n(S_WATER_SWITCH, t.position) * 0.5 + 0.5;
		const T hue = n(S_WATER_HUE, t.position) * 0.09;
		t.albedo = color_hue_shift(interpolate_color(V3<T>(T(40 / 255.0), T(63 / 255.0), T(168 / 255.0)), V3<T>(T(39 / 255.0), T(154 / 255.0), T(186 / 255.0)), sw), hue);
		const T d1 = 1.0 - sqr(range_mask(t.elevation, -25, 3));
		const T d2 = rescale(range_mask(t.elevation, 0, -100), 0, 1, 0.7, 1);
		t.opacity = d1 * d2;
		t.metallic = smoothstep(range_mask(t.elevation, 3, -30));
	}
	void flowers(Tile<T> &t) const { // :658-744
		if (!P.flowers) return;
		const bool lily = t.purpose != PU_LAND;
		if ((t.biome == B_WATER) != lily) return;
		if (val(range_mask(abs(t.temperature - 18.0), 12, 7)) < 1e-5) return;
		if (!lily && val(range_mask(abs(t.precipitation - 200.0), 100, 70)) < 1e-5) return;
		const V3<T> center = voronoi_nearest(P.flower_center, t.position, &t.normal);
		if (val(dot(center - t.position, center - t.position)) > 16.0) return;
		const V3<T> cluster = voronoi_nearest(P.flower_cluster, t.position, &t.normal);
		if (val(dot(center - cluster, center - cluster)) > 400.0) return;
		const T dist = length(center - t.position);
		const T size = smootherstep(smootherstep(saturate(n(S_FLOW_SIZE, t.position) * 0.5 + 0.5))) * 2.0 + 1.5;
		const T bf = range_mask(size - dist, 0, 0.1);
		if (val(bf) < 1e-7) return;
		const V3<T> base = lily ? V3<T>(T(0.2), T(0.14), T(0.0))
		                        : interpolate_color(V3<T>(T(0.5), T(0.0), T(0.35)), V3<T>(T(0.5), T(0.4), T(0.0)), sharpEdge(n(S_FLOW_COLOR, cluster) + 0.4, 0.2));
		const V3<T> color = color_hue_shift(base, n(S_FLOW_HUE1, t.position) * 0.1 + n(S_FLOW_HUE2, t.position) * 0.1);
		const T height = 0.7 + sqr(dist / size) * 0.2;
		t.albedo = interpolate(t.albedo, color, bf);
		t.roughness = interpolate(t.roughness, T(0.8), bf);
		t.metallic = interpolate(t.metallic, T(lily ? 0.85 : 0.0), bf);
		t.height = interpolate(t.height, height, bf);
		t.opacity = interpolate(t.opacity, T(1.0), bf);
	}
	void ice(Tile<T> &t) const { // :746-817
		const T off = n(S_ICE_TEMPOFF, t.position) * 1.5;
		const T bf = sharpEdge(range_mask(t.temperature + off, 0, -3)) * (1.0 - beach_mask(t));
		if (val(bf) < 1e-7) return;
		if (val(bf) > 0.1 && t.type != TT_CLIFFS) t.type = TT_ROUGH;
		const T freq = n(S_ICE_FREQ, t.position) * 0.08 + 1.0;
		const T thick = sharpEdge(saturate(n(S_ICE_THICK, t.position * freq) * 0.5 + 0.8), 0.1) * 0.6 + 0.4;
		const T crack = 1.0 - pow(n(S_ICE_CRACKS, t.position * freq) * 0.5 + 0.5, 0.3);
		V3<T> color = vmax(V3<T>(T(122 / 255.0), T(162 / 255.0), T(164 / 255.0)) - V3<T>(crack * 0.3, crack * 0.3, crack * 0.3), 0.0);
		color = interpolate_color(t.albedo, color, thick);
		T roughness = 0.15 + crack * 0.6;
		roughness = interpolate(t.roughness, roughness, thick);
		const T height = thick * 0.5 * (1.0 - crack * 0.8);
		t.albedo = interpolate(t.albedo, color, bf);
		t.roughness = interpolate(t.roughness, roughness, bf);
		t.metallic = interpolate(t.metallic, T(0.0), bf);
		t.height = interpolate(t.height, height, bf);
		t.opacity = interpolate(t.opacity, t.opacity * 0.9 + thick * 0.5, bf);
	}
	void snow(Tile<T> &t) const { // :819-855
		T bf = sharpEdge(range_mask(t.elevation + n(S_SNOW_ELEVOFF, t.position) * 20.0, 220, 240) * steep(t.slope, 25, 5));
		const T thick = n(S_SNOW_THICK, t.position) * 0.5 + 0.5;
		bf = bf * saturate(thick * 0.5 + 0.7);
		if (val(bf) < 1e-7) return;
		t.albedo = interpolate(t.albedo, V3<T>(T(230 / 255.0), T(230 / 255.0), T(230 / 255.0)), bf);
		t.roughness = interpolate(t.roughness, thick * 0.3 + 0.2, bf);
		t.metallic = interpolate(t.metallic, T(0.0), bf);
		t.height = interpolate(t.height, 0.6 + t.height * 0.1 + thick * 0.3, bf);
	}
	static void visualization(Tile<T> &t) { // :857-893
		static const double C[12][3] = {{187, 187, 187}, {175, 226, 255}, {193, 225, 221}, {200, 110, 62}, {239, 252, 143}, {151, 183, 102},
			{118, 169, 92}, {221, 187, 76}, {253, 213, 120}, {161, 151, 0}, {50, 122, 30}, {0, 0, 255}};
		if (t.biome >= 0 && t.biome < 12) t.albedo = V3<T>(T(C[t.biome][0] / 255), T(C[t.biome][1] / 255), T(C[t.biome][2] / 255));
		else t.albedo = V3<T>(T(NAN), T(NAN), T(NAN));
		t.roughness = T(0.7);
	}
	static void finalization(Tile<T> &t) { // :895-902
		t.albedo = vsat(t.albedo);
		t.roughness = saturate(t.roughness);
		t.metallic = saturate(t.metallic);
		t.height = saturate(t.height);
		t.opacity = saturate(t.opacity);
	}
	void run(Tile<T> &t) const {
		if (P.coloring == 0) { // coloringDefault :905-930
			elevation(t); precipitation(t); temperature(t); slope(t); biome(t); type(t);
			if (t.purpose == PU_WATER) water(t);
			else { bedrock(t); cliffs(t); mica(t); dirt(t); sand(t); grass(t); boulders(t); }
			flowers(t); ice(t);
			if (t.purpose != PU_WATER) snow(t);
			finalization(t);
		} else if (P.coloring == 1) { // coloringBarren :932-952
			elevation(t); slope(t);
			if (t.purpose == PU_WATER) { t.biome = B_WATER; t.type = TT_WATER; water(t); }
			else { t.biome = B_BARE; t.type = TT_FLAT; bedrock(t); cliffs(t); mica(t); boulders(t); }
			finalization(t);
		} else { // coloringDebug :954-966
			elevation(t); precipitation(t); temperature(t); slope(t); biome(t); type(t); visualization(t);
			if (t.purpose == PU_WATER) t.opacity = T(0.5);
			finalization(t);
		}
	}
};

// ---------------------------------------------------------------------------
// synthetic texel program (for synthetic contexts): albedo from a 3-octave
// value-noise field, roughness from a 2-octave simplex field, height from the
// elevation, each evaluated at the texel's surface position
// ---------------------------------------------------------------------------
template<class T> void synth_texel(const up_synth_program &prog, const V3<T> &pos, V3<T> &albedo, T &rough, T &height) {
	const uint32_t s0 = prog.n_layers > 0 ? prog.layer[0].seed : 0u;
	NoiseCfg ca; ca.type = NT_VALUE; ca.fractal = FR_FBM; ca.octaves = 3; ca.frequency = 4.0; ca.seed = s0 + 100;
	NoiseCfg cr; cr.type = NT_SIMPLEX; cr.fractal = FR_FBM; cr.octaves = 2; cr.frequency = 8.0; cr.seed = s0 + 200;
	const T a = noise_eval(make_noise(ca), pos) * 0.5 + 0.5;
	albedo = interpolate(V3<T>(T(0.35), T(0.27), T(0.18)), V3<T>(T(0.72), T(0.66), T(0.52)), saturate(a));
	rough = saturate(noise_eval(make_noise(cr), pos) * 0.5 + 0.5);
	// height = 0.5 + elevation / (2 sum |amp|)
	double tot = 0;
	T e = T(0.0);
	for (int l = 0; l < prog.n_layers; l++) {
		const up_noise_layer &L = prog.layer[l];
		for (int i = 0; i < L.octaves; i++) {
			tot += std::fabs(L.amp[i]);
			const T f = T((double)L.freq[i]);
			T n = noise_single(L.type, V3<T>(pos.x * f, pos.y * f, pos.z * f), seed_key(L.seed + (uint32_t)i), L.distance, L.operation);
			if (L.fractal == UP_FRACTAL_RIDGED) n = 1.0 - 2.0 * abs(n);
			e = e + n * (double)L.amp[i];
		}
	}
	height = saturate(0.5 + e / (2.0 * (tot > 0 ? tot : 1.0)));
}

// ---------------------------------------------------------------------------
// UV rasterisation (replaces meshGenerateTexture, textures.cpp:66-71):
// vertices snapped to 1/256 texel (int64 fixed point), texel centres at
// (x + 0.5, y + 0.5), edge functions exact; a texel on an edge belongs to the
// triangle for which that edge has dy > 0, or dy == 0 and dx < 0 (each
// triangle oriented to positive area); overlaps go to the highest triangle id.
// Weights are the edge functions divided by twice the area (FP64).
// ---------------------------------------------------------------------------
struct Raster {
	std::vector<int32_t> owner; // -1 = not covered
	std::vector<double> w;      // 3 per texel
};
inline int64_t snap(float u, uint32_t size) { return (int64_t)std::llrint((double)u * (double)size * 256.0); }
inline bool edge_in(int64_t e, int64_t dx, int64_t dy) { return e > 0 || (e == 0 && (dy > 0 || (dy == 0 && dx < 0))); }
inline void rasterize(const float *uv, const uint32_t *idx, uint64_t ntri, uint32_t W, uint32_t H, Raster &R) {
	R.owner.assign((size_t)W * H, -1);
	R.w.assign((size_t)W * H * 3, 0.0);
	for (uint64_t t = 0; t < ntri; t++) {
		int64_t X[3], Y[3];
		for (int k = 0; k < 3; k++) { X[k] = snap(uv[2 * idx[3 * t + k]], W); Y[k] = snap(uv[2 * idx[3 * t + k] + 1], H); }
		int64_t area = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
		if (area == 0) continue;
		int o[3] = {0, 1, 2};
		if (area < 0) { o[1] = 2; o[2] = 1; area = -area; }
		const int64_t ax = X[o[0]], ay = Y[o[0]], bx = X[o[1]], by = Y[o[1]], cx = X[o[2]], cy = Y[o[2]];
		const int64_t xmin = std::min(ax, std::min(bx, cx)), xmax = std::max(ax, std::max(bx, cx));
		const int64_t ymin = std::min(ay, std::min(by, cy)), ymax = std::max(ay, std::max(by, cy));
		const int64_t tx0 = std::max<int64_t>(0, (xmin - 128 + 255) / 256), tx1 = std::min<int64_t>(W - 1, (xmax - 128) / 256);
		const int64_t ty0 = std::max<int64_t>(0, (ymin - 128 + 255) / 256), ty1 = std::min<int64_t>(H - 1, (ymax - 128) / 256);
		for (int64_t y = ty0; y <= ty1; y++)
			for (int64_t x = tx0; x <= tx1; x++) {
				const int64_t px = x * 256 + 128, py = y * 256 + 128;
				const int64_t e0 = (cx - bx) * (py - by) - (cy - by) * (px - bx); // edge b->c, weight of a
				const int64_t e1 = (ax - cx) * (py - cy) - (ay - cy) * (px - cx); // edge c->a, weight of b
				const int64_t e2 = (bx - ax) * (py - ay) - (by - ay) * (px - ax); // edge a->b, weight of c
				if (!edge_in(e0, cx - bx, cy - by) || !edge_in(e1, ax - cx, ay - cy) || !edge_in(e2, bx - ax, by - ay)) continue;
				const size_t q = (size_t)y * W + (size_t)x;
				if (R.owner[q] >= (int32_t)t) continue;
				R.owner[q] = (int32_t)t;
				double wt[3];
				wt[o[0]] = (double)e0 / (double)area;
				wt[o[1]] = (double)e1 / (double)area;
				wt[o[2]] = (double)e2 / (double)area;
				for (int k = 0; k < 3; k++) R.w[3 * q + k] = wt[k];
			}
	}
}

// imageDilation(img, rounds, useNan) (textures.cpp:73-77): each round, every
// NaN texel with a valid 8-neighbour becomes the mean of its valid
// 8-neighbours of the previous round
inline void dilate(std::vector<float> &img, uint32_t W, uint32_t H, int ch, int rounds) {
	for (int r = 0; r < rounds; r++) {
		std::vector<float> prev = img;
		for (uint32_t y = 0; y < H; y++)
			for (uint32_t x = 0; x < W; x++) {
				const size_t q = ((size_t)y * W + x) * ch;
				if (!std::isnan(prev[q])) continue;
				double acc[4] = {0, 0, 0, 0};
				int cnt = 0;
				for (int dy = -1; dy <= 1; dy++)
					for (int dx = -1; dx <= 1; dx++) {
						if (!dx && !dy) continue;
						const int64_t xx = (int64_t)x + dx, yy = (int64_t)y + dy;
						if (xx < 0 || yy < 0 || xx >= W || yy >= H) continue;
						const size_t s = ((size_t)yy * W + (size_t)xx) * ch;
						if (std::isnan(prev[s])) continue;
						for (int c = 0; c < ch; c++) acc[c] += prev[s + c];
						cnt++;
					}
				if (cnt)
					for (int c = 0; c < ch; c++) img[q + c] = (float)(acc[c] / cnt);
			}
	}
}
// imageConvert(U8) (textures.cpp:79-81): round(saturate(v) * 255), NaN -> 0
inline uint8_t to_u8(float v) { return std::isnan(v) ? 0 : (uint8_t)(std::min(std::max(v, 0.0f), 1.0f) * 255.0f + 0.5f); }

} // namespace orc
