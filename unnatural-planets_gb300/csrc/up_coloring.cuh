// Device per-texel coloring: the Tile record (sources/planets.h:63-83), the
// coloring stages and the three pipelines of sources/coloringModes.cpp, the
// colour helpers of sources/math.cpp:40-71, the cage colour conversions
// (HSV: Smith 1978; HSLuv: hsluv.org), and the synthetic texel program.
// FP32, one thread per texel or tile.
#pragma once
#include "up_modes.cuh"
#include "up_synth.cuh"

namespace up {

struct TileD {
	V3f position, normal, albedo;
	float roughness, metallic, height, elevation, slope, temperature, precipitation, opacity;
	int biome, type, purpose;
};
UP_HD TileD tile_init(V3f p, V3f n, int purpose) {
	TileD t;
	t.position = p; t.normal = n; t.albedo = zero3();
	t.roughness = t.metallic = t.height = t.elevation = t.slope = t.temperature = t.precipitation = 0.f;
	t.opacity = 1.f;
	t.biome = 12; t.type = 5; t.purpose = purpose;
	return t;
}

UP_HD V3f vlerp(V3f a, V3f b, float f) { return a + (b - a) * f; }
UP_HD V3f vsat3(V3f a) { return v3(saturatef(a.x), saturatef(a.y), saturatef(a.z)); }
UP_HD float frac1(float x) { return x - floorf(x); }
UP_HD float sharpf(float v, float p = 0.05f) { return (fminf(fmaxf(v, 0.5f - p), 0.5f + p) - (0.5f - p)) / (2.f * p); }
UP_HD float range_mask(float v, float z, float o) { return saturatef((v - z) / (o - z)); }        // coloringModes.cpp:29-32
UP_HD float steep_mask(float slope, float thr, float sm) {                                          // :23-27
	const float d2r = 0.017453292519943295f;
	return saturatef((thr * d2r + sm * d2r - slope) / (2.f * sm * d2r));
}
UP_HD float smoothstepf(float x) { return x * x * (3.f - 2.f * x); }
UP_HD float smootherstepf(float x) { return x * x * x * (x * (x * 6.f - 15.f) + 10.f); }

// ---------------------------------------------------------------- colour conversions
UP_HD V3f rgb_to_hsv(V3f c) {
	const float mx = fmaxf(c.x, fmaxf(c.y, c.z)), mn = fminf(c.x, fminf(c.y, c.z)), d = mx - mn;
	float h = 0.f;
	if (d > 0.f) {
		if (mx == c.x) h = (c.y - c.z) / d;
		else if (mx == c.y) h = (c.z - c.x) / d + 2.f;
		else h = (c.x - c.y) / d + 4.f;
		h *= (1.f / 6.f);
		if (h < 0.f) h += 1.f;
	}
	return v3(h, mx > 0.f ? d / mx : 0.f, mx);
}
UP_HD V3f hsv_to_rgb(V3f hsv) {
	const float h6 = frac1(hsv.x) * 6.f, s = hsv.y, v = hsv.z;
	int i = (int)floorf(h6);
	i = i < 0 ? 0 : (i > 5 ? 5 : i);
	const float f = h6 - (float)i;
	const float p = v * (1.f - s), q = v * (1.f - s * f), t = v * (1.f - s * (1.f - f));
	switch (i) {
		case 0: return v3(v, t, p);
		case 1: return v3(q, v, p);
		case 2: return v3(p, v, t);
		case 3: return v3(p, q, v);
		case 4: return v3(t, p, v);
		default: return v3(v, p, q);
	}
}
// HSLuv with h, s, l in [0, 1]
UP_HD float hl_to_linear(float c) { return c > 0.04045f ? powf((c + 0.055f) / 1.055f, 2.4f) : c / 12.92f; }
UP_HD float hl_from_linear(float c) { return c <= 0.0031308f ? 12.92f * c : 1.055f * powf(c, 1.f / 2.4f) - 0.055f; }
UP_HD float hl_max_chroma(float L, float H) {
	const float Mx[3][3] = {{3.240969941904521f, -1.537383177570093f, -0.498610760293f},
		{-0.96924363628087f, 1.87596750150772f, 0.041555057407175f}, {0.055630079696993f, -0.20397695888897f, 1.056971514242878f}};
	const float sub1 = (L + 16.f) * (L + 16.f) * (L + 16.f) / 1560896.f;
	const float sub2 = sub1 > 0.0088564516f ? sub1 : L / 903.2962962f;
	float sh, ch;
	sincosf(H, &sh, &ch);
	float best = 1e30f;
	#pragma unroll
	for (int c = 0; c < 3; c++) {
		const float m1 = Mx[c][0], m2 = Mx[c][1], m3 = Mx[c][2];
		#pragma unroll
		for (int t = 0; t < 2; t++) {
			const float top1 = (284517.f * m1 - 94839.f * m3) * sub2;
			const float top2 = (838422.f * m3 + 769860.f * m2 + 731718.f * m1) * L * sub2 - 769860.f * (float)t * L;
			const float bottom = (632260.f * m3 - 126452.f * m2) * sub2 + 126452.f * (float)t;
			const float len = (top2 / bottom) / (sh - (top1 / bottom) * ch);
			if (len >= 0.f && len < best) best = len;
		}
	}
	return best;
}
UP_HD V3f rgb_to_hsluv(V3f c) {
	const float r = hl_to_linear(c.x), g = hl_to_linear(c.y), b = hl_to_linear(c.z);
	const float X = 0.41239079926595f * r + 0.35758433938387f * g + 0.18048078840183f * b;
	const float Y = 0.21263900587151f * r + 0.71516867876775f * g + 0.072192315360733f * b;
	const float Z = 0.019330818715591f * r + 0.11919477979462f * g + 0.95053215224966f * b;
	const float L = Y <= 0.0088564516f ? Y * 903.2962962f : 116.f * cbrtf(Y) - 16.f;
	if (L < 1e-8f) return zero3();
	const float den = X + 15.f * Y + 3.f * Z;
	const float U = 13.f * L * (4.f * X / den - 0.19783000664283f), V = 13.f * L * (9.f * Y / den - 0.46831999493879f);
	float H = atan2f(V, U);
	if (H < 0.f) H += 6.283185307179586f;
	if (L > 99.9999999f) return v3(H / 6.283185307179586f, 0.f, 1.f);
	return v3(H / 6.283185307179586f, sqrtf(U * U + V * V) / hl_max_chroma(L, H), L / 100.f);
}
UP_HD V3f hsluv_to_rgb(V3f hsl) {
	const float L = hsl.z * 100.f;
	if (L > 99.9999999f) return v3(1.f, 1.f, 1.f);
	if (L < 1e-8f) return zero3();
	const float H = hsl.x * 6.283185307179586f;
	const float C = hl_max_chroma(L, H) * hsl.y;
	float sh, ch;
	sincosf(H, &sh, &ch);
	const float vu = ch * C / (13.f * L) + 0.19783000664283f, vv = sh * C / (13.f * L) + 0.46831999493879f;
	const float Y = L <= 8.f ? L / 903.2962962f : (L + 16.f) * (L + 16.f) * (L + 16.f) / 1560896.f;
	const float X = -(9.f * Y * vu) / ((vu - 4.f) * vv - vu * vv);
	const float Z = (9.f * Y - 15.f * vv * Y - vv * X) / (3.f * vv);
	return v3(hl_from_linear(3.240969941904521f * X - 1.537383177570093f * Y - 0.498610760293f * Z),
		hl_from_linear(-0.96924363628087f * X + 1.87596750150772f * Y + 0.041555057407175f * Z),
		hl_from_linear(0.055630079696993f * X - 0.20397695888897f * Y + 1.056971514242878f * Z));
}
// interpolateColor: HSLuv, hue along the shorter arc
UP_HD V3f interpolate_color(V3f a, V3f b, float f) {
	const V3f ha = rgb_to_hsluv(a), hb = rgb_to_hsluv(b);
	float dh = hb.x - ha.x;
	if (dh > 0.5f) dh -= 1.f;
	if (dh < -0.5f) dh += 1.f;
	return hsluv_to_rgb(v3(frac1(ha.x + dh * f), lerpf(ha.y, hb.y, f), lerpf(ha.z, hb.z, f)));
}
UP_HD V3f color_hue_shift(V3f rgb, float shift) { // math.cpp:47-52
	V3f hsv = rgb_to_hsv(rgb);
	hsv.x = frac1(hsv.x + shift + 1.f);
	return hsv_to_rgb(hsv);
}
// math.cpp:40-45 with the random triple hashed from the 0.25 m cell of pos
UP_HD V3f color_deviation(const ModesDesc &M, V3f color, float dev, V3f pos) {
	const uint32_t h = lattice_hash((int)floorf(pos.x * 4.f), (int)floorf(pos.y * 4.f), (int)floorf(pos.z * 4.f), M.deviation_key);
	V3f hsl = rgb_to_hsluv(color);
	hsl.x += (jitter(h, 0) - 0.5f) * dev;
	hsl.y += (jitter(h, 10) - 0.5f) * dev;
	hsl.z += (jitter(h, 20) - 0.5f) * dev;
	hsl.x = frac1(hsl.x + 1.f);
	return hsluv_to_rgb(vsat3(hsl));
}
UP_HD V3f any_perpendicular(V3f a) { // math.cpp:64-71
	const V3f b = fabsf(a.x) > 0.9f ? v3(0.f, 1.f, 0.f) : v3(1.f, 0.f, 0.f);
	const V3f c = cross(a, b);
	return c * (1.f / length(c));
}

// ---------------------------------------------------------------- coloring stages
struct Colorer {
	const ModesDesc &M;
	UP_HD float n(int slot, V3f p) const { return noise_dev(M.color[slot - N_ELEV_NOISE], vs(p.x, p.y, p.z)); }
	UP_HD float n1(int slot, float x) const { return noise_dev(M.color[slot - N_ELEV_NOISE], vs(x, 0.f, 0.f)); }
	UP_HD float sdf_elev(V3f p) const { return shape_eval(M, vs(p.x, p.y, p.z)) * 10.f; } // terrainSdfElevation
	UP_HD float beach(const TileD &t) const { // :34-49
		if (t.biome == 11) return 0.f;
		return range_mask(t.elevation + n1(NS_BEACH, t.elevation) * 20.f, 10.f, 15.f);
	}
	UP_HD void elevation(TileD &t) const { // :51-57
		t.elevation = t.purpose == UP_PURPOSE_LAND ? sdf_elev(t.position) : elevation_eval(M, vs(t.position.x, t.position.y, t.position.z));
	}
	UP_HD void precipitation(TileD &t) const { // :59-80
		float p = saturatef(n(NS_PRECIP, t.position) * 0.5f + 0.5f);
		p = smootherstepf(smootherstepf(p));
		p = powf(fmaxf(p + 0.2f, 0.f), 3.f) * 0.6f * 400.f;
		p += fmaxf(120.f - fabsf(t.elevation), 0.f) * 0.2f;
		t.precipitation = fmaxf(p, 0.f);
	}
	UP_HD void temperature(TileD &t) const { // :82-120
		float x = smoothstepf(saturatef(n(NS_TEMP, t.position) * 0.5f + 0.5f)) * 2.f - 1.f;
		if (M.poles) {
			float polar = fabsf(atanf(t.position.y / sqrtf(t.position.x * t.position.x + t.position.z * t.position.z))) / 3.14159265358979f * 2.f;
			polar = powf(polar, 1.7f) + n(NS_POLAR, t.position) * 0.1f;
			x += 0.6f - polar * 3.2f;
		}
		t.temperature = 15.f + x * 30.f - fmaxf(t.elevation, 0.f) * 0.02f;
	}
	UP_HD void slope(TileD &t) const { // :122-151
		V3f a = any_perpendicular(t.normal);
		V3f b = cross(t.normal, a);
		a *= 0.5f;
		b *= 0.5f;
		const float div = 0.70710678118654752f;
		const V3f c = (a + b) * div, d = (a - b) * div;
		const V3f taps[8] = {t.position + a, t.position + b, t.position - a, t.position - b, t.position + c, t.position + d, t.position - c, t.position - d};
		float e1 = sdf_elev(taps[0]), e2 = e1;
		#pragma unroll 1
		for (int i = 1; i < 8; i++) {
			const float e = sdf_elev(taps[i]);
			e1 = fminf(e1, e);
			e2 = fmaxf(e2, e);
		}
		t.slope = atanf((e2 - e1) * 0.1f / 0.5f);
	}
	UP_HD static void biome(TileD &t) { // :153-190
		const float e = t.elevation, tp = t.temperature, pr = t.precipitation;
		if (e < 0.f) t.biome = 11;
		else if (tp > 20.f) t.biome = pr < 40.f ? 7 : (pr < 130.f ? 8 : (pr < 230.f ? 9 : 10));
		else if (tp > 5.f) t.biome = pr < 30.f ? 3 : (pr < 100.f ? 4 : (pr < 200.f ? 5 : 6));
		else if (tp > -5.f) t.biome = pr < 30.f ? 0 : 2;
		else t.biome = pr < 10.f ? 0 : 1;
	}
	UP_HD static void type(TileD &t) { // :192-200
		if (t.elevation < 0.f) t.type = 4;
		else if (t.slope > 0.3490658503988659f) t.type = 3;
		else t.type = 1;
	}
	UP_HD void bedrock(TileD &t) const { // :202-261
		const float dn = n(NS_BED_DEPTH, t.position) * 0.5f + 0.501f;
		const float depth = dn * dn * 2.f;
		const float freq = n(NS_BED_FREQ, t.position) * 0.15f + 1.f;
		const float cracks = saturatef(powf(n(NS_BED_CRACKS, t.position * freq) * 0.5f + 0.5f, 0.7f));
		const float value = n(NS_BED_VALUE, t.position * freq);
		const float sat = saturatef(n(NS_BED_SAT, t.position) * 0.35f + 0.3f);
		t.albedo = hsv_to_rgb(v3(0.07f, sat, saturatef(value * 0.1f + 0.7f) * (cracks * 0.4f + 0.6f)));
		t.roughness = lerpf(0.9f, value * -0.15f + 0.65f, cracks);
		t.height = cracks * depth;
	}
	UP_HD void cliffs(TileD &t) const { // :263-293
		const float bf = steep_mask(t.slope, 19.f, 4.f);
		if (bf > 0.99999f) return;
		V3f hsv = rgb_to_hsv(t.albedo);
		hsv.x = lerpf(155.f / 255.f, hsv.x, sharpf(bf, 0.005f));
		hsv.y *= bf * 0.4f + 0.6f;
		hsv.z = lerpf(0.7f, hsv.y, bf * 0.8f + 0.2f);
		t.albedo = hsv_to_rgb(hsv);
		t.roughness *= bf * 0.2f + 0.8f;
		const float cr = sharpf(saturatef(n(NS_CLIFF_CRACKS, t.position) * 2.f - 1.1f), 0.2f);
		t.height *= lerpf(1.f, 0.8f, cr);
		t.albedo *= lerpf(1.f, 0.9f, cr);
		t.roughness = lerpf(t.roughness, 0.9f, cr);
	}
	UP_HD void mica(TileD &t) const { // :295-336
		if (!M.flowers) return;
		const float bf = saturatef((n(NS_MICA_MASK, t.position) - 0.98f) * 10.f);
		if (bf < 1e-7f) return;
		const float cr = sharpf(saturatef(n(NS_MICA_CRACKS, t.position) + 0.6f));
		const V3f color = vlerp(v3(122.f / 255.f, 90.f / 255.f, 88.f / 255.f), v3(184.f / 255.f, 209.f / 255.f, 187.f / 255.f), cr);
		t.albedo = vlerp(t.albedo, color, bf);
		t.roughness = lerpf(t.roughness, cr * 0.3f + 0.4f, bf);
		t.metallic = lerpf(t.metallic, 1.f, bf);
		t.height = lerpf(t.height, t.height * 0.5f, bf);
	}
	UP_HD void dirt(TileD &t) const { // :338-402
		float height = n(NS_DIRT_HEIGHT, t.position) * 0.2f + 0.5f;
		const float bf = sharpf(saturatef(height - t.height + 0.4f)) * steep_mask(t.slope, 20.f, 5.f);
		if (bf < 1e-7f) return;
		V3f hsv = rgb_to_hsv(v3(168.f / 255.f, 94.f / 255.f, 28.f / 255.f));
		hsv.y *= range_mask(t.precipitation, 0.f, 50.f) * 0.7f;
		hsv.z *= 0.8f;
		V3f color = hsv_to_rgb(hsv);
		float roughness = 0.8f;
		float cr = sharpf(saturatef(n(NS_DIRT_CRACKS, t.position) * 2.f - 1.2f), 0.15f);
		const float cm = smoothstepf(saturatef(n(NS_DIRT_CMASK, t.position) * 0.5f + 0.5f));
		cr *= cm * cm * 0.9f + 0.1f;
		cr *= range_mask(t.precipitation, 70.f, 20.f) * 0.9f + 0.1f;
		height = lerpf(height, height * 0.5f, cr);
		color = vlerp(color, v3(0.1f, 0.1f, 0.1f), cr);
		roughness = lerpf(roughness, 0.9f, cr);
		t.albedo = vlerp(t.albedo, color, bf);
		t.roughness = lerpf(t.roughness, roughness, bf);
		t.metallic = lerpf(t.metallic, 0.f, bf);
		t.height = lerpf(t.height, height, bf);
	}
	UP_HD void sand(TileD &t) const { // :404-465
		const float bf = range_mask(t.temperature, 24.f, 28.f) * steep_mask(t.slope, 19.f, 10.f);
		if (bf < 1e-7f) return;
		const float hs = n(NS_SAND_HSCALE, t.position) * 0.3f + 1.f;
		const float height = (n(NS_SAND_HEIGHT, t.position * hs) * 0.2f) * (range_mask(t.precipitation, 100.f, 50.f) * 0.4f + 0.6f) + 0.5f;
		const float cs = smootherstepf(smootherstepf(n(NS_SAND_COLOR, t.position) * 0.5f + 0.5f));
		const float hue = n(NS_SAND_HUE, t.position) * 0.1f;
		V3f color = color_hue_shift(v3(189.f / 255.f, 174.f / 255.f, 152.f / 255.f), hue);
		color = interpolate_color(color, v3(187.f / 255.f, 104.f / 255.f, 50.f / 255.f), cs);
		color = color_deviation(M, color, 0.08f, t.position);
		const V3f hsv = rgb_to_hsv(color);
		color = hsv_to_rgb(v3(hsv.x, hsv.y * 0.7f, hsv.z * 0.8f));
		t.albedo = vlerp(t.albedo, color, bf);
		t.roughness = lerpf(t.roughness, (hs - 1.f) * 0.7f + 0.55f + hue, bf);
		t.metallic = lerpf(t.metallic, 0.f, bf);
		t.height = lerpf(t.height, height, bf);
	}
	UP_HD void grass(TileD &t) const { // :467-533
		const float bf = range_mask(t.temperature, 35.f, 25.f) * range_mask(t.precipitation, 15.f, 35.f) * steep_mask(t.slope, 22.f, 3.f) * beach(t);
		if (bf < 1e-7f) return;
		const float dryness = fminf(fmaxf(t.temperature - (t.precipitation + 100.f) * 30.f / 400.f, 0.f), 5.f) / 5.f;
		const float hb = n(NS_GRASS_HUE, t.position);
		V3f color = color_hue_shift(v3(114.f / 255.f, 187.f / 255.f, 77.f / 255.f), hb * 0.09f - dryness * 0.1f);
		const float pm = sharpf(n(NS_GRASS_PCELLS, t.position) * 0.5f + 0.2f);
		const float patches = powf(n(NS_GRASS_PDIST, t.position) * 0.5f + 0.5f, 0.5f) * pm * (1.f - dryness * 0.8f);
		color *= 1.f - patches * 0.09f;
		const float scratches = saturatef(n(NS_GRASS_SCRATCH, t.position) - 0.2f) * (1.f - dryness * 0.5f);
		color *= 1.f - scratches * 0.1f;
		const float roughness = 0.6f + dryness * 0.1f + patches * 0.1f + scratches * 0.1f - hb * 0.1f;
		const float height = lerpf(t.height, 0.5f, 0.7f) + (0.5f - dryness) * 0.2f + patches * 0.05f - scratches * 0.02f + hb * 0.1f + 0.1f;
		t.albedo = vlerp(t.albedo, color, bf);
		t.roughness = lerpf(t.roughness, roughness, bf);
		t.metallic = lerpf(t.metallic, 0.f, bf);
		t.height = lerpf(t.height, height, bf);
	}
	UP_HD void boulders(TileD &t) const { // :535-615
		if (!M.flowers) return;
		if (n(NS_BOUL_THRESH, t.position) < 0.15f) return;
		const V3S<float> c3 = voronoi_nearest(M.boulders, vs(t.position.x, t.position.y, t.position.z), &t.normal);
		const V3f center = v3(c3.x, c3.y, c3.z);
		const float dist = length(center - t.position);
		const float size = smootherstepf(smootherstepf(saturatef(n(NS_BOUL_SIZE, t.position) * 0.5f + 0.5f))) * 3.f + 3.f;
		const float bf = range_mask(size - dist, 0.f, 0.5f);
		if (bf < 1e-7f) return;
		V3f color = rgb_to_hsv(v3(154.f / 255.f, 154.f / 255.f, 154.f / 255.f));
		color.x = frac1(color.x + n(NS_BOUL_HUE, t.position) * 0.12f + 1.f);
		color.z = saturatef(color.z + n(NS_BOUL_VALUE, t.position) * 0.18f);
		color = hsv_to_rgb(color);
		const float q = dist / size;
		t.albedo = vlerp(t.albedo, color, bf);
		t.roughness = lerpf(t.roughness, n(NS_BOUL_SCRATCH, t.position) * 0.1f + 0.4f, bf);
		t.metallic = lerpf(t.metallic, 0.f, bf);
		t.height = lerpf(t.height, 1.f - q * q * 0.5f, bf);
	}
	UP_HD void water(TileD &t) const { // :617-656
		const float sw = n(NS_WATER_SWITCH, t.position) * 0.5f + 0.5f;
		const float hue = n(NS_WATER_HUE, t.position) * 0.09f;
		t.albedo = color_hue_shift(interpolate_color(v3(40.f / 255.f, 63.f / 255.f, 168.f / 255.f), v3(39.f / 255.f, 154.f / 255.f, 186.f / 255.f), sw), hue);
		const float r1 = range_mask(t.elevation, -25.f, 3.f);
		const float d2 = range_mask(t.elevation, 0.f, -100.f) * 0.3f + 0.7f;
		t.opacity = (1.f - r1 * r1) * d2;
		t.metallic = smoothstepf(range_mask(t.elevation, 3.f, -30.f));
	}
	UP_HD void flowers(TileD &t) const { // :658-744
		if (!M.flowers) return;
		const bool lily = t.purpose != UP_PURPOSE_LAND;
		if ((t.biome == 11) != lily) return;
		if (range_mask(fabsf(t.temperature - 18.f), 12.f, 7.f) < 1e-5f) return;
		if (!lily && range_mask(fabsf(t.precipitation - 200.f), 100.f, 70.f) < 1e-5f) return;
		const V3S<float> c3 = voronoi_nearest(M.flower_center, vs(t.position.x, t.position.y, t.position.z), &t.normal);
		const V3f center = v3(c3.x, c3.y, c3.z);
		if (dot(center - t.position, center - t.position) > 16.f) return;
		const V3S<float> k3 = voronoi_nearest(M.flower_cluster, vs(t.position.x, t.position.y, t.position.z), &t.normal);
		const V3f cluster = v3(k3.x, k3.y, k3.z);
		if (dot(center - cluster, center - cluster) > 400.f) return;
		const float dist = length(center - t.position);
		const float size = smootherstepf(smootherstepf(saturatef(n(NS_FLOW_SIZE, t.position) * 0.5f + 0.5f))) * 2.f + 1.5f;
		const float bf = range_mask(size - dist, 0.f, 0.1f);
		if (bf < 1e-7f) return;
		const V3f base = lily ? v3(0.2f, 0.14f, 0.f) : interpolate_color(v3(0.5f, 0.f, 0.35f), v3(0.5f, 0.4f, 0.f), sharpf(n(NS_FLOW_COLOR, cluster) + 0.4f, 0.2f));
		const V3f color = color_hue_shift(base, n(NS_FLOW_HUE1, t.position) * 0.1f + n(NS_FLOW_HUE2, t.position) * 0.1f);
		const float q = dist / size;
		t.albedo = vlerp(t.albedo, color, bf);
		t.roughness = lerpf(t.roughness, 0.8f, bf);
		t.metallic = lerpf(t.metallic, lily ? 0.85f : 0.f, bf);
		t.height = lerpf(t.height, 0.7f + q * q * 0.2f, bf);
		t.opacity = lerpf(t.opacity, 1.f, bf);
	}
	UP_HD void ice(TileD &t) const { // :746-817
		const float off = n(NS_ICE_TEMPOFF, t.position) * 1.5f;
		const float bf = sharpf(range_mask(t.temperature + off, 0.f, -3.f)) * (1.f - beach(t));
		if (bf < 1e-7f) return;
		if (bf > 0.1f && t.type != 3) t.type = 2;
		const float freq = n(NS_ICE_FREQ, t.position) * 0.08f + 1.f;
		const float thick = sharpf(saturatef(n(NS_ICE_THICK, t.position * freq) * 0.5f + 0.8f), 0.1f) * 0.6f + 0.4f;
		const float crack = 1.f - powf(n(NS_ICE_CRACKS, t.position * freq) * 0.5f + 0.5f, 0.3f);
		V3f color = v3(fmaxf(122.f / 255.f - crack * 0.3f, 0.f), fmaxf(162.f / 255.f - crack * 0.3f, 0.f), fmaxf(164.f / 255.f - crack * 0.3f, 0.f));
		color = interpolate_color(t.albedo, color, thick);
		const float roughness = lerpf(t.roughness, 0.15f + crack * 0.6f, thick);
		t.albedo = vlerp(t.albedo, color, bf);
		t.roughness = lerpf(t.roughness, roughness, bf);
		t.metallic = lerpf(t.metallic, 0.f, bf);
		t.height = lerpf(t.height, thick * 0.5f * (1.f - crack * 0.8f), bf);
		t.opacity = lerpf(t.opacity, t.opacity * 0.9f + thick * 0.5f, bf);
	}
	UP_HD void snow(TileD &t) const { // :819-855
		float bf = sharpf(range_mask(t.elevation + n(NS_SNOW_ELEVOFF, t.position) * 20.f, 220.f, 240.f) * steep_mask(t.slope, 25.f, 5.f));
		const float thick = n(NS_SNOW_THICK, t.position) * 0.5f + 0.5f;
		bf *= saturatef(thick * 0.5f + 0.7f);
		if (bf < 1e-7f) return;
		t.albedo = vlerp(t.albedo, v3(230.f / 255.f, 230.f / 255.f, 230.f / 255.f), bf);
		t.roughness = lerpf(t.roughness, thick * 0.3f + 0.2f, bf);
		t.metallic = lerpf(t.metallic, 0.f, bf);
		t.height = lerpf(t.height, 0.6f + t.height * 0.1f + thick * 0.3f, bf);
	}
	UP_HD static void visualization(TileD &t) { // :857-893
		const unsigned char C[12][3] = {{187, 187, 187}, {175, 226, 255}, {193, 225, 221}, {200, 110, 62}, {239, 252, 143}, {151, 183, 102},
			{118, 169, 92}, {221, 187, 76}, {253, 213, 120}, {161, 151, 0}, {50, 122, 30}, {0, 0, 255}};
		if (t.biome >= 0 && t.biome < 12) t.albedo = v3(C[t.biome][0] / 255.f, C[t.biome][1] / 255.f, C[t.biome][2] / 255.f);
		else t.albedo = v3(NAN, NAN, NAN);
		t.roughness = 0.7f;
	}
	UP_HD static void finalization(TileD &t) { // :895-902
		t.albedo = vsat3(t.albedo);
		t.roughness = saturatef(t.roughness);
		t.metallic = saturatef(t.metallic);
		t.height = saturatef(t.height);
		t.opacity = saturatef(t.opacity);
	}
	UP_HD void pipeline(TileD &t) const {
		if (M.coloring == 0) { // coloringDefault :905-930
			elevation(t); precipitation(t); temperature(t); slope(t); biome(t); type(t);
			if (t.purpose == UP_PURPOSE_WATER) water(t);
			else { bedrock(t); cliffs(t); mica(t); dirt(t); sand(t); grass(t); boulders(t); }
			flowers(t); ice(t);
			if (t.purpose != UP_PURPOSE_WATER) snow(t);
		} else if (M.coloring == 1) { // coloringBarren :932-952
			elevation(t); slope(t);
			if (t.purpose == UP_PURPOSE_WATER) { t.biome = 11; t.type = 4; water(t); }
			else { t.biome = 0; t.type = 1; bedrock(t); cliffs(t); mica(t); boulders(t); }
		} else { // coloringDebug :954-966
			elevation(t); precipitation(t); temperature(t); slope(t); biome(t); type(t); visualization(t);
			if (t.purpose == UP_PURPOSE_WATER) t.opacity = 0.5f;
		}
		finalization(t);
	}
};

// the three pipelines, out of line (one copy per translation unit)
UP_HD_NOINLINE void color_tile(const ModesDesc &M, TileD &t) { Colorer{M}.pipeline(t); }

// synthetic texel program: albedo from 3-octave value noise (freq 4),
// roughness from 2-octave simplex noise (freq 8), height = 0.5 + elevation /
// (2 sum|amp|); seeds offset from the first layer's seed by 100 and 200.
// T0/T1: compile-time noise type of layer 0/1 (noise_t; -1 = run time)
template<int T0 = -1, int T1 = -1>
UP_HD void synth_texel(const up_synth_program &P, V3f p, V3f &albedo, float &rough, float &height) {
	const uint32_t s0 = P.n_layers > 0 ? P.layer[0].seed : 0u;
	float a = 0.f, r = 0.f;
	float amp = 1.f / 1.75f, f = 4.f;
	#pragma unroll 1
	for (int i = 0; i < 3; i++) { a += value_v(p * f, seed_key(s0 + 100u + (uint32_t)i)) * amp; amp *= 0.5f; f *= 2.f; }
	amp = 1.f / 1.5f; f = 8.f;
	#pragma unroll 1
	for (int i = 0; i < 2; i++) { r += simplex_n<false, false>(p * f, seed_key(s0 + 200u + (uint32_t)i)).v * amp; amp *= 0.5f; f *= 2.f; }
	albedo = vlerp(v3(0.35f, 0.27f, 0.18f), v3(0.72f, 0.66f, 0.52f), saturatef(a * 0.5f + 0.5f));
	rough = saturatef(r * 0.5f + 0.5f);
	float tot = 0.f, e = 0.f;
	for (int l = 0; l < P.n_layers; l++) {
		const up_noise_layer &L = P.layer[l];
		#pragma unroll 1
		for (int i = 0; i < L.octaves; i++) {
			tot += fabsf(L.amp[i]);
			const uint32_t key = seed_key(L.seed + (uint32_t)i);
			float v = l == 0 ? noise_t<false, T0>(L, p * L.freq[i], key).v : noise_t<false, T1>(L, p * L.freq[i], key).v;
			if (L.fractal == UP_FRACTAL_RIDGED) v = 1.f - 2.f * fabsf(v);
			e += v * L.amp[i];
		}
	}
	height = saturatef(0.5f + e / (2.f * (tot > 0.f ? tot : 1.f)));
}

} // namespace up
