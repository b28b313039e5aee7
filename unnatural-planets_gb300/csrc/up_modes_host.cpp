// Host side of mode selection: resolves the reference's mode names and
// expands every NoiseFunction / Voronoi configuration of the reference into
// a ModesDesc. Replaces chooseShapeFunction / chooseElevationFunction /
// chooseColoringFunction (sources/modesConfiguration.cpp:38-226) and the lazy
// static noise construction in sdf.cpp, elevationModes.cpp and
// coloringModes.cpp (configurations cited per instance below).
#include "up_modes_desc.h"
#include "up_noise.cuh"
#include "up_synth.cuh"
#include "../../include/up_abi.h"

#include <cmath>
#include <cstring>
#include <string>

namespace up {

const char *const kShapeNames[34] = {"asteroid", "belt", "bowl", "box", "bunny", "capsule", "cube", "disk", "doubletorus", "fibers",
	"gear", "h2o", "h3o", "h4o", "hemispheres", "hexagon", "hexagonalprism", "insidecube", "knot", "mandelbulb", "mobiusstrip",
	"monkeyhead", "octahedron", "pipe", "sphere", "square", "tetrahedron", "torus", "toruscross", "triangularprism", "tube",
	"twistedhexagonalprism", "twistedplane", "wormhole"};
const char *const kElevationNames[6] = {"none", "simple", "legacy", "lakes", "islands", "craters"};
const char *const kColoringNames[3] = {"default", "barren", "debug"};

uint32_t instance_seed(uint32_t seed, uint32_t slot) { return mix32(seed + 0x9E3779B9U * (slot + 1U)); }

namespace {

struct Cfg {
	int type = UP_NOISE_SIMPLEX, fractal = UP_FRACTAL_NONE, octaves = 3, dist = UP_DIST_EUCLIDEAN, op = UP_OP_DISTANCE;
	double frequency = 1, lacunarity = 2, gain = 0.5;
	uint32_t seed = 0;
};

// fractal expansion: f_i = f lac^i, a_i = gain^i / sum_j |gain|^j (FBM/ridged)
NoiseDev expand(const Cfg &c) {
	NoiseDev n;
	std::memset(&n, 0, sizeof(n));
	n.type = (int8_t)c.type; n.fractal = (int8_t)c.fractal; n.dist = (int8_t)c.dist; n.op = (int8_t)c.op;
	n.octaves = c.fractal == UP_FRACTAL_NONE ? 1 : (c.octaves < 1 ? 1 : (c.octaves > 8 ? 8 : c.octaves));
	n.seed = c.seed;
	double bound = 0, g = 1;
	for (int i = 0; i < n.octaves; i++) { bound += std::fabs(g); g *= c.gain; }
	double f = c.frequency;
	g = 1;
	for (int i = 0; i < n.octaves; i++) {
		n.freq[i] = (float)f;
		n.amp[i] = c.fractal == UP_FRACTAL_NONE ? 1.f : (float)(g / bound);
		f *= c.lacunarity;
		g *= c.gain;
	}
	return n;
}

Cfg mk(int type, double freq, uint32_t seed, int fractal = UP_FRACTAL_NONE, int octaves = 3, double gain = 0.5, double lac = 2.0) {
	Cfg c;
	c.type = type; c.frequency = freq; c.seed = seed; c.fractal = fractal; c.octaves = octaves; c.gain = gain; c.lacunarity = lac;
	return c;
}
Cfg mkcell(double freq, uint32_t seed, int dist, int op, int fractal = UP_FRACTAL_NONE, int octaves = 3) {
	Cfg c = mk(UP_NOISE_CELLULAR, freq, seed, fractal, octaves);
	c.dist = dist; c.op = op;
	return c;
}

// voronoi.cpp:17 seedHashes; h = the project hash mix32
VoronoiDev voronoi(uint32_t seed, double cell, int ppc) {
	VoronoiDev v;
	const uint32_t h1 = mix32(seed), h2 = mix32(h1), h3 = mix32(h2);
	v.seed_hash[0] = (int32_t)h1; v.seed_hash[1] = (int32_t)h2; v.seed_hash[2] = (int32_t)h3;
	v.cell_size = (float)cell;
	v.frequency = (float)(1.0 / cell);
	v.points_per_cell = ppc;
	return v;
}

// uniform [0,1) from a slot seed and a draw index
double unit_draw(uint32_t seed, uint32_t i) { return (mix32(seed ^ (0x85EBCA6BU * (i + 1U))) >> 8) * (1.0 / 16777216.0); }

} // namespace

// returns UP_OK or UP_ERR_INVALID_MODE with err filled
// |noise_dev(n)| <= this everywhere: the per-type bound (noise_abs_bound)
// times the sum of |amplitudes|, through 1 - 2|v| for ridged octaves
static double noise_dev_bound(const NoiseDev &n) {
	const double nm = noise_abs_bound(n.type, n.dist, n.op);
	const double sm = n.fractal == UP_FRACTAL_RIDGED ? std::fmax(1.0, 2.0 * nm - 1.0) : nm;
	double b = 0;
	for (int i = 0; i < n.octaves; i++) b += std::fabs((double)n.amp[i]) * sm;
	return b;
}

// Range [lo, hi] of the elevation of the planet's mode (elevation_eval in
// up_modes.cuh, elevationModes.cpp), from the noise bounds:
//  none: 100; simple: 100 - 1000 ((0.3 - n) 1.3 - 0.35)^3 - 100, monotone in n;
//  legacy: 2500 g(n + 0.11), g(a) = -(-a)^0.85 or a^1.7, monotone;
//  lakes/islands: land = 150 (x / (|x| + 0.17) + 0.15), |x| <= 1, plus the
//    mountains, >= 0 and <= max(1000 (r - 0.1)^1.6, 250 (2.5 (t + 0.1) + 1))
//    + 50 / 4 (smooth max over max; terrace(x) <= x + 1);
//  craters: 200 + 190 h, h = 10 (x^4 - 0.9 x^5 - 0.1) in [-1, 0.25] for x in [0, 1].
void elevation_range(const ModesDesc &D, double &lo, double &hi) {
	switch (D.elevation) {
		case 0: lo = hi = 100.0; return;
		case 1: {
			const double b = noise_dev_bound(D.elev[NS_SIMPLE]);
			const double t0 = (0.3 - b) * 1.3 - 0.35, t1 = (0.3 + b) * 1.3 - 0.35;
			lo = 100.0 - (t1 * t1 * t1 + 0.1) * 1000.0;
			hi = 100.0 - (t0 * t0 * t0 + 0.1) * 1000.0;
			return;
		}
		case 2: {
			const double b = noise_dev_bound(D.elev[NS_LEGACY_ELEV]);
			auto g = [](double a) { return a < 0 ? -std::pow(-a, 0.85) : std::pow(a, 1.7); };
			lo = g(0.11 - b) * 2500.0;
			hi = g(0.11 + b) * 2500.0;
			return;
		}
		case 3: case 4: {
			const double x = 1.0 / 1.17;
			const double ridge = std::pow(std::fmax(noise_dev_bound(D.elev[NS_MTN_RIDGE]) - 0.1, 0.0), 1.6) * 1000.0;
			const double terr = (std::fmax(noise_dev_bound(D.elev[NS_MTN_TERRACE]) + 0.1, 0.0) * 2.5 + 1.0) * 250.0;
			lo = (-x + 0.15) * 150.0;
			hi = (x + 0.15) * 150.0 + std::fmax(ridge, terr) + 12.5;
			return;
		}
		default: lo = 10.0; hi = 200.0 + 0.25 * 190.0; return;
	}
}

// Narrow band of contouring a reference-mode field (see contour_band in
// up_sdf.cu for the argument): the land field is shape - elevation / 10 and
// navigation shape - max(elevation / 10, 0), so where |shape| exceeds the
// bound of that term plus the longest grid step, the field has the sign of
// the shape, and so do its grid neighbours, provided the shape is
// 1-Lipschitz. That holds for the exact distance functions and their smooth
// unions, isometries and uniform scalings listed here (sdf.cpp); the other
// shapes (noise, sine networks, twists, folds, polar repetition, the
// Mandelbulb estimator) take no band. Returns 0 for no band.
float modes_contour_band(const ModesDesc &D, int field, const float step[3]) {
	static const int kLipschitz[] = {2, 3, 5, 6, 7, 8, 11, 12, 13, 15, 17, 22, 24, 25, 26, 27, 28, 30};
	bool ok = false;
	for (int s : kLipschitz) ok = ok || D.shape == s;
	if (!ok || (field != UP_FIELD_LAND && field != UP_FIELD_NAVIGATION)) return 0.f;
	double lo, hi;
	elevation_range(D, lo, hi);
	const double B = field == UP_FIELD_LAND ? std::fmax(std::fabs(lo), std::fabs(hi)) * 0.1 : std::fmax(hi, 0.0) * 0.1;
	const double st = std::fmax(step[0], std::fmax(step[1], step[2]));
	const double band = (B + st) * 1.001 + 0.01;
	return std::isfinite(band) ? (float)band : 0.f;
}

int build_modes(const up_modes &m, uint32_t seed, ModesDesc &D, std::string &shape_name, bool &double_sided, std::string &err) {
	std::memset(&D, 0, sizeof(D));
	auto S = [&](uint32_t slot) { return instance_seed(seed, slot); };
	const std::string shape = m.shape ? m.shape : "";
	const std::string elev = m.elevation ? m.elevation : "";
	const std::string col = m.coloring ? m.coloring : "";
	D.shape = -1;
	if (shape == "random") {
		// modesConfiguration.cpp:119-125: uniform pick among the 34 shapes
		D.shape = (int)(unit_draw(S(90), 0) * 34.0);
		if (D.shape > 33) D.shape = 33;
	} else {
		for (int i = 0; i < 34; i++) if (shape == kShapeNames[i]) D.shape = i;
	}
	if (D.shape < 0) { err = "unknown shape mode configuration: '" + shape + "'"; return UP_ERR_INVALID_MODE; }
	shape_name = kShapeNames[D.shape];
	D.elevation = -1;
	for (int i = 0; i < 6; i++) if (elev == kElevationNames[i]) D.elevation = i;
	if (D.elevation < 0) { err = "unknown elevation mode configuration: '" + elev + "'"; return UP_ERR_INVALID_MODE; }
	D.coloring = -1;
	for (int i = 0; i < 3; i++) if (col == kColoringNames[i]) D.coloring = i;
	if (D.coloring < 0) { err = "unknown coloring mode configuration: '" + col + "'"; return UP_ERR_INVALID_MODE; }
	D.poles = m.poles ? 1 : 0;
	D.flowers = m.flowers ? 1 : 0;
	// modesConfiguration.cpp:139-160
	static const char *const ds[] = {"belt", "bowl", "hemispheres", "hexagon", "insidecube", "square", "tube", "twistedplane", "wormhole"};
	double_sided = false;
	for (const char *n : ds) if (shape_name == n) double_sided = true;

	// random draws of sdf.cpp:133 and :342
	for (int a = 0; a < 3; a++) D.fibers_offset[a] = (float)(unit_draw(S(XS_FIBERS_OFFSET), a) * 200.0 - 100.0);
	const double asteroid_freq = 0.65 + 0.1 * unit_draw(S(XS_ASTEROID_FREQ), 0);
	D.deviation_key = S(XS_COLOR_DEVIATION);

	// sdf.cpp:335-345
	D.elev[NS_ASTEROID] = expand(mk(UP_NOISE_SIMPLEX, asteroid_freq, S(NS_ASTEROID), UP_FRACTAL_FBM, 2, 0.3));
	// elevationModes.cpp
	D.elev[NS_SIMPLE] = expand(mk(UP_NOISE_SIMPLEX, 0.0005, S(NS_SIMPLE), UP_FRACTAL_RIDGED, 6, 0.4));        // :16-26
	D.elev[NS_LEGACY_SCALE] = expand(mk(UP_NOISE_VALUE, 0.0005, S(NS_LEGACY_SCALE), UP_FRACTAL_FBM, 4));       // :36-45
	D.elev[NS_LEGACY_ELEV] = expand(mk(UP_NOISE_VALUE, 1.0, S(NS_LEGACY_ELEV), UP_FRACTAL_FBM, 4));            // :46-54
	D.elev[NS_MTN_MASK] = expand(mk(UP_NOISE_PERLIN, 0.0015, S(NS_MTN_MASK)));                                 // :70-77
	D.elev[NS_MTN_RIDGE] = expand(mk(UP_NOISE_SIMPLEX, 0.001, S(NS_MTN_RIDGE), UP_FRACTAL_RIDGED, 4, -0.4, 1.5)); // :78-89
	D.elev[NS_MTN_TERRACE] = expand(mk(UP_NOISE_PERLIN, 0.002, S(NS_MTN_TERRACE), UP_FRACTAL_FBM, 3, 0.3));    // :90-100
	D.elev[NS_LAKES_LAND] = expand(mk(UP_NOISE_VALUE, 0.0013, S(NS_LAKES_LAND), UP_FRACTAL_FBM, 4));           // :131-140
	D.elev[NS_ISLANDS_LAND] = expand(mk(UP_NOISE_VALUE, 0.0013, S(NS_ISLANDS_LAND), UP_FRACTAL_FBM, 4));       // :153-162
	D.elev[NS_CRATERS_SCALE] = expand(mk(UP_NOISE_VALUE, 1.0, S(NS_CRATERS_SCALE)));                           // :183-190
	D.craters = voronoi(S(XS_CRATERS_VORONOI), 300, 2);                                                        // :175-182

	// coloringModes.cpp
	const uint32_t bed = S(XS_SHARED_BEDROCK), grass = S(XS_SHARED_GRASS), ice = S(XS_SHARED_ICE);
	NoiseDev *C = D.color - N_ELEV_NOISE; // index by NoiseSlot
	C[NS_BEACH] = expand(mk(UP_NOISE_VALUE, 0.035, S(NS_BEACH)));                                              // :36-43
	C[NS_PRECIP] = expand(mk(UP_NOISE_CUBIC, 0.001, S(NS_PRECIP), UP_FRACTAL_FBM, 2));                          // :61-70
	C[NS_TEMP] = expand(mk(UP_NOISE_SIMPLEX, 0.0003, S(NS_TEMP), UP_FRACTAL_FBM, 2, 0.4));                      // :84-94
	C[NS_POLAR] = expand(mk(UP_NOISE_VALUE, 0.007, S(NS_POLAR), UP_FRACTAL_FBM, 3));                            // :95-104
	C[NS_BED_DEPTH] = expand(mk(UP_NOISE_CUBIC, 0.0031, S(NS_BED_DEPTH)));                                     // :205-212
	C[NS_BED_FREQ] = expand(mk(UP_NOISE_CUBIC, 0.013, S(NS_BED_FREQ)));                                        // :213-220
	C[NS_BED_CRACKS] = expand(mkcell(0.017, bed, UP_DIST_HYBRID, UP_OP_SUBTRACT));                             // :221-230
	C[NS_BED_VALUE] = expand(mkcell(0.017, bed, UP_DIST_HYBRID, UP_OP_CELL));                                  // :231-240
	C[NS_BED_SAT] = expand(mk(UP_NOISE_CUBIC, 0.0022, S(NS_BED_SAT), UP_FRACTAL_FBM, 2));                       // :241-250
	C[NS_CLIFF_CRACKS] = expand(mk(UP_NOISE_SIMPLEX_REDUCED, 0.047, S(NS_CLIFF_CRACKS), UP_FRACTAL_RIDGED, 2)); // :265-274
	C[NS_MICA_MASK] = expand(mkcell(0.02, S(NS_MICA_MASK), UP_DIST_HYBRID, UP_OP_MULTIPLY));                   // :297-306
	C[NS_MICA_CRACKS] = expand(mkcell(0.05, S(NS_MICA_CRACKS), UP_DIST_MANHATTAN, UP_OP_DIVIDE));              // :307-317
	C[NS_DIRT_HEIGHT] = expand(mk(UP_NOISE_PERLIN, 0.05, S(NS_DIRT_HEIGHT), UP_FRACTAL_FBM, 3, 0.4, 2.3));      // :340-351
	C[NS_DIRT_CRACKS] = expand(mk(UP_NOISE_SIMPLEX_REDUCED, 0.07, S(NS_DIRT_CRACKS), UP_FRACTAL_RIDGED, 2));   // :352-361
	C[NS_DIRT_CMASK] = expand(mk(UP_NOISE_CUBIC, 0.02, S(NS_DIRT_CMASK), UP_FRACTAL_FBM, 4));                   // :362-371
	C[NS_SAND_HSCALE] = expand(mk(UP_NOISE_SIMPLEX, 0.001, S(NS_SAND_HSCALE), UP_FRACTAL_FBM, 3));             // :406-415
	C[NS_SAND_HEIGHT] = expand(mk(UP_NOISE_SIMPLEX, 0.01, S(NS_SAND_HEIGHT), UP_FRACTAL_RIDGED, 3, 0.7));      // :416-426
	C[NS_SAND_COLOR] = expand(mk(UP_NOISE_PERLIN, 0.0008, S(NS_SAND_COLOR)));                                  // :427-433
	C[NS_SAND_HUE] = expand(mk(UP_NOISE_CUBIC, 0.02, S(NS_SAND_HUE), UP_FRACTAL_FBM, 2));                       // :435-444
	C[NS_GRASS_HUE] = expand(mk(UP_NOISE_PERLIN, 0.01, S(NS_GRASS_HUE), UP_FRACTAL_FBM, 2));                    // :470-479
	C[NS_GRASS_PCELLS] = expand(mkcell(0.1, grass, UP_DIST_HYBRID, UP_OP_CELL));                               // :480-489
	C[NS_GRASS_PDIST] = expand(mkcell(0.1, grass, UP_DIST_HYBRID, UP_OP_SUBTRACT));                            // :490-499
	C[NS_GRASS_SCRATCH] = expand(mkcell(0.3, S(NS_GRASS_SCRATCH), UP_DIST_HYBRID, UP_OP_MULTIPLY));            // :500-509
	C[NS_BOUL_THRESH] = expand(mk(UP_NOISE_PERLIN, 0.01, S(NS_BOUL_THRESH)));                                  // :537-544
	C[NS_BOUL_SIZE] = expand(mk(UP_NOISE_PERLIN, 0.09, S(NS_BOUL_SIZE)));                                      // :553-560
	C[NS_BOUL_HUE] = expand(mk(UP_NOISE_PERLIN, 0.3, S(NS_BOUL_HUE)));                                         // :561-567
	C[NS_BOUL_VALUE] = expand(mk(UP_NOISE_PERLIN, 0.5, S(NS_BOUL_VALUE)));                                     // :569-576
	C[NS_BOUL_SCRATCH] = expand(mk(UP_NOISE_PERLIN, 0.5, S(NS_BOUL_SCRATCH)));                                 // :577-584
	C[NS_WATER_SWITCH] = expand(mk(UP_NOISE_PERLIN, 0.0015, S(NS_WATER_SWITCH), UP_FRACTAL_FBM, 2));            // :619-628
	C[NS_WATER_HUE] = expand(mk(UP_NOISE_CUBIC, 0.004, S(NS_WATER_HUE), UP_FRACTAL_FBM, 3));                    // :629-638
	C[NS_FLOW_SIZE] = expand(mk(UP_NOISE_PERLIN, 0.35, S(NS_FLOW_SIZE)));                                      // :674-681
	C[NS_FLOW_COLOR] = expand(mk(UP_NOISE_PERLIN, 0.02, S(NS_FLOW_COLOR)));                                    // :682-689
	C[NS_FLOW_HUE1] = expand(mk(UP_NOISE_PERLIN, 0.005, S(NS_FLOW_HUE1)));                                     // :690-697
	C[NS_FLOW_HUE2] = expand(mk(UP_NOISE_PERLIN, 0.4, S(NS_FLOW_HUE2)));                                       // :698-705
	C[NS_ICE_TEMPOFF] = expand(mk(UP_NOISE_VALUE, 0.035, S(NS_ICE_TEMPOFF)));                                  // :749-756
	C[NS_ICE_FREQ] = expand(mk(UP_NOISE_VALUE, 0.01, S(NS_ICE_FREQ), UP_FRACTAL_FBM, 3));                       // :757-766
	C[NS_ICE_THICK] = expand(mkcell(0.05, ice, UP_DIST_HYBRID, UP_OP_CELL, UP_FRACTAL_FBM, 2));                // :767-778
	C[NS_ICE_CRACKS] = expand(mkcell(0.05, ice, UP_DIST_HYBRID, UP_OP_SUBTRACT, UP_FRACTAL_FBM, 2));           // :779-790
	C[NS_SNOW_ELEVOFF] = expand(mk(UP_NOISE_VALUE, 0.055, S(NS_SNOW_ELEVOFF)));                                // :821-828
	C[NS_SNOW_THICK] = expand(mk(UP_NOISE_CUBIC, 0.05, S(NS_SNOW_THICK), UP_FRACTAL_FBM, 3));                   // :829-838
	D.boulders = voronoi(S(XS_BOUL_VORONOI), 200, 2);        // :545-552
	D.flower_cluster = voronoi(S(XS_FLOW_CLUSTER), 200, 1);  // :660-666
	D.flower_center = voronoi(S(XS_FLOW_CENTER), 35, 1);     // :667-673
	return UP_OK;
}

} // namespace up
