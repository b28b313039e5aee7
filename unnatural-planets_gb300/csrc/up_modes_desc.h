// Plain description of a reference-mode planet (shape, elevation and
// coloring modes with every noise instance expanded), built once on the host
// at context creation and passed by value to the kernels (kernel parameter
// space, read through the constant cache).
#pragma once
#include <stdint.h>

namespace up {

// one configured noise function (cage NoiseFunctionCreateConfig call sites)
// expanded into per-octave frequency/amplitude; octave i uses seed + i
struct NoiseDev {
	int8_t type, fractal, dist, op;
	int32_t octaves;
	uint32_t seed;
	float freq[8];
	float amp[8];
};

// sources/voronoi.cpp:10-91 configuration
struct VoronoiDev {
	int32_t seed_hash[3]; // (h(s), h(h(s)), h(h(h(s))))  voronoi.cpp:17
	float cell_size;
	float frequency;      // 1 / cellSize
	int32_t points_per_cell;
};

// Noise instance slots. The reference draws seeds from a global generator in
// lazy-initialisation order (math.cpp:73-77); here slot i of planet seed s
// gets up_instance_seed(s, i). Instances that share a seed in the reference
// (coloringModes.cpp:204,228,238; :469,487,497; :748,776,789) share a slot.
enum NoiseSlot {
	// sdf.cpp
	NS_ASTEROID = 0,              // sdf.cpp:335-345
	// elevationModes.cpp
	NS_SIMPLE,                    // :16-26
	NS_LEGACY_SCALE,              // :36-45
	NS_LEGACY_ELEV,               // :46-54
	NS_MTN_MASK,                  // :70-77
	NS_MTN_RIDGE,                 // :78-89
	NS_MTN_TERRACE,               // :90-100
	NS_LAKES_LAND,                // :131-140
	NS_ISLANDS_LAND,              // :153-162
	NS_CRATERS_SCALE,             // :183-190
	N_ELEV_NOISE,
	// coloringModes.cpp
	NS_BEACH = N_ELEV_NOISE,      // :36-43
	NS_PRECIP,                    // :61-70
	NS_TEMP,                      // :84-94
	NS_POLAR,                     // :95-104
	NS_BED_DEPTH,                 // :205-212
	NS_BED_FREQ,                  // :213-220
	NS_BED_CRACKS,                // :221-230 (shared seed :204)
	NS_BED_VALUE,                 // :231-240 (shared seed :204)
	NS_BED_SAT,                   // :241-250
	NS_CLIFF_CRACKS,              // :265-274
	NS_MICA_MASK,                 // :297-306
	NS_MICA_CRACKS,               // :307-317
	NS_DIRT_HEIGHT,               // :340-351
	NS_DIRT_CRACKS,               // :352-361
	NS_DIRT_CMASK,                // :362-371
	NS_SAND_HSCALE,               // :406-415
	NS_SAND_HEIGHT,               // :416-426
	NS_SAND_COLOR,                // :427-433
	NS_SAND_HUE,                  // :435-444
	NS_GRASS_HUE,                 // :470-479
	NS_GRASS_PCELLS,              // :480-489 (shared seed :469)
	NS_GRASS_PDIST,               // :490-499 (shared seed :469)
	NS_GRASS_SCRATCH,             // :500-509
	NS_BOUL_THRESH,               // :537-544
	NS_BOUL_SIZE,                 // :553-560
	NS_BOUL_HUE,                  // :561-567
	NS_BOUL_VALUE,                // :569-576
	NS_BOUL_SCRATCH,              // :577-584
	NS_WATER_SWITCH,              // :619-628
	NS_WATER_HUE,                 // :629-638
	NS_FLOW_SIZE,                 // :674-681
	NS_FLOW_COLOR,                // :682-689
	NS_FLOW_HUE1,                 // :690-697
	NS_FLOW_HUE2,                 // :698-705
	NS_ICE_TEMPOFF,               // :749-756
	NS_ICE_FREQ,                  // :757-766
	NS_ICE_THICK,                 // :767-778 (shared seed :748)
	NS_ICE_CRACKS,                // :779-790 (shared seed :748)
	NS_SNOW_ELEVOFF,              // :821-828
	NS_SNOW_THICK,                // :829-838
	N_NOISE_SLOTS
};
// Voronoi and random-draw slots (seed slots after the noise slots)
enum ExtraSlot {
	XS_CRATERS_VORONOI = 64,      // elevationModes.cpp:175-182
	XS_BOUL_VORONOI,              // coloringModes.cpp:545-552
	XS_FLOW_CLUSTER,              // coloringModes.cpp:660-666
	XS_FLOW_CENTER,               // coloringModes.cpp:667-673
	XS_FIBERS_OFFSET,             // sdf.cpp:133 randomRange3(-100, 100)
	XS_ASTEROID_FREQ,             // sdf.cpp:342 randomRange(0.65, 0.75)
	XS_COLOR_DEVIATION,           // math.cpp:40-45 randomChance3 per texel
	XS_SHARED_BEDROCK,            // coloringModes.cpp:204
	XS_SHARED_GRASS,              // coloringModes.cpp:469
	XS_SHARED_ICE                 // coloringModes.cpp:748
};

constexpr int N_COLOR_NOISE = N_NOISE_SLOTS - N_ELEV_NOISE;

struct ModesDesc {
	int32_t shape;       // index into the 34 shape names (modesConfiguration.cpp:79-114)
	int32_t elevation;   // index into the 6 elevation names (:176-183)
	int32_t coloring;    // index into the 3 coloring names (:208-212)
	int32_t poles, flowers;
	float fibers_offset[3];
	uint32_t deviation_key;
	NoiseDev elev[N_ELEV_NOISE];      // incl. NS_ASTEROID at index 0
	VoronoiDev craters;
	NoiseDev color[N_COLOR_NOISE];
	VoronoiDev boulders, flower_cluster, flower_center;
};

} // namespace up
