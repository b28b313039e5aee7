/*
 * up_abi.h -- C ABI of the GB300 planet SDF -> contour -> texel path.
 *
 * This header is the drop-in boundary for the data-parallel hot path of
 * unnatural-planets. Each entry point names the reference interface it
 * replaces (paths relative to the reference project). All calls:
 *   - have C linkage and never let a C++ exception cross the boundary;
 *   - return an int status (UP_OK == 0, else a UP_ERR_* code; the message of
 *     the last failure on a context is available from up_last_error);
 *   - take caller-owned buffers as plain pointers plus explicit sizes; each
 *     pointer may be host memory or device memory (the library inspects it
 *     with cudaPointerGetAttributes: device memory of the context's GPU and
 *     managed memory are used in place, host memory and memory of another
 *     GPU are copied through the context's own device scratch);
 *   - are re-entrant across contexts; one context serves one host thread or
 *     one CUDA stream at a time (the per-point shims make a copy per thread);
 *   - mark their span with an NVTX range named after the entry point.
 * Coordinates are FP32 in the reference's units. Grids are x-fastest:
 * index = (iz * ny + iy) * nx + ix.
 */
#ifndef UP_ABI_H
#define UP_ABI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UP_ABI_VERSION 1

/* ---------------------------------------------------------------- status */
enum up_status {
	UP_OK = 0,
	UP_ERR_INVALID_ARGUMENT = 1, /* null pointer, zero size, bad enum */
	UP_ERR_INVALID_MODE = 2,     /* unknown shape/elevation/coloring name
	                                (modesConfiguration.cpp:131-134,190-194,219-223) */
	UP_ERR_NAN = 3,              /* an SDF value was NaN ("invalid ... sdf value",
	                                modesConfiguration.cpp:234-235,243-244,255-256,264-265,276-277) */
	UP_ERR_OOM = 4,              /* device allocation failed */
	UP_ERR_CUDA = 5,             /* a CUDA runtime call failed */
	UP_ERR_CAPACITY = 6,         /* output buffers too small; required counts reported */
	UP_ERR_TIMEOUT = 7,          /* a bounded device wait expired */
	UP_ERR_EMPTY_MESH = 8,       /* contour produced no triangles (meshGeneration.cpp:51-52,104-105) */
	UP_ERR_NO_DEVICE = 9         /* no CUDA device, or the library was not built for it */
};

/* ---------------------------------------------------------------- enums */
/* SDF fields (modesConfiguration.cpp:230-279) */
enum up_field {
	UP_FIELD_LAND = 0,          /* shape(p) - elevation(p)/10        :248-258 */
	UP_FIELD_WATER = 1,         /* shape(p)                          :260-267 */
	UP_FIELD_NAVIGATION = 2,    /* shape(p) - max(elevation(p),0)/10 :269-279 */
	UP_FIELD_ELEVATION = 3,     /* shape(p) * 10                     :230-237 */
	UP_FIELD_ELEVATION_RAW = 4  /* elevation(p)                      :239-246 */
};
#define UP_FIELDS_MASK_LAND (1u << UP_FIELD_LAND)
#define UP_FIELDS_MASK_WATER (1u << UP_FIELD_WATER)
#define UP_FIELDS_MASK_NAVIGATION (1u << UP_FIELD_NAVIGATION)

/* mesh purpose (planets.h:53-59) */
enum up_purpose { UP_PURPOSE_UNDEFINED = 0, UP_PURPOSE_LAND = 1, UP_PURPOSE_WATER = 2, UP_PURPOSE_NAVIGATION = 3 };

/* noise family (cage NoiseFunction call sites, e.g. elevationModes.cpp:16-26) */
enum up_noise_type { UP_NOISE_VALUE = 0, UP_NOISE_CUBIC = 1, UP_NOISE_PERLIN = 2, UP_NOISE_SIMPLEX = 3, UP_NOISE_SIMPLEX_REDUCED = 4, UP_NOISE_CELLULAR = 5 };
enum up_fractal { UP_FRACTAL_NONE = 0, UP_FRACTAL_FBM = 1, UP_FRACTAL_RIDGED = 2 };
enum up_distance { UP_DIST_EUCLIDEAN = 0, UP_DIST_MANHATTAN = 1, UP_DIST_HYBRID = 2 };
enum up_cell_op { UP_OP_CELL = 0, UP_OP_DISTANCE = 1, UP_OP_DISTANCE2 = 2, UP_OP_ADD = 3, UP_OP_SUBTRACT = 4, UP_OP_MULTIPLY = 5, UP_OP_DIVIDE = 6 };

/* ---------------------------------------------------------------- configuration */
/* Mode selection by the reference's lower-case names (main.cpp:19-29,
 * modesConfiguration.cpp:79-114,176-183,208-212). shape may be "random". */
typedef struct up_modes {
	const char *shape;      /* e.g. "sphere" */
	const char *elevation;  /* e.g. "lakes" */
	const char *coloring;   /* e.g. "default" */
	int32_t poles;          /* unnatural-planets/poles/enable   (coloringModes.cpp:18,111) */
	int32_t flowers;        /* unnatural-planets/flowers/enable (coloringModes.cpp:19,319) */
} up_modes;

/* The reference draws every noise seed from one process-global generator
 * (math.cpp:73-77) in lazy static-initialisation order; here all draws derive
 * from one explicit seed (noise instance i gets a fixed slot, see
 * up_instance_seed), which makes planets reproducible. */
typedef struct up_seeds {
	uint32_t seed;
} up_seeds;

/* One noise layer of a synthetic program: per-octave amplitude and frequency
 * are explicit so they can be differentiated. octave i samples
 * n(freq[i] * p, seed + i); the layer adds sum_i amp[i] * s(n) with
 * s(n) = n (NONE, FBM) or 1 - 2|n| (RIDGED). */
typedef struct up_noise_layer {
	int32_t type;      /* up_noise_type */
	int32_t fractal;   /* up_fractal */
	int32_t octaves;   /* 1..8 */
	int32_t distance;  /* cellular only */
	int32_t operation; /* cellular only */
	uint32_t seed;
	float amp[8];
	float freq[8];
} up_noise_layer;

enum up_base { UP_BASE_SPHERE = 0, UP_BASE_TORUS = 1, UP_BASE_ROUNDED_BOX = 2, UP_BASE_TORUS_SPHERES = 3 };

/* Synthetic unit-scale planet: d(p) = base(p) - sum(layers)(p).
 *   SPHERE:        |p| - R                               (param[0] = R)
 *   TORUS:         |(|p.xy| - R, p.z)| - r               (param[0..1] = R, r)
 *   ROUNDED_BOX:   box(p, h) - rr                        (param[0..1] = h, rr)
 *   TORUS_SPHERES: TORUS smooth-unioned (smoothMin, math.cpp:28-33, width k)
 *                  with n_spheres spheres, in order
 * Differentiable parameter vector theta (up_synth_theta_count entries):
 *   for each layer: amp[0..octaves), freq[0..octaves)
 *   then base: R | R, r | h, rr | R, r, radius[0..n_spheres), k */
typedef struct up_synth_program {
	int32_t base;
	float param[2];
	int32_t n_spheres;   /* 0..8 */
	float sphere[8][4];  /* cx, cy, cz, radius */
	float k;
	int32_t n_layers;    /* 0..2 */
	up_noise_layer layer[2];
} up_synth_program;

/* Regular sampling grid: sample (i,j,k) sits at lo + (i,j,k) * step with
 * step = (hi - lo) / (n - 1), computed in FP32 as a rounded multiply then a
 * rounded add (no fused multiply-add) so host and device agree bit-exactly.
 * Replaces MarchingCubesCreateConfig (meshGeneration.cpp:35-37). */
typedef struct up_grid {
	float lo[3];
	float hi[3];
	uint32_t n[3]; /* samples per axis, >= 2 */
} up_grid;

/* Mesh produced by up_contour (caller-owned buffers). */
typedef struct up_mesh_out {
	float *positions;   /* 3 * vertex_capacity floats */
	float *normals;     /* 3 * vertex_capacity floats, or NULL */
	uint32_t *indices;  /* index_capacity entries (3 per triangle) */
	uint64_t vertex_capacity;
	uint64_t index_capacity;
	uint64_t vertex_count; /* out: vertices written (or required) */
	uint64_t index_count;  /* out: indices written (or required) */
} up_mesh_out;

/* Mesh input of up_texture (the unwrapped render mesh). */
typedef struct up_mesh_in {
	const float *positions; /* 3 * vertex_count */
	const float *normals;   /* 3 * vertex_count */
	const float *uvs;       /* 2 * vertex_count, atlas coordinates in [0,1] */
	const uint32_t *indices;/* index_count, 3 per triangle */
	uint64_t vertex_count;
	uint64_t index_count;
} up_mesh_in;

/* Texel outputs of up_texture, 8-bit, row-major width x height. Any pointer
 * may be NULL to skip that image. Float outputs (before quantisation) can be
 * requested instead through the *_f32 pointers. */
typedef struct up_texture_out {
	uint8_t *albedo;   /* RGB8 (land) or RGBA8 (water, alpha = opacity) */
	uint8_t *special;  /* RG8: roughness, metallic */
	uint8_t *height;   /* R8 */
	float *albedo_f32; /* 3 or 4 floats per texel, NaN where not covered */
	float *special_f32;
	float *height_f32;
} up_texture_out;

typedef struct up_context up_context;

/* ---------------------------------------------------------------- context */
/* Replaces terrainApplyConfig + terrainPreseed (modesConfiguration.cpp:288-315):
 * resolves the mode names (UP_ERR_INVALID_MODE on an unknown name), derives
 * every noise instance from seeds->seed and uploads the planet description
 * to the current CUDA device. */
int up_context_create(const up_modes *modes, const up_seeds *seeds, up_context **out);
/* A context evaluating a synthetic program (no reference counterpart; used
 * for the unit-scale benchmark planets and the parameter adjoint). Coloring
 * uses the synthetic texel program (albedo from value noise, roughness from
 * simplex noise, height from elevation). */
int up_context_create_synthetic(const up_synth_program *program, up_context **out);
int up_context_destroy(up_context *ctx);
/* Stream for all subsequent work on ctx (a cudaStream_t; NULL = legacy default). */
int up_context_set_stream(up_context *ctx, void *cuda_stream);
/* Name of the resolved shape (after "random"), and the doubleSided flag
 * (modesConfiguration.cpp:139-160, 325-328). */
int up_context_shape_name(const up_context *ctx, char *buf, size_t buf_size);
int up_context_double_sided(const up_context *ctx);
/* Replace the synthetic program's parameter vector (theta layout above). */
int up_context_set_theta(up_context *ctx, const float *theta, size_t n);
size_t up_synth_theta_count(const up_synth_program *program);
const char *up_status_string(int status);
const char *up_last_error(const up_context *ctx);
/* Bytes of device scratch the context holds now (staging and work buffers,
 * grown on demand and kept for reuse; not the planet description). No
 * reference counterpart. */
size_t up_context_device_bytes(const up_context *ctx);
/* Fault injection for tests, on the host only: the next count scratch
 * allocations of any context fail as if the device were out of memory
 * (the call returns UP_ERR_OOM). No reference counterpart. */
void up_debug_fail_allocations(uint32_t count);
/* Wait limit, in nanoseconds of the GPU's global timer, of every grid-wide
 * barrier of the persistent batch launch (up_batch_run); 0 restores the
 * default of 2 s. A wait that runs out makes the call return UP_ERR_TIMEOUT
 * and leaves the launch without blocking. For tests of that path; no
 * reference counterpart. */
void up_debug_set_wait_limit(uint64_t ns);
/* Which form up_batch_run replays for chunk lists planned after this call:
 * 0 (default) the faster of the two, timed on the list when it is planned;
 * 1 the stage launches; 2 the persistent launch (where the device supports
 * cooperative launches). For tests and measurements; no reference
 * counterpart. Returns UP_ERR_INVALID_ARGUMENT for another value. */
int up_debug_set_batch_form(int form);
/* Seed of noise instance slot i for planet seed s (math.cpp:73-77 replaced). */
uint32_t up_instance_seed(uint32_t seed, uint32_t slot);

/* ---------------------------------------------------------------- SDF */
/* Batched form of the reference's TerrainFunctor Real(*)(const Vec3&)
 * (modesConfiguration.cpp:29; terrainSdfLand/Water/Navigation/Elevation/
 * ElevationRaw :230-279). xyz holds n points (3 floats each); d receives n
 * values; grad (3 floats per point) receives the analytic gradient dd/dp when
 * not NULL. Returns UP_ERR_NAN if any value is NaN. */
int up_sdf_eval_points(up_context *ctx, int field, const float *xyz, size_t n, float *d, float *grad);

/* Per-point shims with the reference callback's exact signature
 * (meshGeneration.cpp:12-15): up_sdf_land, up_sdf_water and
 * up_sdf_navigation evaluate the LAND, WATER and NAVIGATION fields of the
 * context installed with up_set_current_context. The reference calls its
 * terrain functors from several threads at once (the navmesh, land and water
 * pipelines and their chunk tasks, generator.cpp:159,215,432-439), so each
 * calling thread evaluates on its own copy of the installed context (same
 * planet; its own stream, flag and scratch), made on the thread's first call
 * after the context was installed or its parameters changed
 * (up_context_set_theta), and freed when the thread exits. Installing another
 * context, or destroying the installed one, retires the copies. Returns NaN
 * on any error. One call is one device round trip; batch callers use
 * up_sdf_eval_points. */
int up_set_current_context(up_context *ctx);
float up_sdf_land(const float p[3]);
float up_sdf_water(const float p[3]);
float up_sdf_navigation(const float p[3]);

/* Grid sampling: replaces MarchingCubes::updateByPosition(terrainSdf*)
 * (meshGeneration.cpp:39), called once per field per planet at
 * meshGeneration.cpp:50,60,103. fields_mask selects up to three of
 * LAND/WATER/NAVIGATION written in ONE pass (shape and elevation evaluated
 * once per sample); out[f] receives nx*ny*nz floats for each selected field f
 * (index by up_field). grad, when not NULL, receives 3*nx*ny*nz floats
 * (planes gx, gy, gz) of the analytic gradient of the lowest selected field.
 * Outputs may be host or device memory; when all are host memory the grid is
 * sampled in z-slabs whose device-to-host copies overlap the sampling of the
 * next slab. Values are exact everywhere (no narrow band). */
int up_sdf_grid(up_context *ctx, uint32_t fields_mask, const up_grid *grid, float *const out[3], float *grad);

/* ---------------------------------------------------------------- contour */
/* Dual contouring of one field: replaces MarchingCubes::makeMesh
 * (meshGeneration.cpp:40) and the flow of meshGenerateGeneric (:32-44).
 * Samples the field on grid (or takes it from values when not NULL: a
 * host or device array of nx*ny*nz floats; a synthetic context samples only
 * a narrow band exactly: where |base| exceeds the bound of its noise layers
 * plus one grid step, only the sign is needed and the base gives it, so the
 * mesh equals the mesh of the fully sampled grid), finds sign-change edges, places
 * one vertex per active cell by a QEF solve on analytic Hermite normals
 * (FP32; FP64 for cells whose eigenvalue truncation is within FP32
 * rounding of the threshold), and emits two triangles per interior sign-change edge, wound so
 * that normals point to increasing field values (outwards). Vertex order is
 * the linear cell order; triangle order is (grid point, axis) order.
 * When capacities are too small returns UP_ERR_CAPACITY with the required
 * vertex_count/index_count filled in. UP_ERR_EMPTY_MESH if no triangles. */
int up_contour(up_context *ctx, int field, const up_grid *grid, const float *values, up_mesh_out *mesh);

/* Base mesh of one field, as meshGenerateBaseLand / Water / Navigation
 * (meshGeneration.cpp:46-108): the up_contour mesh, then
 *  - only the largest connected component kept (meshRemoveDisconnected,
 *    :41): components of the vertex graph joined by triangles, largest =
 *    most triangles, ties to the component holding the lowest vertex index;
 *  - meshFlipNormals (:42) needs nothing: up_contour already emits that
 *    orientation;
 *  - WATER only (:62-95): a vertex is valid when the raw elevation there is
 *    below 0.1; validity spreads twice to all vertices of every triangle
 *    holding a valid vertex; triangles with an invalid vertex and invalid
 *    vertices are removed (meshRemoveInvalid).
 * Kept vertices and triangles keep their order. Same capacity protocol and
 * errors as up_contour (UP_ERR_EMPTY_MESH when nothing is left). */
int up_mesh_generate_base(up_context *ctx, int field, const up_grid *grid, const float *values, up_mesh_out *mesh);

/* ---------------------------------------------------------------- images */
/* imageConvertSpecialToGltfPbr (generator.cpp:135): special (width*height*2
 * u8: roughness, metallic) -> pbr (width*height*3 u8) = (255, roughness,
 * metallic), the glTF metallicRoughness channel convention. Host or device
 * buffers. */
int up_image_special_to_gltf_pbr(up_context *ctx, const uint8_t *special, uint32_t width, uint32_t height, uint8_t *pbr);
/* imageConvertHeigthToNormal(height, strength) (generator.cpp:137): height
 * map (width*height u8) -> tangent-space normal map (width*height*3 u8):
 * h = height/255, n = normalize(-strength dh/dx, -strength dh/dy, 1) with
 * central differences in texels (one-sided at the border, x along a row, y
 * down the rows), stored as (n + 1)/2 * 255 rounded. Host or device buffers. */
int up_image_height_to_normal(up_context *ctx, const uint8_t *height_map, uint32_t width, uint32_t height, float strength, uint8_t *normal);

/* ---------------------------------------------------------------- texels */
/* Per-texel material of an unwrapped mesh: replaces Generator<Water>::generate
 * (textures.cpp:45-82): UV rasterisation (meshGenerateTexture, :66-71), the
 * per-texel Generator::pixel -> terrainTile -> coloring pipeline (:24-43,
 * coloringModes.cpp:905-966), imageDilation(7) (:73-77, when dilation != 0)
 * and imageConvert to U8 (:79-81). purpose is UP_PURPOSE_LAND or
 * UP_PURPOSE_WATER. */
int up_texture(up_context *ctx, int purpose, const up_mesh_in *mesh, uint32_t width, uint32_t height, int dilation, up_texture_out *out);

/* Batched terrainTile for points with normals (tileProperties.cpp:256-273,
 * purpose NAVIGATION there). Per point outputs (any may be NULL):
 * albedo 3f, roughness, metallic, height, opacity, elevation, slope (rad),
 * temperature, precipitation as floats; biome and type as uint8. */
typedef struct up_tile_out {
	float *albedo;
	float *roughness, *metallic, *height, *opacity;
	float *elevation, *slope, *temperature, *precipitation;
	uint8_t *biome, *type;
} up_tile_out;
int up_tiles(up_context *ctx, int purpose, const float *positions, const float *normals, size_t n, up_tile_out *out);

/* ---------------------------------------------------------------- adjoint */
/* Parameter adjoint of a synthetic context: dtheta[j] = sum_i dL_dd[i] *
 * dd(points_i)/dtheta_j for the context's theta (up_synth_theta_count
 * entries). Noise octaves are recomputed, nothing is stored per point. Per
 * block partial sums are reduced in a fixed order (deterministic). No
 * reference counterpart. */
int up_sdf_param_backward(up_context *ctx, const float *points, size_t n, const float *dL_dd, float *dtheta);

/* Allocation-free variant of up_sdf_param_backward. It has no counterpart in
 * the reference. It is for callers that cannot allocate device memory: an
 * engine that hands out all device memory from its own pool, or a process
 * that must not grow its device footprint after start-up. points, dL_dd and
 * dtheta must be device memory of the context's GPU (host buffers and
 * buffers of another GPU are rejected with UP_ERR_INVALID_ARGUMENT: staging
 * them would need an allocation). The only scratch is a static device array
 * of 2048 x 43 floats (352 KiB) that every GPU that loads the library keeps
 * until the process exits; the kernel never launches more than 2048 blocks,
 * so any point count fits, and a parameter vector longer than 43 entries is
 * rejected. Creating the context looks up the array's device address (with
 * the context's device current), so the call itself makes no runtime query;
 * after a device reset (cudaDeviceReset) that address is gone with the old
 * device state, so create a new context. All calls share the array: calls
 * that overlap on the GPU race. */
int up_sdf_param_backward_noalloc(up_context *ctx, const float *points, size_t n, const float *dL_dd, float *dtheta);

/* ---------------------------------------------------------------- batching */
/* One chunk of a batched run: a synthetic program (per planet), a grid
 * (chunk box and resolution), and output offsets. */
typedef struct up_chunk {
	uint32_t planet;   /* index into the planets array */
	up_grid grid;
} up_chunk;
typedef struct up_batch_out {
	float *positions;     /* 3 * vertex_capacity, device or host */
	uint32_t *indices;    /* index_capacity */
	uint64_t vertex_capacity, index_capacity;
	uint64_t *chunk_vertex_offset; /* nchunks + 1 entries, out (host) */
	uint64_t *chunk_index_offset;  /* nchunks + 1 entries, out (host) */
	uint64_t vertex_count, index_count; /* out */
	float *values;        /* optional: the sampled grids of all chunks, concatenated (x-fastest per chunk) */
	uint64_t values_capacity;
} up_batch_out;
/* Samples and contours many chunks of uneven size (from many planets). The
 * first call for a chunk list runs one launch per stage over all chunks (the
 * host sizes the lists from the counts), autotunes the sampling tile shape,
 * and captures a CUDA graph for later calls with the same list: either one
 * persistent, cooperatively launched kernel that runs every stage as a phase
 * separated by grid-wide barriers (bounded waits: UP_ERR_TIMEOUT when one runs
 * out), or the stage launches, whichever ran faster on the list when it was
 * planned (up_debug_set_batch_form fixes the choice).
 * The closest reference counterpart is the per-chunk tasksRunBlocking fan-out
 * (generator.cpp:159,215).
 * Indices of chunk c are local to chunk c's vertices. Without a values buffer
 * the chunks are sampled with the narrow band of contouring (see up_contour;
 * the meshes are the same); with one, every sample is exact. */
int up_batch_run(up_context *ctx, const up_synth_program *planets, size_t nplanets, const up_chunk *chunks, size_t nchunks, up_batch_out *out);

#ifdef __cplusplus
}
#endif

#endif /* UP_ABI_H */
