// Internal host-side interface between the C ABI (up_abi.cu) and the kernel
// translation units. Not part of the public boundary.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include "../../include/up_abi.h"

namespace up {

struct GridDev {
	float lo[3], step[3];
	uint32_t n[3];
	uint32_t k0 = 0; // z index of the first plane (sampling of z-slabs of a larger grid)
};
GridDev make_grid(const up_grid &g);

// Reference-mode planet description (defined in up_modes.cuh)
struct ModesDesc;

// ---- SDF sampling (up_sdf.cu / up_modes.cu)
// band > 0: narrow band of contouring (samples with |base| > band keep the
// base value); 0: exact values everywhere. flags: three device words, [0]
// the NaN flag (set, never cleared, by the kernel), [1] the task counter of
// the x-coherent grid kernels and [2] their count of listed tasks (both
// zeroed by the launcher, in stream order). task_list (runs_task_count
// words, or null): lets a narrow-band value launch sample only the tasks
// near the surface; the others get one value of the right sign per task.
// signs (dc_sign_words, or null; only where synth_grid_signs holds and with
// task_list): the launch writes the sign words of contouring, and values only
// in the listed tasks (the others hold no sample that contouring reads by
// value: NegFromBits in up_contour.cuh).
cudaError_t launch_synth_grid(const up_synth_program &P, const GridDev &g, float *out, float *grad, unsigned *flags, cudaStream_t s,
	float band = 0.f, uint32_t *task_list = nullptr, uint32_t *signs = nullptr);
bool synth_grid_signs(const up_synth_program &P, const GridDev &g, float band);
// zeroes the sign words before a launch writes them (runs_row_signs)
cudaError_t runs_signs_clear(uint32_t *signs, const GridDev &g, cudaStream_t s);
// work units (tasks) of the x-coherent grid kernels on grid g
uint64_t runs_task_count(const GridDev &g);
// narrow band of contouring for program P on grid g (0 when unbounded)
float contour_band(const up_synth_program &P, const GridDev &g);
cudaError_t launch_synth_points(const up_synth_program &P, const float *xyz, uint64_t n, float *d, float *grad, unsigned *nanflag, cudaStream_t s);
// band > 0: narrow band of contouring one field (modes_contour_band)
// task_list, signs: as launch_synth_grid (signs only where modes_grid_signs holds)
cudaError_t launch_modes_grid(const ModesDesc *M, const ModesDesc &host, uint32_t fields_mask, const GridDev &g, float *o0, float *o1, float *o2, float *grad, unsigned *flags,
	cudaStream_t s, float band = 0.f, uint32_t *task_list = nullptr, uint32_t *signs = nullptr);
bool modes_grid_signs(const ModesDesc &host, uint32_t fields_mask, const GridDev &g, float band);
cudaError_t launch_modes_points(const ModesDesc *M, int field, const float *xyz, uint64_t n, float *d, float *grad, unsigned *nanflag, cudaStream_t s);

// adjoint: partial sums per block into partials (nblocks x ACC stride), then
// a fixed-order reduction into dtheta (compact layout)
int synth_bwd_blocks(uint64_t n);
cudaError_t launch_synth_bwd(const up_synth_program &P, const float *xyz, uint64_t n, const float *w, float *partials, int nblocks,
	float *dtheta, cudaStream_t s);

// ---- dual contouring (up_contour.cu)
struct DcScratch {
	uint32_t *blk_counts;   // dc_scan_words(nblocks)
	uint32_t *totals;       // 4 (device)
	uint32_t *cell_map;     // cells
	uint32_t *edge_map;     // 3 * points
	uint32_t *cell_list;    // capacity cells
	uint32_t *edge_list;    // capacity edges
	uint32_t *quad_list;    // capacity quads
	float *edge_t;         // capacity edges
	float *edge_n;          // 3 * capacity edges
	uint32_t *signs;        // dc_sign_words(grid): bit-packed d < 0
	uint32_t *fb_list;      // capacity cells: cells left to the FP64 QEF (count in totals[3])
	uint8_t *fb_flag;       // capacity cells: 1 = left to the FP64 QEF
	cudaStream_t side;      // optional: the FP64 QEF runs there (forked and joined with the two events)
	cudaEvent_t ev_fork, ev_join;
};
uint32_t dc_num_blocks(const GridDev &g);
uint64_t dc_sign_words(const GridDev &g);
// words of the block-count buffer for nb blocks (3 arrays + chunk sums)
size_t dc_scan_words(uint32_t nb);
// exclusive scan of the three block-count arrays in place; totals[a] = sums
cudaError_t dc_scan_blocks(uint32_t *blk, uint32_t nb, uint32_t *totals, cudaStream_t s);
// pass 1: counts -> totals[0]=cells, [1]=edges, [2]=quads (device), returns after enqueue
// signs_ready: S.signs already holds the sign words of d (written by the
// sampling launch), so the sign pass is skipped
cudaError_t dc_count(const float *d, const GridDev &g, DcScratch &S, cudaStream_t s, bool signs_ready = false);
// pass 2 (after the host knows the totals and sized the lists)
cudaError_t dc_emit(const float *d, const GridDev &g, DcScratch &S, cudaStream_t s);
cudaError_t dc_geometry_synth(const up_synth_program &P, const float *d, const GridDev &g, DcScratch &S, uint32_t ncells, uint32_t nedges,
	uint32_t nquads, float *pos, float *nrm, uint32_t *idx, cudaStream_t s);
cudaError_t dc_geometry_modes(const ModesDesc *M, int field, const float *d, const GridDev &g, DcScratch &S, uint32_t ncells,
	uint32_t nedges, uint32_t nquads, float *pos, float *nrm, uint32_t *idx, cudaStream_t s);

// ---- mesh hygiene (up_mesh.cu)
struct MeshFilterArgs {
	uint32_t V, T;                 // vertices, triangles
	const float *pos, *nrm;        // device; nrm may be null
	const uint32_t *idx;           // device, 3 T
	const float *elev;             // water: elevationRaw at the vertices; null for land/navigation
	uint32_t *parent, *label, *cnt, *newidx; // V each
	uint32_t *blk, *totals;        // dc_scan_words(mesh_blocks(V, T)), 4
	unsigned long long *best;      // 1
	uint8_t *keep_v, *valid2;      // V each
	uint8_t *keep_t;               // T
	unsigned *err;                 // union-find iteration limit flag
};
uint32_t mesh_blocks(uint32_t V, uint32_t T);
// keep flags and their counts: totals[0] = kept vertices, totals[1] = kept triangles
cudaError_t mesh_filter(const MeshFilterArgs &a, cudaStream_t s);
// ordered compaction into device outputs (after mesh_filter)
cudaError_t mesh_compact(const MeshFilterArgs &a, float *pos_out, float *nrm_out, uint32_t *idx_out, cudaStream_t s);

// ---- texture post-processing (up_image.cu)
cudaError_t image_pbr_run(const uint8_t *special, uint32_t W, uint32_t H, uint8_t *pbr, cudaStream_t s);
cudaError_t image_normal_run(const uint8_t *height, uint32_t W, uint32_t H, float strength, uint8_t *normal, cudaStream_t s);

// occupancy-derived persistent grid size
int persistent_blocks(const void *kernel, int threads, size_t smem = 0);

} // namespace up
