// Kernels of the reference modes (the planet description is read from device
// memory, uploaded once per context): grid sampling of up to three fields in one
// pass (land, water, navigation share the shape and elevation evaluation),
// scattered points with optional analytic gradient, and the contouring
// Hermite/QEF instantiation.
//
// Replaces the three MarchingCubes::updateByPosition passes per planet
// (sources/meshGeneration.cpp:39, called at :50, :60 and :103) and the
// per-point terrainSdf* callbacks (sources/modesConfiguration.cpp:230-279).
#include "up_contour.cuh"
#include "up_modes.cuh"
#include "up_modes_runs.cuh"

namespace up {

__device__ __forceinline__ float mgrid_coord(const GridDev &g, int a, uint32_t i) {
	return __fadd_rn(__fmul_rn((float)i, g.step[a]), g.lo[a]);
}

// land = s - e/10, water = s, navigation = s - max(e/10, 0)
template<class S>
__device__ __forceinline__ void fields_of(const ModesDesc &M, uint32_t mask, V3S<S> p, S out[3]) {
	const S s = shape_eval(M, p);
	S e = mk<S>(0.f);
	if (mask & 5u) e = elevation_eval(M, p) * 0.1f;
	out[0] = s - e;
	out[1] = s;
	out[2] = s - s_max(e, mk<S>(0.f));
}

// band > 0 (one field, no gradient): samples with |shape| > band take the
// shape value (narrow band of contouring, modes_contour_band)
template<bool GRAD>
__global__ void __launch_bounds__(128) modes_grid_kernel(const ModesDesc *__restrict__ Mp, uint32_t mask, const GridDev g, float *__restrict__ o0,
	float *__restrict__ o1, float *__restrict__ o2, float *__restrict__ grad, unsigned *__restrict__ nanflag, float band) {
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint64_t plane = (uint64_t)nx * ny * g.n[2];
	const uint32_t total = (uint32_t)plane;
	const ModesDesc &M = *Mp;
	const int gf = (mask & 1u) ? 0 : ((mask & 2u) ? 1 : 2); // gradient of the lowest selected field
	bool bad = false;
	for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
		const uint32_t i = idx % nx, r = idx / nx, j = r % ny, k = r / ny;
		const V3f p = v3(mgrid_coord(g, 0, i), mgrid_coord(g, 1, j), mgrid_coord(g, 2, k + g.k0));
		float v[3];
		if (GRAD) {
			Df f[3];
			fields_of(M, mask, dual_point(p), f);
			v[0] = f[0].v; v[1] = f[1].v; v[2] = f[2].v;
			grad[idx] = f[gf].d.x;
			grad[plane + idx] = f[gf].d.y;
			grad[2 * plane + idx] = f[gf].d.z;
		} else {
			const float sh = band > 0.f ? shape_eval(M, vs(p.x, p.y, p.z)) : 0.f;
			if (band > 0.f && fabsf(sh) > band) v[0] = v[1] = v[2] = sh;
			else fields_of(M, mask, vs(p.x, p.y, p.z), v);
		}
		if (mask & 1u) { o0[idx] = v[0]; bad |= isnan(v[0]); }
		if (mask & 2u) { o1[idx] = v[1]; bad |= isnan(v[1]); }
		if (mask & 4u) { o2[idx] = v[2]; bad |= isnan(v[2]); }
	}
	if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(nanflag, 1u);
}

// ---------------------------------------------------------------- x-coherent grid (lakes, islands, legacy)
// Lattice instances per run from a table (up_modes_runs.cuh). Work mapping,
// narrow band and stores follow synth_grid_runs_kernel: a warp takes RUN_R
// samples along x of an 8 (y) x 4 (z) tile of rows.
constexpr int MRUNS_T = 32 * RUNS_WARPS;
constexpr int MRUN_SLOTS = 4; // slots 0-2: noise instances, then the three fields (in place); 3: shape values

// Narrow band at the task level (synth_task_band_kernel, with the shape as
// the base and the margin of modes_run_shape): tasks whose sample box lies
// farther than the band from the shape's surface get shape(centre) in every
// selected field; the others are listed for modes_grid_runs_kernel.
__global__ void __launch_bounds__(256) modes_task_band_kernel(const ModesDesc *__restrict__ Mp, uint32_t mask, const GridDev g, float band,
	float *__restrict__ o0, float *__restrict__ o1, float *__restrict__ o2, uint32_t *__restrict__ task_list, unsigned *__restrict__ list_count,
	uint32_t *__restrict__ signs) {
	const ModesDesc &M = *Mp;
	const uint32_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const uint32_t ntasks = ((nx + RUN_R - 1) / RUN_R) * ((ny + 7) / 8) * ((nz + 3) / 4); // < 2^31
	const uint32_t ngroups = (ntasks + 31) / 32;
	const uint32_t lane = threadIdx.x & 31;
	float *const outs[3] = {o0, o1, o2};
	for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < ngroups; w += (gridDim.x * blockDim.x) >> 5) {
		const uint32_t t = w * 32 + lane;
		bool far = false;
		float fv = 0.f;
		if (t < ntasks) {
			V3f c;
			float hd;
			runs_task_box(g, t, c, hd);
			fv = shape_eval(M, vs(c.x, c.y, c.z));
			far = fabsf(fv) > (band + hd) * 1.001f + 1e-3f * (1.f + fabsf(fv)); // false for NaN
		}
		const unsigned near = __ballot_sync(0xFFFFFFFFu, t < ntasks && !far);
		uint32_t slot = 0;
		if (lane == 0 && near) slot = atomicAdd(list_count, (unsigned)__popc(near));
		slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
		if (near & (1u << lane)) task_list[slot + __popc(near & ((1u << lane) - 1u))] = t;
		#pragma unroll 1
		for (unsigned fm = __ballot_sync(0xFFFFFFFFu, far); fm != 0u; fm &= fm - 1u) {
			const int src = __ffs(fm) - 1;
			const float v = __shfl_sync(0xFFFFFFFFu, fv, src);
			if (signs) { // one field; contouring reads no value of these samples
				runs_task_signs(signs, nx, ny, nz, w * 32 + (uint32_t)src, v < 0.f);
				continue;
			}
			#pragma unroll 1
			for (int f = 0; f < 3; f++)
				if (mask & (1u << f)) runs_task_fill(outs[f], nx, ny, nz, w * 32 + (uint32_t)src, v);
		}
	}
}

// task_list (narrow band only, or null): the tasks to sample, *list_count of
// them, listed by modes_task_band_kernel, which has written the others.
// signs (one field, with task_list; or null): the sign words of contouring
// that field (synth_grid_runs_kernel).
template<int EM>
__global__ void __launch_bounds__(MRUNS_T, 3) modes_grid_runs_kernel(const ModesDesc *__restrict__ Mp, uint32_t mask, const GridDev g,
	float *__restrict__ o0, float *__restrict__ o1, float *__restrict__ o2, unsigned *__restrict__ nanflag, unsigned *__restrict__ tasks,
	float band, const uint32_t *__restrict__ task_list, const unsigned *__restrict__ list_count, uint32_t *__restrict__ signs) {
	extern __shared__ __align__(16) float mruns_smem[];
	constexpr int R = RUN_R;
	float *tab = mruns_smem + threadIdx.x;
	float *shv = tab + 3 * R * MRUNS_T;
	const ModesDesc &M = *Mp;
	const uint32_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const uint32_t nruns = (nx + R - 1) / R;
	const uint32_t tny = (ny + 7) / 8, tnz = (nz + 3) / 4;
	// a task holds at least two samples of a grid of 2 .. 2^32 - 1 samples:
	// ntasks < 2^31, and the counter (ntasks plus one failed take per warp)
	// cannot wrap
	const uint32_t ntasks = task_list ? *list_count : nruns * tny * tnz;
	const uint32_t lane = threadIdx.x & 31;
	const bool need_e = (mask & 5u) != 0;
	float *const outs[3] = {o0, o1, o2};
	runs_tables_init();
	RunCtx rc;
	rc.lo_x = g.lo[0];
	rc.step_x = g.step[0];
	rc.nx = nx;
	bool bad = false;
	// tasks in order from the launcher-zeroed counter (synth_grid_runs_kernel)
	uint32_t t = 0;
	if (lane == 0) t = atomicAdd(tasks, 1u);
	t = __shfl_sync(0xFFFFFFFFu, t, 0);
	while (t < ntasks) {
		uint32_t t_next = 0;
		if (lane == 0) t_next = atomicAdd(tasks, 1u); // taken ahead; read after the task
		const uint32_t tt = task_list ? task_list[t] : t;
		const uint32_t run = tt % nruns, tile = tt / nruns;
		const uint32_t jr = (tile % tny) * 8 + (lane & 7), kr = (tile / tny) * 4 + (lane >> 3);
		const bool live = jr < ny && kr < nz;
		const uint32_t j = jr < ny ? jr : ny - 1, k = kr < nz ? kr : nz - 1;
		rc.i0 = run * R;
		rc.py = mgrid_coord(g, 1, j);
		rc.pz = mgrid_coord(g, 2, k + g.k0);
		bool far = modes_run_shape(M, rc, R, band, shv, MRUNS_T);
		far = __all_sync(0xFFFFFFFFu, far); // every lane of the warp runs every task
		if (need_e && !far) modes_run_fill<EM>(M, rc, R, tab, MRUNS_T);
		// fields of sample r into slots 0-2 at r (after its table entries are read)
		#pragma unroll 1
		for (int r = 0; r < R; r++) {
			float v[3];
			modes_run_fields<EM>(M, rc, r, shv[r * MRUNS_T], need_e, band, tab, MRUNS_T, v);
			#pragma unroll
			for (int f = 0; f < 3; f++) tab[(f * R + r) * MRUNS_T] = v[f];
		}
		if (live) {
			const uint64_t base = ((uint64_t)k * ny + j) * nx + rc.i0;
			const bool full = rc.i0 + R <= nx;
			#pragma unroll 1
			for (int f = 0; f < 3; f++) {
				if (!(mask & (1u << f))) continue;
				float *o = outs[f];
				const float *src = tab + f * R * MRUNS_T;
				// 16-byte stores only where the destination is 16-byte aligned
				const bool vec = full && ((uintptr_t)(o + base) & 15) == 0;
				#pragma unroll 1
				for (int r = 0; r < R; r += 4) {
					float x[4];
					#pragma unroll
					for (int q = 0; q < 4; q++) {
						x[q] = src[(r + q) * MRUNS_T];
						bad |= isnan(x[q]);
					}
					if (vec) {
						*(float4 *)(o + base + r) = make_float4(x[0], x[1], x[2], x[3]);
					} else {
						#pragma unroll
						for (int q = 0; q < 4; q++)
							if (rc.i0 + r + q < nx) o[base + r + q] = x[q];
					}
				}
				if (signs) {
					uint32_t neg = 0; // bit r: sample r < 0 (samples past the row clear)
					#pragma unroll
					for (int r = 0; r < R; r++) neg |= (src[r * MRUNS_T] < 0.f && rc.i0 + r < nx ? 1u : 0u) << r;
					runs_row_signs(signs, base, neg, nx % R == 0);
				}
			}
		}
		t = __shfl_sync(0xFFFFFFFFu, t_next, 0);
	}
	if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(nanflag, 1u);
}

template<bool GRAD>
__global__ void __launch_bounds__(128) modes_points_kernel(const ModesDesc *__restrict__ Mp, int field, const float *__restrict__ xyz, uint64_t n,
	float *__restrict__ out, float *__restrict__ grad, unsigned *__restrict__ nanflag) {
	const ModesDesc &M = *Mp;
	bool bad = false;
	for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (uint64_t)gridDim.x * blockDim.x) {
		const V3f p = v3(xyz[3 * idx], xyz[3 * idx + 1], xyz[3 * idx + 2]);
		float v;
		if (GRAD) {
			const Df f = field_eval(M, field, dual_point(p));
			v = f.v;
			grad[3 * idx] = f.d.x;
			grad[3 * idx + 1] = f.d.y;
			grad[3 * idx + 2] = f.d.z;
		} else {
			v = field_eval(M, field, vs(p.x, p.y, p.z));
		}
		out[idx] = v;
		bad |= isnan(v);
	}
	if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(nanflag, 1u);
}

template<class K, class... A>
static cudaError_t launch_p(K kernel, uint64_t work, cudaStream_t s, A... args) {
	const int threads = 128;
	int blocks = persistent_blocks((const void *)kernel, threads);
	const uint64_t need = (work + threads - 1) / threads;
	if ((uint64_t)blocks > need) blocks = (int)(need > 0 ? need : 1);
	kernel<<<blocks, threads, 0, s>>>(args...);
	return cudaGetLastError();
}

// tasks: the kernel's task counter, zeroed here in stream order
template<class K, class... A>
static cudaError_t launch_mruns(K kernel, const GridDev &g, cudaStream_t s, unsigned *tasks, A... args) {
	constexpr size_t smem = (size_t)MRUN_SLOTS * RUN_R * MRUNS_T * sizeof(float); // 64 KiB
	cudaError_t e = cudaFuncSetAttribute((const void *)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	if ((e = cudaMemsetAsync(tasks, 0, sizeof(unsigned), s)) != cudaSuccess) return e;
	uint64_t blocks = (uint64_t)persistent_blocks((const void *)kernel, MRUNS_T, smem);
	const uint64_t ntasks = (uint64_t)((g.n[0] + RUN_R - 1) / RUN_R) * ((g.n[1] + 7) / 8) * ((g.n[2] + 3) / 4);
	const uint64_t need = (ntasks + MRUNS_T / 32 - 1) / (MRUNS_T / 32);
	if (blocks > need) blocks = need > 0 ? need : 1;
	kernel<<<(unsigned)blocks, MRUNS_T, smem, s>>>(args...);
	return cudaGetLastError();
}

bool modes_grid_signs(const ModesDesc &H, uint32_t mask, const GridDev &g, float band) {
	return band > 0.f && (mask == 1u || mask == 4u) && mrun_applies(H);
}
cudaError_t launch_modes_grid(const ModesDesc *M, const ModesDesc &H, uint32_t mask, const GridDev &g, float *o0, float *o1, float *o2, float *grad,
	unsigned *flags, cudaStream_t s, float band, uint32_t *task_list, uint32_t *signs) {
	if (signs && (grad || !task_list || !modes_grid_signs(H, mask, g, band))) return cudaErrorInvalidValue;
	unsigned *const nanflag = flags, *const tasks = flags + 1, *const list_count = flags + 2;
	const uint64_t n = (uint64_t)g.n[0] * g.n[1] * g.n[2];
	if (n >= (1ull << 32)) return cudaErrorInvalidValue;
	if (grad) return launch_p(modes_grid_kernel<true>, n, s, M, mask, g, o0, o1, o2, grad, nanflag, 0.f);
	if ((mask & 5u) && mrun_applies(H)) {
		const uint32_t *tl = nullptr;
		const unsigned *tc = nullptr;
		uint32_t *sg = nullptr;
		if (band > 0.f && task_list) {
			cudaError_t e = cudaMemsetAsync(list_count, 0, sizeof(unsigned), s);
			if (e != cudaSuccess) return e;
			if (signs) {
				if ((e = runs_signs_clear(signs, g, s)) != cudaSuccess) return e;
				sg = signs;
			}
			const uint64_t groups = (runs_task_count(g) + 31) / 32;
			uint64_t blocks = (uint64_t)persistent_blocks((const void *)modes_task_band_kernel, 256);
			if (blocks > (groups + 7) / 8) blocks = (groups + 7) / 8;
			modes_task_band_kernel<<<(unsigned)blocks, 256, 0, s>>>(M, mask, g, band, o0, o1, o2, task_list, list_count, sg);
			if ((e = cudaGetLastError()) != cudaSuccess) return e;
			tl = task_list;
			tc = list_count;
		}
		if (H.elevation == 2) return launch_mruns(modes_grid_runs_kernel<2>, g, s, tasks, M, mask, g, o0, o1, o2, nanflag, tasks, band, tl, tc, sg);
		if (H.elevation == 3) return launch_mruns(modes_grid_runs_kernel<3>, g, s, tasks, M, mask, g, o0, o1, o2, nanflag, tasks, band, tl, tc, sg);
		return launch_mruns(modes_grid_runs_kernel<4>, g, s, tasks, M, mask, g, o0, o1, o2, nanflag, tasks, band, tl, tc, sg);
	}
	return launch_p(modes_grid_kernel<false>, n, s, M, mask, g, o0, o1, o2, grad, nanflag, band);
}

cudaError_t launch_modes_points(const ModesDesc *M, int field, const float *xyz, uint64_t n, float *d, float *grad, unsigned *nanflag, cudaStream_t s) {
	if (grad) return launch_p(modes_points_kernel<true>, n, s, M, field, xyz, n, d, grad, nanflag);
	return launch_p(modes_points_kernel<false>, n, s, M, field, xyz, n, d, grad, nanflag);
}

struct ModesEvalF {
	const ModesDesc *M;
	int field;
	__device__ __forceinline__ NG operator()(V3f p) const {
		const Df f = field_eval(*M, field, dual_point(p));
		return ng(f.v, f.d);
	}
};

cudaError_t dc_geometry_modes(const ModesDesc *M, int field, const float *d, const GridDev &g, DcScratch &S, uint32_t ncells, uint32_t nedges,
	uint32_t nquads, float *pos, float *nrm, uint32_t *idx, cudaStream_t s) {
	ModesEvalF ev{M, field};
	return dc_geometry_t(ev, d, g, S, ncells, nedges, nquads, pos, nrm, idx, s);
}

} // namespace up
