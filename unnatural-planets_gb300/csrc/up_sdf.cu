// SDF sampling kernels for synthetic programs: grid (value or fused
// value+gradient), scattered points, and the parameter adjoint.
//
// Replaces the reference's per-sample callback loop
// MarchingCubes::updateByPosition(terrainSdf*) (sources/meshGeneration.cpp:39)
// for the unit-scale synthetic planets. One thread per sample in a
// grid-stride loop sized from the occupancy of the kernel (a multiple of the
// SM count); the noise octaves run in registers; stores are coalesced 4-byte
// writes to x-fastest planes.
#include "up_internal.h"
#include "up_synth.cuh"
#include "up_grid_runs.cuh"
#include <cmath>


namespace up {

GridDev make_grid(const up_grid &g) {
	GridDev d;
	for (int a = 0; a < 3; a++) {
		d.lo[a] = g.lo[a];
		d.n[a] = g.n[a];
		d.step[a] = (g.hi[a] - g.lo[a]) / (float)(g.n[a] - 1);
	}
	return d;
}

int persistent_blocks(const void *kernel, int threads, size_t smem) {
	int dev = 0, sms = 0, per = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess || per < 1) per = 1;
	return sms * per;
}

__device__ __forceinline__ float grid_coord(const GridDev &g, int a, uint32_t i) {
	return __fadd_rn(__fmul_rn((float)i, g.step[a]), g.lo[a]);
}

// band > 0: samples with |base| > band take the base value (narrow band of
// contouring, see synth_run)
template<bool GRAD, int T0, int T1>
__global__ void __launch_bounds__(256) synth_grid_kernel(const up_synth_program P, const GridDev g, float *__restrict__ out,
	float *__restrict__ grad, unsigned *__restrict__ nanflag, float band) {
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint64_t plane = (uint64_t)nx * ny * g.n[2];
	const uint32_t total = (uint32_t)plane;
	bool bad = false;
	for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
		const uint32_t i = idx % nx, r = idx / nx, j = r % ny, k = r / ny;
		const V3f p = v3(grid_coord(g, 0, i), grid_coord(g, 1, j), grid_coord(g, 2, k + g.k0));
		NG d;
		if (band > 0.f) {
			d = synth_base<GRAD>(P, p);
			if (!(fabsf(d.v) > band)) d = synth_eval<GRAD, T0, T1>(P, p);
		} else {
			d = synth_eval<GRAD, T0, T1>(P, p);
		}
		out[idx] = d.v;
		if (GRAD) {
			grad[idx] = d.g.x;
			grad[plane + idx] = d.g.y;
			grad[2 * plane + idx] = d.g.z;
		}
		bad |= isnan(d.v);
	}
	if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(nanflag, 1u);
}

// x-coherent runs (up_grid_runs.cuh): a warp task is RUN_R consecutive x
// samples of 32 rows, the rows an 8 (y) x 4 (z) tile (a compact task skips the
// noise more often under the narrow band of contouring); accumulators in
// dynamic shared memory, RUNS_T slots per sample index, so thread t owns
// acc[r * RUNS_T + t]
constexpr int RUNS_T = 256;
static_assert(RUNS_T == 32 * RUNS_WARPS, "the x tables of up_grid_runs.cuh hold one row per warp");
// 3 blocks of 8 warps per SM: the value + gradient form's shared memory
// (64 KiB of accumulators plus 10 KiB of tables per block) admits 3, and the
// cap keeps the registers (80) from admitting fewer. Timed against 4-warp
// blocks (5 per SM, shared-memory bound: 5.25 ms at 512^3) and 2-warp blocks.
// task_list (narrow band only, or null): the tasks to sample, *list_count of
// them, listed by synth_task_band_kernel, which has written the others.
// signs (value form with task_list, or null): the bit-packed d < 0 words of
// contouring (dc_sign_words), written per row segment (runs_row_signs).
template<bool GRAD, int T0, int T1>
__global__ void __launch_bounds__(RUNS_T, 3) synth_grid_runs_kernel(const up_synth_program P, const GridDev g, float *__restrict__ out,
	float *__restrict__ grad, unsigned *__restrict__ nanflag, unsigned *__restrict__ tasks, float band,
	const uint32_t *__restrict__ task_list, const unsigned *__restrict__ list_count, uint32_t *__restrict__ signs) {
	typedef typename AccOf<GRAD>::T A;
	extern __shared__ __align__(16) unsigned char runs_smem[];
	A *acc = (A *)runs_smem + threadIdx.x;
	constexpr int R = RUN_R;
	constexpr int S = RUNS_T;
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint32_t nz = g.n[2];
	const uint32_t nrows = ny * nz;
	const uint32_t nruns = (nx + R - 1) / R;
	const uint32_t tny = (ny + 7) / 8, tnz = (nz + 3) / 4;
	// a task holds at least two samples of a grid of 2 .. 2^32 - 1 samples:
	// ntasks < 2^31, and the counter (ntasks plus one failed take per warp)
	// cannot wrap
	const uint32_t ntasks = task_list ? *list_count : nruns * tny * tnz;
	const uint64_t plane = (uint64_t)nx * nrows;
	const uint32_t lane = threadIdx.x & 31;
	runs_tables_init();
	RunCtx rc;
	rc.lo_x = g.lo[0];
	rc.step_x = g.step[0];
	rc.nx = nx;
	bool bad = false;
	// Warps take tasks in order from a counter that the launcher zeroes: task
	// costs differ (under the narrow band a task near the surface evaluates
	// the noise and one far from it stores the base), and a fixed
	// assignment of every nwarps-th task left some warps twice the mean work.
	uint32_t t = 0;
	if (lane == 0) t = atomicAdd(tasks, 1u);
	t = __shfl_sync(0xFFFFFFFFu, t, 0);
	while (t < ntasks) {
		uint32_t t_next = 0;
		if (lane == 0) t_next = atomicAdd(tasks, 1u); // taken ahead; read after the task
		const uint32_t tt = task_list ? task_list[t] : t;
		const uint32_t run = tt % nruns, tile = tt / nruns;
		const uint32_t j0 = (tile % tny) * 8, k0 = (tile / tny) * 4;
		// this lane's row (rows past the grid evaluate its last row, unstored)
		const uint32_t jr = j0 + (lane & 7), kr = k0 + (lane >> 3);
		const uint32_t j = jr < ny ? jr : ny - 1, k = kr < nz ? kr : nz - 1;
		rc.i0 = run * R;
		rc.py = grid_coord(g, 1, j);
		rc.pz = grid_coord(g, 2, k + g.k0);
		synth_run<GRAD, T0, T1>(P, rc, R, acc, S, band);
		if (GRAD) {
			// value + gradient: the task's 32 rows, 8 per store instruction,
			// lane l taking row 8 q + (l & 7) and samples 4 (l >> 3) .. + 3
			// from another lane's accumulators (16-byte reads in phases of 8
			// lanes, 8 consecutive slots); with a lane per row, each store
			// instruction half-filled 32 sectors (1.3 % slower at 512^3).
			// 16-byte stores only where every destination address is 16-byte
			// aligned (caller pointers and plane offsets need not be).
			__syncwarp(); // every lane's accumulators are complete
			const Acc4 *wacc = (const Acc4 *)runs_smem + (threadIdx.x & ~31u);
			const bool full = rc.i0 + R <= nx;
			const uint32_t x0 = 4 * (lane >> 3);
			#pragma unroll 1
			for (uint32_t q = 0; q < 4; q++) {
				const uint32_t rr = 8 * q + (lane & 7);
				const uint32_t jj = j0 + (lane & 7), kk = k0 + q;
				float v[4], gx[4], gy[4], gz[4];
				#pragma unroll
				for (int i = 0; i < 4; i++) {
					const Acc4 x = wacc[(x0 + i) * S + rr];
					v[i] = x.v; gx[i] = x.gx; gy[i] = x.gy; gz[i] = x.gz;
				}
				if (jj < ny && kk < nz && rc.i0 + x0 < nx) {
					#pragma unroll
					for (int i = 0; i < 4; i++) bad |= isnan(v[i]);
					const uint64_t base = ((uint64_t)kk * ny + jj) * nx + rc.i0 + x0;
					const bool vec = full && ((uintptr_t)(out + base) & 15) == 0;
					const bool vecg = full &&
						(((uintptr_t)(grad + base) | (uintptr_t)(grad + plane + base) | (uintptr_t)(grad + 2 * plane + base)) & 15) == 0;
					if (vec) {
						*(float4 *)(out + base) = make_float4(v[0], v[1], v[2], v[3]);
					} else {
						#pragma unroll
						for (int i = 0; i < 4; i++)
							if (rc.i0 + x0 + i < nx) out[base + i] = v[i];
					}
					if (vecg) {
						*(float4 *)(grad + base) = make_float4(gx[0], gx[1], gx[2], gx[3]);
						*(float4 *)(grad + plane + base) = make_float4(gy[0], gy[1], gy[2], gy[3]);
						*(float4 *)(grad + 2 * plane + base) = make_float4(gz[0], gz[1], gz[2], gz[3]);
					} else {
						#pragma unroll
						for (int i = 0; i < 4; i++)
							if (rc.i0 + x0 + i < nx) {
								grad[base + i] = gx[i];
								grad[plane + base + i] = gy[i];
								grad[2 * plane + base + i] = gz[i];
							}
					}
				}
			}
			__syncwarp(); // the reads are done before the next task writes
		} else if (jr < ny && kr < nz) {
			// values: each lane stores its own row (timed 1.3 % faster than
			// the row-wise form above, whose 4-byte reads cost more)
			const uint64_t base = ((uint64_t)kr * ny + jr) * nx + rc.i0;
			const bool full = rc.i0 + R <= nx;
			const bool vec = full && ((uintptr_t)(out + base) & 15) == 0;
			#pragma unroll 1
			for (int r = 0; r < R; r += 4) {
				float v[4];
				#pragma unroll
				for (int q = 0; q < 4; q++) {
					v[q] = ((const float *)acc)[(r + q) * S];
					bad |= isnan(v[q]);
				}
				if (vec) {
					*(float4 *)(out + base + r) = make_float4(v[0], v[1], v[2], v[3]);
				} else {
					#pragma unroll
					for (int q = 0; q < 4; q++)
						if (rc.i0 + r + q < nx) out[base + r + q] = v[q];
				}
			}
			if (signs) {
				uint32_t neg = 0; // bit r: sample r < 0 (samples past the row clear)
				#pragma unroll
				for (int r = 0; r < R; r++) neg |= (((const float *)acc)[r * S] < 0.f && rc.i0 + r < nx ? 1u : 0u) << r;
				runs_row_signs(signs, base, neg, nx % R == 0);
			}
		}
		t = __shfl_sync(0xFFFFFFFFu, t_next, 0);
	}
	if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(nanflag, 1u);
}

// Narrow band at the task level (a task: RUN_R samples along x of 8 x 4
// rows, the work unit of synth_grid_runs_kernel). The base is 1-Lipschitz, so
// a task whose sample box lies farther from the base's surface than the band
// (|base(centre)| above band plus the box's half diagonal; margins as in
// synth_run) holds no sample with |base| <= band, and base(centre) has the
// sign of every one of its samples. This kernel lists the other tasks (order
// unspecified) for the runs kernel and gives such tasks that sign: with sign
// words (signs non-null) it writes their bits and leaves their values
// unwritten, else it stores base(centre) to every sample. Lane i of a warp
// tests task 32 w + i, then the warp writes the far tasks of its 32 one after
// the other (runs_task_signs, runs_task_fill).
__global__ void __launch_bounds__(256) synth_task_band_kernel(const up_synth_program P, const GridDev g, float band, float *__restrict__ out,
	uint32_t *__restrict__ task_list, unsigned *__restrict__ list_count, uint32_t *__restrict__ signs) {
	const uint32_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const uint32_t ntasks = ((nx + RUN_R - 1) / RUN_R) * ((ny + 7) / 8) * ((nz + 3) / 4); // < 2^31 (synth_grid_runs_kernel)
	const uint32_t ngroups = (ntasks + 31) / 32;
	const uint32_t lane = threadIdx.x & 31;
	for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < ngroups; w += (gridDim.x * blockDim.x) >> 5) {
		const uint32_t t = w * 32 + lane;
		bool far = false;
		float fv = 0.f;
		if (t < ntasks) {
			V3f c;
			float hd;
			runs_task_box(g, t, c, hd);
			fv = synth_base<false>(P, c).v;
			far = fabsf(fv) > (band + hd) * 1.001f + 1e-5f; // false for NaN
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
			// with sign words, contouring reads no value of these samples
			// (NegFromBits in up_contour.cuh)
			if (signs) runs_task_signs(signs, nx, ny, nz, w * 32 + (uint32_t)src, v < 0.f);
			else runs_task_fill(out, nx, ny, nz, w * 32 + (uint32_t)src, v);
		}
	}
}

// Every lane of a warp runs every step (lanes past n evaluate the last point
// and store nothing), so the warp-cooperative cellular noise (cellular_warp)
// can share cell hashes between the lanes of spatially close points.
static_assert(256 / 32 <= PT_WARPS, "the per-warp cell tables of cellular_warp");
template<bool GRAD, int T0, int T1>
__global__ void __launch_bounds__(256) synth_points_kernel(const up_synth_program P, const float *__restrict__ xyz, uint64_t n,
	float *__restrict__ out, float *__restrict__ grad, unsigned *__restrict__ nanflag) {
	bool bad = false;
	const uint32_t lane = threadIdx.x & 31;
	for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += (uint64_t)gridDim.x * blockDim.x) {
		const uint64_t idx = base + lane;
		const bool valid = idx < n;
		const uint64_t q = valid ? idx : n - 1;
		const V3f p = v3(xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2]);
		const NG d = synth_eval<GRAD, T0, T1, true>(P, p);
		if (!valid) continue;
		out[idx] = d.v;
		if (GRAD) {
			grad[3 * idx] = d.g.x;
			grad[3 * idx + 1] = d.g.y;
			grad[3 * idx + 2] = d.g.z;
		}
		bad |= isnan(d.v);
	}
	if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(nanflag, 1u);
}


template<class K, class... A>
static cudaError_t launch_persistent(K kernel, uint64_t work, cudaStream_t s, A... args) {
	const int threads = 256;
	int blocks = persistent_blocks((const void *)kernel, threads);
	const uint64_t need = (work + threads - 1) / threads;
	if ((uint64_t)blocks > need) blocks = (int)(need > 0 ? need : 1);
	kernel<<<blocks, threads, 0, s>>>(args...);
	return cudaGetLastError();
}

// tasks: the kernel's task counter, zeroed here in stream order
template<bool GRAD, class K, class... A>
static cudaError_t launch_runs(K kernel, const GridDev &g, cudaStream_t s, unsigned *tasks, A... args) {
	// 64 KiB (value + gradient) or 16 KiB of accumulators
	constexpr size_t smem = (size_t)RUN_R * RUNS_T * sizeof(typename AccOf<GRAD>::T);
	cudaError_t e = cudaFuncSetAttribute((const void *)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	if ((e = cudaMemsetAsync(tasks, 0, sizeof(unsigned), s)) != cudaSuccess) return e;
	uint64_t blocks = (uint64_t)persistent_blocks((const void *)kernel, RUNS_T, smem);
	const uint64_t ntasks = (uint64_t)((g.n[0] + RUN_R - 1) / RUN_R) * ((g.n[1] + 7) / 8) * ((g.n[2] + 3) / 4);
	const uint64_t need = (ntasks + RUNS_T / 32 - 1) / (RUNS_T / 32);
	if (blocks > need) blocks = need > 0 ? need : 1;
	kernel<<<(unsigned)blocks, RUNS_T, smem, s>>>(args...);
	return cudaGetLastError();
}

// Narrow band of contouring for a synthetic program. |layers| <= B everywhere
// (synth_noise_bound) and the base is 1-Lipschitz (exact SDFs and their
// polynomial smooth union), so a sample with |base| > B + (longest grid step)
// has the sign of the base, and so has every grid neighbour: it is neither an
// end of a sign-change edge nor decides an active cell by anything but its
// sign, and its value is not needed. The margins absorb FP32 rounding.
// Returns 0 (sample everything exactly) when the bound is not finite.
float contour_band(const up_synth_program &P, const GridDev &g) {
	const float B = synth_noise_bound(P);
	float st = g.step[0];
	if (g.step[1] > st) st = g.step[1];
	if (g.step[2] > st) st = g.step[2];
	const float band = (B + st) * 1.001f + 1e-5f;
	return std::isfinite(band) ? band : 0.f;
}
uint64_t runs_task_count(const GridDev &g) {
	return (uint64_t)((g.n[0] + RUN_R - 1) / RUN_R) * ((g.n[1] + 7) / 8) * ((g.n[2] + 3) / 4);
}
bool synth_grid_signs(const up_synth_program &P, const GridDev &g, float band) {
	return band > 0.f && spec_of(P) == SPEC_PERLIN_CELL;
}
// Zeroes the sign words that runs_row_signs does not store: with the x extent
// a multiple of 16, those past the last sample (and the upper half of the
// last word when the samples end mid-word); otherwise all (bits are OR-ed).
cudaError_t runs_signs_clear(uint32_t *signs, const GridDev &g, cudaStream_t s) {
	const uint64_t npts = (uint64_t)g.n[0] * g.n[1] * g.n[2];
	const uint64_t w0 = g.n[0] % RUN_R == 0 ? npts / 32 : 0;
	return cudaMemsetAsync(signs + w0, 0, (dc_sign_words(g) - w0) * 4, s);
}
cudaError_t launch_synth_grid(const up_synth_program &P, const GridDev &g, float *out, float *grad, unsigned *flags, cudaStream_t s, float band,
	uint32_t *task_list, uint32_t *signs) {
	if (signs && (grad || !task_list || !synth_grid_signs(P, g, band))) return cudaErrorInvalidValue;
	unsigned *const nanflag = flags, *const tasks = flags + 1, *const list_count = flags + 2;
	const uint64_t n = (uint64_t)g.n[0] * g.n[1] * g.n[2];
	if (n >= (1ull << 32)) return cudaErrorInvalidValue;
	const Spec sp = spec_of(P);
	if (sp == SPEC_PERLIN_CELL) {
		if (grad) return launch_runs<true>(synth_grid_runs_kernel<true, 2, CELL_EU_SUB>, g, s, tasks, P, g, out, grad, nanflag, tasks, band,
			(const uint32_t *)nullptr, (const unsigned *)nullptr, (uint32_t *)nullptr);
		if (band > 0.f && task_list) {
			cudaError_t e = cudaMemsetAsync(list_count, 0, sizeof(unsigned), s);
			if (e != cudaSuccess) return e;
			if (signs && (e = runs_signs_clear(signs, g, s)) != cudaSuccess) return e;
			const uint64_t groups = (runs_task_count(g) + 31) / 32;
			uint64_t blocks = (uint64_t)persistent_blocks((const void *)synth_task_band_kernel, 256);
			if (blocks > (groups + 7) / 8) blocks = (groups + 7) / 8;
			synth_task_band_kernel<<<(unsigned)blocks, 256, 0, s>>>(P, g, band, out, task_list, list_count, signs);
			if ((e = cudaGetLastError()) != cudaSuccess) return e;
			return launch_runs<false>(synth_grid_runs_kernel<false, 2, CELL_EU_SUB>, g, s, tasks, P, g, out, grad, nanflag, tasks, band,
				(const uint32_t *)task_list, (const unsigned *)list_count, signs);
		}
		return launch_runs<false>(synth_grid_runs_kernel<false, 2, CELL_EU_SUB>, g, s, tasks, P, g, out, grad, nanflag, tasks, band,
			(const uint32_t *)nullptr, (const unsigned *)nullptr, (uint32_t *)nullptr);
	}
	if (grad) {
		if (sp == SPEC_PERLIN_CELL) return launch_persistent(synth_grid_kernel<true, 2, CELL_EU_SUB>, n, s, P, g, out, grad, nanflag, band);
		if (sp == SPEC_SIMPLEX) return launch_persistent(synth_grid_kernel<true, 3, -1>, n, s, P, g, out, grad, nanflag, band);
		return launch_persistent(synth_grid_kernel<true, -1, -1>, n, s, P, g, out, grad, nanflag, band);
	}
	if (sp == SPEC_PERLIN_CELL) return launch_persistent(synth_grid_kernel<false, 2, CELL_EU_SUB>, n, s, P, g, out, grad, nanflag, band);
	if (sp == SPEC_SIMPLEX) return launch_persistent(synth_grid_kernel<false, 3, -1>, n, s, P, g, out, grad, nanflag, band);
	return launch_persistent(synth_grid_kernel<false, -1, -1>, n, s, P, g, out, grad, nanflag, band);
}

cudaError_t launch_synth_points(const up_synth_program &P, const float *xyz, uint64_t n, float *d, float *grad, unsigned *nanflag, cudaStream_t s) {
	const Spec sp = spec_of(P);
	if (grad) {
		if (sp == SPEC_PERLIN_CELL) return launch_persistent(synth_points_kernel<true, 2, CELL_EU_SUB>, n, s, P, xyz, n, d, grad, nanflag);
		if (sp == SPEC_SIMPLEX) return launch_persistent(synth_points_kernel<true, 3, -1>, n, s, P, xyz, n, d, grad, nanflag);
		return launch_persistent(synth_points_kernel<true, -1, -1>, n, s, P, xyz, n, d, grad, nanflag);
	}
	if (sp == SPEC_PERLIN_CELL) return launch_persistent(synth_points_kernel<false, 2, CELL_EU_SUB>, n, s, P, xyz, n, d, grad, nanflag);
	if (sp == SPEC_SIMPLEX) return launch_persistent(synth_points_kernel<false, 3, -1>, n, s, P, xyz, n, d, grad, nanflag);
	return launch_persistent(synth_points_kernel<false, -1, -1>, n, s, P, xyz, n, d, grad, nanflag);
}

// ---------------------------------------------------------------- adjoint
constexpr int BWD_THREADS = 256;

template<int T0, int T1>
__global__ void __launch_bounds__(BWD_THREADS) synth_bwd_kernel(const up_synth_program P, const float *__restrict__ xyz, uint64_t n,
	const float *__restrict__ w, float *__restrict__ partials) {
	float acc[ACC_N];
	#pragma unroll
	for (int i = 0; i < ACC_N; i++) acc[i] = 0.f;
	// every lane of a warp runs every step (as synth_points_kernel)
	const uint32_t lane0 = threadIdx.x & 31;
	for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += (uint64_t)gridDim.x * blockDim.x) {
		const uint64_t idx = base + lane0;
		const uint64_t q = idx < n ? idx : n - 1;
		// a point of weight 0 adds w * dd/dtheta = 0 (the derivatives are
		// finite for finite parameters): a hinge loss leaves most weights 0,
		// and a warp whose weights are all 0 skips its step
		const float wi = idx < n ? w[idx] : 0.f;
		if (__all_sync(0xFFFFFFFFu, wi == 0.f)) continue;
		const V3f p = v3(xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2]);
		synth_bwd<T0, T1, true>(P, p, wi, acc);
	}
	// warp sums, then warps in a fixed order: deterministic per block
	__shared__ float red[BWD_THREADS / 32][ACC_N];
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	#pragma unroll
	for (int i = 0; i < ACC_N; i++) {
		float v = acc[i];
		#pragma unroll
		for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
		if (lane == 0) red[wid][i] = v;
	}
	__syncthreads();
	if (threadIdx.x < ACC_N) {
		float v = 0.f;
		#pragma unroll
		for (int k = 0; k < BWD_THREADS / 32; k++) v += red[k][threadIdx.x];
		partials[(uint64_t)blockIdx.x * ACC_N + threadIdx.x] = v;
	}
}

struct SlotMap { int slot[64]; int n; };

// one block: each thread owns theta entries, sums the block partials in order
__global__ void synth_bwd_reduce(const float *__restrict__ partials, int nblocks, const SlotMap m, float *__restrict__ dtheta) {
	for (int t = threadIdx.x; t < m.n; t += blockDim.x) {
		const int s = m.slot[t];
		double v = 0.0;
		for (int b = 0; b < nblocks; b++) v += partials[(uint64_t)b * ACC_N + s];
		dtheta[t] = (float)v;
	}
}

int synth_bwd_blocks(uint64_t n) {
	int blocks = persistent_blocks((const void *)synth_bwd_kernel<-1, -1>, BWD_THREADS);
	const uint64_t need = (n + BWD_THREADS - 1) / BWD_THREADS;
	if ((uint64_t)blocks > need) blocks = (int)(need > 0 ? need : 1);
	return blocks;
}

cudaError_t launch_synth_bwd(const up_synth_program &P, const float *xyz, uint64_t n, const float *w, float *partials, int nblocks,
	float *dtheta, cudaStream_t s) {
	const Spec sp = spec_of(P);
	if (sp == SPEC_PERLIN_CELL) synth_bwd_kernel<2, CELL_EU_SUB><<<nblocks, BWD_THREADS, 0, s>>>(P, xyz, n, w, partials);
	else if (sp == SPEC_SIMPLEX) synth_bwd_kernel<3, -1><<<nblocks, BWD_THREADS, 0, s>>>(P, xyz, n, w, partials);
	else synth_bwd_kernel<-1, -1><<<nblocks, BWD_THREADS, 0, s>>>(P, xyz, n, w, partials);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	SlotMap m;
	m.n = theta_slots(P, m.slot);
	synth_bwd_reduce<<<1, 64, 0, s>>>(partials, nblocks, m, dtheta);
	return cudaGetLastError();
}

// ---------------------------------------------------------------- adjoint without allocation
// Variant of the parameter adjoint for callers that cannot allocate device
// memory: an engine that hands out all device memory from its own pool, or a
// host process that must not grow its device footprint after start-up (a
// fixed budget shared with a renderer or another engine). Its only scratch -- one row of ACC_N partial sums per block -- is
// this file-scope device array, which every GPU that loads the library keeps
// until the process exits. The kernel launches at most NOALLOC_MAX_BLOCKS
// blocks (grid-stride loop), so every point count fits; the array is shared by
// every call, and each launched block overwrites its whole row before the
// reduction reads it, so nothing needs clearing. Calls that overlap on the GPU
// (different streams or host threads) race on the array.
constexpr int NOALLOC_MAX_BLOCKS = 2048;
static __device__ __align__(256) float g_noalloc_partials[NOALLOC_MAX_BLOCKS * ACC_N];
static const size_t NOALLOC_SCRATCH_BYTES = sizeof(float) * NOALLOC_MAX_BLOCKS * ACC_N;

// Host code cannot pass g_noalloc_partials itself: in host code the name is a
// host-side stand-in, not a device address. Every context looks the device
// address up once, at its creation (init_context in up_abi.cu, with the
// context's device current), and passes it to each launch. Creating the
// context also loads this file's module, so the array is resident from then
// on, and no later call queries the runtime (a call inside a stream capture
// makes no lookup). A device reset frees the array with everything else: the
// contexts made before it are dead, and contexts made after it look the new
// address up.
cudaError_t noalloc_scratch_address(float **out) {
	void *p = nullptr;
	const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
	*out = e == cudaSuccess ? (float *)p : nullptr;
	return e;
}

size_t noalloc_scratch_bytes() { return NOALLOC_SCRATCH_BYTES; }
int noalloc_max_blocks() { return NOALLOC_MAX_BLOCKS; }

cudaError_t launch_synth_bwd_noalloc(const up_synth_program &P, const float *xyz, uint64_t n, const float *w, float *dtheta, float *scratch,
	cudaStream_t s) {
	if (!scratch) return cudaErrorInvalidDevicePointer;
	int nblocks = synth_bwd_blocks(n);
	if (nblocks > NOALLOC_MAX_BLOCKS) nblocks = NOALLOC_MAX_BLOCKS;
	return launch_synth_bwd(P, xyz, n, w, scratch, nblocks, dtheta, s);
}

} // namespace up
