// Dual contouring: classification, ordered compaction, quad emission, and
// the synthetic-program instantiation of the Hermite/QEF kernels.
// Rules and pipeline: see up_contour.cuh.
#include "up_contour.cuh"
#include "up_synth.cuh"

namespace up {

// per-point flags packed as cells | edges << 21 | quads << 42 (counts per
// point: cells <= 1, edges <= 3, quads <= 3), plus the per-axis bits
struct PointFlags { uint32_t bits; }; // bit0 cell, bit1..3 edge x/y/z, bit4..6 quad x/y/z

__device__ __forceinline__ PointFlags point_flags(const float *__restrict__ d, const GridDev &g, uint32_t p) {
	PointFlags f{0};
	const uint32_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const uint32_t i = p % nx, r = p / nx, j = r % ny, k = r / ny;
	const uint32_t sxy = nx * ny;
	const bool in0 = __ldg(d + p) < 0.f;
	const bool hx = i + 1 < nx, hy = j + 1 < ny, hz = k + 1 < nz;
	const bool inx = hx && (__ldg(d + p + 1) < 0.f);
	const bool iny = hy && (__ldg(d + p + nx) < 0.f);
	const bool inz = hz && (__ldg(d + p + sxy) < 0.f);
	const bool iix = i >= 1 && i + 1 < nx, ijy = j >= 1 && j + 1 < ny, ikz = k >= 1 && k + 1 < nz;
	if (hx && inx != in0) { f.bits |= 2u; if (ijy && ikz) f.bits |= 16u; }
	if (hy && iny != in0) { f.bits |= 4u; if (iix && ikz) f.bits |= 32u; }
	if (hz && inz != in0) { f.bits |= 8u; if (iix && ijy) f.bits |= 64u; }
	if (hx && hy && hz) {
		const uint32_t m = (uint32_t)in0 | ((uint32_t)inx << 1) | ((uint32_t)iny << 2) | ((uint32_t)(__ldg(d + p + nx + 1) < 0.f) << 3) |
			((uint32_t)inz << 4) | ((uint32_t)(__ldg(d + p + sxy + 1) < 0.f) << 5) | ((uint32_t)(__ldg(d + p + sxy + nx) < 0.f) << 6) |
			((uint32_t)(__ldg(d + p + sxy + nx + 1) < 0.f) << 7);
		if (m != 0u && m != 255u) f.bits |= 1u;
	}
	return f;
}
__device__ __forceinline__ uint64_t pack_counts(PointFlags f) {
	const uint64_t c = f.bits & 1u;
	const uint64_t e = __popc(f.bits & 14u);
	const uint64_t q = __popc(f.bits & 112u);
	return c | (e << 21) | (q << 42);
}

// block-wide exclusive scan of one 64-bit value per thread
template<int T>
__device__ __forceinline__ uint64_t block_exscan(uint64_t v, uint64_t &total) {
	__shared__ uint64_t ws[T / 32];
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	uint64_t x = v;
	#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
		if (lane >= o) x += y;
	}
	if (lane == 31) ws[wid] = x;
	__syncthreads();
	if (wid == 0) {
		uint64_t w = lane < T / 32 ? ws[lane] : 0;
		#pragma unroll
		for (int o = 1; o < T / 32; o <<= 1) {
			const uint64_t y = __shfl_up_sync(0xffffffffu, w, o);
			if (lane >= o) w += y;
		}
		if (lane < T / 32) ws[lane] = w;
	}
	__syncthreads();
	const uint64_t off = wid > 0 ? ws[wid - 1] : 0;
	total = ws[T / 32 - 1];
	__syncthreads();
	return off + x - v;
}

// each thread owns DC_ITEMS consecutive points of the block's DC_PB points
__global__ void __launch_bounds__(DC_T) dc_count_kernel(const float *__restrict__ d, const GridDev g, uint32_t npts, uint32_t nblocks,
	uint32_t *__restrict__ blk) {
	const uint32_t base = blockIdx.x * DC_PB + threadIdx.x * DC_ITEMS;
	uint64_t c = 0;
	#pragma unroll
	for (int it = 0; it < DC_ITEMS; it++) {
		const uint32_t p = base + it;
		if (p < npts) c += pack_counts(point_flags(d, g, p));
	}
	uint64_t tot;
	block_exscan<DC_T>(c, tot);
	if (threadIdx.x == 0) {
		blk[blockIdx.x] = (uint32_t)(tot & 0x1FFFFF);
		blk[nblocks + blockIdx.x] = (uint32_t)((tot >> 21) & 0x1FFFFF);
		blk[2 * nblocks + blockIdx.x] = (uint32_t)(tot >> 42);
	}
}

// one block of 1024 threads: exclusive scan of the three block-count arrays
// in place; totals[a] = sum
__global__ void __launch_bounds__(1024) dc_scan_kernel(uint32_t *__restrict__ blk, uint32_t nblocks, uint32_t *__restrict__ totals) {
	const uint32_t per = (nblocks + 1023) / 1024;
	for (int a = 0; a < 3; a++) {
		uint32_t *arr = blk + (uint64_t)a * nblocks;
		const uint32_t b0 = threadIdx.x * per;
		uint64_t s = 0;
		for (uint32_t b = b0; b < b0 + per && b < nblocks; b++) s += arr[b];
		uint64_t tot;
		uint64_t run = block_exscan<1024>(s, tot);
		for (uint32_t b = b0; b < b0 + per && b < nblocks; b++) {
			const uint32_t v = arr[b];
			arr[b] = (uint32_t)run;
			run += v;
		}
		if (threadIdx.x == 0) totals[a] = (uint32_t)tot;
		__syncthreads();
	}
}

__global__ void __launch_bounds__(DC_T) dc_emit_kernel(const float *__restrict__ d, const GridDev g, uint32_t npts, uint32_t nblocks,
	const uint32_t *__restrict__ blk, uint32_t *__restrict__ cell_list, uint32_t *__restrict__ cell_map, uint32_t *__restrict__ edge_list,
	uint32_t *__restrict__ edge_map, uint32_t *__restrict__ quad_list) {
	const uint32_t base = blockIdx.x * DC_PB + threadIdx.x * DC_ITEMS;
	PointFlags f[DC_ITEMS];
	uint64_t c = 0;
	#pragma unroll
	for (int it = 0; it < DC_ITEMS; it++) {
		const uint32_t p = base + it;
		f[it].bits = 0;
		if (p < npts) f[it] = point_flags(d, g, p);
		c += pack_counts(f[it]);
	}
	uint64_t tot;
	const uint64_t off = block_exscan<DC_T>(c, tot);
	uint32_t co = blk[blockIdx.x] + (uint32_t)(off & 0x1FFFFF);
	uint32_t eo = blk[nblocks + blockIdx.x] + (uint32_t)((off >> 21) & 0x1FFFFF);
	uint32_t qo = blk[2 * nblocks + blockIdx.x] + (uint32_t)(off >> 42);
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint32_t cx = nx - 1, cy = ny - 1;
	#pragma unroll
	for (int it = 0; it < DC_ITEMS; it++) {
		const uint32_t p = base + it;
		const uint32_t b = f[it].bits;
		if (!b) continue;
		if (b & 1u) {
			const uint32_t i = p % nx, r = p / nx, j = r % ny, k = r / ny;
			cell_list[co] = p;
			cell_map[(k * cy + j) * cx + i] = co;
			co++;
		}
		#pragma unroll
		for (int a = 0; a < 3; a++) {
			if (b & (2u << a)) {
				const uint32_t code = 3 * p + a;
				edge_list[eo] = code;
				edge_map[code] = eo;
				if (b & (16u << a)) quad_list[qo++] = eo;
				eo++;
			}
		}
	}
}

__global__ void __launch_bounds__(256) dc_quads_kernel(const float *__restrict__ d, const GridDev g, const uint32_t *__restrict__ quad_list,
	uint32_t nquads, const uint32_t *__restrict__ edge_list, const uint32_t *__restrict__ cell_map, uint32_t *__restrict__ idx) {
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint32_t cx = nx - 1, cy = ny - 1;
	for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nquads; q += gridDim.x * blockDim.x) {
		const uint32_t code = edge_list[quad_list[q]];
		const uint32_t p = code / 3, a = code % 3;
		const uint32_t i = p % nx, r = p / nx, j = r % ny, k = r / ny;
		auto C = [&](uint32_t ci, uint32_t cj, uint32_t ck) { return cell_map[(ck * cy + cj) * cx + ci]; };
		uint32_t v0, v1, v2, v3;
		if (a == 0) { v0 = C(i, j - 1, k - 1); v1 = C(i, j, k - 1); v2 = C(i, j, k); v3 = C(i, j - 1, k); }
		else if (a == 1) { v0 = C(i - 1, j, k - 1); v1 = C(i - 1, j, k); v2 = C(i, j, k); v3 = C(i, j, k - 1); }
		else { v0 = C(i - 1, j - 1, k); v1 = C(i, j - 1, k); v2 = C(i, j, k); v3 = C(i - 1, j, k); }
		uint32_t *o = idx + 6 * (uint64_t)q;
		if (d[p] < 0.f) { o[0] = v0; o[1] = v1; o[2] = v2; o[3] = v0; o[4] = v2; o[5] = v3; }
		else { o[0] = v0; o[1] = v2; o[2] = v1; o[3] = v0; o[4] = v3; o[5] = v2; }
	}
}

uint32_t dc_num_blocks(const GridDev &g) {
	const uint64_t n = (uint64_t)g.n[0] * g.n[1] * g.n[2];
	return (uint32_t)((n + DC_PB - 1) / DC_PB);
}

cudaError_t dc_count(const float *d, const GridDev &g, DcScratch &S, cudaStream_t s) {
	const uint32_t npts = g.n[0] * g.n[1] * g.n[2];
	const uint32_t nb = dc_num_blocks(g);
	dc_count_kernel<<<nb, DC_T, 0, s>>>(d, g, npts, nb, S.blk_counts);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	dc_scan_kernel<<<1, 1024, 0, s>>>(S.blk_counts, nb, S.totals);
	return cudaGetLastError();
}

cudaError_t dc_emit(const float *d, const GridDev &g, DcScratch &S, cudaStream_t s) {
	const uint32_t npts = g.n[0] * g.n[1] * g.n[2];
	const uint32_t nb = dc_num_blocks(g);
	dc_emit_kernel<<<nb, DC_T, 0, s>>>(d, g, npts, nb, S.blk_counts, S.cell_list, S.cell_map, S.edge_list, S.edge_map, S.quad_list);
	return cudaGetLastError();
}

cudaError_t dc_quads_launch(const float *d, const GridDev &g, const DcScratch &S, uint32_t nquads, uint32_t *idx, cudaStream_t s) {
	if (!nquads) return cudaSuccess;
	const int b = persistent_blocks((const void *)dc_quads_kernel, 256);
	const uint32_t need = (nquads + 255) / 256;
	dc_quads_kernel<<<need < (uint32_t)b ? need : (uint32_t)b, 256, 0, s>>>(d, g, S.quad_list, nquads, S.edge_list, S.cell_map, idx);
	return cudaGetLastError();
}

struct SynthEvalF {
	up_synth_program P;
	__device__ __forceinline__ NG operator()(V3f p) const { return synth_eval<true, -1, -1>(P, p); }
};

cudaError_t dc_geometry_synth(const up_synth_program &P, const float *d, const GridDev &g, DcScratch &S, uint32_t ncells, uint32_t nedges,
	uint32_t nquads, float *pos, float *nrm, uint32_t *idx, cudaStream_t s) {
	SynthEvalF ev{P};
	return dc_geometry_t(ev, d, g, S, ncells, nedges, nquads, pos, nrm, idx, s);
}

} // namespace up
