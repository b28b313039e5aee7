// Dual contouring: classification, ordered compaction, quad emission, and
// the synthetic-program instantiation of the Hermite/QEF kernels.
// Rules and pipeline: see up_contour.cuh.
#include "up_contour.cuh"
#include "up_synth.cuh"

namespace up {

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

// Exclusive scan of the three block-count arrays blk[a * nb + b] in place,
// totals[a] = sum, in three launches: chunks of 1024 entries scanned by one
// block each (coalesced), the chunk sums scanned by one block, the chunk
// offsets added. The chunk sums live after the arrays: part = blk + 3 nb.
__global__ void __launch_bounds__(1024) dc_scan_chunks_kernel(uint32_t *__restrict__ blk, uint32_t nb, uint32_t nch, uint32_t *__restrict__ part) {
	const uint32_t x = blockIdx.x * 1024 + threadIdx.x;
	for (int a = 0; a < 3; a++) {
		uint32_t *arr = blk + (uint64_t)a * nb;
		const uint32_t v = x < nb ? arr[x] : 0u;
		uint64_t tot;
		const uint64_t ex = block_exscan<1024>(v, tot);
		if (x < nb) arr[x] = (uint32_t)ex;
		if (threadIdx.x == 0) part[a * nch + blockIdx.x] = (uint32_t)tot;
	}
}
__global__ void __launch_bounds__(1024) dc_scan_top_kernel(uint32_t *__restrict__ part, uint32_t nch, uint32_t *__restrict__ totals) {
	const uint32_t per = (nch + 1023) / 1024;
	for (int a = 0; a < 3; a++) {
		uint32_t *arr = part + (uint64_t)a * nch;
		const uint32_t b0 = threadIdx.x * per;
		uint64_t s = 0;
		for (uint32_t b = b0; b < b0 + per && b < nch; b++) s += arr[b];
		uint64_t tot;
		uint64_t run = block_exscan<1024>(s, tot);
		for (uint32_t b = b0; b < b0 + per && b < nch; b++) {
			const uint32_t v = arr[b];
			arr[b] = (uint32_t)run;
			run += v;
		}
		if (threadIdx.x == 0) totals[a] = (uint32_t)tot;
	}
}
__global__ void __launch_bounds__(1024) dc_scan_add_kernel(uint32_t *__restrict__ blk, uint32_t nb, uint32_t nch, const uint32_t *__restrict__ part) {
	const uint32_t x = blockIdx.x * 1024 + threadIdx.x;
	if (x >= nb) return;
	#pragma unroll
	for (int a = 0; a < 3; a++) blk[(uint64_t)a * nb + x] += part[a * nch + blockIdx.x];
}

size_t dc_scan_words(uint32_t nb) { return 3 * (size_t)nb + 3 * (size_t)((nb + 1023) / 1024); }

cudaError_t dc_scan_blocks(uint32_t *blk, uint32_t nb, uint32_t *totals, cudaStream_t s) {
	const uint32_t nch = (nb + 1023) / 1024;
	uint32_t *part = blk + 3 * (size_t)nb;
	if (nch) dc_scan_chunks_kernel<<<nch, 1024, 0, s>>>(blk, nb, nch, part);
	dc_scan_top_kernel<<<1, 1024, 0, s>>>(part, nch, totals);
	if (nch) dc_scan_add_kernel<<<nch, 1024, 0, s>>>(blk, nb, nch, part);
	return cudaGetLastError();
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
	for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nquads; q += gridDim.x * blockDim.x)
		dc_quad_item(d, g, edge_list[quad_list[q]], cell_map, 0u, idx + 6 * (uint64_t)q);
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
	return dc_scan_blocks(S.blk_counts, nb, S.totals, s);
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
