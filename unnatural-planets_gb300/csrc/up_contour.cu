// Dual contouring: classification, ordered compaction, quad emission, and
// the synthetic-program instantiation of the Hermite/QEF kernels.
// Rules and pipeline: see up_contour.cuh.
#include "up_contour.cuh"
#include "up_synth.cuh"

namespace up {

// ---- word-parallel kernels (single grids; see dc_word_flags)
// one warp packs DC_SIGN_U consecutive words per step (DC_SIGN_U coalesced
// 128-byte loads in flight per warp); persistent grid
constexpr int DC_SIGN_U = 8;
__global__ void __launch_bounds__(256) dc_signs_kernel(const float *__restrict__ d, uint32_t npts, uint64_t nalloc, uint32_t *__restrict__ bits) {
	const uint32_t lane = threadIdx.x & 31;
	const uint64_t step = (((uint64_t)gridDim.x * blockDim.x) >> 5) * DC_SIGN_U;
	for (uint64_t w0 = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * DC_SIGN_U; w0 < nalloc; w0 += step) { // warp-uniform
		bool in[DC_SIGN_U];
		#pragma unroll
		for (int u = 0; u < DC_SIGN_U; u++) {
			const uint64_t p = 32 * (w0 + u) + lane;
			in[u] = p < npts && __ldg(d + p) < 0.f;
		}
		uint32_t mine = 0;
		#pragma unroll
		for (int u = 0; u < DC_SIGN_U; u++) {
			const uint32_t m = __ballot_sync(0xFFFFFFFFu, in[u]);
			if (lane == (uint32_t)u) mine = m;
		}
		if (lane < DC_SIGN_U && w0 + lane < nalloc) bits[w0 + lane] = mine;
	}
}
__global__ void __launch_bounds__(DC_T) dc_wcount_kernel(const uint32_t *__restrict__ bits, uint64_t nalloc, const GridDev g, uint32_t npts,
	uint32_t nblocks, uint32_t *__restrict__ blk) {
	const WordFlags f = dc_word_flags(bits, nalloc, g, (uint64_t)blockIdx.x * DC_T + threadIdx.x, npts);
	uint64_t tot;
	block_exscan<DC_T>(dc_word_counts(f), tot);
	if (threadIdx.x == 0) {
		blk[blockIdx.x] = (uint32_t)(tot & 0x1FFFFF);
		blk[nblocks + blockIdx.x] = (uint32_t)((tot >> 21) & 0x1FFFFF);
		blk[2 * nblocks + blockIdx.x] = (uint32_t)(tot >> 42);
	}
}
__global__ void __launch_bounds__(DC_T) dc_wemit_kernel(const uint32_t *__restrict__ bits, uint64_t nalloc, const GridDev g, uint32_t npts,
	uint32_t nblocks, const uint32_t *__restrict__ blk, uint32_t *__restrict__ cell_list, uint32_t *__restrict__ cell_map,
	uint32_t *__restrict__ edge_list, uint32_t *__restrict__ edge_map, uint32_t *__restrict__ quad_list) {
	const uint64_t w = (uint64_t)blockIdx.x * DC_T + threadIdx.x;
	const WordFlags f = dc_word_flags(bits, nalloc, g, w, npts);
	uint64_t tot;
	const uint64_t off = block_exscan<DC_T>(dc_word_counts(f), tot);
	uint32_t co = blk[blockIdx.x] + (uint32_t)(off & 0x1FFFFF);
	uint32_t eo = blk[nblocks + blockIdx.x] + (uint32_t)((off >> 21) & 0x1FFFFF);
	uint32_t qo = blk[2 * nblocks + blockIdx.x] + (uint32_t)(off >> 42);
	const uint32_t p0 = (uint32_t)(32 * w);
	const uint32_t nx = g.n[0], ny = g.n[1], cx = nx - 1, cy = ny - 1;
	for (uint32_t m = f.cell; m; m &= m - 1) {
		const uint32_t p = p0 + (uint32_t)(__ffs(m) - 1);
		const uint32_t r = p / nx, i = p - r * nx, j = r % ny, k = r / ny;
		cell_list[co] = p;
		cell_map[(k * cy + j) * cx + i] = co;
		co++;
	}
	for (uint32_t m = f.ex | f.ey | f.ez; m; m &= m - 1) {
		const uint32_t b = (uint32_t)(__ffs(m) - 1);
		const uint32_t p = p0 + b;
		const uint32_t e[3] = {f.ex, f.ey, f.ez}, q[3] = {f.qx, f.qy, f.qz};
		#pragma unroll
		for (int a = 0; a < 3; a++) {
			if (!((e[a] >> b) & 1u)) continue;
			const uint32_t code = 3 * p + a;
			edge_list[eo] = code;
			edge_map[code] = eo;
			if ((q[a] >> b) & 1u) quad_list[qo++] = eo;
			eo++;
		}
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

__global__ void __launch_bounds__(256) dc_quads_kernel(const float *__restrict__ d, const GridDev g, const uint32_t *__restrict__ quad_list,
	uint32_t nquads, const uint32_t *__restrict__ edge_list, const uint32_t *__restrict__ cell_map, uint32_t *__restrict__ idx) {
	for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nquads; q += gridDim.x * blockDim.x)
		dc_quad_item(d, g, edge_list[quad_list[q]], cell_map, 0u, idx + 6 * (uint64_t)q);
}

uint32_t dc_num_blocks(const GridDev &g) {
	const uint64_t n = (uint64_t)g.n[0] * g.n[1] * g.n[2];
	return (uint32_t)((n + DC_WPB - 1) / DC_WPB);
}
uint64_t dc_sign_words(const GridDev &g) { return ((uint64_t)g.n[0] * g.n[1] * g.n[2] + 31) / 32 + 2; }

cudaError_t dc_count(const float *d, const GridDev &g, DcScratch &S, cudaStream_t s, bool signs_ready) {
	const uint32_t npts = g.n[0] * g.n[1] * g.n[2];
	const uint32_t nb = dc_num_blocks(g);
	const uint64_t nalloc = dc_sign_words(g);
	if (!signs_ready) {
		const uint64_t need = (nalloc + DC_SIGN_U * 8 - 1) / (DC_SIGN_U * 8); // 8 warps per block
		const int pb = persistent_blocks((const void *)dc_signs_kernel, 256);
		dc_signs_kernel<<<(unsigned)(need < (uint64_t)pb ? need : (uint64_t)pb), 256, 0, s>>>(d, npts, nalloc, S.signs);
	}
	dc_wcount_kernel<<<nb, DC_T, 0, s>>>(S.signs, nalloc, g, npts, nb, S.blk_counts);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	return dc_scan_blocks(S.blk_counts, nb, S.totals, s);
}


cudaError_t dc_emit(const float *d, const GridDev &g, DcScratch &S, cudaStream_t s) {
	const uint32_t npts = g.n[0] * g.n[1] * g.n[2];
	const uint32_t nb = dc_num_blocks(g);
	dc_wemit_kernel<<<nb, DC_T, 0, s>>>(S.signs, dc_sign_words(g), g, npts, nb, S.blk_counts, S.cell_list, S.cell_map, S.edge_list, S.edge_map,
		S.quad_list);
	return cudaGetLastError();
}

cudaError_t dc_quads_launch(const float *d, const GridDev &g, const DcScratch &S, uint32_t nquads, uint32_t *idx, cudaStream_t s) {
	if (!nquads) return cudaSuccess;
	const int b = persistent_blocks((const void *)dc_quads_kernel, 256);
	const uint32_t need = (nquads + 255) / 256;
	dc_quads_kernel<<<need < (uint32_t)b ? need : (uint32_t)b, 256, 0, s>>>(d, g, S.quad_list, nquads, S.edge_list, S.cell_map, idx);
	return cudaGetLastError();
}

// evaluator of a synthetic program: noise types of the two layers fixed at
// compile time (T0/T1) or read at run time (-1)
template<int T0, int T1>
struct SynthEvalF {
	up_synth_program P;
	__device__ __forceinline__ NG operator()(V3f p) const { return synth_eval<true, T0, T1>(P, p); }
};

cudaError_t dc_geometry_synth(const up_synth_program &P, const float *d, const GridDev &g, DcScratch &S, uint32_t ncells, uint32_t nedges,
	uint32_t nquads, float *pos, float *nrm, uint32_t *idx, cudaStream_t s) {
	// Perlin + Euclidean F2 - F1 cellular: the benchmark program's specialisation
	if (P.n_layers == 2 && P.layer[0].type == UP_NOISE_PERLIN && P.layer[1].type == UP_NOISE_CELLULAR &&
		P.layer[1].distance == UP_DIST_EUCLIDEAN && P.layer[1].operation == UP_OP_SUBTRACT) {
		SynthEvalF<2, cell_spec(UP_DIST_EUCLIDEAN, UP_OP_SUBTRACT)> ev{P};
		return dc_geometry_t(ev, d, g, S, ncells, nedges, nquads, pos, nrm, idx, s);
	}
	SynthEvalF<-1, -1> ev{P};
	return dc_geometry_t(ev, d, g, S, ncells, nedges, nquads, pos, nrm, idx, s);
}

} // namespace up
