// Batched sampling and dual contouring of many chunks of uneven size, from
// many planets, with one launch per stage over all chunks.
//
// No direct reference counterpart: the reference contours one planet field
// at a time (sources/meshGeneration.cpp:32-44) and fans chunk work out over
// CPU tasks (tasksRunBlocking, sources/generator.cpp:159,215).
//
// Stages (each one launch covering every chunk):
//   sample  persistent blocks pull tiles of samples from a device work
//           counter; a tile belongs to one chunk (binary search of the tile
//           table); values go to one concatenated grid, and the sign bits
//           of every chunk, 32 points per word, to chunk c's words from
//           word_off
//   count   per 8192-point block of every chunk: active cells, sign edges,
//           quads from the sign words (dc_word_flags of up_contour.cuh)
//   scan    exclusive scan of all block counts (global order = chunk order)
//   offsets per-chunk list offsets from the scan
//   emit    ordered lists and per-chunk maps
//   hermite / qef / quads  over the global lists, chunk found by binary search
// The first call for a given (planets, chunks) input runs eagerly (the host
// needs the totals to size the lists), autotunes the sampling stage's tile
// shape (1024 to 16384 samples per tile) and block size (128/256/512
// threads) by timing each pair on this input, then captures the stages in a
// CUDA graph on a private stream; later calls with byte-identical inputs
// replay the graph (the same work, recomputed, with the chosen shape) without
// host round trips.
#include "up_contour.cuh"
#include "up_synth.cuh"

#include <atomic>
#include <cstddef>
#include <cstring>
#include <vector>

namespace up {

struct BatchChunkDev {
	GridDev g;
	uint32_t planet;
	uint32_t pt_off, cell_off, blk_off;
	uint32_t word_off, nwords; // sign words: ceil(points / 32) + 2 (zero slack for dc_bits_at)
	float band; // narrow band of contouring (0: exact values, when the caller reads them)
	FastDiv divx, divy; // by n[0] and n[1]
};

// tile shapes of the sampling stage, chosen per input by the autotune
constexpr int BATCH_NTILE = 5;
constexpr uint32_t BATCH_TILES[BATCH_NTILE] = {1024, 2048, 4096, 8192, 16384};
// dynamic shared memory of a tile: its list of band samples and its sign words
__host__ __device__ constexpr size_t batch_tile_smem(uint32_t tile) { return (size_t)tile * 2 + (size_t)tile / 32 * 4; }

__device__ __forceinline__ uint32_t find_chunk(const uint32_t *__restrict__ starts, uint32_t n, uint32_t x) {
	// last c with starts[c] <= x (starts ascending, starts[0] = 0)
	uint32_t lo = 0, hi = n;
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (starts[mid] <= x) lo = mid;
		else hi = mid;
	}
	return lo;
}

__device__ __forceinline__ float bgrid_coord(const GridDev &g, int a, uint32_t i) {
	return __fadd_rn(__fmul_rn((float)i, g.step[a]), g.lo[a]);
}

// value of a tile's sample with the planet's layer types fixed at compile
// time where they are the batch planets' (one Perlin or one simplex layer)
__device__ __forceinline__ float batch_eval(const up_synth_program &P, V3f p) {
	if (P.n_layers == 1 && P.layer[0].type == UP_NOISE_PERLIN) return synth_eval<false, 2, -1>(P, p).v;
	if (P.n_layers == 1 && P.layer[0].type == UP_NOISE_SIMPLEX) return synth_eval<false, 3, -1>(P, p).v;
	return synth_eval<false, -1, -1>(P, p).v;
}

// A tile in two passes: every sample's base shape, stored at once where the
// sample lies outside the narrow band; the others are listed in shared
// memory and evaluated in full by consecutive threads, so the noise runs in
// full warps however the band crosses the tile.
// The tile's sign words (d < 0, 32 samples a word: a warp's samples in the
// first pass) are formed in shared memory and stored with the values.
extern __shared__ uint32_t batch_smem[]; // sampling: TILE / 32 sign words, then TILE list entries

// the sampling stage, run by every block of a launch: tiles are taken from
// *counter until none is left
template<int THREADS>
__device__ __forceinline__ void batch_sample_body(const up_synth_program *__restrict__ planets, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ tile_starts, uint32_t nchunks, uint32_t ntiles, uint32_t TILE, float *__restrict__ d, uint32_t *__restrict__ bits,
	unsigned *__restrict__ counter, unsigned *__restrict__ nanflag) {
	__shared__ uint32_t tile, nnear;
	uint32_t *words = batch_smem;
	uint16_t *near = (uint16_t *)(batch_smem + TILE / 32);
	const uint32_t lane = threadIdx.x & 31;
	bool bad = false;
	for (;;) {
		if (threadIdx.x == 0) { tile = atomicAdd(counter, 1u); nnear = 0; }
		__syncthreads();
		const uint32_t t = tile;
		if (t >= ntiles) break; // the same for every thread
		const uint32_t c = find_chunk(tile_starts, nchunks, t);
		const BatchChunkDev &ch = chunks[c];
		const up_synth_program &P = planets[ch.planet];
		const uint32_t nx = ch.g.n[0], ny = ch.g.n[1];
		const uint32_t npts = nx * ny * ch.g.n[2];
		const uint32_t base = (t - tile_starts[c]) * TILE;
		const FastDiv dx = ch.divx, dy = ch.divy;
		#pragma unroll 1
		for (uint32_t it = threadIdx.x; it < TILE; it += THREADS) { // every thread the same trip count
			const uint32_t s = base + it;
			bool full = false, neg = false;
			if (s < npts) {
				if (ch.band > 0.f) {
					const uint32_t r = dx.div(s), i = s - r * nx, k = dy.div(r), j = r - k * ny;
					const float v = synth_base<false>(P, v3(bgrid_coord(ch.g, 0, i), bgrid_coord(ch.g, 1, j), bgrid_coord(ch.g, 2, k))).v;
					if (fabsf(v) > ch.band) {
						d[ch.pt_off + s] = v;
						neg = v < 0.f;
					} else {
						full = true;
					}
				} else {
					full = true;
				}
			}
			const unsigned m = __ballot_sync(0xFFFFFFFFu, full);
			uint32_t slot = 0;
			if (lane == 0 && m) slot = atomicAdd(&nnear, (uint32_t)__popc(m));
			slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
			if (full) near[slot + __popc(m & ((1u << lane) - 1u))] = (uint16_t)it;
			// signs of the stored samples now; the listed ones are or-ed in below
			const unsigned negs = __ballot_sync(0xFFFFFFFFu, neg);
			if (lane == 0) words[it >> 5] = negs;
		}
		__syncthreads();
		const uint32_t nn = nnear;
		#pragma unroll 1
		for (uint32_t e = threadIdx.x; e < nn; e += THREADS) {
			const uint32_t it = near[e], s = base + it;
			const uint32_t r = dx.div(s), i = s - r * nx, k = dy.div(r), j = r - k * ny;
			const float v = batch_eval(P, v3(bgrid_coord(ch.g, 0, i), bgrid_coord(ch.g, 1, j), bgrid_coord(ch.g, 2, k)));
			d[ch.pt_off + s] = v;
			bad |= isnan(v);
			if (v < 0.f) atomicOr(&words[it >> 5], 1u << (it & 31));
		}
		__syncthreads();
		// the tile's words that belong to the chunk (its data words, and the
		// two zero words after them from its last tile)
		const uint32_t w0 = base >> 5;
		for (uint32_t w = threadIdx.x; w < TILE / 32; w += THREADS)
			if (w0 + w < ch.nwords) bits[ch.word_off + w0 + w] = words[w];
		if (threadIdx.x < 2 && base + TILE >= npts) {
			const uint32_t ws = (npts + 31) / 32 + threadIdx.x; // slack words
			if (ws >= w0 + TILE / 32) bits[ch.word_off + ws] = 0u;
		}
		__syncthreads(); // the tile's list and words are read before the next tile is taken
	}
	if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(nanflag, 1u);
}
template<int THREADS>
__global__ void __launch_bounds__(THREADS) batch_sample_kernel(const up_synth_program *__restrict__ planets, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ tile_starts, uint32_t nchunks, uint32_t ntiles, uint32_t TILE, float *__restrict__ d, uint32_t *__restrict__ bits,
	unsigned *__restrict__ counter, unsigned *__restrict__ nanflag) {
	batch_sample_body<THREADS>(planets, chunks, tile_starts, nchunks, ntiles, TILE, d, bits, counter, nanflag);
}

// counts of word block vb (DC_T threads, DC_WPB points of one chunk)
__device__ __forceinline__ void batch_count_body(const uint32_t *__restrict__ bits, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ blk_starts, uint32_t nchunks, uint32_t nblocks, uint32_t *__restrict__ blk, uint32_t vb) {
	const uint32_t c = find_chunk(blk_starts, nchunks, vb);
	const BatchChunkDev &ch = chunks[c];
	const uint32_t npts = ch.g.n[0] * ch.g.n[1] * ch.g.n[2];
	const uint64_t w = (uint64_t)(vb - ch.blk_off) * DC_T + threadIdx.x;
	const WordFlags f = dc_word_flags(bits + ch.word_off, ch.nwords, ch.g, w, npts);
	uint64_t tot;
	block_exscan<DC_T>(dc_word_counts(f), tot);
	if (threadIdx.x == 0) {
		blk[vb] = (uint32_t)(tot & 0x1FFFFF);
		blk[nblocks + vb] = (uint32_t)((tot >> 21) & 0x1FFFFF);
		blk[2 * nblocks + vb] = (uint32_t)(tot >> 42);
	}
}
__global__ void __launch_bounds__(DC_T) batch_count_kernel(const uint32_t *__restrict__ bits, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ blk_starts, uint32_t nchunks, uint32_t nblocks, uint32_t *__restrict__ blk) {
	batch_count_body(bits, chunks, blk_starts, nchunks, nblocks, blk, blockIdx.x);
}

// per-chunk offsets of the three lists (+ totals at index nchunks)
__device__ __forceinline__ void batch_offsets_body(const BatchChunkDev *__restrict__ chunks, uint32_t nchunks, uint32_t nblocks,
	const uint32_t *__restrict__ blk, const uint32_t *__restrict__ totals, uint32_t *__restrict__ off) {
	for (uint32_t c = threadIdx.x + blockIdx.x * blockDim.x; c <= nchunks; c += blockDim.x * gridDim.x) {
		for (int a = 0; a < 3; a++)
			off[a * (nchunks + 1) + c] = c < nchunks ? __ldcg(blk + (uint64_t)a * nblocks + chunks[c].blk_off) : __ldcg(totals + a);
	}
}
__global__ void batch_offsets_kernel(const BatchChunkDev *__restrict__ chunks, uint32_t nchunks, uint32_t nblocks, const uint32_t *__restrict__ blk,
	const uint32_t *__restrict__ totals, uint32_t *__restrict__ off) {
	batch_offsets_body(chunks, nchunks, nblocks, blk, totals, off);
}

// lists and maps of word block vb (DC_T threads)
__device__ __forceinline__ void batch_emit_body(const uint32_t *__restrict__ bits, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ blk_starts, uint32_t nchunks, uint32_t nblocks, const uint32_t *__restrict__ blk, uint32_t *__restrict__ cell_list,
	uint32_t *__restrict__ cell_map, uint32_t *__restrict__ edge_list, uint32_t *__restrict__ edge_map, uint32_t *__restrict__ quad_list, uint32_t vb) {
	const uint32_t c = find_chunk(blk_starts, nchunks, vb);
	const BatchChunkDev &ch = chunks[c];
	const GridDev g = ch.g;
	const uint32_t npts = g.n[0] * g.n[1] * g.n[2];
	const uint64_t w = (uint64_t)(vb - ch.blk_off) * DC_T + threadIdx.x;
	const WordFlags f = dc_word_flags(bits + ch.word_off, ch.nwords, g, w, npts);
	uint64_t tot;
	const uint64_t o = block_exscan<DC_T>(dc_word_counts(f), tot);
	// (L2-coherent loads: in the persistent kernel other blocks wrote blk in
	// this launch)
	uint32_t co = __ldcg(blk + vb) + (uint32_t)(o & 0x1FFFFF);
	uint32_t eo = __ldcg(blk + nblocks + vb) + (uint32_t)((o >> 21) & 0x1FFFFF);
	uint32_t qo = __ldcg(blk + 2 * nblocks + vb) + (uint32_t)(o >> 42);
	const uint32_t p0 = (uint32_t)(32 * w);
	const uint32_t nx = g.n[0], ny = g.n[1], cx = nx - 1, cy = ny - 1;
	uint32_t *cmap = cell_map + ch.cell_off;
	uint32_t *emap = edge_map + 3 * (uint64_t)ch.pt_off;
	// the same order as the per-point form: cells in point order, then each
	// point's edges x, y, z (lists stay in ascending point order)
	for (uint32_t m = f.cell; m; m &= m - 1) {
		const uint32_t p = p0 + (uint32_t)(__ffs(m) - 1);
		const uint32_t r = p / nx, i = p - r * nx, j = r % ny, k = r / ny;
		cell_list[co] = p;
		cmap[(k * cy + j) * cx + i] = co;
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
			emap[code] = eo;
			if ((q[a] >> b) & 1u) quad_list[qo++] = eo;
			eo++;
		}
	}
}
__global__ void __launch_bounds__(DC_T) batch_emit_kernel(const uint32_t *__restrict__ bits, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ blk_starts, uint32_t nchunks, uint32_t nblocks, const uint32_t *__restrict__ blk, uint32_t *__restrict__ cell_list,
	uint32_t *__restrict__ cell_map, uint32_t *__restrict__ edge_list, uint32_t *__restrict__ edge_map, uint32_t *__restrict__ quad_list) {
	batch_emit_body(bits, chunks, blk_starts, nchunks, nblocks, blk, cell_list, cell_map, edge_list, edge_map, quad_list, blockIdx.x);
}

struct BatchEvalF {
	const up_synth_program *P;
	__device__ __forceinline__ NG operator()(V3f p) const { return synth_eval<true, -1, -1>(*P, p); }
};

// the stages below run grid-stride over their lists, as kernels of their own
// or as phases of the persistent kernel
__device__ __forceinline__ void batch_hermite_body(const up_synth_program *__restrict__ planets, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ off, uint32_t nchunks, const float *__restrict__ d, const uint32_t *__restrict__ edge_list,
	float *__restrict__ edge_t, float *__restrict__ edge_n) {
	const uint32_t *eoff = off + (nchunks + 1);
	const uint32_t nedges = eoff[nchunks];
	for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < nedges; e += gridDim.x * blockDim.x) {
		const uint32_t c = find_chunk(eoff, nchunks, e);
		const BatchChunkDev &ch = chunks[c];
		dc_hermite_item(BatchEvalF{planets + ch.planet}, d + ch.pt_off, ch.g, edge_list[e], edge_t[e], edge_n + 3 * (uint64_t)e);
	}
}
__global__ void __launch_bounds__(256) batch_hermite_kernel(const up_synth_program *__restrict__ planets, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ off, uint32_t nchunks, const float *__restrict__ d, const uint32_t *__restrict__ edge_list,
	float *__restrict__ edge_t, float *__restrict__ edge_n) {
	batch_hermite_body(planets, chunks, off, nchunks, d, edge_list, edge_t, edge_n);
}

// FP32 QEF of every cell; the cells that need the FP64 solver go to fb_list
// (count in *fb_count) for batch_qef_fp64_kernel (see dc_qef_kernel)
__device__ __forceinline__ void batch_qef_body(const up_synth_program *__restrict__ planets, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ off, uint32_t nchunks, const float *__restrict__ d, const uint32_t *__restrict__ cell_list,
	const uint32_t *__restrict__ edge_map, const float *__restrict__ edge_t, const float *__restrict__ edge_n, float *__restrict__ pos,
	uint32_t *__restrict__ fb_list, uint32_t *__restrict__ fb_count) {
	const uint32_t ncells = off[nchunks];
	for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < ncells; q += gridDim.x * blockDim.x) {
		const uint32_t c = find_chunk(off, nchunks, q);
		const BatchChunkDev &ch = chunks[c];
		if (!dc_qef_item(BatchEvalF{planets + ch.planet}, NegFromValues{d + ch.pt_off}, ch.g, cell_list[q], edge_map + 3 * (uint64_t)ch.pt_off, edge_t, edge_n,
				pos + 3 * (uint64_t)q, nullptr))
			fb_list[atomicAdd(fb_count, 1u)] = q;
	}
}
__global__ void __launch_bounds__(128) batch_qef_kernel(const up_synth_program *__restrict__ planets, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ off, uint32_t nchunks, const float *__restrict__ d, const uint32_t *__restrict__ cell_list,
	const uint32_t *__restrict__ edge_map, const float *__restrict__ edge_t, const float *__restrict__ edge_n, float *__restrict__ pos,
	uint32_t *__restrict__ fb_list, uint32_t *__restrict__ fb_count) {
	batch_qef_body(planets, chunks, off, nchunks, d, cell_list, edge_map, edge_t, edge_n, pos, fb_list, fb_count);
}
// one cell per one-warp block, as dc_qef_fp64_kernel
// cells first, first + stride, ... of the FP64 list, by the calling thread
__device__ __forceinline__ void batch_qef_fp64_body(const up_synth_program *__restrict__ planets, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ off, uint32_t nchunks, const float *__restrict__ d, const uint32_t *__restrict__ cell_list,
	const uint32_t *__restrict__ edge_map, const float *__restrict__ edge_t, const float *__restrict__ edge_n, float *__restrict__ pos,
	const uint32_t *__restrict__ fb_list, const uint32_t *__restrict__ fb_count, uint32_t first, uint32_t stride) {
	const uint32_t n = *fb_count;
	for (uint32_t e = first; e < n; e += stride) {
		const uint32_t q = fb_list[e];
		const uint32_t c = find_chunk(off, nchunks, q);
		const BatchChunkDev &ch = chunks[c];
		double vd[3];
		dc_qef_vertex_fp64(NegFromValues{d + ch.pt_off}, ch.g, cell_list[q], edge_map + 3 * (uint64_t)ch.pt_off, edge_t, edge_n, vd);
		const float vc[3] = {(float)vd[0], (float)vd[1], (float)vd[2]};
		dc_vertex_out(BatchEvalF{planets + ch.planet}, ch.g, cell_list[q], vc, pos + 3 * (uint64_t)q, nullptr);
	}
}
__global__ void __launch_bounds__(32) batch_qef_fp64_kernel(const up_synth_program *__restrict__ planets, const BatchChunkDev *__restrict__ chunks,
	const uint32_t *__restrict__ off, uint32_t nchunks, const float *__restrict__ d, const uint32_t *__restrict__ cell_list,
	const uint32_t *__restrict__ edge_map, const float *__restrict__ edge_t, const float *__restrict__ edge_n, float *__restrict__ pos,
	const uint32_t *__restrict__ fb_list, const uint32_t *__restrict__ fb_count) {
	if (threadIdx.x == 0)
		batch_qef_fp64_body(planets, chunks, off, nchunks, d, cell_list, edge_map, edge_t, edge_n, pos, fb_list, fb_count, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void batch_quads_body(const BatchChunkDev *__restrict__ chunks, const uint32_t *__restrict__ off, uint32_t nchunks,
	const float *__restrict__ d, const uint32_t *__restrict__ quad_list, const uint32_t *__restrict__ edge_list,
	const uint32_t *__restrict__ cell_map, uint32_t *__restrict__ idx) {
	const uint32_t *coff = off, *qoff = off + 2 * (nchunks + 1);
	const uint32_t nquads = qoff[nchunks];
	for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nquads; q += gridDim.x * blockDim.x) {
		const uint32_t c = find_chunk(qoff, nchunks, q);
		const BatchChunkDev &ch = chunks[c];
		dc_quad_item(d + ch.pt_off, ch.g, edge_list[quad_list[q]], cell_map + ch.cell_off, coff[c], idx + 6 * (uint64_t)q);
	}
}
__global__ void __launch_bounds__(256) batch_quads_kernel(const BatchChunkDev *__restrict__ chunks, const uint32_t *__restrict__ off, uint32_t nchunks,
	const float *__restrict__ d, const uint32_t *__restrict__ quad_list, const uint32_t *__restrict__ edge_list,
	const uint32_t *__restrict__ cell_map, uint32_t *__restrict__ idx) {
	batch_quads_body(chunks, off, nchunks, d, quad_list, edge_list, cell_map, idx);
}

// ---------------------------------------------------------------- one persistent launch
// Every stage above as a phase of one kernel: persistent blocks of 256
// threads (the count and emit block size), launched cooperatively so that all
// are resident, separated by a grid-wide barrier. Phases: sample | count |
// scan (chunks, top, add) | per-chunk offsets | emit | Hermite data and quads |
// FP32 QEF | FP64 QEF. The outputs are those of the stage launches.

// barrier words (reset before every launch, except gen) and the wait limit
struct BatchBarrier {
	unsigned count, gen, err, pad;
	unsigned long long limit_ns;
};

__device__ __forceinline__ unsigned long long batch_now_ns() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// Grid-wide barrier with a bounded wait: the last block to arrive opens the
// next generation; the others wait for it at most limit_ns (global timer),
// then record err and return false, as they do when another block has
// recorded err. Every block stops at its first false. Memory written before
// the barrier is visible after it (fence before arriving and after leaving,
// as in a cooperative-groups grid sync).
__device__ __noinline__ bool batch_grid_sync(BatchBarrier *b) {
	__shared__ int ok;
	__syncthreads();
	if (threadIdx.x == 0) {
		ok = 1;
		volatile unsigned *vgen = &b->gen, *verr = &b->err;
		const unsigned g = *vgen;
		__threadfence();
		if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
			atomicExch(&b->count, 0u);
			__threadfence();
			atomicAdd(&b->gen, 1u);
		} else {
			const unsigned long long t0 = batch_now_ns(), limit = b->limit_ns;
			while (*vgen == g) {
				if (*verr != 0u || batch_now_ns() - t0 > limit) {
					atomicOr(&b->err, 1u);
					ok = 0;
					break;
				}
				__nanosleep(128);
			}
		}
		__threadfence();
		if (*verr != 0u) ok = 0;
	}
	__syncthreads();
	return ok != 0;
}

// scan of the three block-count arrays (the layout and result of
// dc_scan_blocks: 1024-entry chunks, chunk sums after the arrays), in three
// phases separated by barriers; 256 threads x 4 entries per chunk
__device__ __forceinline__ void batch_scan_chunks_phase(uint32_t *blk, uint32_t nb, uint32_t nch, uint32_t *part) {
	for (uint32_t item = blockIdx.x; item < 3 * nch; item += gridDim.x) {
		const uint32_t a = item / nch, ch = item - a * nch;
		uint32_t *arr = blk + (uint64_t)a * nb;
		const uint32_t x0 = ch * 1024 + threadIdx.x * 4;
		uint32_t v[4];
		uint64_t sum = 0;
		#pragma unroll
		for (int k = 0; k < 4; k++) {
			v[k] = x0 + k < nb ? __ldcg(arr + x0 + k) : 0u;
			sum += v[k];
		}
		uint64_t tot;
		uint64_t run = block_exscan<256>(sum, tot);
		#pragma unroll
		for (int k = 0; k < 4; k++) {
			if (x0 + k < nb) arr[x0 + k] = (uint32_t)run;
			run += v[k];
		}
		if (threadIdx.x == 0) part[a * nch + ch] = (uint32_t)tot;
	}
}
// block 0 only: exclusive scan of the chunk sums, totals[a] = array sums
__device__ __forceinline__ void batch_scan_top_phase(uint32_t *part, uint32_t nch, uint32_t *totals) {
	const uint32_t per = (nch + 255) / 256;
	for (int a = 0; a < 3; a++) {
		uint32_t *arr = part + (uint64_t)a * nch;
		const uint32_t b0 = threadIdx.x * per;
		uint64_t sum = 0;
		for (uint32_t b = b0; b < b0 + per && b < nch; b++) sum += __ldcg(arr + b);
		uint64_t tot;
		uint64_t run = block_exscan<256>(sum, tot);
		for (uint32_t b = b0; b < b0 + per && b < nch; b++) {
			const uint32_t v = __ldcg(arr + b);
			arr[b] = (uint32_t)run;
			run += v;
		}
		if (threadIdx.x == 0) totals[a] = (uint32_t)tot;
	}
}
__device__ __forceinline__ void batch_scan_add_phase(uint32_t *blk, uint32_t nb, uint32_t nch, const uint32_t *part) {
	for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < nb; x += gridDim.x * blockDim.x) {
		#pragma unroll
		for (int a = 0; a < 3; a++) blk[(uint64_t)a * nb + x] = __ldcg(blk + (uint64_t)a * nb + x) + __ldcg(part + a * nch + x / 1024);
	}
}

struct BatchArgs {
	const up_synth_program *planets;
	const BatchChunkDev *chunks;
	const uint32_t *tiles, *blkst;
	uint32_t nchunks, ntiles, tile, nblocks;
	float *grid;
	uint32_t *signs, *blk, *totals, *off, *cmap, *emap, *clist, *elist, *qlist;
	float *et, *en, *pos;
	uint32_t *idx, *fb;
	unsigned *counter, *flag;
	BatchBarrier *bar;
	uint32_t cap_cells, cap_edges, cap_quads; // list capacities (the planned counts)
};

constexpr int BATCH_PT = 256; // threads per block of the persistent kernel (= DC_T)
static_assert(BATCH_PT == DC_T, "the count and emit phases run one word block per thread block");

__global__ void __launch_bounds__(BATCH_PT) batch_persistent_kernel(const BatchArgs A) {
	uint32_t *fb_count = A.totals + 3;
	if (blockIdx.x == 0 && threadIdx.x == 0) *fb_count = 0u; // read after several barriers
	batch_sample_body<BATCH_PT>(A.planets, A.chunks, A.tiles, A.nchunks, A.ntiles, A.tile, A.grid, A.signs, A.counter, A.flag);
	if (!batch_grid_sync(A.bar)) return;
	for (uint32_t vb = blockIdx.x; vb < A.nblocks; vb += gridDim.x) batch_count_body(A.signs, A.chunks, A.blkst, A.nchunks, A.nblocks, A.blk, vb);
	if (!batch_grid_sync(A.bar)) return;
	const uint32_t nch = (A.nblocks + 1023) / 1024;
	uint32_t *part = A.blk + 3 * (size_t)A.nblocks;
	batch_scan_chunks_phase(A.blk, A.nblocks, nch, part);
	if (!batch_grid_sync(A.bar)) return;
	if (blockIdx.x == 0) batch_scan_top_phase(part, nch, A.totals);
	if (!batch_grid_sync(A.bar)) return;
	// the lists were sized from the planned counts: a launch whose counts
	// differ records error bit 2 and stops before writing them (every block
	// reads the same totals, so every block stops here)
	if (__ldcg(A.totals) != A.cap_cells || __ldcg(A.totals + 1) != A.cap_edges || __ldcg(A.totals + 2) != A.cap_quads) {
		if (threadIdx.x == 0) atomicOr(&A.bar->err, 2u);
		return;
	}
	batch_scan_add_phase(A.blk, A.nblocks, nch, part);
	if (!batch_grid_sync(A.bar)) return;
	batch_offsets_body(A.chunks, A.nchunks, A.nblocks, A.blk, A.totals, A.off);
	if (!batch_grid_sync(A.bar)) return;
	for (uint32_t vb = blockIdx.x; vb < A.nblocks; vb += gridDim.x)
		batch_emit_body(A.signs, A.chunks, A.blkst, A.nchunks, A.nblocks, A.blk, A.clist, A.cmap, A.elist, A.emap, A.qlist, vb);
	if (!batch_grid_sync(A.bar)) return;
	batch_hermite_body(A.planets, A.chunks, A.off, A.nchunks, A.grid, A.elist, A.et, A.en);
	batch_quads_body(A.chunks, A.off, A.nchunks, A.grid, A.qlist, A.elist, A.cmap, A.idx);
	if (!batch_grid_sync(A.bar)) return;
	batch_qef_body(A.planets, A.chunks, A.off, A.nchunks, A.grid, A.clist, A.emap, A.et, A.en, A.pos, A.fb, fb_count);
	if (!batch_grid_sync(A.bar)) return;
	// the FP64 cells one per warp, consecutive cells in different blocks so
	// that they spread over every SM first (the FP64 pipe is SM-wide)
	const uint32_t wib = threadIdx.x >> 5, nwarps = gridDim.x * (BATCH_PT / 32);
	if ((threadIdx.x & 31) == 0)
		batch_qef_fp64_body(A.planets, A.chunks, A.off, A.nchunks, A.grid, A.clist, A.emap, A.et, A.en, A.pos, A.fb, fb_count,
			blockIdx.x + wib * gridDim.x, nwarps);
}

// ---------------------------------------------------------------- host side

struct DevBuf {
	void *p = nullptr;
	size_t n = 0;
	cudaError_t ensure(size_t bytes) {
		if (bytes == 0) bytes = 16;
		if (n >= bytes) return cudaSuccess;
		if (p) cudaFree(p);
		p = nullptr;
		n = 0;
		cudaError_t e = cudaMalloc(&p, bytes);
		if (e == cudaSuccess) n = bytes;
		return e;
	}
	~DevBuf() { if (p) cudaFree(p); }
	template<class T> T *as() const { return (T *)p; }
};

struct BatchState {
	std::vector<uint8_t> key;      // bytes of (planets, chunks) of the planned input
	uint32_t nchunks = 0, npts = 0, ncells_all = 0, nblocks = 0;
	uint32_t ncells = 0, nedges = 0, nquads = 0;
	int threads = 256;             // autotuned sampling block size
	int tile_sel = 2;              // autotuned tile shape: BATCH_TILES[tile_sel]
	uint32_t ntiles_of[BATCH_NTILE] = {}; // tiles of the whole input per tile shape
	uint32_t nwords = 0;
	DevBuf planets, chunks, tiles, blkst, grid, signs, blk, totals, off, cmap, emap, clist, elist, qlist, et, en, pos, idx, counter, flag, fb, bar;
	// the persistent form (one cooperative launch) replays when it ran on this
	// input; its tile shape is autotuned separately, its block count fixed by
	// occupancy
	bool persistent = false;
	int ptile = 2;
	int pgrid[BATCH_NTILE] = {};
	unsigned long long limit_host = 0; // wait limit last written to bar
	cudaStream_t stream = nullptr;
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	~BatchState() {
		if (exec) cudaGraphExecDestroy(exec);
		if (graph) cudaGraphDestroy(graph);
		if (stream) cudaStreamDestroy(stream);
	}
};

// Wait limit of the persistent kernel's grid barrier (global timer ns); a
// host-side setting for tests (0 = the default).
static std::atomic<unsigned long long> g_batch_wait_limit{0};
constexpr unsigned long long BATCH_WAIT_DEFAULT_NS = 2000000000ull; // 2 s: far above any phase of a real batch
void batch_set_wait_limit(unsigned long long ns) { g_batch_wait_limit.store(ns); }
// which form the plan replays: 0 the faster of the two on the input (timed),
// 1 the stage launches, 2 the persistent launch when it runs on the device
static std::atomic<int> g_batch_form{0};
void batch_set_form(int form) { g_batch_form.store(form); }
static unsigned long long batch_wait_limit() {
	const unsigned long long v = g_batch_wait_limit.load();
	return v ? v : BATCH_WAIT_DEFAULT_NS;
}

// writes the current wait limit into the barrier block when it changed
static cudaError_t batch_sync_limit(BatchState &S, cudaStream_t s) {
	const unsigned long long want = batch_wait_limit();
	if (S.limit_host == want) return cudaSuccess;
	S.limit_host = want;
	return cudaMemcpyAsync((char *)S.bar.p + offsetof(BatchBarrier, limit_ns), &S.limit_host, sizeof(S.limit_host), cudaMemcpyHostToDevice, s);
}

// the persistent kernel with tile shape BATCH_TILES[ts]: barrier count and
// error word and the tile counter zeroed in stream order, then one
// cooperative launch of pgrid[ts] blocks
static cudaError_t enqueue_persistent(BatchState &S, int ts, cudaStream_t s) {
	cudaError_t e = cudaMemsetAsync(S.counter.p, 0, 4, s);
	if (e == cudaSuccess) e = cudaMemsetAsync((char *)S.bar.p + offsetof(BatchBarrier, count), 0, 4, s);
	if (e == cudaSuccess) e = cudaMemsetAsync((char *)S.bar.p + offsetof(BatchBarrier, err), 0, 4, s);
	if (e != cudaSuccess) return e;
	BatchArgs A;
	A.planets = S.planets.as<up_synth_program>();
	A.chunks = S.chunks.as<BatchChunkDev>();
	A.tiles = S.tiles.as<uint32_t>() + (size_t)ts * S.nchunks;
	A.blkst = S.blkst.as<uint32_t>();
	A.nchunks = S.nchunks; A.ntiles = S.ntiles_of[ts]; A.tile = BATCH_TILES[ts]; A.nblocks = S.nblocks;
	A.grid = S.grid.as<float>();
	A.signs = S.signs.as<uint32_t>(); A.blk = S.blk.as<uint32_t>(); A.totals = S.totals.as<uint32_t>(); A.off = S.off.as<uint32_t>();
	A.cmap = S.cmap.as<uint32_t>(); A.emap = S.emap.as<uint32_t>(); A.clist = S.clist.as<uint32_t>(); A.elist = S.elist.as<uint32_t>();
	A.qlist = S.qlist.as<uint32_t>();
	A.et = S.et.as<float>(); A.en = S.en.as<float>(); A.pos = S.pos.as<float>();
	A.idx = S.idx.as<uint32_t>(); A.fb = S.fb.as<uint32_t>();
	A.counter = S.counter.as<unsigned>(); A.flag = S.flag.as<unsigned>();
	A.bar = S.bar.as<BatchBarrier>();
	A.cap_cells = S.ncells; A.cap_edges = S.nedges; A.cap_quads = S.nquads;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3((unsigned)S.pgrid[ts]);
	cfg.blockDim = dim3(BATCH_PT);
	cfg.dynamicSmemBytes = batch_tile_smem(BATCH_TILES[ts]);
	cfg.stream = s;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeCooperative;
	at[0].val.cooperative = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, batch_persistent_kernel, A);
}

static const void *sample_kernel(int threads) {
	return threads == 128 ? (const void *)batch_sample_kernel<128> : (threads == 512 ? (const void *)batch_sample_kernel<512> : (const void *)batch_sample_kernel<256>);
}

// the sampling stage with block size `threads` and tile shape BATCH_TILES[ts]
// (tile table ts of S.tiles)
static cudaError_t enqueue_sample(BatchState &S, int threads, int ts, cudaStream_t s) {
	cudaError_t e = cudaMemsetAsync(S.counter.p, 0, 4, s);
	if (e != cudaSuccess) return e;
	const uint32_t tile = BATCH_TILES[ts];
	const size_t smem = batch_tile_smem(tile);
	const int b = persistent_blocks(sample_kernel(threads), threads, smem);
	const auto *P = S.planets.as<up_synth_program>();
	const auto *C = S.chunks.as<BatchChunkDev>();
	const uint32_t *T = S.tiles.as<uint32_t>() + (size_t)ts * S.nchunks;
	uint32_t *B = S.signs.as<uint32_t>();
	const uint32_t nt = S.ntiles_of[ts];
	if (threads == 128) batch_sample_kernel<128><<<b, 128, smem, s>>>(P, C, T, S.nchunks, nt, tile, S.grid.as<float>(), B, S.counter.as<unsigned>(), S.flag.as<unsigned>());
	else if (threads == 512) batch_sample_kernel<512><<<b, 512, smem, s>>>(P, C, T, S.nchunks, nt, tile, S.grid.as<float>(), B, S.counter.as<unsigned>(), S.flag.as<unsigned>());
	else batch_sample_kernel<256><<<b, 256, smem, s>>>(P, C, T, S.nchunks, nt, tile, S.grid.as<float>(), B, S.counter.as<unsigned>(), S.flag.as<unsigned>());
	return cudaGetLastError();
}

static cudaError_t enqueue_front(BatchState &S, cudaStream_t s) {
	cudaError_t e = enqueue_sample(S, S.threads, S.tile_sel, s);
	if (e != cudaSuccess) return e;
	batch_count_kernel<<<S.nblocks, DC_T, 0, s>>>(S.signs.as<uint32_t>(), S.chunks.as<BatchChunkDev>(), S.blkst.as<uint32_t>(), S.nchunks, S.nblocks, S.blk.as<uint32_t>());
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	dc_scan_blocks(S.blk.as<uint32_t>(), S.nblocks, S.totals.as<uint32_t>(), s);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	batch_offsets_kernel<<<(S.nchunks + 256) / 256, 256, 0, s>>>(S.chunks.as<BatchChunkDev>(), S.nchunks, S.nblocks, S.blk.as<uint32_t>(), S.totals.as<uint32_t>(), S.off.as<uint32_t>());
	return cudaGetLastError();
}

static cudaError_t enqueue_back(BatchState &S, cudaStream_t s) {
	const auto *P = S.planets.as<up_synth_program>();
	const auto *C = S.chunks.as<BatchChunkDev>();
	batch_emit_kernel<<<S.nblocks, DC_T, 0, s>>>(S.signs.as<uint32_t>(), C, S.blkst.as<uint32_t>(), S.nchunks, S.nblocks, S.blk.as<uint32_t>(),
		S.clist.as<uint32_t>(), S.cmap.as<uint32_t>(), S.elist.as<uint32_t>(), S.emap.as<uint32_t>(), S.qlist.as<uint32_t>());
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	auto grid_of = [](const void *k, int t, uint32_t work) {
		const int b = persistent_blocks(k, t);
		const uint32_t need = (work + t - 1) / t;
		return need < (uint32_t)b ? (need ? need : 1u) : (uint32_t)b;
	};
	batch_hermite_kernel<<<grid_of((const void *)batch_hermite_kernel, 256, S.nedges), 256, 0, s>>>(P, C, S.off.as<uint32_t>(), S.nchunks,
		S.grid.as<float>(), S.elist.as<uint32_t>(), S.et.as<float>(), S.en.as<float>());
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	uint32_t *fb_count = S.totals.as<uint32_t>() + 3;
	if ((e = cudaMemsetAsync(fb_count, 0, 4, s)) != cudaSuccess) return e;
	batch_qef_kernel<<<grid_of((const void *)batch_qef_kernel, 128, S.ncells), 128, 0, s>>>(P, C, S.off.as<uint32_t>(), S.nchunks, S.grid.as<float>(),
		S.clist.as<uint32_t>(), S.emap.as<uint32_t>(), S.et.as<float>(), S.en.as<float>(), S.pos.as<float>(), S.fb.as<uint32_t>(), fb_count);
	batch_qef_fp64_kernel<<<grid_of((const void *)batch_qef_fp64_kernel, 1, S.ncells), 32, 0, s>>>(P, C, S.off.as<uint32_t>(), S.nchunks,
		S.grid.as<float>(), S.clist.as<uint32_t>(), S.emap.as<uint32_t>(), S.et.as<float>(), S.en.as<float>(), S.pos.as<float>(), S.fb.as<uint32_t>(),
		fb_count);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	batch_quads_kernel<<<grid_of((const void *)batch_quads_kernel, 256, S.nquads), 256, 0, s>>>(C, S.off.as<uint32_t>(), S.nchunks, S.grid.as<float>(),
		S.qlist.as<uint32_t>(), S.elist.as<uint32_t>(), S.cmap.as<uint32_t>(), S.idx.as<uint32_t>());
	return cudaGetLastError();
}

// Plans the persistent form on an input whose stage launches have run: the
// barrier block, the block count per tile shape, and one timed trial launch
// per tile shape whose counts must equal the stage launches' (and whose
// barrier must not have run out). The fastest such tile shape is kept and
// timed against one run of the stage launches: the faster form is replayed
// (or the form set by batch_set_form). When no persistent trial qualifies (no
// cooperative launch on this device, a launch error) the stage launches are
// replayed.
static void plan_persistent(BatchState &S, cudaStream_t s) {
	S.persistent = false;
	const int form = g_batch_form.load();
	if (form == 1) return;
	int dev = 0, coop = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) {
		cudaGetLastError();
		return;
	}
	if (S.bar.ensure(sizeof(BatchBarrier)) != cudaSuccess || cudaMemsetAsync(S.bar.p, 0, sizeof(BatchBarrier), s) != cudaSuccess) {
		cudaGetLastError();
		return;
	}
	S.limit_host = 0;
	if (batch_sync_limit(S, s) != cudaSuccess) { cudaGetLastError(); return; }
	for (int ts = 0; ts < BATCH_NTILE; ts++)
		S.pgrid[ts] = persistent_blocks((const void *)batch_persistent_kernel, BATCH_PT, batch_tile_smem(BATCH_TILES[ts]));
	cudaEvent_t a, b;
	cudaEventCreate(&a);
	cudaEventCreate(&b);
	float best = 1e30f;
	for (int ts = 0; ts < BATCH_NTILE; ts++) {
		cudaEventRecord(a, s);
		cudaError_t e = enqueue_persistent(S, ts, s);
		cudaEventRecord(b, s);
		if (e == cudaSuccess) e = cudaEventSynchronize(b);
		if (e != cudaSuccess) {
			cudaGetLastError();
			continue;
		}
		uint32_t tot[4] = {0, 0, 0, 0}, err = 1;
		cudaMemcpyAsync(tot, S.totals.p, 12, cudaMemcpyDeviceToHost, s);
		cudaMemcpyAsync(&err, (char *)S.bar.p + offsetof(BatchBarrier, err), 4, cudaMemcpyDeviceToHost, s);
		if (cudaStreamSynchronize(s) != cudaSuccess) { cudaGetLastError(); continue; }
		if (err || tot[0] != S.ncells || tot[1] != S.nedges || tot[2] != S.nquads) continue;
		float ms = 0.f;
		cudaEventElapsedTime(&ms, a, b);
		if (ms < best) {
			best = ms;
			S.ptile = ts;
			S.persistent = true;
		}
	}
	if (S.persistent && form == 0) {
		// the stage launches of the same input, timed the same way (their last
		// run recomputes the same outputs)
		cudaEventRecord(a, s);
		cudaError_t e = cudaMemsetAsync(S.flag.p, 0, 4, s);
		if (e == cudaSuccess) e = enqueue_front(S, s);
		if (e == cudaSuccess) e = enqueue_back(S, s);
		cudaEventRecord(b, s);
		if (e == cudaSuccess) e = cudaEventSynchronize(b);
		float ms = 1e30f;
		if (e == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
		else cudaGetLastError();
		if (ms < best) S.persistent = false;
	}
	cudaEventDestroy(a);
	cudaEventDestroy(b);
}

void batch_state_free(void *p) { delete (BatchState *)p; }

// Plans (or reuses) the batch for this input and runs it; on return the
// device outputs are in the state's pos/idx buffers and counts are filled.
// Returns cudaSuccess or an error; *nan set when a sample was NaN.
cudaError_t batch_execute(void *&state, const up_synth_program *planets, size_t nplanets, const up_chunk *chunks, size_t nchunks,
	bool exact_values, uint32_t &ncells, uint32_t &nquads, std::vector<uint32_t> &chunk_cells, std::vector<uint32_t> &chunk_quads, const float *&dpos,
	const uint32_t *&didx, const float *&dvalues, uint64_t &nvalues, bool &nan, bool &replayed, unsigned &fault, cudaStream_t caller) {
	fault = 0;
	std::vector<uint8_t> key(nplanets * sizeof(up_synth_program) + nchunks * sizeof(up_chunk) + 1);
	std::memcpy(key.data(), planets, nplanets * sizeof(up_synth_program));
	std::memcpy(key.data() + nplanets * sizeof(up_synth_program), chunks, nchunks * sizeof(up_chunk));
	key.back() = exact_values ? 1 : 0;
	BatchState *S = (BatchState *)state;
	cudaError_t e;
	replayed = false;
	if (S && S->key == key && S->exec) {
		// replay: the same work, recomputed, ordered after the caller's stream
		cudaEvent_t ev;
		if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return e;
		cudaEventRecord(ev, caller);
		cudaStreamWaitEvent(S->stream, ev, 0);
		if (S->persistent && (e = batch_sync_limit(*S, S->stream)) != cudaSuccess) return e;
		e = cudaGraphLaunch(S->exec, S->stream);
		cudaEventRecord(ev, S->stream);
		cudaStreamWaitEvent(caller, ev, 0);
		cudaEventDestroy(ev);
		if (e != cudaSuccess) return e;
		replayed = true;
	} else {
		if (S) { delete S; state = nullptr; }
		S = new BatchState();
		state = S;
		S->key = key;
		if ((e = cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking)) != cudaSuccess) return e;
		// host chunk table
		std::vector<BatchChunkDev> tab(nchunks);
		std::vector<uint32_t> tiles((size_t)BATCH_NTILE * nchunks), blks(nchunks);
		uint64_t pts = 0, cells = 0, nb = 0, nw = 0, nt[BATCH_NTILE] = {};
		for (size_t c = 0; c < nchunks; c++) {
			BatchChunkDev &t = tab[c];
			t.g = make_grid(chunks[c].grid);
			t.planet = chunks[c].planet;
			t.band = exact_values ? 0.f : contour_band(planets[t.planet], t.g);
			t.divx = FastDiv::of(t.g.n[0]);
			t.divy = FastDiv::of(t.g.n[1]);
			const uint64_t n = (uint64_t)t.g.n[0] * t.g.n[1] * t.g.n[2];
			t.pt_off = (uint32_t)pts;
			t.cell_off = (uint32_t)cells;
			t.blk_off = (uint32_t)nb;
			t.word_off = (uint32_t)nw;
			t.nwords = (uint32_t)((n + 31) / 32 + 2);
			for (int ts = 0; ts < BATCH_NTILE; ts++) { // first tile of chunk c per tile shape
				tiles[(size_t)ts * nchunks + c] = (uint32_t)nt[ts];
				nt[ts] += (n + BATCH_TILES[ts] - 1) / BATCH_TILES[ts];
			}
			blks[c] = t.blk_off;
			pts += n;
			cells += (uint64_t)(t.g.n[0] - 1) * (t.g.n[1] - 1) * (t.g.n[2] - 1);
			nb += (n + DC_WPB - 1) / DC_WPB;
			nw += t.nwords;
		}
		if (3 * pts >= (1ull << 32)) return cudaErrorInvalidValue;
		S->nchunks = (uint32_t)nchunks; S->npts = (uint32_t)pts; S->ncells_all = (uint32_t)cells; S->nblocks = (uint32_t)nb;
		for (int ts = 0; ts < BATCH_NTILE; ts++) S->ntiles_of[ts] = (uint32_t)nt[ts];
		S->nwords = (uint32_t)nw;
		if ((e = S->planets.ensure(nplanets * sizeof(up_synth_program))) != cudaSuccess) return e;
		if ((e = S->chunks.ensure(nchunks * sizeof(BatchChunkDev))) != cudaSuccess) return e;
		if ((e = S->tiles.ensure(tiles.size() * 4)) != cudaSuccess) return e;
		if ((e = S->blkst.ensure(nchunks * 4)) != cudaSuccess) return e;
		if ((e = S->signs.ensure(nw * 4)) != cudaSuccess) return e;
		if ((e = S->grid.ensure(pts * 4)) != cudaSuccess) return e;
		if ((e = S->blk.ensure(dc_scan_words((uint32_t)nb) * 4)) != cudaSuccess) return e;
		if ((e = S->totals.ensure(16)) != cudaSuccess) return e;
		if ((e = S->off.ensure((nchunks + 1) * 12)) != cudaSuccess) return e;
		if ((e = S->cmap.ensure(cells * 4)) != cudaSuccess) return e;
		if ((e = S->emap.ensure(pts * 12)) != cudaSuccess) return e;
		if ((e = S->counter.ensure(16)) != cudaSuccess) return e;
		if ((e = S->flag.ensure(16)) != cudaSuccess) return e;
		cudaStream_t s = S->stream;
		cudaEvent_t ev;
		if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return e;
		cudaEventRecord(ev, caller);
		cudaStreamWaitEvent(s, ev, 0);
		cudaEventDestroy(ev);
		cudaMemcpyAsync(S->planets.p, planets, nplanets * sizeof(up_synth_program), cudaMemcpyHostToDevice, s);
		cudaMemcpyAsync(S->chunks.p, tab.data(), nchunks * sizeof(BatchChunkDev), cudaMemcpyHostToDevice, s);
		cudaMemcpyAsync(S->tiles.p, tiles.data(), tiles.size() * 4, cudaMemcpyHostToDevice, s);
		cudaMemcpyAsync(S->blkst.p, blks.data(), nchunks * 4, cudaMemcpyHostToDevice, s);
		cudaMemsetAsync(S->flag.p, 0, 4, s);
		// autotune the sampling stage's tile shape and block size: each
		// (tile, threads) candidate runs the full sampling stage of this input
		// once, after one untimed run that warms the caches; the fastest is
		// kept for this input's plan and its graph
		{
			cudaEvent_t a, b;
			cudaEventCreate(&a);
			cudaEventCreate(&b);
			float best = 1e30f;
			e = enqueue_sample(*S, 256, 2, s);
			for (int ts = 0; ts < BATCH_NTILE && e == cudaSuccess; ts++)
				for (int t : {128, 256, 512}) {
					if (e != cudaSuccess) break;
					cudaEventRecord(a, s);
					if ((e = enqueue_sample(*S, t, ts, s)) != cudaSuccess) break;
					cudaEventRecord(b, s);
					cudaEventSynchronize(b);
					float ms = 0.f;
					cudaEventElapsedTime(&ms, a, b);
					if (ms < best) { best = ms; S->threads = t; S->tile_sel = ts; }
				}
			cudaEventDestroy(a);
			cudaEventDestroy(b);
			if (e != cudaSuccess) return e;
		}
		if ((e = enqueue_front(*S, s)) != cudaSuccess) return e;
		uint32_t tot[4] = {0, 0, 0, 0};
		cudaMemcpyAsync(tot, S->totals.p, 12, cudaMemcpyDeviceToHost, s);
		if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
		S->ncells = tot[0]; S->nedges = tot[1]; S->nquads = tot[2];
		if ((e = S->clist.ensure((size_t)S->ncells * 4)) != cudaSuccess) return e;
		if ((e = S->elist.ensure((size_t)S->nedges * 4)) != cudaSuccess) return e;
		if ((e = S->qlist.ensure((size_t)S->nquads * 4)) != cudaSuccess) return e;
		if ((e = S->et.ensure((size_t)S->nedges * 4)) != cudaSuccess) return e;
		if ((e = S->en.ensure((size_t)S->nedges * 12)) != cudaSuccess) return e;
		if ((e = S->pos.ensure((size_t)S->ncells * 12)) != cudaSuccess) return e;
		if ((e = S->fb.ensure((size_t)S->ncells * 4)) != cudaSuccess) return e;
		if ((e = S->idx.ensure((size_t)S->nquads * 24)) != cudaSuccess) return e;
		if ((e = enqueue_back(*S, s)) != cudaSuccess) return e;
		if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
		// the persistent form, when it runs here (its trial launches recompute
		// the same outputs)
		plan_persistent(*S, s);
		// capture the replayed form: the persistent launch, or every stage
		for (int attempt = 0; attempt < 2; attempt++) {
			if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
			cudaError_t e1 = cudaMemsetAsync(S->flag.p, 0, 4, s);
			if (S->persistent) {
				if (e1 == cudaSuccess) e1 = enqueue_persistent(*S, S->ptile, s);
			} else {
				if (e1 == cudaSuccess) e1 = enqueue_front(*S, s);
				if (e1 == cudaSuccess) e1 = enqueue_back(*S, s);
			}
			e = cudaStreamEndCapture(s, &S->graph);
			if (e1 == cudaSuccess && e == cudaSuccess) e = cudaGraphInstantiate(&S->exec, S->graph, 0);
			else if (e == cudaSuccess) e = e1;
			if (e == cudaSuccess) break;
			cudaGetLastError();
			if (S->graph) { cudaGraphDestroy(S->graph); S->graph = nullptr; }
			if (!S->persistent) return e; // the stage launches could not be captured
			S->persistent = false;        // capture the stage launches instead
		}
		cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
		cudaEventRecord(ev, s);
		cudaStreamWaitEvent(caller, ev, 0);
		cudaEventDestroy(ev);
	}
	// per-chunk offsets and the NaN flag
	std::vector<uint32_t> off(3 * (S->nchunks + 1));
	unsigned fl = 0, berr = 0;
	cudaMemcpyAsync(off.data(), S->off.p, off.size() * 4, cudaMemcpyDeviceToHost, S->stream);
	cudaMemcpyAsync(&fl, S->flag.p, 4, cudaMemcpyDeviceToHost, S->stream);
	if (replayed && S->persistent) // the persistent launch's error word (1: a wait ran out, 2: counts differ)
		cudaMemcpyAsync(&berr, (char *)S->bar.p + offsetof(BatchBarrier, err), 4, cudaMemcpyDeviceToHost, S->stream);
	if ((e = cudaStreamSynchronize(S->stream)) != cudaSuccess) return e;
	fault = berr;
	chunk_cells.assign(off.begin(), off.begin() + S->nchunks + 1);
	chunk_quads.assign(off.begin() + 2 * (S->nchunks + 1), off.end());
	ncells = S->ncells;
	nquads = S->nquads;
	dpos = S->pos.as<float>();
	didx = S->idx.as<uint32_t>();
	dvalues = S->grid.as<float>();
	nvalues = S->npts;
	nan = fl != 0;
	return cudaSuccess;
}

} // namespace up
