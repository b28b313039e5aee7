// Mesh hygiene after contouring, as meshGenerateBase* of the reference
// (sources/meshGeneration.cpp):
//   meshRemoveDisconnected (:41): only the largest connected component is
//     kept (components of the vertex graph joined by triangles; largest = most
//     triangles, ties to the component holding the lowest vertex index);
//   meshFlipNormals (:42): nothing to do, the contour is emitted with the
//     orientation the reference reaches after the flip;
//   water filter (:62-95): a vertex is valid when elevationRaw < 0.1, validity
//     spreads twice to every vertex of a triangle holding a valid vertex, and
//     triangles with an invalid vertex and invalid vertices are removed.
// Kept vertices and triangles keep their order (ordered compaction by block
// counts and the contouring scan).
//
// Components: lock-free union-find. parent[x] <= x always holds (a root is
// only ever hooked under a smaller root by compare-and-swap), so every find
// walks a strictly decreasing chain and ends; reads bypass L1 (other SMs
// write the array). Loops carry iteration limits that raise an error flag.
#include "up_internal.h"
#include "up_contour.cuh"

namespace up {

constexpr uint32_t UF_LIMIT = 1u << 26;

__device__ __forceinline__ uint32_t uf_find(uint32_t *parent, uint32_t x, unsigned *err) {
	for (uint32_t it = 0; it < UF_LIMIT; it++) {
		const uint32_t p = __ldcg(parent + x);
		if (p == x) return x;
		const uint32_t gp = __ldcg(parent + p);
		if (gp != p) parent[x] = gp; // path halving: gp is an ancestor, gp <= p < x
		x = gp;
	}
	atomicOr(err, 1u);
	return x;
}
__device__ __forceinline__ void uf_unite(uint32_t *parent, uint32_t a, uint32_t b, unsigned *err) {
	for (uint32_t it = 0; it < UF_LIMIT; it++) {
		const uint32_t ra = uf_find(parent, a, err), rb = uf_find(parent, b, err);
		if (ra == rb) return;
		const uint32_t lo = ra < rb ? ra : rb, hi = ra < rb ? rb : ra;
		if (atomicCAS(parent + hi, hi, lo) == hi) return;
	}
	atomicOr(err, 2u);
}

__global__ void uf_init_kernel(uint32_t *__restrict__ parent, uint32_t V) {
	for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) parent[v] = v;
}
__global__ void uf_union_kernel(const uint32_t *__restrict__ idx, uint32_t T, uint32_t *parent, unsigned *err) {
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
		const uint32_t a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
		uf_unite(parent, a, b, err);
		uf_unite(parent, a, c, err);
	}
}
// after every union has completed: label = root; roots also count triangles
__global__ void uf_label_kernel(uint32_t *parent, uint32_t V, uint32_t *__restrict__ label, unsigned *err) {
	for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) label[v] = uf_find(parent, v, err);
}
__global__ void comp_count_kernel(const uint32_t *__restrict__ idx, uint32_t T, const uint32_t *__restrict__ label, uint32_t *cnt) {
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) atomicAdd(cnt + label[idx[3 * t]], 1u);
}
// best = max over roots of (triangles << 32 | ~root): most triangles, then lowest root
__global__ void comp_best_kernel(const uint32_t *__restrict__ label, const uint32_t *__restrict__ cnt, uint32_t V, unsigned long long *best) {
	for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
		if (label[v] == v) atomicMax(best, ((unsigned long long)cnt[v] << 32) | (0xFFFFFFFFu - v));
}
__device__ __forceinline__ uint32_t best_root(const unsigned long long *best) { return 0xFFFFFFFFu - (uint32_t)(*best & 0xFFFFFFFFull); }

// keep flags of land/navigation meshes: the largest component
__global__ void keep_component_kernel(const uint32_t *__restrict__ label, uint32_t V, const uint32_t *__restrict__ idx, uint32_t T,
	const unsigned long long *best, uint8_t *__restrict__ keep_v, uint8_t *__restrict__ keep_t) {
	const uint32_t root = best_root(best);
	const uint32_t n = V > T ? V : T;
	for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
		if (x < V) keep_v[x] = label[x] == root;
		if (x < T) keep_t[x] = label[idx[3 * x]] == root;
	}
}
// water: valid = in the largest component and elevationRaw < 0.1
__global__ void water_seed_kernel(const uint32_t *__restrict__ label, const float *__restrict__ elev, uint32_t V, const unsigned long long *best,
	uint8_t *__restrict__ valid) {
	const uint32_t root = best_root(best);
	for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) valid[v] = label[v] == root && elev[v] < 0.1f;
}
// one expansion: every vertex of a triangle (of the kept component) holding a valid vertex
__global__ void water_expand_kernel(const uint32_t *__restrict__ idx, uint32_t T, const uint32_t *__restrict__ label, const unsigned long long *best,
	const uint8_t *__restrict__ valid, uint8_t *__restrict__ valid2) {
	const uint32_t root = best_root(best);
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
		const uint32_t a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
		if (label[a] == root && (valid[a] | valid[b] | valid[c])) valid2[a] = valid2[b] = valid2[c] = 1;
	}
}
__global__ void keep_triangles_kernel(const uint32_t *__restrict__ idx, uint32_t T, const uint8_t *__restrict__ keep_v, uint8_t *__restrict__ keep_t) {
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x)
		keep_t[t] = keep_v[idx[3 * t]] & keep_v[idx[3 * t + 1]] & keep_v[idx[3 * t + 2]];
}

// ordered compaction: per block of DC_PB items, kept vertices | kept triangles << 21
__device__ __forceinline__ uint64_t keep_counts(const uint8_t *keep_v, uint32_t V, const uint8_t *keep_t, uint32_t T, uint32_t x) {
	return (uint64_t)(x < V && keep_v[x]) | ((uint64_t)(x < T && keep_t[x]) << 21);
}
__global__ void __launch_bounds__(DC_T) compact_count_kernel(const uint8_t *__restrict__ keep_v, uint32_t V, const uint8_t *__restrict__ keep_t,
	uint32_t T, uint32_t nb, uint32_t *__restrict__ blk) {
	const uint32_t base = blockIdx.x * DC_PB + threadIdx.x * DC_ITEMS;
	uint64_t c = 0;
	#pragma unroll
	for (int it = 0; it < DC_ITEMS; it++) c += keep_counts(keep_v, V, keep_t, T, base + it);
	uint64_t tot;
	block_exscan<DC_T>(c, tot);
	if (threadIdx.x == 0) {
		blk[blockIdx.x] = (uint32_t)(tot & 0x1FFFFF);
		blk[nb + blockIdx.x] = (uint32_t)((tot >> 21) & 0x1FFFFF);
		blk[2 * nb + blockIdx.x] = 0;
	}
}
// vertices: new index and copies of position and normal
__global__ void __launch_bounds__(DC_T) compact_vertices_kernel(const uint8_t *__restrict__ keep_v, uint32_t V, const uint8_t *__restrict__ keep_t,
	uint32_t T, uint32_t nb, const uint32_t *__restrict__ blk, const float *__restrict__ pos, const float *__restrict__ nrm,
	uint32_t *__restrict__ newidx, float *__restrict__ pos_out, float *__restrict__ nrm_out) {
	const uint32_t base = blockIdx.x * DC_PB + threadIdx.x * DC_ITEMS;
	uint64_t c = 0;
	#pragma unroll
	for (int it = 0; it < DC_ITEMS; it++) c += keep_counts(keep_v, V, keep_t, T, base + it);
	uint64_t tot;
	const uint64_t off = block_exscan<DC_T>(c, tot);
	uint32_t vo = blk[blockIdx.x] + (uint32_t)(off & 0x1FFFFF);
	#pragma unroll
	for (int it = 0; it < DC_ITEMS; it++) {
		const uint32_t v = base + it;
		if (v >= V || !keep_v[v]) continue;
		newidx[v] = vo;
		#pragma unroll
		for (int q = 0; q < 3; q++) {
			pos_out[3 * (uint64_t)vo + q] = pos[3 * (uint64_t)v + q];
			if (nrm_out) nrm_out[3 * (uint64_t)vo + q] = nrm[3 * (uint64_t)v + q];
		}
		vo++;
	}
}
// triangles: remapped indices (after compact_vertices_kernel)
__global__ void __launch_bounds__(DC_T) compact_triangles_kernel(const uint8_t *__restrict__ keep_v, uint32_t V, const uint8_t *__restrict__ keep_t,
	uint32_t T, uint32_t nb, const uint32_t *__restrict__ blk, const uint32_t *__restrict__ idx, const uint32_t *__restrict__ newidx,
	uint32_t *__restrict__ idx_out) {
	const uint32_t base = blockIdx.x * DC_PB + threadIdx.x * DC_ITEMS;
	uint64_t c = 0;
	#pragma unroll
	for (int it = 0; it < DC_ITEMS; it++) c += keep_counts(keep_v, V, keep_t, T, base + it);
	uint64_t tot;
	const uint64_t off = block_exscan<DC_T>(c, tot);
	uint32_t to = blk[nb + blockIdx.x] + (uint32_t)((off >> 21) & 0x1FFFFF);
	#pragma unroll
	for (int it = 0; it < DC_ITEMS; it++) {
		const uint32_t t = base + it;
		if (t >= T || !keep_t[t]) continue;
		#pragma unroll
		for (int q = 0; q < 3; q++) idx_out[3 * (uint64_t)to + q] = newidx[idx[3 * (uint64_t)t + q]];
		to++;
	}
}

static unsigned grid_for(const void *k, uint64_t work) {
	const int b = persistent_blocks(k, 256);
	const uint64_t need = (work + 255) / 256;
	return (unsigned)(need < (uint64_t)b ? (need ? need : 1) : (uint64_t)b);
}

uint32_t mesh_blocks(uint32_t V, uint32_t T) { return ((V > T ? V : T) + DC_PB - 1) / DC_PB; }

cudaError_t mesh_filter(const MeshFilterArgs &a, cudaStream_t s) {
	const uint32_t V = a.V, T = a.T;
	uf_init_kernel<<<grid_for((const void *)uf_init_kernel, V), 256, 0, s>>>(a.parent, V);
	uf_union_kernel<<<grid_for((const void *)uf_union_kernel, T), 256, 0, s>>>(a.idx, T, a.parent, a.err);
	uf_label_kernel<<<grid_for((const void *)uf_label_kernel, V), 256, 0, s>>>(a.parent, V, a.label, a.err);
	cudaError_t e = cudaMemsetAsync(a.cnt, 0, (size_t)V * 4, s);
	if (e != cudaSuccess) return e;
	if ((e = cudaMemsetAsync(a.best, 0, 8, s)) != cudaSuccess) return e;
	comp_count_kernel<<<grid_for((const void *)comp_count_kernel, T), 256, 0, s>>>(a.idx, T, a.label, a.cnt);
	comp_best_kernel<<<grid_for((const void *)comp_best_kernel, V), 256, 0, s>>>(a.label, a.cnt, V, a.best);
	if (!a.elev) {
		keep_component_kernel<<<grid_for((const void *)keep_component_kernel, V > T ? V : T), 256, 0, s>>>(a.label, V, a.idx, T, a.best, a.keep_v,
			a.keep_t);
	} else {
		water_seed_kernel<<<grid_for((const void *)water_seed_kernel, V), 256, 0, s>>>(a.label, a.elev, V, a.best, a.keep_v);
		for (int r = 0; r < 2; r++) {
			if ((e = cudaMemcpyAsync(a.valid2, a.keep_v, V, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
			water_expand_kernel<<<grid_for((const void *)water_expand_kernel, T), 256, 0, s>>>(a.idx, T, a.label, a.best, a.keep_v, a.valid2);
			if ((e = cudaMemcpyAsync(a.keep_v, a.valid2, V, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
		}
		keep_triangles_kernel<<<grid_for((const void *)keep_triangles_kernel, T), 256, 0, s>>>(a.idx, T, a.keep_v, a.keep_t);
	}
	const uint32_t nb = mesh_blocks(V, T);
	compact_count_kernel<<<nb, DC_T, 0, s>>>(a.keep_v, V, a.keep_t, T, nb, a.blk);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	return dc_scan_blocks(a.blk, nb, a.totals, s);
}

cudaError_t mesh_compact(const MeshFilterArgs &a, float *pos_out, float *nrm_out, uint32_t *idx_out, cudaStream_t s) {
	const uint32_t nb = mesh_blocks(a.V, a.T);
	compact_vertices_kernel<<<nb, DC_T, 0, s>>>(a.keep_v, a.V, a.keep_t, a.T, nb, a.blk, a.pos, a.nrm, a.newidx, pos_out, nrm_out);
	compact_triangles_kernel<<<nb, DC_T, 0, s>>>(a.keep_v, a.V, a.keep_t, a.T, nb, a.blk, a.idx, a.newidx, idx_out);
	return cudaGetLastError();
}

} // namespace up
