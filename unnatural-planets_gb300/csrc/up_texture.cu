// Texel pipeline of an unwrapped mesh: UV rasterisation, per-texel coloring,
// dilation and 8-bit quantisation; plus batched tiles for points.
//
// Replaces Generator<Water>::generate (sources/textures.cpp:45-82): the cage
// rasteriser meshGenerateTexture (:66-71) calling Generator::pixel (:24-43)
// for every covered texel, imageDilation(7) (:73-77) and imageConvert U8
// (:79-81); and the per-vertex terrainTile loop of
// sources/tileProperties.cpp:256-273.
//
// Rasterisation rule (the oracle implements the same): vertices snapped to
// 1/256 texel in int64 fixed point, texel centres at (x+0.5, y+0.5), exact
// edge functions; a texel on an edge belongs to the triangle (oriented to
// positive area) for which the edge has dy > 0, or dy == 0 and dx < 0;
// overlaps go to the highest triangle id (atomicMax). Barycentric weights
// and the interpolation of position and normal are FP64.
#include "up_internal.h"
#include "up_coloring.cuh"

namespace up {

struct TexMesh {
	const float *pos, *nrm, *uv;
	const uint32_t *idx;
	uint64_t ntri;
};

struct FixTri {
	long long ax, ay, bx, by, cx, cy, area;
	int o[3];
};
__device__ __forceinline__ bool tri_fixed(const TexMesh &m, uint64_t t, uint32_t W, uint32_t H, FixTri &f) {
	long long X[3], Y[3];
	#pragma unroll
	for (int k = 0; k < 3; k++) {
		const uint32_t v = m.idx[3 * t + k];
		X[k] = __double2ll_rn((double)m.uv[2 * (uint64_t)v] * (double)W * 256.0);
		Y[k] = __double2ll_rn((double)m.uv[2 * (uint64_t)v + 1] * (double)H * 256.0);
	}
	long long area = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
	if (area == 0) return false;
	f.o[0] = 0; f.o[1] = 1; f.o[2] = 2;
	if (area < 0) { f.o[1] = 2; f.o[2] = 1; area = -area; }
	f.ax = X[f.o[0]]; f.ay = Y[f.o[0]]; f.bx = X[f.o[1]]; f.by = Y[f.o[1]]; f.cx = X[f.o[2]]; f.cy = Y[f.o[2]];
	f.area = area;
	return true;
}
__device__ __forceinline__ bool edge_in(long long e, long long dx, long long dy) { return e > 0 || (e == 0 && (dy > 0 || (dy == 0 && dx < 0))); }
__device__ __forceinline__ bool tri_cover(const FixTri &f, long long px, long long py, long long e[3]) {
	e[0] = (f.cx - f.bx) * (py - f.by) - (f.cy - f.by) * (px - f.bx);
	e[1] = (f.ax - f.cx) * (py - f.cy) - (f.ay - f.cy) * (px - f.cx);
	e[2] = (f.bx - f.ax) * (py - f.ay) - (f.by - f.ay) * (px - f.ax);
	return edge_in(e[0], f.cx - f.bx, f.cy - f.by) && edge_in(e[1], f.ax - f.cx, f.ay - f.cy) && edge_in(e[2], f.bx - f.ax, f.by - f.ay);
}

// (also the FP64 reciprocal of each triangle's area, for the shading of its
// texels: one division per triangle instead of one per texel)
__global__ void __launch_bounds__(256) tex_raster_kernel(const TexMesh m, uint32_t W, uint32_t H, int *__restrict__ owner, double *__restrict__ tri_ia) {
	for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m.ntri; t += (uint64_t)gridDim.x * blockDim.x) {
		FixTri f;
		if (!tri_fixed(m, t, W, H, f)) continue;
		tri_ia[t] = 1.0 / (double)f.area;
		const long long xmin = min(f.ax, min(f.bx, f.cx)), xmax = max(f.ax, max(f.bx, f.cx));
		const long long ymin = min(f.ay, min(f.by, f.cy)), ymax = max(f.ay, max(f.by, f.cy));
		// texel x is covered only if x*256 + 128 lies in [xmin, xmax]
		const long long tx0 = max(0ll, (xmin - 128 + 255) >> 8), tx1 = min((long long)W - 1, (xmax - 128) >> 8);
		const long long ty0 = max(0ll, (ymin - 128 + 255) >> 8), ty1 = min((long long)H - 1, (ymax - 128) >> 8);
		for (long long y = ty0; y <= ty1; y++)
			for (long long x = tx0; x <= tx1; x++) {
				long long e[3];
				if (tri_cover(f, x * 256 + 128, y * 256 + 128, e)) atomicMax(owner + (uint64_t)y * W + x, (int)t);
			}
	}
}

// per texel: interpolate position and normal of the owning triangle, color.
// A block takes tiles of TS_TILE consecutive texels in two passes: the
// uncovered texels are written NaN at once and the covered ones listed in
// shared memory, then shaded by consecutive threads, so the coloring runs
// in full warps however the charts cross a row.
constexpr uint32_t TS_TILE = 4096;
// T0/T1: compile-time noise types of the synthetic program's layers (synth_texel)
template<bool SYNTH, int T0 = -1, int T1 = -1>
__global__ void __launch_bounds__(128) tex_shade_kernel(const TexMesh m, uint32_t W, uint32_t H, const int *__restrict__ owner,
	const double *__restrict__ tri_ia, const ModesDesc *__restrict__ Mp, const up_synth_program P, int purpose, float *__restrict__ img, int ach) {
	__shared__ uint16_t cov[TS_TILE];
	__shared__ uint32_t ncov;
	const int nch = ach + 3;
	const uint64_t n = (uint64_t)W * H;
	const uint64_t ntiles = (n + TS_TILE - 1) / TS_TILE;
	const uint32_t lane = threadIdx.x & 31;
	for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
		if (threadIdx.x == 0) ncov = 0;
		__syncthreads();
		const uint64_t q0 = tile * TS_TILE;
		#pragma unroll 1
		for (uint32_t it = threadIdx.x; it < TS_TILE; it += blockDim.x) { // every thread the same trip count
			const uint64_t q = q0 + it;
			bool covered = false;
			if (q < n) {
				covered = owner[q] >= 0;
				if (!covered) {
					float *o = img + q * nch;
					for (int c = 0; c < nch; c++) o[c] = NAN;
				}
			}
			const unsigned mk = __ballot_sync(0xFFFFFFFFu, covered);
			uint32_t slot = 0;
			if (lane == 0 && mk) slot = atomicAdd(&ncov, (uint32_t)__popc(mk));
			slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
			if (covered) cov[slot + __popc(mk & ((1u << lane) - 1u))] = (uint16_t)it;
		}
		__syncthreads();
		const uint32_t nc = ncov;
		#pragma unroll 1
		for (uint32_t e = threadIdx.x; e < nc; e += blockDim.x) {
			const uint64_t q = q0 + cov[e];
			float *o = img + q * nch;
			const int t = owner[q];
			FixTri f;
			tri_fixed(m, (uint64_t)t, W, H, f);
			long long ed[3];
			const uint32_t x = (uint32_t)(q % W), y = (uint32_t)(q / W);
			tri_cover(f, (long long)x * 256 + 128, (long long)y * 256 + 128, ed);
			// barycentric weights from the exact edge functions: FP64 for the
			// position (one reciprocal of the area), FP32 for the normal (its
			// direction does not depend on the area)
			const double ia = tri_ia[t];
			double w[3];
			float wf[3];
			#pragma unroll
			for (int k = 0; k < 3; k++) {
				w[f.o[k]] = (double)ed[k] * ia;
				wf[f.o[k]] = (float)ed[k];
			}
			double p[3] = {0, 0, 0};
			V3f nsum = zero3();
			#pragma unroll
			for (int k = 0; k < 3; k++) {
				const uint64_t v = m.idx[3 * (uint64_t)t + k];
				#pragma unroll
				for (int a = 0; a < 3; a++) p[a] += (double)m.pos[3 * v + a] * w[k];
				if (!SYNTH) nsum = nsum + v3(m.nrm[3 * v], m.nrm[3 * v + 1], m.nrm[3 * v + 2]) * wf[k];
			}
			const V3f pf = v3((float)p[0], (float)p[1], (float)p[2]);
			const V3f nf = SYNTH ? zero3() : nsum * (1.f / sqrtf(dot(nsum, nsum)));
			V3f albedo;
			float rough, metal = 0.f, height, opacity = 1.f;
			if (SYNTH) {
				synth_texel<T0, T1>(P, pf, albedo, rough, height);
			} else {
				TileD tl = tile_init(pf, nf, purpose);
				color_tile(*Mp, tl);
				albedo = tl.albedo; rough = tl.roughness; metal = tl.metallic; height = tl.height; opacity = tl.opacity;
			}
			o[0] = albedo.x; o[1] = albedo.y; o[2] = albedo.z;
			if (ach == 4) o[3] = opacity;
			o[ach] = rough; o[ach + 1] = metal; o[ach + 2] = height;
		}
		__syncthreads(); // the list is read before the next tile's
	}
}

// one dilation round over all channels (shared coverage): a NaN texel with
// valid 8-neighbours becomes their mean
__global__ void __launch_bounds__(256) tex_dilate_kernel(const float *__restrict__ src, float *__restrict__ dst, uint32_t W, uint32_t H, int nch) {
	const uint64_t n = (uint64_t)W * H;
	for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (uint64_t)gridDim.x * blockDim.x) {
		const float *s = src + q * nch;
		float *d = dst + q * nch;
		if (!isnan(s[0])) {
			for (int c = 0; c < nch; c++) d[c] = s[c];
			continue;
		}
		const int x = (int)(q % W), y = (int)(q / W);
		float acc[7] = {0, 0, 0, 0, 0, 0, 0};
		int cnt = 0;
		for (int dy = -1; dy <= 1; dy++)
			for (int dx = -1; dx <= 1; dx++) {
				if (!dx && !dy) continue;
				const int xx = x + dx, yy = y + dy;
				if (xx < 0 || yy < 0 || xx >= (int)W || yy >= (int)H) continue;
				const float *r = src + ((uint64_t)yy * W + xx) * nch;
				if (isnan(r[0])) continue;
				for (int c = 0; c < nch; c++) acc[c] += r[c];
				cnt++;
			}
		const float ic = cnt ? 1.f / (float)cnt : 0.f;
		for (int c = 0; c < nch; c++) d[c] = cnt ? acc[c] * ic : NAN;
	}
}

__device__ __forceinline__ uint8_t to_u8(float v) { return isnan(v) ? (uint8_t)0 : (uint8_t)(fminf(fmaxf(v, 0.f), 1.f) * 255.f + 0.5f); }

// All dilation rounds and the output split in one kernel: a block loads a
// DT_X x DT_Y tile with a halo of `rounds` texels into shared memory, runs
// the rounds there and writes the tile's final texels to the caller's images.
// One buffer is updated in place: tag[i] is the round after which texel i is
// valid (0 = covered, DT_ABSENT = outside the image, DT_NAN = not yet), and
// round k fills a NaN texel from the neighbours with tag < k (the texels
// valid before round k, exactly those tex_dilate_kernel reads), so texels
// filled in round k are not read in round k, and the order in which a round
// visits its texels does not matter. Round k updates the region k texels in
// from the loaded edge. The rounds visit only the tile's NaN texels (a list
// built while loading; a tile without any skips the rounds). Same arithmetic
// and neighbour order as tex_dilate_kernel. RT > 0: the round count is RT at
// compile time (the reference's 7), else `rounds`.
constexpr int DT_X = 32, DT_Y = 16, DT_MAX_ROUNDS = 16;
constexpr uint8_t DT_ABSENT = 254, DT_NAN = 255;
__host__ __device__ inline size_t dilate_smem(int rounds, int nch) {
	const size_t t = (size_t)(DT_X + 2 * rounds) * (DT_Y + 2 * rounds);
	return sizeof(float) * t * (nch | 1) + ((t + 15) & ~(size_t)15) + sizeof(uint32_t) * t;
}
template<int RT>
__global__ void __launch_bounds__(256) tex_dilate_fused_kernel(const float *__restrict__ img, uint32_t W, uint32_t H, int nch, int ach, int rounds_rt,
	uint8_t *__restrict__ a8, uint8_t *__restrict__ s8, uint8_t *__restrict__ h8, float *__restrict__ af, float *__restrict__ sf,
	float *__restrict__ hf) {
	extern __shared__ float dsm[];
	__shared__ int nlist;
	const int rounds = RT > 0 ? RT : rounds_rt;
	const int SX = DT_X + 2 * rounds, SY = DT_Y + 2 * rounds;
	float *A = dsm;
	const int NS = nch | 1; // odd texel stride in shared memory: conflict-free
	uint8_t *tag = (uint8_t *)(dsm + (size_t)SX * SY * NS);
	uint32_t *list = (uint32_t *)(tag + ((SX * SY + 15) & ~15)); // (ly << 16) | lx of the NaN texels
	const int x0 = (int)(blockIdx.x * DT_X) - rounds, y0 = (int)(blockIdx.y * DT_Y) - rounds;
	const unsigned lane = threadIdx.x & 31;
	if (threadIdx.x == 0) nlist = 0;
	__syncthreads();
	for (int i0 = 0; i0 < SX * SY; i0 += blockDim.x) { // uniform trip count: the ballot below has every lane
		const int i = i0 + (int)threadIdx.x;
		const int lx = i % SX, ly = i / SX;
		bool empty = false;
		if (i < SX * SY) {
			const int gx = x0 + lx, gy = y0 + ly;
			const bool in = gx >= 0 && gy >= 0 && gx < (int)W && gy < (int)H;
			const float *src = img + ((uint64_t)(in ? gy : 0) * W + (in ? gx : 0)) * nch;
			if (nch == 6) {
				const float2 *s2 = (const float2 *)src;
				#pragma unroll
				for (int c = 0; c < 3; c++) {
					const float2 v = in ? s2[c] : make_float2(NAN, NAN);
					A[i * NS + 2 * c] = v.x;
					A[i * NS + 2 * c + 1] = v.y;
				}
			} else {
				for (int c = 0; c < nch; c++) A[i * NS + c] = in ? src[c] : NAN;
			}
			const uint8_t t = !in ? DT_ABSENT : (isnan(src[0]) ? DT_NAN : 0);
			tag[i] = t;
			empty = t == DT_NAN && lx >= 1 && lx < SX - 1 && ly >= 1 && ly < SY - 1;
		}
		const unsigned m = __ballot_sync(0xFFFFFFFFu, empty);
		int base = 0;
		if (lane == 0 && m) base = atomicAdd(&nlist, __popc(m));
		base = __shfl_sync(0xFFFFFFFFu, base, 0);
		if (empty) list[base + __popc(m & ((1u << lane) - 1u))] = ((uint32_t)ly << 16) | (uint32_t)lx;
	}
	__syncthreads();
	const int nl = nlist;
	for (int k = 1; k <= rounds && nl > 0; k++) {
		for (int e = threadIdx.x; e < nl; e += blockDim.x) {
			const int lx = (int)(list[e] & 0xFFFFu), ly = (int)(list[e] >> 16);
			if (lx < k || lx >= SX - k || ly < k || ly >= SY - k) continue;
			const int i = ly * SX + lx;
			if (tag[i] != DT_NAN) continue;
			float acc[7] = {0, 0, 0, 0, 0, 0, 0};
			int cnt = 0;
			for (int dy = -1; dy <= 1; dy++)
				for (int dx = -1; dx <= 1; dx++) {
					if (!dx && !dy) continue;
					const int ni = (ly + dy) * SX + lx + dx;
					if (tag[ni] >= k) continue; // not valid before this dilation pass (or absent)
					const float *r = A + ni * NS;
					for (int c = 0; c < nch; c++) acc[c] += r[c];
					cnt++;
				}
			if (!cnt) continue;
			const float ic = 1.f / (float)cnt;
			for (int c = 0; c < nch; c++) A[i * NS + c] = acc[c] * ic;
			tag[i] = (uint8_t)k;
		}
		__syncthreads();
	}
	for (int j = threadIdx.x; j < DT_X * DT_Y; j += blockDim.x) {
		const int gx = (int)(blockIdx.x * DT_X) + j % DT_X, gy = (int)(blockIdx.y * DT_Y) + j / DT_X;
		if (gx >= (int)W || gy >= (int)H) continue;
		const float *v = A + ((rounds + j / DT_X) * SX + rounds + j % DT_X) * NS;
		const uint64_t q = (uint64_t)gy * W + gx;
		for (int c = 0; c < ach; c++) {
			if (a8) a8[q * ach + c] = to_u8(v[c]);
			if (af) af[q * ach + c] = v[c];
		}
		if (s8) { s8[2 * q] = to_u8(v[ach]); s8[2 * q + 1] = to_u8(v[ach + 1]); }
		if (sf) { sf[2 * q] = v[ach]; sf[2 * q + 1] = v[ach + 1]; }
		if (h8) h8[q] = to_u8(v[ach + 2]);
		if (hf) hf[q] = v[ach + 2];
	}
}

// split the interleaved working image into the caller's images
__global__ void __launch_bounds__(256) tex_output_kernel(const float *__restrict__ img, uint64_t n, int ach, uint8_t *__restrict__ a8,
	uint8_t *__restrict__ s8, uint8_t *__restrict__ h8, float *__restrict__ af, float *__restrict__ sf, float *__restrict__ hf) {
	const int nch = ach + 3;
	for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (uint64_t)gridDim.x * blockDim.x) {
		const float *s = img + q * nch;
		for (int c = 0; c < ach; c++) {
			if (a8) a8[q * ach + c] = to_u8(s[c]);
			if (af) af[q * ach + c] = s[c];
		}
		if (s8) { s8[2 * q] = to_u8(s[ach]); s8[2 * q + 1] = to_u8(s[ach + 1]); }
		if (sf) { sf[2 * q] = s[ach]; sf[2 * q + 1] = s[ach + 1]; }
		if (h8) h8[q] = to_u8(s[ach + 2]);
		if (hf) hf[q] = s[ach + 2];
	}
}

// tiles as SoA planes: out[k * n + i] for the 11 float channels (albedo r,
// g, b, roughness, metallic, height, opacity, elevation, slope, temperature,
// precipitation), bt[i] = biome, bt[n + i] = type
__global__ void __launch_bounds__(128) tiles_kernel(const ModesDesc *__restrict__ Mp, int purpose, const float *__restrict__ pos,
	const float *__restrict__ nrm, uint64_t n, float *__restrict__ out, uint8_t *__restrict__ bt) {
	for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
		TileD t = tile_init(v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), v3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]), purpose);
		color_tile(*Mp, t);
		const float v[11] = {t.albedo.x, t.albedo.y, t.albedo.z, t.roughness, t.metallic, t.height, t.opacity, t.elevation, t.slope,
			t.temperature, t.precipitation};
		#pragma unroll
		for (int k = 0; k < 11; k++) out[k * n + i] = v[k];
		bt[i] = (uint8_t)t.biome;
		bt[n + i] = (uint8_t)t.type;
	}
}

static int blocks_for(const void *k, int threads, uint64_t work) {
	int b = persistent_blocks(k, threads);
	const uint64_t need = (work + threads - 1) / threads;
	if ((uint64_t)b > need) b = (int)(need ? need : 1);
	return b;
}

cudaError_t texture_run(const ModesDesc *M, const up_synth_program *synth, int purpose, const float *pos, const float *nrm, const float *uv,
	const uint32_t *idx, uint64_t nidx, uint32_t W, uint32_t H, int dilation, int *owner, double *tri_ia, float *img0, float *img1, uint8_t *a8, uint8_t *s8,
	uint8_t *h8, float *af, float *sf, float *hf, int *launches, cudaStream_t s) {
	const uint64_t n = (uint64_t)W * H;
	const int ach = purpose == UP_PURPOSE_WATER ? 4 : 3;
	const int nch = ach + 3;
	TexMesh m{pos, nrm, uv, idx, nidx / 3};
	cudaError_t e = cudaMemsetAsync(owner, 0xFF, n * sizeof(int), s);
	if (e != cudaSuccess) return e;
	int L = 0;
	if (m.ntri) {
		tex_raster_kernel<<<blocks_for((const void *)tex_raster_kernel, 256, m.ntri), 256, 0, s>>>(m, W, H, owner, tri_ia);
		L++;
	}
	up_synth_program P{};
	const uint64_t nsh = (n + TS_TILE - 1) / TS_TILE * 128; // one block per tile at most
	if (synth) {
		P = *synth;
		if (spec_of(P) == SPEC_PERLIN_CELL)
			tex_shade_kernel<true, 2, CELL_EU_SUB><<<blocks_for((const void *)tex_shade_kernel<true, 2, CELL_EU_SUB>, 128, nsh), 128, 0, s>>>(m, W, H,
				owner, tri_ia, M, P, purpose, img0, ach);
		else
			tex_shade_kernel<true><<<blocks_for((const void *)tex_shade_kernel<true>, 128, nsh), 128, 0, s>>>(m, W, H, owner, tri_ia, M, P, purpose, img0, ach);
	} else {
		tex_shade_kernel<false><<<blocks_for((const void *)tex_shade_kernel<false>, 128, nsh), 128, 0, s>>>(m, W, H, owner, tri_ia, M, P, purpose, img0, ach);
	}
	L++;
	if (dilation > 0 && dilation <= DT_MAX_ROUNDS) {
		// every round and the output split in one launch (shared-memory tiles)
		const size_t smem = dilate_smem(dilation, nch);
		const void *kern = dilation == 7 ? (const void *)tex_dilate_fused_kernel<7> : (const void *)tex_dilate_fused_kernel<0>;
		e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
		const dim3 grid((W + DT_X - 1) / DT_X, (H + DT_Y - 1) / DT_Y);
		if (dilation == 7) tex_dilate_fused_kernel<7><<<grid, 256, smem, s>>>(img0, W, H, nch, ach, dilation, a8, s8, h8, af, sf, hf);
		else tex_dilate_fused_kernel<0><<<grid, 256, smem, s>>>(img0, W, H, nch, ach, dilation, a8, s8, h8, af, sf, hf);
		L++;
	} else {
		float *cur = img0, *nxt = img1;
		for (int r = 0; r < dilation; r++) {
			tex_dilate_kernel<<<blocks_for((const void *)tex_dilate_kernel, 256, n), 256, 0, s>>>(cur, nxt, W, H, nch);
			L++;
			float *t = cur; cur = nxt; nxt = t;
		}
		tex_output_kernel<<<blocks_for((const void *)tex_output_kernel, 256, n), 256, 0, s>>>(cur, n, ach, a8, s8, h8, af, sf, hf);
		L++;
	}
	if (launches) *launches = L;
	return cudaGetLastError();
}

cudaError_t tiles_run(const ModesDesc *M, int purpose, const float *pos, const float *nrm, uint64_t n, float *out11, uint8_t *bt, cudaStream_t s) {
	tiles_kernel<<<blocks_for((const void *)tiles_kernel, 128, n), 128, 0, s>>>(M, purpose, pos, nrm, n, out11, bt);
	return cudaGetLastError();
}

} // namespace up
