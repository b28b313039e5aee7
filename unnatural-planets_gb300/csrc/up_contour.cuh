// Dual contouring kernels (templated on the SDF evaluator).
//
// Replaces cage's MarchingCubes::makeMesh (sources/meshGeneration.cpp:40).
// Rules (the CPU oracle implements the same rules independently):
//   inside(d) = d < 0; a cell is active when its 8 corner signs differ; a
//   sign edge joins two samples of different sign; the Hermite point is
//   x0 + t (x1 - x0), t = d0 / (d0 - d1) (FP32; the oracle uses FP64, a
//   difference of ~1e-7 of a cell); the Hermite normal is the
//   analytic gradient at that point; the cell vertex minimises the QEF
//   (cell-local units, mass-point centred, eight cyclic Jacobi sweeps,
//   eigenvalues below 1e-2 of the largest truncated, clamped to the cell)
//   in FP32, and in FP64 for the cells whose truncation decision lies
//   within FP32 rounding;
//   every sign edge with four cells emits two triangles wound outwards.
// Pipeline (single grids): signs (d < 0 bit-packed, 32 points a word) ->
// count (per word: active cells, sign edges, quads; dc_word_flags) ->
// exclusive scan of block counts -> emit (ordered lists and dense maps; order
// fixed by the scan, no atomics) -> Hermite per edge -> QEF per cell -> quads.
// Batches of chunks run the same word kernels per chunk (up_batch.cu).
#pragma once
#include "up_internal.h"
#include "up_fastdiv.h"
#include "up_noise.cuh"

namespace up {

constexpr int DC_T = 256, DC_ITEMS = 4, DC_PB = DC_T * DC_ITEMS;

__device__ __forceinline__ float dc_coord(const GridDev &g, int a, uint32_t i) {
	return __fadd_rn(__fmul_rn((float)i, g.step[a]), g.lo[a]);
}

// ---- word-parallel classification
// The signs (d < 0) of 32 consecutive points form one word (bit b = point
// 32 w + b; 0 past the grid; two words of zero padding). One thread
// classifies a word: the neighbour signs along +x, +y, +z are the same
// bitfield read at offsets 1, nx, nx * ny (funnel shifts of two words), so
// sign-change edges, quads and active cells are bitwise expressions, gated
// by per-word masks of the grid boundary: point (i, j, k) has an edge along
// x when i + 1 < nx (likewise y, z); that edge emits a quad when the other
// two indices are interior (1 <= j < ny - 1, 1 <= k < nz - 1); the point is
// an active cell when i + 1 < nx, j + 1 < ny, k + 1 < nz and the cell's
// eight corners do not all share one sign.
constexpr uint32_t DC_WPB = DC_T * 32; // points per block of the word kernels

__device__ __forceinline__ uint32_t dc_bits_at(const uint32_t *__restrict__ B, uint64_t q, uint64_t nalloc) {
	const uint64_t wi = q >> 5;
	const uint32_t lo = wi < nalloc ? __ldg(B + wi) : 0u, hi = wi + 1 < nalloc ? __ldg(B + wi + 1) : 0u;
	return __funnelshift_r(lo, hi, (uint32_t)(q & 31));
}
struct WordFlags { uint32_t cell, ex, ey, ez, qx, qy, qz; };
__device__ __forceinline__ WordFlags dc_word_flags(const uint32_t *__restrict__ B, uint64_t nalloc, const GridDev &g, uint64_t w, uint32_t npts) {
	WordFlags f{0, 0, 0, 0, 0, 0, 0};
	const uint32_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const uint64_t p0 = 32 * w;
	if (p0 >= npts) return f;
	// boundary masks: bits of points with i + 1 < nx (hx), 1 <= i < nx - 1 (iix),
	// j + 1 < ny (hy), 1 <= j < ny - 1 (ijy) and likewise in k
	uint32_t valid = 0, hx = 0, iix = 0, hy = 0, ijy = 0, hz = 0, ikz = 0;
	uint32_t r = (uint32_t)(p0 / nx), i = (uint32_t)(p0 - (uint64_t)r * nx), pos = 0;
	while (pos < 32 && p0 + pos < npts) {
		uint32_t seg = 32 - pos;
		if (nx - i < seg) seg = nx - i;
		if (npts - (p0 + pos) < seg) seg = (uint32_t)(npts - (p0 + pos));
		const uint32_t sm = (seg >= 32 ? 0xFFFFFFFFu : ((1u << seg) - 1u)) << pos;
		const uint32_t j = r % ny, k = r / ny;
		valid |= sm;
		if (j + 1 < ny) hy |= sm;
		if (j >= 1 && j + 1 < ny) ijy |= sm;
		if (k + 1 < nz) hz |= sm;
		if (k >= 1 && k + 1 < nz) ikz |= sm;
		uint32_t mx = sm, mi = sm;
		if (i + seg == nx) { mx &= ~(1u << (pos + seg - 1)); mi &= ~(1u << (pos + seg - 1)); }
		if (i == 0) mi &= ~(1u << pos);
		hx |= mx;
		iix |= mi;
		pos += seg;
		i = 0;
		r++;
	}
	const uint64_t sxy = (uint64_t)nx * ny;
	const uint32_t A = dc_bits_at(B, p0, nalloc), X = dc_bits_at(B, p0 + 1, nalloc);
	const uint32_t Y = dc_bits_at(B, p0 + nx, nalloc), XY = dc_bits_at(B, p0 + nx + 1, nalloc);
	const uint32_t Z = dc_bits_at(B, p0 + sxy, nalloc), ZX = dc_bits_at(B, p0 + sxy + 1, nalloc);
	const uint32_t ZY = dc_bits_at(B, p0 + sxy + nx, nalloc), ZXY = dc_bits_at(B, p0 + sxy + nx + 1, nalloc);
	f.ex = (A ^ X) & hx;
	f.ey = (A ^ Y) & hy;
	f.ez = (A ^ Z) & hz;
	f.qx = f.ex & ijy & ikz;
	f.qy = f.ey & iix & ikz;
	f.qz = f.ez & iix & ijy;
	f.cell = ((A ^ X) | (A ^ Y) | (A ^ XY) | (A ^ Z) | (A ^ ZX) | (A ^ ZY) | (A ^ ZXY)) & hx & hy & hz;
	return f;
}
__device__ __forceinline__ uint64_t dc_word_counts(const WordFlags &f) {
	return (uint64_t)__popc(f.cell) | ((uint64_t)(__popc(f.ex) + __popc(f.ey) + __popc(f.ez)) << 21) |
		((uint64_t)(__popc(f.qx) + __popc(f.qy) + __popc(f.qz)) << 42);
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

// FP64 QEF vertex in cell-local coordinates (cell = unit cube)
__device__ inline void dc_qef_solve(int ne, const double (*pt)[3], const double (*nm)[3], double out[3]) {
	double a[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, atb[3] = {0, 0, 0}, m[3] = {0, 0, 0};
	for (int e = 0; e < ne; e++) {
		const double b = nm[e][0] * pt[e][0] + nm[e][1] * pt[e][1] + nm[e][2] * pt[e][2];
		#pragma unroll
		for (int i = 0; i < 3; i++) {
			#pragma unroll
			for (int j = 0; j < 3; j++) a[i][j] += nm[e][i] * nm[e][j];
			atb[i] += nm[e][i] * b;
			m[i] += pt[e][i];
		}
	}
	#pragma unroll
	for (int i = 0; i < 3; i++) m[i] /= (double)ne;
	double r[3];
	#pragma unroll
	for (int i = 0; i < 3; i++) r[i] = atb[i] - (a[i][0] * m[0] + a[i][1] * m[1] + a[i][2] * m[2]);
	double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
	#pragma unroll 1
	for (int sweep = 0; sweep < 8; sweep++) {
		#pragma unroll
		for (int rr = 0; rr < 3; rr++) {
			const int p = rr == 2 ? 1 : 0, q = rr == 0 ? 1 : 2;
			const double apq = a[p][q];
			if (fabs(apq) < 1e-300) continue;
			const double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
			const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
			const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
			#pragma unroll
			for (int k = 0; k < 3; k++) {
				const double akp = a[k][p], akq = a[k][q];
				a[k][p] = c * akp - s * akq;
				a[k][q] = s * akp + c * akq;
			}
			#pragma unroll
			for (int k = 0; k < 3; k++) {
				const double apk = a[p][k], aqk = a[q][k];
				a[p][k] = c * apk - s * aqk;
				a[q][k] = s * apk + c * aqk;
			}
			#pragma unroll
			for (int k = 0; k < 3; k++) {
				const double vkp = v[k][p], vkq = v[k][q];
				v[k][p] = c * vkp - s * vkq;
				v[k][q] = s * vkp + c * vkq;
			}
		}
	}
	const double lmax = fmax(fabs(a[0][0]), fmax(fabs(a[1][1]), fabs(a[2][2])));
	double c3[3] = {0, 0, 0};
	#pragma unroll
	for (int k = 0; k < 3; k++) {
		const double l = a[k][k];
		if (fabs(l) < 1e-2 * lmax || fabs(l) < 1e-12) continue;
		const double proj = (v[0][k] * r[0] + v[1][k] * r[1] + v[2][k] * r[2]) / l;
		#pragma unroll
		for (int i = 0; i < 3; i++) c3[i] += v[i][k] * proj;
	}
	#pragma unroll
	for (int i = 0; i < 3; i++) out[i] = fmin(fmax(m[i] + c3[i], 0.0), 1.0);
}

// Hermite data of one sign edge (code = 3 * point + axis): the crossing
// parameter t = d0 / (d0 - d1) and the unit analytic normal at the crossing
template<class E>
__device__ __forceinline__ void dc_hermite_item(const E &ev, const float *__restrict__ d, const GridDev &g, uint32_t code, float &t_out,
	float *n_out) {
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint32_t p = code / 3, a = code % 3;
	const uint32_t i = p % nx, r = p / nx, j = r % ny, k = r / ny;
	const uint32_t stride = a == 0 ? 1u : (a == 1 ? nx : nx * ny);
	const float d0 = d[p], d1 = d[p + stride];
	const float t = d0 / (d0 - d1);
	float x[3] = {dc_coord(g, 0, i), dc_coord(g, 1, j), dc_coord(g, 2, k)};
	const uint32_t ii[3] = {i, j, k};
	const float x1 = dc_coord(g, a, ii[a] + 1);
	x[a] = x[a] + t * (x1 - x[a]);
	const NG s = ev(v3(x[0], x[1], x[2]));
	const float ln = sqrtf(dot(s.g, s.g));
	const float il = ln > 0.f ? 1.f / ln : 0.f;
	t_out = t;
	n_out[0] = s.g.x * il;
	n_out[1] = s.g.y * il;
	n_out[2] = s.g.z * il;
}

// Sign sources (neg(q): sample q has d < 0) for the sign-change tests of the
// QEF kernels, which look at all 12 edges of an active cell: the sampled
// values, or the bit-packed sign words of contouring (dc_sign_words). A
// narrow-band grid sampled with its sign words holds values only near the
// surface (synth_task_band_kernel); its words are complete. The Hermite and
// quad kernels read values only at the ends of sign-change edges, which lie
// near the surface.
struct NegFromValues {
	const float *d;
	__device__ __forceinline__ bool operator()(uint32_t q) const { return __ldg(d + q) < 0.f; }
};
struct NegFromBits {
	const uint32_t *w;
	__device__ __forceinline__ bool operator()(uint32_t q) const { return (__ldg(w + (q >> 5)) >> (q & 31)) & 1u; }
};

// FP64 QEF vertex (cell-local) of one active cell whose origin is grid point p
template<class N>
static __device__ __noinline__ void dc_qef_vertex_fp64(const N neg, const GridDev &g, uint32_t p, const uint32_t *__restrict__ edge_map,
	const float *__restrict__ edge_t, const float *__restrict__ edge_n, double v[3]) {
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint32_t sxy = nx * ny;
	const uint32_t i = p % nx, r = p / nx, j = r % ny, k = r / ny;
	const double o[3] = {dc_coord(g, 0, i), dc_coord(g, 1, j), dc_coord(g, 2, k)};
	const double st[3] = {g.step[0], g.step[1], g.step[2]};
	double pts[12][3], nms[12][3];
	int ne = 0;
	#pragma unroll 1
	for (int a = 0; a < 3; a++) {
		const uint32_t stride = a == 0 ? 1u : (a == 1 ? nx : sxy);
		#pragma unroll 1
		for (int e = 0; e < 4; e++) {
			const uint32_t u = e & 1, w = e >> 1;
			uint32_t ii = i, jj = j, kk = k;
			if (a == 0) { jj += u; kk += w; }
			else if (a == 1) { ii += u; kk += w; }
			else { ii += u; jj += w; }
			const uint32_t pe = (kk * ny + jj) * nx + ii;
			if (neg(pe) == neg(pe + stride)) continue;
			const uint32_t eid = edge_map[3 * (uint64_t)pe + a];
			const double t = (double)edge_t[eid];
			double h[3] = {dc_coord(g, 0, ii), dc_coord(g, 1, jj), dc_coord(g, 2, kk)};
			const uint32_t iv[3] = {ii, jj, kk};
			const double x1 = dc_coord(g, a, iv[a] + 1);
			h[a] = h[a] + t * (x1 - h[a]);
			double nl[3], nn = 0;
			#pragma unroll
			for (int q = 0; q < 3; q++) {
				pts[ne][q] = (h[q] - o[q]) / st[q];
				nl[q] = (double)edge_n[3 * (uint64_t)eid + q] * st[q];
				nn += nl[q] * nl[q];
			}
			nn = sqrt(nn);
			#pragma unroll
			for (int q = 0; q < 3; q++) nms[ne][q] = nn > 0 ? nl[q] / nn : 0.0;
			ne++;
		}
	}
	dc_qef_solve(ne, pts, nms, v);
}

// FP32 form of dc_qef_solve for the accumulated A = sum n n^T and
// r = sum n (n . (p - m)) about the mass point m: the same eight cyclic
// Jacobi sweeps and truncation rule. Returns false when an eigenvalue lies
// within 2e-6 lmax of the truncation threshold 1e-2 lmax, or lmax is below
// 1e-6 (the FP32 eigenvalues of this backward-stable iteration on a
// matrix accumulated in FP32 are within a few 1e-7 lmax of the FP64 ones,
// so every other truncation decision equals the FP64 one); the caller then
// solves in FP64.
__device__ __forceinline__ bool dc_qef_solve_f32(float a[3][3], const float r[3], const float m[3], float out[3]) {
	float v[3][3] = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}};
	#pragma unroll 1
	for (int sweep = 0; sweep < 8; sweep++) {
		#pragma unroll
		for (int rr = 0; rr < 3; rr++) {
			const int p = rr == 2 ? 1 : 0, q = rr == 0 ? 1 : 2;
			const float apq = a[p][q];
			if (fabsf(apq) < 1e-30f) continue;
			const float theta = (a[q][q] - a[p][p]) / (2.f * apq);
			const float t = (theta >= 0.f ? 1.f : -1.f) / (fabsf(theta) + sqrtf(theta * theta + 1.f));
			const float c = 1.f / sqrtf(t * t + 1.f), s = t * c;
			#pragma unroll
			for (int k = 0; k < 3; k++) {
				const float akp = a[k][p], akq = a[k][q];
				a[k][p] = c * akp - s * akq;
				a[k][q] = s * akp + c * akq;
			}
			#pragma unroll
			for (int k = 0; k < 3; k++) {
				const float apk = a[p][k], aqk = a[q][k];
				a[p][k] = c * apk - s * aqk;
				a[q][k] = s * apk + c * aqk;
			}
			#pragma unroll
			for (int k = 0; k < 3; k++) {
				const float vkp = v[k][p], vkq = v[k][q];
				v[k][p] = c * vkp - s * vkq;
				v[k][q] = s * vkp + c * vkq;
			}
		}
	}
	const float lmax = fmaxf(fabsf(a[0][0]), fmaxf(fabsf(a[1][1]), fabsf(a[2][2])));
	if (!(lmax >= 1e-6f)) return false;
	float c3[3] = {0.f, 0.f, 0.f};
	#pragma unroll
	for (int k = 0; k < 3; k++) {
		const float l = fabsf(a[k][k]);
		if (fabsf(l - 1e-2f * lmax) <= 2e-6f * lmax) return false;
		if (l < 1e-2f * lmax) continue;
		const float proj = (v[0][k] * r[0] + v[1][k] * r[1] + v[2][k] * r[2]) / a[k][k];
		#pragma unroll
		for (int i = 0; i < 3; i++) c3[i] += v[i][k] * proj;
	}
	#pragma unroll
	for (int i = 0; i < 3; i++) out[i] = fminf(fmaxf(m[i] + c3[i], 0.f), 1.f);
	return true;
}

// vertex position of cell p from its cell-local solution vc, and the unit
// SDF gradient there (the vertex normal)
template<class E>
__device__ __forceinline__ void dc_vertex_out(const E &ev, const GridDev &g, uint32_t p, const float vc[3], float *vpos, float *vnrm) {
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint32_t i = p % nx, r = p / nx, j = r % ny, k = r / ny;
	const V3f vp = v3(dc_coord(g, 0, i) + vc[0] * g.step[0], dc_coord(g, 1, j) + vc[1] * g.step[1], dc_coord(g, 2, k) + vc[2] * g.step[2]);
	vpos[0] = vp.x;
	vpos[1] = vp.y;
	vpos[2] = vp.z;
	if (vnrm) {
		const NG s = ev(vp);
		const float ln = sqrtf(dot(s.g, s.g));
		const float il = ln > 0.f ? 1.f / ln : 0.f;
		vnrm[0] = s.g.x * il;
		vnrm[1] = s.g.y * il;
		vnrm[2] = s.g.z * il;
	}
}

// QEF vertex and normal of one active cell whose origin is grid point p.
// Pass 1 gathers the Hermite points of the cell's sign edges (cell-local:
// 0/1 on the two other axes, t along the edge axis) and their mass point;
// pass 2 accumulates the normal matrix and residual about the mass point in
// FP32 (no cancellation: the points are centred first). Returns false,
// writing nothing, when the truncation decision is within FP32 rounding:
// the cell then needs the FP64 solver (dc_qef_vertex_fp64, dc_vertex_out).
template<class E, class N>
__device__ __forceinline__ bool dc_qef_item(const E &ev, const N &neg, const GridDev &g, uint32_t p,
	const uint32_t *__restrict__ edge_map, const float *__restrict__ edge_t, const float *__restrict__ edge_n, float *vpos, float *vnrm) {
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint32_t sxy = nx * ny;
	const uint32_t i = p % nx, r = p / nx, j = r % ny, k = r / ny;
	float P[12][3];
	uint32_t eid[12];
	uint32_t present = 0;
	float ms[3] = {0.f, 0.f, 0.f};
	int ne = 0;
	#pragma unroll
	for (int sl = 0; sl < 12; sl++) {
		const int a = sl >> 2;
		const uint32_t u = sl & 1, w = (sl >> 1) & 1;
		const uint32_t stride = a == 0 ? 1u : (a == 1 ? nx : sxy);
		const uint32_t ii = i + (a == 0 ? 0u : u), jj = j + (a == 0 ? u : (a == 1 ? 0u : w)), kk = k + (a == 2 ? 0u : w);
		const uint32_t pe = (kk * ny + jj) * nx + ii;
		eid[sl] = 0;
		P[sl][0] = P[sl][1] = P[sl][2] = 0.f;
		if (neg(pe) == neg(pe + stride)) continue;
		eid[sl] = __ldg(edge_map + 3 * (uint64_t)pe + a);
		const float t = __ldg(edge_t + eid[sl]);
		P[sl][0] = a == 0 ? t : (float)u;
		P[sl][1] = a == 0 ? (float)u : (a == 1 ? t : (float)w);
		P[sl][2] = a == 2 ? t : (float)w;
		present |= 1u << sl;
		ne++;
		ms[0] += P[sl][0]; ms[1] += P[sl][1]; ms[2] += P[sl][2];
	}
	const float ine = ne > 0 ? 1.f / (float)ne : 0.f;
	const float m[3] = {ne > 0 ? ms[0] * ine : 0.5f, ne > 0 ? ms[1] * ine : 0.5f, ne > 0 ? ms[2] * ine : 0.5f};
	float A[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}}, rv[3] = {0.f, 0.f, 0.f};
	#pragma unroll
	for (int sl = 0; sl < 12; sl++) {
		if (!(present >> sl & 1u)) continue;
		const float *en = edge_n + 3 * (uint64_t)eid[sl];
		const float nl[3] = {__ldg(en) * g.step[0], __ldg(en + 1) * g.step[1], __ldg(en + 2) * g.step[2]};
		const float nn = sqrtf(nl[0] * nl[0] + nl[1] * nl[1] + nl[2] * nl[2]);
		const float inn = nn > 0.f ? 1.f / nn : 0.f;
		const float n[3] = {nl[0] * inn, nl[1] * inn, nl[2] * inn};
		const float b = n[0] * (P[sl][0] - m[0]) + n[1] * (P[sl][1] - m[1]) + n[2] * (P[sl][2] - m[2]);
		#pragma unroll
		for (int x = 0; x < 3; x++) {
			#pragma unroll
			for (int y = 0; y < 3; y++) A[x][y] += n[x] * n[y];
			rv[x] += n[x] * b;
		}
	}
	float vc[3];
	if (!dc_qef_solve_f32(A, rv, m, vc)) return false;
	dc_vertex_out(ev, g, p, vc, vpos, vnrm);
	return true;
}

// quad of one interior sign edge: six indices into the cell -> vertex map
__device__ __forceinline__ void dc_quad_item(const float *__restrict__ d, const GridDev &g, uint32_t code, const uint32_t *__restrict__ cell_map,
	uint32_t vbase, uint32_t *o) {
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint32_t cx = nx - 1, cy = ny - 1;
	const uint32_t p = code / 3, a = code % 3;
	const uint32_t i = p % nx, r = p / nx, j = r % ny, k = r / ny;
	auto C = [&](uint32_t ci, uint32_t cj, uint32_t ck) { return cell_map[(ck * cy + cj) * cx + ci] - vbase; };
	uint32_t v0, v1, v2, v3;
	if (a == 0) { v0 = C(i, j - 1, k - 1); v1 = C(i, j, k - 1); v2 = C(i, j, k); v3 = C(i, j - 1, k); }
	else if (a == 1) { v0 = C(i - 1, j, k - 1); v1 = C(i - 1, j, k); v2 = C(i, j, k); v3 = C(i, j, k - 1); }
	else { v0 = C(i - 1, j - 1, k); v1 = C(i, j - 1, k); v2 = C(i, j, k); v3 = C(i - 1, j, k); }
	if (d[p] < 0.f) { o[0] = v0; o[1] = v1; o[2] = v2; o[3] = v0; o[4] = v2; o[5] = v3; }
	else { o[0] = v0; o[1] = v2; o[2] = v1; o[3] = v0; o[4] = v3; o[5] = v2; }
}

// Hermite data of every sign edge
template<class E>
__global__ void __launch_bounds__(256) dc_hermite_kernel(const E ev, const float *__restrict__ d, const GridDev g,
	const uint32_t *__restrict__ edge_list, uint32_t nedges, float *__restrict__ edge_t, float *__restrict__ edge_n) {
	for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < nedges; e += gridDim.x * blockDim.x)
		dc_hermite_item(ev, d, g, edge_list[e], edge_t[e], edge_n + 3 * (uint64_t)e);
}

// QEF vertex of every active cell (positions only). Cells whose FP32
// truncation decision is not certain are flagged, appended to fb_list (count
// in *fb_count) and solved, normal included, by dc_qef_fp64_kernel: packed
// into full warps there, the few FP64 cells do not hold whole warps of this
// kernel on the slow FP64 pipe, and their latency overlaps dc_normal_kernel.
template<class E>
__global__ void __launch_bounds__(128) dc_qef_kernel(const E ev, const uint32_t *__restrict__ signs, const GridDev g,
	const uint32_t *__restrict__ cell_list, uint32_t ncells, const uint32_t *__restrict__ edge_map,
	const float *__restrict__ edge_t, const float *__restrict__ edge_n, float *__restrict__ pos, uint8_t *__restrict__ fb_flag,
	uint32_t *__restrict__ fb_list, uint32_t *__restrict__ fb_count) {
	for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
		const bool ok = dc_qef_item(ev, NegFromBits{signs}, g, cell_list[c], edge_map, edge_t, edge_n, pos + 3 * (uint64_t)c, nullptr);
		fb_flag[c] = ok ? 0 : 1;
		if (!ok) fb_list[atomicAdd(fb_count, 1u)] = c;
	}
}
// unit SDF gradient at the vertex of every cell solved in FP32
template<class E>
__global__ void __launch_bounds__(256) dc_normal_kernel(const E ev, const float *__restrict__ pos, const uint8_t *__restrict__ fb_flag,
	uint32_t ncells, float *__restrict__ nrm) {
	for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
		if (fb_flag[c]) continue;
		const float *vp = pos + 3 * (uint64_t)c;
		const NG s = ev(v3(vp[0], vp[1], vp[2]));
		const float ln = sqrtf(dot(s.g, s.g));
		const float il = ln > 0.f ? 1.f / ln : 0.f;
		float *o = nrm + 3 * (uint64_t)c;
		o[0] = s.g.x * il;
		o[1] = s.g.y * il;
		o[2] = s.g.z * il;
	}
}
// One cell per block (thread 0 of a one-warp block): the FP64 pipe is an
// SM-wide resource on this part, so the few FP64 cells are spread over as
// many SMs as there are cells (timed against 32 and 128 cells per block).
template<class E>
__global__ void __launch_bounds__(32) dc_qef_fp64_kernel(const E ev, const uint32_t *__restrict__ signs, const GridDev g,
	const uint32_t *__restrict__ cell_list, const uint32_t *__restrict__ edge_map, const float *__restrict__ edge_t,
	const float *__restrict__ edge_n, float *__restrict__ pos, float *__restrict__ nrm, const uint32_t *__restrict__ fb_list,
	const uint32_t *__restrict__ fb_count) {
	const uint32_t n = *fb_count;
	if (threadIdx.x != 0) return;
	for (uint32_t e = blockIdx.x; e < n; e += gridDim.x) {
		const uint32_t c = fb_list[e], p = cell_list[c];
		double vd[3];
		dc_qef_vertex_fp64(NegFromBits{signs}, g, p, edge_map, edge_t, edge_n, vd);
		const float vc[3] = {(float)vd[0], (float)vd[1], (float)vd[2]};
		dc_vertex_out(ev, g, p, vc, pos + 3 * (uint64_t)c, nrm ? nrm + 3 * (uint64_t)c : nullptr);
	}
}

cudaError_t dc_quads_launch(const float *d, const GridDev &g, const DcScratch &S, uint32_t nquads, uint32_t *idx, cudaStream_t s);

// Hermite -> QEF -> quads for evaluator E
template<class E>
cudaError_t dc_geometry_t(const E &ev, const float *d, const GridDev &g, DcScratch &S, uint32_t ncells, uint32_t nedges, uint32_t nquads,
	float *pos, float *nrm, uint32_t *idx, cudaStream_t s) {
	if (nedges) {
		const int b = persistent_blocks((const void *)dc_hermite_kernel<E>, 256);
		const uint32_t need = (nedges + 255) / 256;
		dc_hermite_kernel<E><<<need < (uint32_t)b ? need : (uint32_t)b, 256, 0, s>>>(ev, d, g, S.edge_list, nedges, S.edge_t, S.edge_n);
		cudaError_t e = cudaGetLastError();
		if (e != cudaSuccess) return e;
	}
	if (!ncells) return dc_quads_launch(d, g, S, nquads, idx, s);
	uint32_t *fb_count = S.totals + 3;
	cudaError_t e = cudaMemsetAsync(fb_count, 0, sizeof(uint32_t), s);
	if (e != cudaSuccess) return e;
	const int b = persistent_blocks((const void *)dc_qef_kernel<E>, 128);
	const uint32_t need = (ncells + 127) / 128;
	dc_qef_kernel<E><<<need < (uint32_t)b ? need : (uint32_t)b, 128, 0, s>>>(ev, S.signs, g, S.cell_list, ncells, S.edge_map, S.edge_t, S.edge_n, pos,
		S.fb_flag, S.fb_list, fb_count);
	// the FP64 cells (a grid as large as the count could need; blocks past it
	// exit) on the side stream, beside the normals and quads on s
	cudaStream_t s64 = s;
	if (S.side) {
		if ((e = cudaEventRecord(S.ev_fork, s)) != cudaSuccess || (e = cudaStreamWaitEvent(S.side, S.ev_fork, 0)) != cudaSuccess) return e;
		s64 = S.side;
	}
	const int b64 = persistent_blocks((const void *)dc_qef_fp64_kernel<E>, 32);
	dc_qef_fp64_kernel<E><<<ncells < (uint32_t)b64 ? ncells : (uint32_t)b64, 32, 0, s64>>>(ev, S.signs, g, S.cell_list, S.edge_map, S.edge_t, S.edge_n, pos,
		nrm, S.fb_list, fb_count);
	if (nrm) {
		const int bn = persistent_blocks((const void *)dc_normal_kernel<E>, 256);
		const uint32_t needn = (ncells + 255) / 256;
		dc_normal_kernel<E><<<needn < (uint32_t)bn ? needn : (uint32_t)bn, 256, 0, s>>>(ev, pos, S.fb_flag, ncells, nrm);
	}
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	e = dc_quads_launch(d, g, S, nquads, idx, s);
	if (e == cudaSuccess && S.side) {
		if ((e = cudaEventRecord(S.ev_join, S.side)) != cudaSuccess) return e;
		e = cudaStreamWaitEvent(s, S.ev_join, 0);
	}
	return e;
}

} // namespace up
