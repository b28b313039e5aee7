// Dual contouring kernels (templated on the SDF evaluator).
//
// Replaces cage's MarchingCubes::makeMesh (sources/meshGeneration.cpp:40).
// Rules (the CPU oracle implements the same rules independently):
//   inside(d) = d < 0; a cell is active when its 8 corner signs differ; a
//   sign edge joins two samples of different sign; the Hermite point is
//   x0 + t (x1 - x0), t = d0 / (d0 - d1) in FP64; the Hermite normal is the
//   analytic gradient at that point; the cell vertex minimises the QEF in
//   FP64 (cell-local units, mass-point centred, eight cyclic Jacobi sweeps,
//   eigenvalues below 1e-2 of the largest truncated, clamped to the cell);
//   every sign edge with four cells emits two triangles wound outwards.
// Pipeline: count (per 1024-point block: active cells, sign edges, quads) ->
// exclusive scan of block counts -> emit (ordered lists and dense maps; order
// fixed by the scan, no atomics) -> Hermite per edge -> QEF per cell -> quads.
#pragma once
#include "up_internal.h"
#include "up_noise.cuh"

namespace up {

constexpr int DC_T = 256, DC_ITEMS = 4, DC_PB = DC_T * DC_ITEMS;

__device__ __forceinline__ float dc_coord(const GridDev &g, int a, uint32_t i) {
	return __fadd_rn(__fmul_rn((float)i, g.step[a]), g.lo[a]);
}

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

// Hermite data of one sign edge (code = 3 * point + axis)
template<class E>
__device__ __forceinline__ void dc_hermite_item(const E &ev, const float *__restrict__ d, const GridDev &g, uint32_t code, double &t_out,
	float *n_out) {
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint32_t p = code / 3, a = code % 3;
	const uint32_t i = p % nx, r = p / nx, j = r % ny, k = r / ny;
	const uint32_t stride = a == 0 ? 1u : (a == 1 ? nx : nx * ny);
	const double d0 = d[p], d1 = d[p + stride];
	const double t = d0 / (d0 - d1);
	double x[3] = {dc_coord(g, 0, i), dc_coord(g, 1, j), dc_coord(g, 2, k)};
	const uint32_t ii[3] = {i, j, k};
	const double x1 = dc_coord(g, a, ii[a] + 1);
	x[a] = x[a] + t * (x1 - x[a]);
	const NG s = ev(v3((float)x[0], (float)x[1], (float)x[2]));
	const float ln = sqrtf(dot(s.g, s.g));
	const float il = ln > 0.f ? 1.f / ln : 0.f;
	t_out = t;
	n_out[0] = s.g.x * il;
	n_out[1] = s.g.y * il;
	n_out[2] = s.g.z * il;
}

// QEF vertex and normal of one active cell whose origin is grid point p
template<class E>
__device__ __forceinline__ void dc_qef_item(const E &ev, const float *__restrict__ d, const GridDev &g, uint32_t p,
	const uint32_t *__restrict__ edge_map, const double *__restrict__ edge_t, const float *__restrict__ edge_n, float *vpos, float *vnrm) {
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
			if ((d[pe] < 0.f) == (d[pe + stride] < 0.f)) continue;
			const uint32_t eid = edge_map[3 * (uint64_t)pe + a];
			const double t = edge_t[eid];
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
	double v[3];
	dc_qef_solve(ne, pts, nms, v);
	const V3f vp = v3((float)(o[0] + v[0] * st[0]), (float)(o[1] + v[1] * st[1]), (float)(o[2] + v[2] * st[2]));
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
	const uint32_t *__restrict__ edge_list, uint32_t nedges, double *__restrict__ edge_t, float *__restrict__ edge_n) {
	for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < nedges; e += gridDim.x * blockDim.x)
		dc_hermite_item(ev, d, g, edge_list[e], edge_t[e], edge_n + 3 * (uint64_t)e);
}

// QEF vertex and normal of every active cell
template<class E>
__global__ void __launch_bounds__(128) dc_qef_kernel(const E ev, const float *__restrict__ d, const GridDev g,
	const uint32_t *__restrict__ cell_list, uint32_t ncells, const uint32_t *__restrict__ edge_map,
	const double *__restrict__ edge_t, const float *__restrict__ edge_n, float *__restrict__ pos, float *__restrict__ nrm) {
	for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x)
		dc_qef_item(ev, d, g, cell_list[c], edge_map, edge_t, edge_n, pos + 3 * (uint64_t)c, nrm ? nrm + 3 * (uint64_t)c : nullptr);
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
	if (ncells) {
		const int b = persistent_blocks((const void *)dc_qef_kernel<E>, 128);
		const uint32_t need = (ncells + 127) / 128;
		dc_qef_kernel<E><<<need < (uint32_t)b ? need : (uint32_t)b, 128, 0, s>>>(ev, d, g, S.cell_list, ncells, S.edge_map, S.edge_t, S.edge_n, pos, nrm);
		cudaError_t e = cudaGetLastError();
		if (e != cudaSuccess) return e;
	}
	return dc_quads_launch(d, g, S, nquads, idx, s);
}

} // namespace up
