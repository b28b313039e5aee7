// Oracle: dual contouring of an FP32 sample grid. TEST INFRASTRUCTURE,
// parity unpinned: the reference contours with cage's MarchingCubes
// (sources/meshGeneration.cpp:32-44), which is absent; the project's target
// is dual contouring (T. Ju, F. Losasso, S. Schaefer, J. Warren, "Dual
// contouring of Hermite data", SIGGRAPH 2002) with the rules below, which the
// CUDA path implements independently.
//
//   inside(d)      d < 0
//   active cell    its 8 corner signs are not all equal
//   sign edge      grid edge whose two end samples differ in sign
//   Hermite point  x = p0 + t (p1 - p0), t = d0 / (d0 - d1) (FP64 from the
//                  FP32 samples and FP32 sample positions)
//   Hermite normal normalize(grad d(x)) (analytic; supplied by the caller)
//   cell vertex    FP64 QEF in cell-local units (cell = unit cube): minimise
//                  sum (n.(v - x_e))^2 around the mass point with a truncated
//                  eigen pseudo-inverse (eight cyclic Jacobi sweeps,
//                  eigenvalues below 1e-2 * max dropped), clamped to the cell
//   vertex normal  normalize(grad d(vertex))
//   triangles      each sign edge whose four cells exist emits the quad of
//                  those cells' vertices as two triangles (v0 v1 v2)(v0 v2 v3),
//                  wound so the normal points to increasing d (outwards,
//                  which is the orientation meshFlipNormals produces at
//                  sources/meshGeneration.cpp:42)
//   order          vertices by linear cell index; triangles by (grid point,
//                  axis)
#pragma once
#include "oracle_core.hpp"
#include "../include/up_abi.h"
#include <array>
#include <functional>
#include <unordered_map>
#include <vector>

namespace orc {

struct GridF {
	float lo[3], step[3];
	uint32_t n[3];
	explicit GridF(const up_grid &g) {
		for (int a = 0; a < 3; a++) {
			lo[a] = g.lo[a];
			n[a] = g.n[a];
			step[a] = (g.hi[a] - g.lo[a]) / (float)(g.n[a] - 1);
		}
	}
	// FP32 sample coordinate: rounded multiply then rounded add
	float coord(int a, uint32_t i) const {
		volatile float m = (float)i * step[a];
		return m + lo[a];
	}
};

struct Jacobi3 {
	// symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (fixed
	// count): on return a holds eigenvalues on its diagonal, v the eigenvectors
	// as columns.
	static void run(double a[3][3], double v[3][3]) {
		for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) v[i][j] = i == j ? 1.0 : 0.0;
		static const int P[3] = {0, 0, 1}, Q[3] = {1, 2, 2};
		for (int sweep = 0; sweep < 8; sweep++)
			for (int r = 0; r < 3; r++) {
				const int p = P[r], q = Q[r];
				const double apq = a[p][q];
				if (std::fabs(apq) < 1e-300) continue;
				const double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
				const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
				const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
				for (int k = 0; k < 3; k++) { // A <- A J
					const double akp = a[k][p], akq = a[k][q];
					a[k][p] = c * akp - s * akq;
					a[k][q] = s * akp + c * akq;
				}
				for (int k = 0; k < 3; k++) { // A <- J^T A
					const double apk = a[p][k], aqk = a[q][k];
					a[p][k] = c * apk - s * aqk;
					a[q][k] = s * apk + c * aqk;
				}
				for (int k = 0; k < 3; k++) { // V <- V J
					const double vkp = v[k][p], vkq = v[k][q];
					v[k][p] = c * vkp - s * vkq;
					v[k][q] = s * vkp + c * vkq;
				}
			}
	}
};

// QEF vertex in cell-local coordinates from up to 12 (point, normal) pairs.
inline void qef_solve(int ne, const double (*pt)[3], const double (*nm)[3], double out[3]) {
	double ata[3][3] = {}, atb[3] = {}, m[3] = {};
	for (int e = 0; e < ne; e++) {
		const double *n = nm[e], *x = pt[e];
		const double b = n[0] * x[0] + n[1] * x[1] + n[2] * x[2];
		for (int i = 0; i < 3; i++) {
			for (int j = 0; j < 3; j++) ata[i][j] += n[i] * n[j];
			atb[i] += n[i] * b;
			m[i] += x[i];
		}
	}
	for (int i = 0; i < 3; i++) m[i] /= ne;
	double r[3];
	for (int i = 0; i < 3; i++) r[i] = atb[i] - (ata[i][0] * m[0] + ata[i][1] * m[1] + ata[i][2] * m[2]);
	double a[3][3], v[3][3];
	for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) a[i][j] = ata[i][j];
	Jacobi3::run(a, v);
	const double lmax = std::max(std::fabs(a[0][0]), std::max(std::fabs(a[1][1]), std::fabs(a[2][2])));
	double c[3] = {0, 0, 0};
	for (int k = 0; k < 3; k++) {
		const double l = a[k][k];
		if (std::fabs(l) < 1e-2 * lmax || std::fabs(l) < 1e-12) continue;
		const double proj = (v[0][k] * r[0] + v[1][k] * r[1] + v[2][k] * r[2]) / l;
		for (int i = 0; i < 3; i++) c[i] += v[i][k] * proj;
	}
	for (int i = 0; i < 3; i++) out[i] = std::min(std::max(m[i] + c[i], 0.0), 1.0);
}

struct ContourResult {
	std::vector<uint64_t> cells;      // active cell linear indices (vertex order)
	std::vector<float> positions;     // 3 per vertex
	std::vector<float> normals;       // 3 per vertex
	std::vector<uint32_t> indices;    // 3 per triangle
	std::vector<uint64_t> edges;      // sign edges: point index * 3 + axis
};

using GradFn = std::function<void(const double p[3], double g[3])>;

inline void contour(const up_grid &gspec, const float *d, const GradFn &grad, ContourResult &res) {
	const GridF g(gspec);
	const uint64_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const uint64_t cx = nx - 1, cy = ny - 1, cz = nz - 1;
	auto P = [&](uint64_t i, uint64_t j, uint64_t k) { return (k * ny + j) * nx + i; };
	auto C = [&](uint64_t i, uint64_t j, uint64_t k) { return (k * cy + j) * cx + i; };
	auto in = [&](uint64_t idx) { return d[idx] < 0.0f; };

	// sign edges with Hermite data, keyed by point*3+axis
	std::vector<uint64_t> &edges = res.edges;
	std::vector<std::array<double, 6>> herm;
	std::unordered_map<uint64_t, uint32_t> emap;
	for (uint64_t k = 0; k < nz; k++)
		for (uint64_t j = 0; j < ny; j++)
			for (uint64_t i = 0; i < nx; i++) {
				const uint64_t p0 = P(i, j, k);
				for (int a = 0; a < 3; a++) {
					uint64_t i1 = i, j1 = j, k1 = k;
					if (a == 0) { if (i + 1 >= nx) continue; i1++; }
					if (a == 1) { if (j + 1 >= ny) continue; j1++; }
					if (a == 2) { if (k + 1 >= nz) continue; k1++; }
					const uint64_t p1 = P(i1, j1, k1);
					if (in(p0) == in(p1)) continue;
					const double d0 = d[p0], d1 = d[p1];
					const double t = d0 / (d0 - d1);
					double x0[3] = {g.coord(0, (uint32_t)i), g.coord(1, (uint32_t)j), g.coord(2, (uint32_t)k)};
					double x1[3] = {g.coord(0, (uint32_t)i1), g.coord(1, (uint32_t)j1), g.coord(2, (uint32_t)k1)};
					std::array<double, 6> h;
					for (int c = 0; c < 3; c++) h[c] = x0[c] + t * (x1[c] - x0[c]);
					double gr[3];
					grad(h.data(), gr);
					const double ln = std::sqrt(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
					for (int c = 0; c < 3; c++) h[3 + c] = ln > 0 ? gr[c] / ln : 0.0;
					emap[p0 * 3 + a] = (uint32_t)edges.size();
					edges.push_back(p0 * 3 + a);
					herm.push_back(h);
				}
			}

	// active cells and QEF vertices
	std::unordered_map<uint64_t, uint32_t> vmap;
	for (uint64_t k = 0; k < cz; k++)
		for (uint64_t j = 0; j < cy; j++)
			for (uint64_t i = 0; i < cx; i++) {
				int mask = 0;
				for (int b = 0; b < 8; b++)
					if (in(P(i + (b & 1), j + ((b >> 1) & 1), k + (b >> 2)))) mask |= 1 << b;
				if (mask == 0 || mask == 255) continue;
				const double o[3] = {g.coord(0, (uint32_t)i), g.coord(1, (uint32_t)j), g.coord(2, (uint32_t)k)};
				const double st[3] = {g.step[0], g.step[1], g.step[2]};
				double pts[12][3], nms[12][3];
				int ne = 0;
				for (int a = 0; a < 3; a++)
					for (int e = 0; e < 4; e++) {
						const int u = e & 1, w = e >> 1; // offsets along the two other axes (increasing order)
						uint64_t ii = i, jj = j, kk = k;
						if (a == 0) { jj += u; kk += w; }
						if (a == 1) { ii += u; kk += w; }
						if (a == 2) { ii += u; jj += w; }
						auto it = emap.find(P(ii, jj, kk) * 3 + a);
						if (it == emap.end()) continue;
						const auto &h = herm[it->second];
						double nl[3], nn = 0;
						for (int c = 0; c < 3; c++) { pts[ne][c] = (h[c] - o[c]) / st[c]; nl[c] = h[3 + c] * st[c]; nn += nl[c] * nl[c]; }
						nn = std::sqrt(nn);
						for (int c = 0; c < 3; c++) nms[ne][c] = nn > 0 ? nl[c] / nn : 0.0;
						ne++;
					}
				double v[3];
				qef_solve(ne, pts, nms, v);
				float vp[3];
				for (int c = 0; c < 3; c++) vp[c] = (float)(o[c] + v[c] * st[c]);
				const uint64_t cid = C(i, j, k);
				vmap[cid] = (uint32_t)res.cells.size();
				res.cells.push_back(cid);
				double vd[3] = {vp[0], vp[1], vp[2]}, gr[3];
				grad(vd, gr);
				const double ln = std::sqrt(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
				for (int c = 0; c < 3; c++) {
					res.positions.push_back(vp[c]);
					res.normals.push_back(ln > 0 ? (float)(gr[c] / ln) : 0.0f);
				}
			}

	// quads
	for (uint64_t e : edges) {
		const uint64_t p0 = e / 3;
		const int a = (int)(e % 3);
		const uint64_t i = p0 % nx, j = (p0 / nx) % ny, k = p0 / (nx * ny);
		uint64_t c4[4];
		if (a == 0) {
			if (j < 1 || j > cy - 1 || k < 1 || k > cz - 1) continue;
			c4[0] = C(i, j - 1, k - 1); c4[1] = C(i, j, k - 1); c4[2] = C(i, j, k); c4[3] = C(i, j - 1, k);
		} else if (a == 1) {
			if (i < 1 || i > cx - 1 || k < 1 || k > cz - 1) continue;
			c4[0] = C(i - 1, j, k - 1); c4[1] = C(i - 1, j, k); c4[2] = C(i, j, k); c4[3] = C(i, j, k - 1);
		} else {
			if (i < 1 || i > cx - 1 || j < 1 || j > cy - 1) continue;
			c4[0] = C(i - 1, j - 1, k); c4[1] = C(i, j - 1, k); c4[2] = C(i, j, k); c4[3] = C(i - 1, j, k);
		}
		uint32_t v[4];
		for (int q = 0; q < 4; q++) v[q] = vmap.at(c4[q]);
		if (in(p0)) {
			const uint32_t t[6] = {v[0], v[1], v[2], v[0], v[2], v[3]};
			res.indices.insert(res.indices.end(), t, t + 6);
		} else {
			const uint32_t t[6] = {v[0], v[2], v[1], v[0], v[3], v[2]};
			res.indices.insert(res.indices.end(), t, t + 6);
		}
	}
}

} // namespace orc
