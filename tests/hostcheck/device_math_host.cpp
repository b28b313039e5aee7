// Test harness: compiles the CUDA path's device arithmetic headers as plain
// host C++ so the CPU test suite can compare them with the oracle without a
// GPU. It exercises arithmetic only; the kernels themselves run in the GPU
// tests. Built by tests/hostcheck/build_hostcheck.py into tests/hostcheck/_build.
#include "../../unnatural-planets_gb300/csrc/up_synth.cuh"
#include "../../unnatural-planets_gb300/csrc/up_grid_runs.cuh"
#include "../../unnatural-planets_gb300/csrc/up_modes.cuh"
#include "../../unnatural-planets_gb300/csrc/up_modes_runs.cuh"
#include "../../unnatural-planets_gb300/csrc/up_coloring.cuh"
#include "../../unnatural-planets_gb300/csrc/up_fastdiv.h"
#include "../../unnatural-planets_gb300/csrc/up_ptr.h"
#include <string>

namespace up {
int build_modes(const up_modes &m, uint32_t seed, ModesDesc &D, std::string &shape_name, bool &double_sided, std::string &err);
void elevation_range(const ModesDesc &D, double &lo, double &hi);
float modes_contour_band(const ModesDesc &D, int field, const float step[3]);
}

using namespace up;

// grid of the host checks (the fields of GridDev that the task helpers read)
struct HostGrid { uint32_t n[3]; float lo[3], step[3]; uint32_t k0; };

extern "C" {

void hc_noise(int type, int dist, int op, uint32_t key, const float *xyz, uint64_t n, float *out, float *grad) {
	for (uint64_t i = 0; i < n; i++) {
		const V3f p = v3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
		if (grad) {
			const NG r = noise_single<true>(type, p, key, dist, op);
			out[i] = r.v;
			grad[3 * i] = r.g.x; grad[3 * i + 1] = r.g.y; grad[3 * i + 2] = r.g.z;
		} else {
			out[i] = noise_single<false>(type, p, key, dist, op).v;
		}
	}
}

void hc_synth(const up_synth_program *P, const float *xyz, uint64_t n, float *out, float *grad) {
	for (uint64_t i = 0; i < n; i++) {
		const V3f p = v3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
		if (grad) {
			const NG r = synth_eval<true, -1, -1>(*P, p);
			out[i] = r.v;
			grad[3 * i] = r.g.x; grad[3 * i + 1] = r.g.y; grad[3 * i + 2] = r.g.z;
		} else {
			out[i] = synth_eval<false, -1, -1>(*P, p).v;
		}
	}
}

// sum_i w_i d d(p_i) / d theta in the compact theta layout
int hc_synth_bwd(const up_synth_program *P, const float *xyz, uint64_t n, const float *w, double *dtheta) {
	float acc[ACC_N];
	double tot[ACC_N] = {};
	for (uint64_t i = 0; i < n; i++) {
		for (int k = 0; k < ACC_N; k++) acc[k] = 0.f;
		synth_bwd<-1, -1>(*P, v3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), w[i], acc);
		for (int k = 0; k < ACC_N; k++) tot[k] += acc[k];
	}
	int slots[64];
	const int m = theta_slots(*P, slots);
	for (int j = 0; j < m; j++) dtheta[j] = tot[slots[j]];
	return m;
}

uint32_t hc_lattice_hash(int x, int y, int z, uint32_t key) { return lattice_hash(x, y, z, key); }
// where the C ABI takes a caller's buffer from (up_ptr.h): 0 host, 1 in place, 2 other GPU
int hc_ptr_kind(int query_ok, int type, int device, int ctx_device) { return (int)ptr_kind(query_ok != 0, type, device, ctx_device); }
uint32_t hc_corner_hash(int x, int y, int z, uint32_t key, int b) {
	Cell c; c.ix = x; c.iy = y; c.iz = z; c.fx = c.fy = c.fz = 0.f;
	return corner_hashes(c, key).h[b];
}

// reference-mode planet built by the product's host builder
void *hc_modes_create(const char *shape, const char *elevation, const char *coloring, int poles, int flowers, uint32_t seed) {
	up_modes m{shape, elevation, coloring, poles, flowers};
	auto *D = new ModesDesc();
	std::string name, err;
	bool ds;
	if (build_modes(m, seed, *D, name, ds, err) != UP_OK) { delete D; return nullptr; }
	return D;
}
void hc_modes_free(void *d) { delete (ModesDesc *)d; }
void hc_elevation_range(void *d, double *lo, double *hi) { elevation_range(*(ModesDesc *)d, *lo, *hi); }
float hc_modes_band(void *d, int field, const float *step) { return modes_contour_band(*(ModesDesc *)d, field, step); }
void hc_modes_field(void *d, int field, const float *xyz, uint64_t n, float *out, float *grad) {
	const ModesDesc &M = *(ModesDesc *)d;
	for (uint64_t i = 0; i < n; i++) {
		const V3f p = v3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
		if (grad) {
			const Df f = field_eval(M, field, dual_point(p));
			out[i] = f.v;
			grad[3 * i] = f.d.x; grad[3 * i + 1] = f.d.y; grad[3 * i + 2] = f.d.z;
		} else {
			out[i] = field_eval(M, field, vs(p.x, p.y, p.z));
		}
	}
}

// per-point tiles with the device coloring pipeline (11 floats + biome, type)
void hc_tiles(void *d, int purpose, const float *pos, const float *nrm, uint64_t n, float *out11, int32_t *bt) {
	const ModesDesc &M = *(ModesDesc *)d;
	for (uint64_t i = 0; i < n; i++) {
		TileD t = tile_init(v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), v3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]), purpose);
		color_tile(M, t);
		float *o = out11 + 11 * i;
		o[0] = t.albedo.x; o[1] = t.albedo.y; o[2] = t.albedo.z; o[3] = t.roughness; o[4] = t.metallic; o[5] = t.height; o[6] = t.opacity;
		o[7] = t.elevation; o[8] = t.slope; o[9] = t.temperature; o[10] = t.precipitation;
		bt[2 * i] = t.biome; bt[2 * i + 1] = t.type;
	}
}
void hc_synth_texel(const up_synth_program *P, const float *pos, uint64_t n, float *out5) {
	for (uint64_t i = 0; i < n; i++) {
		V3f a; float r, h;
		synth_texel(*P, v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), a, r, h);
		out5[5 * i] = a.x; out5[5 * i + 1] = a.y; out5[5 * i + 2] = a.z; out5[5 * i + 3] = r; out5[5 * i + 4] = h;
	}
}

// whole grid of the torus/spheres/ridged-Perlin/cellular program through the
// run-based evaluation (runs of RUN_R samples along x, the kernel's order)
float hc_noise_bound(int type, int dist, int op) { return noise_abs_bound(type, dist, op); }
float hc_synth_noise_bound(const up_synth_program *P) { return synth_noise_bound(*P); }

// value-only runs with a narrow band (the internal sampling of contouring)
void hc_grid_runs_band(const up_synth_program *P, const float *lo, const float *step, const uint32_t *n, float band, float *out) {
	constexpr int R = RUN_R;
	constexpr int T1 = cell_spec(UP_DIST_EUCLIDEAN, UP_OP_SUBTRACT);
	auto coord = [&](int a, uint32_t i) { volatile float m = (float)i * step[a]; return m + lo[a]; };
	RunCtx rc;
	rc.lo_x = lo[0];
	rc.step_x = step[0];
	rc.nx = n[0];
	for (uint32_t k = 0; k < n[2]; k++)
		for (uint32_t j = 0; j < n[1]; j++)
			for (uint32_t i0 = 0; i0 < n[0]; i0 += R) {
				rc.i0 = i0;
				rc.py = coord(1, j);
				rc.pz = coord(2, k);
				float acc[R];
				synth_run<false, 2, T1>(*P, rc, R, acc, 1, band);
				for (int r = 0; r < R && i0 + r < n[0]; r++) out[((uint64_t)k * n[1] + j) * n[0] + i0 + r] = acc[r];
			}
}

void hc_grid_runs(const up_synth_program *P, const float *lo, const float *step, const uint32_t *n, float *out, float *grad) {
	constexpr int R = RUN_R;
	constexpr int T1 = cell_spec(UP_DIST_EUCLIDEAN, UP_OP_SUBTRACT);
	const uint64_t plane = (uint64_t)n[0] * n[1] * n[2];
	auto coord = [&](int a, uint32_t i) { volatile float m = (float)i * step[a]; return m + lo[a]; };
	RunCtx rc;
	rc.lo_x = lo[0];
	rc.step_x = step[0];
	rc.nx = n[0];
	for (uint32_t k = 0; k < n[2]; k++)
		for (uint32_t j = 0; j < n[1]; j++)
			for (uint32_t i0 = 0; i0 < n[0]; i0 += R) {
				rc.i0 = i0;
				rc.py = coord(1, j);
				rc.pz = coord(2, k);
				if (grad) {
					Acc4 acc[R];
					synth_run<true, 2, T1>(*P, rc, R, acc, 1);
					for (int r = 0; r < R && i0 + r < n[0]; r++) {
						const uint64_t idx = ((uint64_t)k * n[1] + j) * n[0] + i0 + r;
						out[idx] = acc[r].v;
						grad[idx] = acc[r].gx; grad[plane + idx] = acc[r].gy; grad[2 * plane + idx] = acc[r].gz;
					}
				} else {
					float acc[R];
					synth_run<false, 2, T1>(*P, rc, R, acc, 1);
					for (int r = 0; r < R && i0 + r < n[0]; r++) out[((uint64_t)k * n[1] + j) * n[0] + i0 + r] = acc[r];
				}
			}
}

// land, water, navigation over a grid through the run tables of
// up_modes_runs.cuh (the x-coherent modes kernel's arithmetic, one run at a
// time); returns 0 when the mode has no run tables
int hc_modes_grid_runs(void *d, const float *lo, const float *step, const uint32_t *n, float band, float *o0, float *o1, float *o2) {
	const ModesDesc &M = *(ModesDesc *)d;
	if (!mrun_applies(M)) return 0;
	constexpr int R = RUN_R;
	auto coord = [&](int a, uint32_t i) { volatile float m = (float)i * step[a]; return m + lo[a]; };
	RunCtx rc;
	rc.lo_x = lo[0];
	rc.step_x = step[0];
	rc.nx = n[0];
	float tab[3 * R], *outs[3] = {o0, o1, o2};
	for (uint32_t k = 0; k < n[2]; k++)
		for (uint32_t j = 0; j < n[1]; j++)
			for (uint32_t i0 = 0; i0 < n[0]; i0 += R) {
				rc.i0 = i0;
				rc.py = coord(1, j);
				rc.pz = coord(2, k);
				if (M.elevation == 2) modes_run_fill<2>(M, rc, R, tab, 1);
				else if (M.elevation == 3) modes_run_fill<3>(M, rc, R, tab, 1);
				else modes_run_fill<4>(M, rc, R, tab, 1);
				float shv[R];
				modes_run_shape(M, rc, R, band, shv, 1);
				for (int r = 0; r < R && i0 + r < n[0]; r++) {
					const float sh = shv[r];
					float v[3];
					if (M.elevation == 2) modes_run_fields<2>(M, rc, r, sh, true, band, tab, 1, v);
					else if (M.elevation == 3) modes_run_fields<3>(M, rc, r, sh, true, band, tab, 1, v);
					else modes_run_fields<4>(M, rc, r, sh, true, band, tab, 1, v);
					const uint64_t idx = ((uint64_t)k * n[1] + j) * n[0] + i0 + r;
					for (int f = 0; f < 3; f++) outs[f][idx] = v[f];
				}
			}
	return 1;
}

// synth_base at R samples of the segment x in [x0, x1] at (y, z): with the
// sphere mask of synth_segment_spheres (v, g into out_m) and testing every
// sphere (out_f); returns the mask
uint32_t hc_segment_base(const up_synth_program *P, float x0, float x1, float y, float z, int R, float *out_m, float *out_f) {
	const uint32_t live = synth_segment_spheres(*P, x0, x1, y, z);
	for (int r = 0; r < R; r++) {
		const float x = R > 1 ? x0 + (x1 - x0) * (float)r / (float)(R - 1) : x0;
		const NG a = synth_base<true>(*P, v3(fminf(x, x1), y, z), live), b = synth_base<true>(*P, v3(fminf(x, x1), y, z));
		out_m[4 * r] = a.v; out_m[4 * r + 1] = a.g.x; out_m[4 * r + 2] = a.g.y; out_m[4 * r + 3] = a.g.z;
		out_f[4 * r] = b.v; out_f[4 * r + 1] = b.g.x; out_f[4 * r + 2] = b.g.y; out_f[4 * r + 3] = b.g.z;
	}
	return live;
}

// FastDiv (up_fastdiv.h): q[i] = n[i] / d by the multiply-shift
// narrow band at the task level (synth_task_band_kernel): task_val[t] =
// base(centre) for the tasks classified outside the band, NaN for the
// listed ones; band as contour_band (noise bound + longest step, margins)
float hc_task_band(const up_synth_program *P, const float *lo, const float *step, const uint32_t *n, float *task_val) {
	HostGrid g{{n[0], n[1], n[2]}, {lo[0], lo[1], lo[2]}, {step[0], step[1], step[2]}, 0u};
	const float st = fmaxf(step[0], fmaxf(step[1], step[2]));
	const float band = (synth_noise_bound(*P) + st) * 1.001f + 1e-5f;
	const uint32_t ntasks = ((n[0] + RUN_R - 1) / RUN_R) * ((n[1] + 7) / 8) * ((n[2] + 3) / 4);
	for (uint32_t t = 0; t < ntasks; t++) {
		V3f c;
		float hd;
		runs_task_box(g, t, c, hd);
		const float fv = synth_base<false>(*P, c).v;
		task_val[t] = fabsf(fv) > (band + hd) * 1.001f + 1e-5f ? fv : NAN;
	}
	return band;
}
// reference-mode narrow band at the task level (modes_task_band_kernel):
// task_val[t] = shape(centre) for the tasks classified outside the band,
// NaN for the listed ones
void hc_modes_task_band(void *d, const float *lo, const float *step, const uint32_t *n, float band, float *task_val) {
	const ModesDesc &M = *(ModesDesc *)d;
	HostGrid g{{n[0], n[1], n[2]}, {lo[0], lo[1], lo[2]}, {step[0], step[1], step[2]}, 0u};
	const uint32_t ntasks = ((n[0] + RUN_R - 1) / RUN_R) * ((n[1] + 7) / 8) * ((n[2] + 3) / 4);
	for (uint32_t t = 0; t < ntasks; t++) {
		V3f c;
		float hd;
		runs_task_box(g, t, c, hd);
		const float fv = shape_eval(M, vs(c.x, c.y, c.z));
		task_val[t] = fabsf(fv) > (band + hd) * 1.001f + 1e-3f * (1.f + fabsf(fv)) ? fv : NAN;
	}
}
// base value at every grid sample (coordinates as the grid kernels form them)
void hc_base_grid(const up_synth_program *P, const float *lo, const float *step, const uint32_t *n, float *out) {
	uint64_t q = 0;
	for (uint32_t k = 0; k < n[2]; k++)
		for (uint32_t j = 0; j < n[1]; j++)
			for (uint32_t i = 0; i < n[0]; i++)
				out[q++] = synth_base<false>(*P, v3(runs_coord(lo[0], step[0], i), runs_coord(lo[1], step[1], j), runs_coord(lo[2], step[2], k))).v;
}

// sign words of row segments (p0[i], bits m[i]) OR-ed as the unaligned
// path of the grid kernels does (row_sign_parts)
void hc_row_signs(const uint64_t *p0, const uint32_t *m, uint64_t count, uint32_t *words) {
	for (uint64_t i = 0; i < count; i++) {
		const up::RowSignParts q = up::row_sign_parts(p0[i], m[i]);
		words[q.w] |= q.lo;
		if (q.hi) words[q.w + 1] |= q.hi;
	}
}
void hc_fastdiv(uint32_t d, const uint32_t *n, uint64_t count, uint32_t *q) {
	const FastDiv f = FastDiv::of(d);
	for (uint64_t i = 0; i < count; i++) q[i] = f.div(n[i]);
}

// mix32 of a ^ b against its split form (the lattice runs hash a corner as
// mix32_tail of the x and y/z halves, each through mix32_head): out[i] = 1
// where they agree
void hc_mix32_split(const uint32_t *a, const uint32_t *b, uint64_t n, uint8_t *out) {
	for (uint64_t i = 0; i < n; i++) out[i] = mix32(a[i] ^ b[i]) == mix32_tail(mix32_head(a[i]) ^ mix32_head(b[i]));
}
// the ridged derivative factor of the lattice runs (n != 0 ? mul_sign(k2, n)
// : 0) against its select form (k2 for n > 0, -k2 for n < 0, 0 at n = 0):
// out[i] = 1 where the bits agree
void hc_ridged_sign(const float *k2, const float *nv, uint64_t n, uint8_t *out) {
	for (uint64_t i = 0; i < n; i++) {
		const float a = nv[i] != 0.f ? mul_sign(k2[i], nv[i]) : 0.f;
		const float b = nv[i] > 0.f ? k2[i] : (nv[i] < 0.f ? -k2[i] : 0.f);
		out[i] = f_bits(a) == f_bits(b);
	}
}

// Warp-wide pruning of the cellular table (the helpers of up_grid_runs.cuh
// that cellular_subrun uses), checked against the unpruned search: random
// warps of 32 lanes (table cells ty, tz in 1 .. t*max, fractions fy, fz) and
// sub-runs of 8 samples along x, table entries made by cell_entry from
// random hashes; every lane and sample ranks its candidates by the kernel's
// keys (metric bits with the entry id in the low 6 bits) over the lane's 3 x 3
// window and the columns of its x cell, once over every entry and once over
// the entries the pruning keeps. spread: the sub-run's extent along x, and
// lane_spread the lanes' extent along y and z, in cells (at most 1 each).
// Returns the number of (lane, sample) pairs whose two keys differ; *kept
// and *total count the kept and the present entries over all trials.
int hc_prune_check(uint32_t seed, int trials, double spread, double lane_spread, uint64_t *kept, uint64_t *total) {
	constexpr int S = 8;
	uint32_t st = seed * 2654435761u + 12345u;
	auto next = [&]() { st = mix32(st + 0x9E3779B9u); return st; };
	auto unit = [&]() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }; // [0, 1)
	int bad = 0;
	*kept = 0; *total = 0;
	for (int t = 0; t < trials; t++) {
		// the sub-run's x positions in the first column frame: increasing, below 2
		const float x0 = unit(), dx = unit() * (float)spread / S;
		float sx[S];
		int split = S;
		for (int r = 0; r < S; r++) {
			const float x = x0 + dx * (float)r;
			sx[r] = x < 1.f ? x : 1.f + (x - 1.f); // cell ixa + 1 from x = 1 on
			if (x >= 1.f && split == S) split = r;
		}
		const int ncol = split < S ? 4 : 3;
		// the lanes' cells and fractions along y and z, table cells counted from
		// the lowest lane cell (which is table cell 1), as in cellular_subrun
		int ty[32], tz[32];
		float fy[32], fz[32];
		const float y0 = unit(), z0 = unit();
		int iymin = 2, izmin = 2;
		for (int l = 0; l < 32; l++) {
			const float ly = y0 + unit() * (float)lane_spread, lz = z0 + unit() * (float)lane_spread;
			const float fly = floorf(ly), flz = floorf(lz);
			ty[l] = (int)fly; tz[l] = (int)flz;
			fy[l] = ly - fly; fz[l] = lz - flz;
			iymin = ty[l] < iymin ? ty[l] : iymin;
			izmin = tz[l] < izmin ? tz[l] : izmin;
		}
		int tymax = 1, tzmax = 1;
		for (int l = 0; l < 32; l++) {
			ty[l] += 1 - iymin; tz[l] += 1 - izmin;
			tymax = ty[l] > tymax ? ty[l] : tymax;
			tzmax = tz[l] > tzmax ? tz[l] : tzmax;
		}
		CellEntry ce[64];
		for (int e = 0; e < 64; e++) ce[e] = cell_entry(next(), e);
		// the warp's box and the pruning, as cellular_subrun forms them
		CellBox box;
		box.x0 = sx[0]; box.x1 = sx[0];
		for (int r = 1; r < S; r++) { box.x0 = fminf(box.x0, sx[r]); box.x1 = fmaxf(box.x1, sx[r]); }
		box.y0 = box.z0 = 3e38f; box.y1 = box.z1 = -3e38f;
		for (int l = 0; l < 32; l++) {
			const float ly = (float)ty[l] + fy[l], lz = (float)tz[l] + fz[l];
			box.y0 = fminf(box.y0, ly); box.y1 = fmaxf(box.y1, ly);
			box.z0 = fminf(box.z0, lz); box.z1 = fmaxf(box.z1, lz);
		}
		const int n = ncol * 16;
		float lb[64], ub[64];
		float u1 = 3e38f, u2 = 3e38f; // the two smallest ub of the entries seen everywhere
		for (int e = 0; e < n; e++) {
			cell_box_bounds<0>(ce[e], box, lb[e], ub[e]);
			if (!cell_entry_everywhere(e, ncol, tymax, tzmax)) continue;
			if (ub[e] < u1) { u2 = u1; u1 = ub[e]; }
			else if (ub[e] < u2) u2 = ub[e];
		}
		const float thr = cell_prune_bound(u2);
		bool keep[64];
		for (int e = 0; e < n; e++) {
			keep[e] = lb[e] <= thr && cell_entry_in_some_window(e, tymax, tzmax);
			*kept += keep[e];
			*total += 1;
		}
		// every lane and sample: the full search and the pruned one
		for (int l = 0; l < 32; l++) {
			const float tyf = (float)ty[l], tzf = (float)tz[l];
			for (int r = 0; r < S; r++) {
				uint32_t K[2][2] = {{0xFFFFFFFFu, 0xFFFFFFFFu}, {0xFFFFFFFFu, 0xFFFFFFFFu}};
				for (int e = 0; e < n; e++) {
					const int col = e >> 4, yy = (e >> 2) & 3, zz = e & 3;
					if (abs(yy - ty[l]) > 1 || abs(zz - tz[l]) > 1) continue;    // outside the lane's window
					if ((col == 0 && r >= split) || (col == 3 && r < split)) continue; // outside the sample's columns
					const float vy = (ce[e].jy - tyf) - fy[l];
					const float vz = (ce[e].jz - tzf) - fz[l];
					const float d = cell_metric<0>(ce[e].jx - sx[r], vy * vy + vz * vz, fabsf(vy) + fabsf(vz));
					const uint32_t k = (f_bits(d) & ~63u) | (uint32_t)e;
					for (int v = 0; v < 2; v++) {
						if (v == 1 && !keep[e]) continue;
						K[v][1] = umin32(K[v][1], umax32(K[v][0], k));
						K[v][0] = umin32(K[v][0], k);
					}
				}
				if (K[0][0] != K[1][0] || K[0][1] != K[1][1]) bad++;
			}
		}
	}
	return bad;
}
}

