// x-coherent grid sampling of synthetic programs ("runs").
//
// A warp evaluates RUN_R consecutive samples along x for 32 different (y, z)
// rows: every lane sees the same x coordinates, so a lattice-cell change
// along x happens for all lanes at the same sample (warp-uniform control
// flow). Per-sample accumulators (value and gradient) live in shared memory
// as acc[r * stride + lane-slot], so the sample loops stay rolled and
// every code block appears once (the unrolled form overflowed the
// instruction cache).
// Lattice noise (value, Perlin): per octave, the y/z fade weights are formed
// once per run; corner hashes and gradients are formed only when the x cell
// changes (once per segment of samples sharing a cell; 4 of the 8 corners
// when the new cell is the next one along x, whose low face is the old high
// face) and folded into 12 coefficients (x halves h = 0/1 of
//   A_h(t) = t GX_h + C_h,  dA_h/dy = t P_hy + Q_hy,  dA_h/dz = t P_hz + Q_hz),
// after which a sample's value and analytic gradient cost a few FMAs:
//   n = A0(fx) + u (A1(fx - 1) - A0(fx)),
//   dn/dx = GX0 + u (GX1 - GX0) + u' (A1 - A0), dn/dy, dn/dz likewise
// (the trilinear form of I. Quilez's gradient-noise derivatives).
// Cellular noise: in sub-runs of 8 samples, candidates outer and samples
// inner -- each of the 3 or 4 x columns of 9 candidate cells is hashed once
// per sub-run, a sample ignores columns outside its own 3x3x3 neighbourhood
// (so the candidate set equals the per-sample search); with the warp's
// shared cell table, candidates that cannot be among any sample's two
// nearest are skipped warp-wide. The two nearest are kept as integer keys
// (distance bits with the candidate id in the low 6 mantissa bits), and the
// winners' distances and difference vectors are rebuilt from the ids (the
// value-only form on the device takes the winners' metrics from the keys
// themselves, the middle of their 2^-17 relative quantum, and rebuilds
// nothing). Values equal the per-sample kernels up to FP32 reassociation
// and, on the device, the approximate square root of the winners' distances
// (sqrt_hd) and the value-only form's quantised metrics (within 2^-18
// relative; 1e-7 of the benchmark planet's value);
// the key's 2^-17 relative quantisation can only reorder candidates whose
// distances agree to that level (F1/F2 near-ties, where the gradient of
// F2 - F1 is discontinuous anyway).
#pragma once
#include "up_synth.cuh"

namespace up {

constexpr int RUN_R = 16;   // samples per run
constexpr int CELL_SUB = 8; // cellular sub-run

// sample coordinates of a run: x(r) = lo + (i0 + r) step (clamped to the grid)
struct RunCtx {
	float lo_x, step_x;
	uint32_t i0, nx;
	float py, pz;
	UP_HD float px(int r) const {
		const uint32_t i = i0 + (uint32_t)r < nx ? i0 + (uint32_t)r : nx - 1;
#ifdef __CUDA_ARCH__
		return __fadd_rn(__fmul_rn((float)i, step_x), lo_x);
#else
		volatile float m = (float)i * step_x;
		return m + lo_x;
#endif
	}
};

// Perlin gradient vectors (grad_vec of h & 15) in shared memory: a lookup is
// one shared load instead of a chain of integer selects on the ALU pipe.
// runs_tables_init() fills it at the start of every kernel that calls
// synth_run (host builds compute grad_vec directly).
#ifdef __CUDACC__
__shared__ float4 g_runs_gradtab[16];
__device__ __forceinline__ void runs_tables_init() {
	if (threadIdx.x < 16) {
		const V3f v = grad_vec(threadIdx.x);
		g_runs_gradtab[threadIdx.x] = make_float4(v.x, v.y, v.z, 0.f);
	}
	__syncthreads();
}
#endif
UP_HD V3f grad_lookup(uint32_t h) {
#ifdef __CUDA_ARCH__
	const float4 t = g_runs_gradtab[h & 15u];
	return v3(t.x, t.y, t.z);
#else
	return grad_vec(h);
#endif
}

// Per-warp table of the x quantities of one lattice octave: every lane of a
// warp shares the run's x coordinates, so lanes 0..R-1 fill entry r = lane
// once per octave and all lanes read it (shared-memory broadcast) instead of
// each forming x, floor, fade and fade' per sample.
struct XTab { float fx, u, du; int cx; };
constexpr int RUNS_WARPS = 8; // warps per block of the runs kernels
#ifdef __CUDACC__
__shared__ XTab g_runs_xtab[RUNS_WARPS * RUN_R];
#endif
UP_HD XTab xtab_entry(const RunCtx &rc, int r, float f) {
	const float qx = rc.px(r) * f;
	const float fx0 = floorf(qx);
	XTab e;
	e.fx = qx - fx0;
	e.u = fade(e.fx);
	e.du = dfade(e.fx);
	e.cx = (int)fx0;
	return e;
}

// per-sample accumulator: value and gradient (Acc4) or value only (float);
// acc[r * stride] belongs to sample r
struct alignas(16) Acc4 { float v, gx, gy, gz; };
template<bool GRAD> struct AccOf { typedef Acc4 T; };
template<> struct AccOf<false> { typedef float T; };
UP_HD void acc_set(Acc4 *a, int i, float v, float gx, float gy, float gz) { Acc4 t; t.v = v; t.gx = gx; t.gy = gy; t.gz = gz; a[i] = t; }
UP_HD void acc_set(float *a, int i, float v, float, float, float) { a[i] = v; }
UP_HD void acc_add(Acc4 *a, int i, float v, float gx, float gy, float gz) {
	Acc4 t = a[i];
	t.v += v; t.gx += gx; t.gy += gy; t.gz += gz;
	a[i] = t;
}
UP_HD void acc_add(float *a, int i, float v, float, float, float) { a[i] += v; }
// value term a * b added with one rounding (fmaf), on the device and the host
// alike, so the value-only and value+gradient forms agree bit for bit
UP_HD void acc_add_fma(Acc4 *acc, int i, float a, float b, float gx, float gy, float gz) {
	Acc4 t = acc[i];
	t.v = fmaf(a, b, t.v); t.gx += gx; t.gy += gy; t.gz += gz;
	acc[i] = t;
}
UP_HD void acc_add_fma(float *acc, int i, float a, float b, float, float, float) { acc[i] = fmaf(a, b, acc[i]); }

// one octave of lattice noise (VALUE = value noise, else Perlin); subtracts
// amp * s(n) (s = n or 1 - 2|n|) from every sample of the run
// RIDGED: 1 ridged, 0 not, both fixed at compile time (the per-sample loop
// carries no branch on it); -1 taken from ridged_rt at run time (one
// instantiation for callers that hold many noise instances in one kernel)
template<bool GRAD, bool VALUE, int RIDGED>
UP_HD void lattice_octave_run_t(const RunCtx &rc, int R, float f, float amp, uint32_t key, typename AccOf<GRAD>::T *acc, int stride,
	bool ridged_rt = false) {
	const bool ridged = RIDGED < 0 ? ridged_rt : RIDGED == 1;
	const float qy = rc.py * f, qz = rc.pz * f;
	const float fy0 = floorf(qy), fz0 = floorf(qz);
	const int iy = (int)fy0, iz = (int)fz0;
	const float fy = qy - fy0, fz = qz - fz0;
	// fade and fade' of y and z as FP32 pairs: t^3 (t (6 t - 15) + 10) and
	// 30 t^2 (t (t - 2) + 1)
	const P2 t = p2(fy, fz), t2 = mul2(t, t);
	const P2 fd = mul2(mul2(t2, t), fma2(t, fma2(t, p2s(6.f), p2s(-15.f)), p2s(10.f)));
	const float v = fd.x, w = fd.y;
	float dv = 0.f, dw = 0.f;
	if (GRAD) {
		const P2 dd = mul2(mul2(p2s(30.f), t2), fma2(t, add2(t, p2s(-2.f)), p2s(1.f)));
		dv = dd.x; dw = dd.y;
	}
	// y/z corners c = by + 2 bz
	const float Wyz[4] = {(1.f - v) * (1.f - w), v * (1.f - w), (1.f - v) * w, v * w};
	const float dWy[4] = {-dv * (1.f - w), dv * (1.f - w), -dv * w, dv * w};
	const float dWz[4] = {-(1.f - v) * dw, -v * dw, (1.f - v) * dw, v * dw};
	const uint32_t y0 = (uint32_t)iy * HY, z0 = ((uint32_t)iz * HZ) ^ key, z1 = ((uint32_t)iz * HZ + HZ) ^ key;
	// the y/z half of each corner's hash, its first mixing step applied
	const uint32_t yz[4] = {mix32_head(y0 ^ z0), mix32_head((y0 + HY) ^ z0), mix32_head(y0 ^ z1), mix32_head((y0 + HY) ^ z1)};
	const float ys[4] = {fy, fy - 1.f, fy, fy - 1.f}, zs[4] = {fz, fz, fz - 1.f, fz - 1.f};
	// starts: bit r set when sample r begins a segment (its x cell differs
	// from sample r - 1's), the same for every lane
#ifdef __CUDA_ARCH__
	XTab *tab = g_runs_xtab + (threadIdx.x >> 5) * RUN_R;
	__syncwarp(); // every lane has finished reading the previous octave's table
	const int lane = (int)(threadIdx.x & 31);
	int mycx = 0;
	if (lane < R) {
		const XTab e = xtab_entry(rc, lane, f);
		tab[lane] = e;
		mycx = e.cx;
	}
	const int leftcx = __shfl_up_sync(0xFFFFFFFFu, mycx, 1);
	const uint32_t starts = __ballot_sync(0xFFFFFFFFu, lane < R && (lane == 0 || mycx != leftcx));
	__syncwarp();
#else
	XTab tab[RUN_R];
	uint32_t starts = 0;
	for (int q = 0; q < R; q++) {
		tab[q] = xtab_entry(rc, q, f);
		if (q == 0 || tab[q].cx != tab[q - 1].cx) starts |= 1u << q;
	}
#endif
	// coefficients of the two x faces of the current cell; when the next
	// segment is the neighbouring cell, its low face is the old high face
	float GX[2], Cc[2], Py[2], Qy[2], Pz[2], Qz[2];
	int cx_prev = 0;
	int r = 0;
	#pragma unroll 1
	while (r < R) { // one segment of samples sharing an x cell (the same for every lane)
		const int cx = tab[r].cx;
		// the segment's end: the next start after r, or R
		const uint32_t later = starts & ~((2u << r) - 1u);
		const int r1 = later ? lowest_bit(later) : R;
		const bool carry = r > 0 && cx == cx_prev + 1;
		cx_prev = cx;
		if (carry) { GX[0] = GX[1]; Cc[0] = Cc[1]; Py[0] = Py[1]; Qy[0] = Qy[1]; Pz[0] = Pz[1]; Qz[0] = Qz[1]; }
		#pragma unroll
		for (int h = 0; h < 2; h++) {
			if (h == 0 && carry) continue;
			const uint32_t xh = mix32_head((uint32_t)(cx + h) * HX);
			V3f cg[4]; // corner c: gradient vector, or the value in .x
			#pragma unroll
			for (int c = 0; c < 4; c++) {
				const uint32_t hh = mix32_tail(xh ^ yz[c]); // == mix32(x part ^ y/z part)
				cg[c] = VALUE ? v3(hash_signed(hh), 0.f, 0.f) : grad_lookup(hh);
			}
			// the face's coefficients, summed over its 4 corners in pairs:
			// (GX, C) += W (g.x, cyz); (Py, Pz) += (dWy, dWz) g.x;
			// (Qy, Qz) += W (g.y, g.z) + (dWy, dWz) cyz
			P2 gc = p2(0.f, 0.f), pyz = p2(0.f, 0.f), qyz = p2(0.f, 0.f);
			#pragma unroll
			for (int c = 0; c < 4; c++) {
				const P2 dW = p2(dWy[c], dWz[c]);
				if (VALUE) {
					const float val = cg[c].x;
					gc.y += Wyz[c] * val;
					if (GRAD) qyz = fma2(dW, p2s(val), qyz);
				} else {
					const V3f g = cg[c];
					const float cyz = g.y * ys[c] + g.z * zs[c];
					gc = fma2(p2s(Wyz[c]), p2(g.x, cyz), gc);
					if (GRAD) {
						pyz = fma2(dW, p2s(g.x), pyz);
						qyz = fma2(dW, p2s(cyz), fma2(p2s(Wyz[c]), p2(g.y, g.z), qyz));
					}
				}
			}
			GX[h] = gc.x; Cc[h] = gc.y; Py[h] = pyz.x; Qy[h] = qyz.x; Pz[h] = pyz.y; Qz[h] = qyz.y;
		}
		// per segment: the high face minus the low one as linear functions of
		// fx (A1 - A0 = fx DG + DC, likewise for the y and z derivatives)
		const float DG = VALUE ? 0.f : GX[1] - GX[0], DC = VALUE ? Cc[1] - Cc[0] : (Cc[1] - GX[1]) - Cc[0];
		const float DPy = VALUE ? 0.f : Py[1] - Py[0], DQy = VALUE ? Qy[1] - Qy[0] : (Qy[1] - Py[1]) - Qy[0];
		const float DPz = VALUE ? 0.f : Pz[1] - Pz[0], DQz = VALUE ? Qz[1] - Qz[0] : (Qz[1] - Pz[1]) - Qz[0];
		const float k2 = 2.f * amp * f;
		// two samples per step in the reference-mode instantiation (RIDGED < 0:
		// value only, several noise instances per kernel), one elsewhere (both
		// measured fastest for their kernel)
		constexpr int SAMPLE_UNROLL = RIDGED < 0 ? 2 : 1;
		#pragma unroll SAMPLE_UNROLL
		for (; r < r1; r++) {
			const XTab e = tab[r];
			const float fx = e.fx;
			const float u = e.u;
			const float A0 = VALUE ? Cc[0] : fx * GX[0] + Cc[0];
			const float dA = VALUE ? DC : fx * DG + DC;
			const float n = A0 + u * dA;
			const float s = ridged ? 1.f - 2.f * fabsf(n) : n;
			if (GRAD) {
				const float du = e.du;
				const float dnx = (VALUE ? 0.f : GX[0] + u * DG) + du * dA;
				const float y0v = VALUE ? Qy[0] : fx * Py[0] + Qy[0], dyv = VALUE ? DQy : fx * DPy + DQy;
				const float z0v = VALUE ? Qz[0] : fx * Pz[0] + Qz[0], dzv = VALUE ? DQz : fx * DPz + DQz;
				// -amp ds f with ds = -2 sign(n) (ridged) or 1
				const float k = ridged ? (n != 0.f ? mul_sign(k2, n) : 0.f) : -amp * f;
				acc_add_fma(acc, r * stride, -amp, s, k * dnx, k * (y0v + u * dyv), k * (z0v + u * dzv));
			} else {
				acc_add_fma(acc, r * stride, -amp, s, 0.f, 0.f, 0.f);
			}
		}
	}
}
template<bool GRAD, bool VALUE>
UP_HD void lattice_octave_run(const RunCtx &rc, int R, float f, float amp, bool ridged, uint32_t key, typename AccOf<GRAD>::T *acc, int stride) {
	if (ridged) lattice_octave_run_t<GRAD, VALUE, 1>(rc, R, f, amp, key, acc, stride);
	else lattice_octave_run_t<GRAD, VALUE, 0>(rc, R, f, amp, key, acc, stride);
}

// cellular noise (one octave) over samples [r0, r0 + CELL_SUB); DIST/OP fixed
// at compile time. Returns false (nothing accumulated) when the sub-run spans
// more than two x cells; the caller then evaluates those samples one by one.
// The x cells are the same for every lane. A candidate is ranked by its
// distance with the low 6 mantissa bits replaced by its id
// col * 16 + (dy + 1) * 4 + (dz + 1): the two smallest keys per sample are
// kept with integer min/max, and the winners' exact distances and difference
// vectors are rebuilt from the ids.
UP_HD uint32_t umin32(uint32_t a, uint32_t b) { return a < b ? a : b; }
template<bool B> struct BoolTag { static constexpr bool value = B; };
template<int I> struct IntTag { static constexpr int value = I; };
UP_HD uint32_t umax32(uint32_t a, uint32_t b) { return a > b ? a : b; }
template<int DIST>
UP_HD float cell_metric(float vx, float e2yz, float m1yz) {
	if (DIST == 0) return vx * vx + e2yz;
	if (DIST == 1) return fabsf(vx) + m1yz;
	return (vx * vx + e2yz) + (fabsf(vx) + m1yz);
}
// Candidate cells of a warp's cellular sub-run, shared: when the lanes' y and
// z cells span at most two values each, the union of their 3x3 neighbourhoods
// times the sub-run's columns fits a 4 x 4 x 4 table that the lanes hash
// together (two cells each) and every lane reads (broadcasts); otherwise each
// lane hashes its own candidates. Entry e = col * 16 + yy * 4 + zz holds the
// cell's feature point relative to the table's corner cell (col - 1 + jx,
// yy + jy, zz + jz; exact in FP32) and its hash, so a lane's candidate with id
// col * 16 + (dy + 1) * 4 + (dz + 1) sits at id + (ty - 1) * 4 + (tz - 1) and
// its offset is (jy - ty) - fy along y (lane mode: the lane's own 3 x 3 x 3
// block is the table, ty = 1).
struct CellEntry { float jx, jy, jz; uint32_t h; };
constexpr int CT = 4;
#ifdef __CUDACC__
__shared__ CellEntry g_runs_cells[RUNS_WARPS * CT * CT * CT];
#endif
UP_HD CellEntry cell_entry(uint32_t h, int e) {
	CellEntry c;
	c.jx = (float)((e >> 4) - 1) + jitter(h, 0);
	c.jy = (float)((e >> 2) & 3) + jitter(h, 10);
	c.jz = (float)(e & 3) + jitter(h, 20);
	c.h = h;
	return c;
}

// Warp-wide pruning of a sub-run's shared cell table (cellular_subrun). In
// table coordinates every sample of the warp lies in the box [x0, x1] x
// [y0, y1] x [z0, z1]: x spans the sub-run's sx (a sample's x difference to an
// entry is jx - sx), y and z the lanes' positions ty + fy and tz + fz.
struct CellBox { float x0, x1, y0, y1, z0, z1; };
// the smallest (lb) and the largest (ub) metric of entry c over the box
template<int DIST>
UP_HD void cell_box_bounds(const CellEntry &c, const CellBox &b, float &lb, float &ub) {
	const float ax = b.x0 - c.jx, bx = c.jx - b.x1;
	const float ay = b.y0 - c.jy, by = c.jy - b.y1;
	const float az = b.z0 - c.jz, bz = c.jz - b.z1;
	const float nx = fmaxf(fmaxf(ax, bx), 0.f), ny = fmaxf(fmaxf(ay, by), 0.f), nz = fmaxf(fmaxf(az, bz), 0.f);
	const float fx = fmaxf(-ax, -bx), fy = fmaxf(-ay, -by), fz = fmaxf(-az, -bz);
	lb = cell_metric<DIST>(nx, ny * ny + nz * nz, ny + nz);
	ub = cell_metric<DIST>(fx, fy * fy + fz * fz, fy + fz);
}
// entry e is seen by every sample: a column of both x cells (of the sub-run's
// ncol), y and z inside every lane's 3 x 3 window (the lanes' own table cells
// are 1 .. tymax along y and 1 .. tzmax along z)
UP_HD bool cell_entry_everywhere(int e, int ncol, int tymax, int tzmax) {
	const int c = e >> 4, yy = (e >> 2) & 3, zz = e & 3;
	return c >= (ncol == 4 ? 1 : 0) && c <= 2 && yy >= tymax - 1 && yy <= 2 && zz >= tzmax - 1 && zz <= 2;
}
// entry e lies inside some lane's window
UP_HD bool cell_entry_in_some_window(int e, int tymax, int tzmax) { return ((e >> 2) & 3) <= tymax + 1 && (e & 3) <= tzmax + 1; }
// The pruning bound from ub2, the second smallest ub of the entries seen
// everywhere: an entry whose lb exceeds it (by 0.1 % + 1e-4, far beyond FP32
// rounding and the keys' 2^-17 quantisation) is outranked by both of those
// entries at every sample, so it is never one of a sample's two keys.
UP_HD float cell_prune_bound(float ub2) { return ub2 * 1.001f + 1e-4f; }

// tab: the run's x table at frequency f (xtab_entry, shared by the warp)
template<bool GRAD, int DIST, int OP>
UP_HD bool cellular_subrun(const RunCtx &rc, const XTab *tab, int r0, float f, float amp, bool ridged, uint32_t key,
	typename AccOf<GRAD>::T *acc, int stride) {
	constexpr int S = CELL_SUB;
	const float qy = rc.py * f, qz = rc.pz * f;
	const float fy0 = floorf(qy), fz0 = floorf(qz);
	const int iy = (int)fy0, iz = (int)fz0;
	const float fy = qy - fy0, fz = qz - fz0;
	const int ixa = tab[r0].cx;
	const int ixb = tab[r0 + S - 1].cx;
	if (ixb - ixa > 1) return false;
	// sx[r] = (ix_r - ixa) + fx_r: then x difference to a candidate in column
	// cxi = ixa - 1 + col is ((col - 1) + jitter) - sx[r]
	float sx[S];
	int split = S; // samples [0, split) are in cell ixa, the rest in ixa + 1
	#pragma unroll
	for (int r = S - 1; r >= 0; r--) {
		const XTab e = tab[r0 + r];
		const bool second = e.cx != ixa;
		sx[r] = second ? 1.f + e.fx : e.fx;
		if (second) split = r;
	}
	uint32_t K1[S], K2[S];
	#pragma unroll
	for (int r = 0; r < S; r++) { K1[r] = 0xFFFFFFFFu; K2[r] = 0xFFFFFFFFu; }
	const int ncol = ixb - ixa + 3;
	int ty = 1, tz = 1; // table cell of this lane's own cell
	bool table = false;
	const CellEntry *ct = nullptr; // the warp's shared candidate table (device builds)
#ifdef __CUDA_ARCH__
	const int iymin = __reduce_min_sync(0xFFFFFFFFu, iy), iymax = __reduce_max_sync(0xFFFFFFFFu, iy);
	const int izmin = __reduce_min_sync(0xFFFFFFFFu, iz), izmax = __reduce_max_sync(0xFFFFFFFFu, iz);
	table = iymax - iymin <= 1 && izmax - izmin <= 1; // the same for every lane
	ct = g_runs_cells + (threadIdx.x >> 5) * (CT * CT * CT);
	if (table) {
		CellEntry *w = g_runs_cells + (threadIdx.x >> 5) * (CT * CT * CT);
		__syncwarp(); // the previous sub-run's readers are done
		for (int e = (int)(threadIdx.x & 31); e < ncol * CT * CT; e += 32)
			w[e] = cell_entry(mix32(((uint32_t)(ixa - 1 + (e >> 4)) * HX) ^ ((uint32_t)(iymin - 1 + ((e >> 2) & 3)) * HY) ^
				(((uint32_t)(izmin - 1 + (e & 3)) * HZ) ^ key)), e);
		__syncwarp();
		ty = iy - iymin + 1;
		tz = iz - izmin + 1;
	}
#endif
	const float tyf = (float)ty, tzf = (float)tz;
	// candidate (feature point ce, key id) against the sub-run's samples; with
	// MASKED, samples r outside [rlo, rhi) do not see it (pushed far away)
	auto visit = [&](auto masked_tag, uint32_t id, const CellEntry &ce, float T, int rlo, int rhi) {
		constexpr bool MASKED = decltype(masked_tag)::value;
		const float vy = (ce.jy - tyf) - fy;
		const float vz = (ce.jz - tzf) - fz;
		const float e2yz = vy * vy + vz * vz, m1yz = fabsf(vy) + fabsf(vz);
		#pragma unroll
		for (int r = 0; r < S; r++) {
			const float s = MASKED && (r < rlo || r >= rhi) ? -1e18f : sx[r];
			const uint32_t k = (f_bits(cell_metric<DIST>(T - s, e2yz, m1yz)) & ~63u) | id;
			K2[r] = umin32(K2[r], umax32(K1[r], k));
			K1[r] = umin32(K1[r], k);
		}
	};
	// the candidate search and the winners, compiled once for the shared
	// table (TABLE) and once for per-lane hashing, so that neither loop
	// branches per candidate
	auto search = [&](auto table_tag) {
		constexpr bool TABLE = decltype(table_tag)::value;
		// TABLE: the candidate of table index id (keys carry table indices:
		// the lane's own ids plus the per-lane constant (ty - 1) * 4 + (tz - 1),
		// so the order by key is that of the per-lane search); otherwise the
		// lane's candidate (column, dy + 1, dz + 1)
		auto cand = [&](int id) -> CellEntry {
			if (TABLE) return ct[id];
			return cell_entry(mix32(((uint32_t)(ixa - 1 + (id >> 4)) * HX) ^ ((uint32_t)(iy - 1 + ((id >> 2) & 3)) * HY) ^
				(((uint32_t)(iz - 1 + (id & 3)) * HZ) ^ key)), id);
		};
		if (!TABLE) {
			#pragma unroll 1
			for (int col = 0; col < ncol; col++) {
				// a column outside a sample's 3x3x3 neighbourhood: samples of the
				// other x cell only
				const int rlo = col == 3 ? split : 0, rhi = col == 0 ? split : S;
				#pragma unroll 1
				for (int dy = -1; dy <= 1; dy++) {
					#pragma unroll
					for (int dz = -1; dz <= 1; dz++) {
						const uint32_t id = (uint32_t)(col * 16 + (dy + 1) * 4 + (dz + 1));
						const CellEntry ce = cand((int)id);
						visit(BoolTag<true>(), id, ce, ce.jx, rlo, rhi);
					}
				}
			}
		}
#ifdef __CUDA_ARCH__
		if (TABLE) {
			// Warp-wide pruning (CellBox and the helpers above). Two entries
			// that every sample sees bound F2 by the second smallest of their
			// largest metrics over the warp's box; an entry whose smallest
			// metric over the box exceeds that bound (cell_prune_bound) is
			// never one of a sample's two keys and is skipped. The surviving
			// entries are the same for every lane (no divergence).
			const uint32_t FULL = 0xFFFFFFFFu;
			const int lane = (int)(threadIdx.x & 31);
			float sxmin = sx[0], sxmax = sx[0];
			#pragma unroll
			for (int r = 1; r < S; r++) { sxmin = fminf(sxmin, sx[r]); sxmax = fmaxf(sxmax, sx[r]); }
			// lane positions are positive (ty >= 1): their bits order as the floats
			const uint32_t ly = f_bits(tyf + fy), lz = f_bits(tzf + fz);
			const float ymin = bits_f(__reduce_min_sync(FULL, ly)), ymax = bits_f(__reduce_max_sync(FULL, ly));
			const float zmin = bits_f(__reduce_min_sync(FULL, lz)), zmax = bits_f(__reduce_max_sync(FULL, lz));
			const int tymax = iymax - iymin + 1, tzmax = izmax - izmin + 1;
			const int n = ncol * CT * CT;
			const CellBox box = {sxmin, sxmax, ymin, ymax, zmin, zmax};
			auto bounds = [&](int e, float &lb, float &ub) { cell_box_bounds<DIST>(ct[e], box, lb, ub); };
			auto everywhere = [&](int e) { return cell_entry_everywhere(e, ncol, tymax, tzmax); };
			float lb0, ub0, lb1 = 3e38f, ub1 = 3e38f;
			const bool has1 = lane + 32 < n; // n >= 48
			bounds(lane, lb0, ub0);
			if (has1) bounds(lane + 32, lb1, ub1);
			const float u0 = everywhere(lane) ? ub0 : 3e38f, u1 = has1 && everywhere(lane + 32) ? ub1 : 3e38f;
			const uint32_t a1 = f_bits(fminf(u0, u1)), a2 = f_bits(fmaxf(u0, u1));
			const uint32_t m1 = __reduce_min_sync(FULL, a1);
			const uint32_t first = __ffs(__ballot_sync(FULL, a1 == m1)) - 1;
			const float thr = cell_prune_bound(bits_f(__reduce_min_sync(FULL, lane == (int)first ? a2 : a1)));
			auto keep = [&](int e, float lb) { return lb <= thr && cell_entry_in_some_window(e, tymax, tzmax); };
			uint32_t s0 = __ballot_sync(FULL, keep(lane, lb0));
			uint32_t s1 = __ballot_sync(FULL, has1 && keep(lane + 32, lb1));
			// survivors of the 16 entries of column col (bits of m), all seen by
			// samples [rlo, rhi) only (MASKED) or by every sample
			auto visit_col = [&](auto masked_tag, uint32_t m, int col, int rlo, int rhi) {
				#pragma unroll 1
				while (m) {
					const int e = col * 16 + __ffs(m) - 1;
					m &= m - 1u;
					const CellEntry ce = ct[e];
					const int yy = (e >> 2) & 3, zz = e & 3;
					// outside this lane's 3 x 3 window: no sample of the lane sees it
					const float T = abs(yy - ty) <= 1 && abs(zz - tz) <= 1 ? ce.jx : 1e18f;
					visit(masked_tag, (uint32_t)e, ce, T, rlo, rhi);
				}
			};
			// column 0 serves the samples of cell ixa, column 3 those of ixa + 1
			if (split < S) visit_col(BoolTag<true>(), s0 & 0xFFFFu, 0, 0, split);
			else visit_col(BoolTag<false>(), s0 & 0xFFFFu, 0, 0, S);
			visit_col(BoolTag<false>(), (s0 >> 16) | ((s1 & 0xFFFFu) << 16), 1, 0, S); // columns 1 and 2
			visit_col(BoolTag<true>(), s1 >> 16, 3, split, S);
		}
#endif
		#pragma unroll 2
		for (int r = 0; r < S; r++) {
			float Fw[2];
			V3f vw[2], dFw[2] = {zero3(), zero3()};
			uint32_t h1 = 0;
			#pragma unroll
			for (int wsel = 0; wsel < 2; wsel++) {
#ifdef __CUDA_ARCH__
				if (!GRAD && OP != 0) {
					// value only (device): the winner's metric from its key, the
					// middle of the key's 2^-17 relative quantum; no rebuild
					const float d = bits_f(((wsel ? K2[r] : K1[r]) & ~63u) | 32u);
					Fw[wsel] = DIST == 0 ? sqrt_hd(d) : d;
					continue;
				}
#endif
				const int id = (int)((wsel ? K2[r] : K1[r]) & 63u);
				const CellEntry ce = cand(id);
				const float vy = (ce.jy - tyf) - fy;
				const float vz = (ce.jz - tzf) - fz;
				const float vx = ce.jx - sx[r];
				const float d = cell_metric<DIST>(vx, vy * vy + vz * vz, fabsf(vy) + fabsf(vz));
				Fw[wsel] = DIST == 0 ? sqrt_hd(d) : d;
				vw[wsel] = v3(vx, vy, vz);
				// d F / d p for v = q - p (dv/dp = -I); Euclidean: -v / |v|
				if (GRAD) dFw[wsel] = cell_dist_grad(vw[wsel], d, DIST);
				if (!wsel) h1 = ce.h;
			}
			const float a = Fw[0], b = Fw[1];
			const V3f dF1 = dFw[0], dF2 = dFw[1];
			float n;
			V3f dn;
			switch (OP) {
				case 0: n = hash_signed(mix32(h1)); dn = zero3(); break;
				case 1: n = a - 1.f; dn = dF1; break;
				case 2: n = b - 1.f; dn = dF2; break;
				case 3: n = (a + b) * 0.5f - 1.f; dn = (dF1 + dF2) * 0.5f; break;
				case 4: n = b - a - 1.f; dn = dF2 - dF1; break;
				case 5: n = a * b * 0.5f - 1.f; dn = (dF1 * b + dF2 * a) * 0.5f; break;
				default: n = a / b - 1.f; dn = (dF1 * b - dF2 * a) * (1.f / (b * b)); break;
			}
			// ridged: s = 1 - 2|n|, selected without a branch
			const float s = ridged ? 1.f - 2.f * fabsf(n) : n;
			const float k = ridged ? (n != 0.f ? mul_sign(2.f * amp * f, n) : 0.f) : -amp * f;
			acc_add(acc, (r0 + r) * stride, -amp * s, k * dn.x, k * dn.y, k * dn.z);
		}
	};
	if (table) search(BoolTag<true>());
	else search(BoolTag<false>());
	return true;
}

// a layer over a run: TYPE 0 value, 2 Perlin, cellular spec (see cell_spec)
template<bool GRAD, int TYPE>
UP_HD void layer_run(const up_noise_layer &L, const RunCtx &rc, int R, typename AccOf<GRAD>::T *acc, int stride) {
	const bool ridged = L.fractal == UP_FRACTAL_RIDGED;
	#pragma unroll 1
	for (int i = 0; i < L.octaves; i++) {
		const float f = L.freq[i], a = L.amp[i];
		const uint32_t key = seed_key(L.seed + (uint32_t)i);
		if (TYPE == 0) lattice_octave_run<GRAD, true>(rc, R, f, a, ridged, key, acc, stride);
		else if (TYPE == 2) lattice_octave_run<GRAD, false>(rc, R, f, a, ridged, key, acc, stride);
		else {
			constexpr int DIST = ((TYPE >> 4) & 15) - 1, OP = ((TYPE >> 8) & 15) - 1;
#ifdef __CUDA_ARCH__
			XTab *tab = g_runs_xtab + (threadIdx.x >> 5) * RUN_R;
			__syncwarp(); // every lane has finished reading the previous table
			if ((int)(threadIdx.x & 31) < R) tab[threadIdx.x & 31] = xtab_entry(rc, (int)(threadIdx.x & 31), f);
			__syncwarp();
#else
			XTab tab[RUN_R];
			for (int q = 0; q < R; q++) tab[q] = xtab_entry(rc, q, f);
#endif
			#pragma unroll 1
			for (int r0 = 0; r0 < R; r0 += CELL_SUB) {
				if (cellular_subrun<GRAD, DIST, OP>(rc, tab, r0, f, a, ridged, key, acc, stride)) continue;
				#pragma unroll 1
				for (int r = r0; r < r0 + CELL_SUB; r++) {
					const NG n = cellular_n<GRAD, DIST, OP>(v3(rc.px(r) * f, rc.py * f, rc.pz * f), key, DIST, OP);
					float s = n.v, ds = 1.f;
					if (ridged) { s = 1.f - 2.f * fabsf(n.v); ds = n.v > 0.f ? -2.f : (n.v < 0.f ? 2.f : 0.f); }
					const float k = -a * ds * f;
					acc_add(acc, r * stride, -a * s, k * n.g.x, k * n.g.y, k * n.g.z);
				}
			}
		}
	}
}

// Grid coordinate lo + i step, rounded as the grid kernels form it
UP_HD float runs_coord(float lo, float step, uint32_t i) {
#ifdef __CUDA_ARCH__
	return __fadd_rn(__fmul_rn((float)i, step), lo);
#else
	volatile float m = (float)i * step;
	return m + lo;
#endif
}
// Sample box of task t of the x-coherent grid kernels (below) on grid g
// (fields n, lo, step, k0 of GridDev; coordinates as the kernels form them):
// its centre c and half diagonal hd.
template<class G>
UP_HD void runs_task_box(const G &g, uint32_t t, V3f &c, float &hd) {
	const uint32_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const uint32_t nruns = (nx + RUN_R - 1) / RUN_R, tny = (ny + 7) / 8;
	const uint32_t run = t % nruns, tile = t / nruns;
	const uint32_t lo[3] = {run * RUN_R, (tile % tny) * 8, (tile / tny) * 4};
	const uint32_t ext[3] = {RUN_R - 1, 7, 3}, last[3] = {nx - 1, ny - 1, nz - 1};
	float cc[3], h2 = 0.f;
	for (int a = 0; a < 3; a++) {
		const uint32_t off = a == 2 ? g.k0 : 0u;
		const uint32_t hi = lo[a] + ext[a] < last[a] ? lo[a] + ext[a] : last[a];
		const float x0 = runs_coord(g.lo[a], g.step[a], lo[a] + off);
		const float x1 = runs_coord(g.lo[a], g.step[a], hi + off);
		const float h = 0.5f * fabsf(x1 - x0);
		cc[a] = 0.5f * (x0 + x1);
		h2 += h * h;
	}
	c = v3(cc[0], cc[1], cc[2]);
	hd = sqrtf(h2);
}

#ifdef __CUDACC__
// Task t of the x-coherent grid kernels (RUN_R samples along x of an 8 (y) x
// 4 (z) tile of rows; tasks numbered x-run fastest) of an nx x ny x nz grid:
// stores v at every sample, warp-wide (every lane calls it with the same t
// and v). The task's 32 rows of RUN_R samples go out as 128 16-byte pieces,
// 8 whole rows per store instruction (with a lane per row, each store
// instruction half-filled 32 sectors: 2.9x slower).
__device__ __forceinline__ void runs_task_fill(float *__restrict__ out, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t t, float v) {
	static_assert(RUN_R == 16, "four 16-byte pieces per row");
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t nruns = (nx + RUN_R - 1) / RUN_R, tny = (ny + 7) / 8;
	const uint32_t run = t % nruns, tile = t / nruns;
	const uint32_t i0 = run * RUN_R, j0 = (tile % tny) * 8, k0 = (tile / tny) * 4;
	#pragma unroll
	for (uint32_t q = 0; q < 4; q++) {
		const uint32_t piece = q * 32 + lane, rr = piece >> 2, x = i0 + (piece & 3) * 4;
		const uint32_t jr = j0 + (rr & 7), kr = k0 + (rr >> 3);
		if (jr >= ny || kr >= nz || x >= nx) continue;
		float *o = out + ((uint64_t)kr * ny + jr) * nx + x;
		if (x + 4 <= nx && ((uintptr_t)o & 15) == 0) {
			*(float4 *)o = make_float4(v, v, v, v);
		} else {
			#pragma unroll 1
			for (uint32_t r = 0; r < 4 && x + r < nx; r++) o[r] = v;
		}
	}
}
#endif

// The bits that a row segment's sign bits m (bit r: sample p0 + r; at most
// 16 bits) occupy in the bit-packed words (bit p of word p / 32: sample p):
// lo = m << (p0 % 32) in word w = p0 / 32, and hi = the bits past bit 31, in
// word w + 1 (0 when none).
struct RowSignParts { uint64_t w; uint32_t lo, hi; };
UP_HD RowSignParts row_sign_parts(uint64_t p0, uint32_t m) {
	const uint32_t sh = (uint32_t)(p0 & 31);
	RowSignParts r;
	r.w = p0 >> 5;
	r.lo = m << sh;
	r.hi = sh > 16 ? m >> (32 - sh) : 0u;
	return r;
}

#ifdef __CUDACC__
// Sign bits of one row segment (bit p of the words: sample p < 0): samples
// p0 .. p0 + 15 get the bits of m (bit r: sample p0 + r; bits past the row's
// end clear). With the x extent a multiple of 16 (aligned) the segment is
// an aligned half-word of its own, stored; otherwise its bits may share a
// word with another task's and are OR-ed into words zeroed beforehand.
__device__ __forceinline__ void runs_row_signs(uint32_t *__restrict__ signs, uint64_t p0, uint32_t m, bool aligned) {
	if (aligned) {
		((uint16_t *)signs)[p0 >> 4] = (uint16_t)m;
		return;
	}
	if (!m) return;
	const RowSignParts q = row_sign_parts(p0, m);
	atomicOr(signs + q.w, q.lo);
	if (q.hi) atomicOr(signs + q.w + 1, q.hi);
}
// Sign bits of task t of an nx x ny x nz grid all of whose samples have the
// sign neg; warp-wide, lane = row (runs_row_signs).
__device__ __forceinline__ void runs_task_signs(uint32_t *__restrict__ signs, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t t, bool neg) {
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t nruns = (nx + RUN_R - 1) / RUN_R, tny = (ny + 7) / 8;
	const uint32_t run = t % nruns, tile = t / nruns;
	const uint32_t jr = (tile % tny) * 8 + (lane & 7), kr = (tile / tny) * 4 + (lane >> 3);
	const uint32_t i0 = run * RUN_R, len = nx - i0 < RUN_R ? nx - i0 : RUN_R;
	if (jr < ny && kr < nz)
		runs_row_signs(signs, ((uint64_t)kr * ny + jr) * nx + i0, neg ? (1u << len) - 1u : 0u, nx % RUN_R == 0);
}
#endif

// one run: base shape plus layers into acc (R must be a multiple of CELL_SUB).
// band > 0 (narrow band of contouring, values only): when every sample of the
// warp's task has |base| > band, the layers are skipped and acc holds the
// base (such samples have the sign of the base and are not ends of
// sign-change edges: contouring reads only their signs). A lane whose whole
// run lies that far (|base| at the run's midpoint above band + half the run:
// the base shapes are 1-Lipschitz) stores the midpoint's value for all its
// samples, which has their sign, without evaluating the base per sample.
template<bool GRAD, int T0, int T1>
UP_HD void synth_run(const up_synth_program &P, const RunCtx &rc, int R, typename AccOf<GRAD>::T *acc, int stride, float band = 0.f) {
	bool far = !GRAD && band > 0.f; // the narrow band is a value-only mode
	const float x0 = rc.px(0), x1 = rc.px(R - 1);
	const uint32_t spheres = synth_segment_spheres(P, x0, x1, rc.py, rc.pz);
	bool filled = false;
	if (!GRAD && band > 0.f) {
		const float xm = 0.5f * (x0 + x1), half = 0.5f * (x1 - x0);
		const float bm = synth_base<false>(P, v3(xm, rc.py, rc.pz), spheres).v;
		if (fabsf(bm) > (band + half) * 1.001f + 1e-5f) {
			#pragma unroll 1
			for (int r = 0; r < R; r++) acc_set(acc, r * stride, bm, 0.f, 0.f, 0.f);
			filled = true;
		}
	}
	// the base at every sample, the shape's switch taken once per run
	auto base_loop = [&](auto base_tag) {
		constexpr int B = decltype(base_tag)::value;
		#pragma unroll 1
		for (int r = 0; r < R && !filled; r++) {
			const NG b = synth_base<GRAD, B>(P, v3(rc.px(r), rc.py, rc.pz), spheres);
			acc_set(acc, r * stride, b.v, b.g.x, b.g.y, b.g.z);
			far = far && fabsf(b.v) > band;
		}
	};
	switch (P.base) {
		case UP_BASE_SPHERE: base_loop(IntTag<UP_BASE_SPHERE>()); break;
		case UP_BASE_TORUS: base_loop(IntTag<UP_BASE_TORUS>()); break;
		case UP_BASE_ROUNDED_BOX: base_loop(IntTag<UP_BASE_ROUNDED_BOX>()); break;
		default: base_loop(IntTag<UP_BASE_TORUS_SPHERES>()); break;
	}
#ifdef __CUDA_ARCH__
	if (!GRAD) far = __all_sync(0xFFFFFFFFu, far); // every lane of the warp runs every task
#endif
	if (far) return;
	if (P.n_layers > 0) layer_run<GRAD, T0>(P.layer[0], rc, R, acc, stride);
	if (P.n_layers > 1) layer_run<GRAD, T1>(P.layer[1], rc, R, acc, stride);
}

} // namespace up
