// x-coherent evaluation of the reference elevation modes over grid runs.
//
// The lattice-noise instances that an elevation mode evaluates at the sample
// position itself (value and Perlin FBM: lakes and islands land, mountain
// mask and terraces; legacy scale) are filled for a run of RUN_R samples
// along x with the segment form of up_grid_runs.cuh (corner hashes once per
// lattice cell and run instead of once per sample). The rest of the mode
// (simplex ridges, noise at moved positions, the composition of
// sources/elevationModes.cpp) runs per sample and reads those instances from
// the table through NoiseRun. Table entry (q, r) sits at
// tab[(q * RUN_R + r) * stride].
#pragma once
#include "up_grid_runs.cuh"
#include "up_modes.cuh"

namespace up {

// elevation noise instance held in table slot q (0-2) under mode EM, or -1
template<int EM> UP_HD int mrun_instance(int q) {
	if (EM == 2) return q == 0 ? NS_LEGACY_SCALE : -1;
	if (EM == 3 || EM == 4) return q == 0 ? (EM == 3 ? NS_LAKES_LAND : NS_ISLANDS_LAND) : (q == 1 ? NS_MTN_MASK : NS_MTN_TERRACE);
	return -1;
}

// true when mode em has table instances and every one is value or Perlin noise
UP_HD bool mrun_applies(const ModesDesc &M) {
	const int em = M.elevation;
	if (em != 2 && em != 3 && em != 4) return false;
	for (int q = 0; q < 3; q++) {
		const int ns = em == 2 ? mrun_instance<2>(q) : (em == 3 ? mrun_instance<3>(q) : mrun_instance<4>(q));
		if (ns < 0) break;
		const int t = M.elev[ns].type;
		if (t != UP_NOISE_VALUE && t != UP_NOISE_PERLIN) return false;
	}
	return true;
}

// noise source of elevation_nz for sample r of a filled run table
template<int EM> struct NoiseRun {
	const float *tab;
	int r, stride;
	UP_HD float operator()(const ModesDesc &M, int ns, V3S<float> pos) const {
		#pragma unroll
		for (int q = 0; q < 3; q++)
			if (mrun_instance<EM>(q) == ns) return tab[(q * RUN_R + r) * stride];
		return noise_dev(M.elev[ns], pos);
	}
};

// fills slots 0-2 over samples [0, R) of the run: slot q = noise_dev of
// instance mrun_instance(q) (octaves summed in order from 0, as noise_dev)
template<int EM> UP_HD void modes_run_fill(const ModesDesc &M, const RunCtx &rc, int R, float *tab, int stride) {
	#pragma unroll 1
	for (int q = 0; q < 3; q++) {
		const int ns = mrun_instance<EM>(q);
		if (ns < 0) break;
		const NoiseDev &n = M.elev[ns];
		float *slot = tab + q * RUN_R * stride;
		#pragma unroll 1
		for (int r = 0; r < R; r++) slot[r * stride] = 0.f;
		// lattice_octave_run subtracts amp * s(n): -amp adds it
		#pragma unroll 1
		for (int i = 0; i < n.octaves; i++) {
			const uint32_t key = seed_key(n.seed + (uint32_t)i);
			const bool ridged = n.fractal == UP_FRACTAL_RIDGED;
			// the ridged flag at run time: one instantiation per noise type keeps
			// this kernel's code small
			if (n.type == UP_NOISE_VALUE) lattice_octave_run_t<false, true, -1>(rc, R, n.freq[i], -n.amp[i], key, slot, stride, ridged);
			else lattice_octave_run_t<false, false, -1>(rc, R, n.freq[i], -n.amp[i], key, slot, stride, ridged);
		}
	}
}

// shape values of the run's samples into sh[r * stride]; returns true when
// every sample lies outside the band (band > 0). The band is given only for
// 1-Lipschitz shapes (modes_contour_band): a run whose midpoint lies further
// than band + half the run is outside it everywhere, and its samples take the
// midpoint's value (their sign; contouring reads nothing else of them).
UP_HD bool modes_run_shape(const ModesDesc &M, const RunCtx &rc, int R, float band, float *sh, int stride) {
	if (band > 0.f) {
		const float x0 = rc.px(0), x1 = rc.px(R - 1);
		const float xm = 0.5f * (x0 + x1), half = 0.5f * (x1 - x0);
		const float sm = shape_eval(M, vs(xm, rc.py, rc.pz));
		if (fabsf(sm) > (band + half) * 1.001f + 1e-3f * (1.f + fabsf(sm))) {
			#pragma unroll 1
			for (int r = 0; r < R; r++) sh[r * stride] = sm;
			return true;
		}
	}
	bool far = band > 0.f;
	#pragma unroll 1
	for (int r = 0; r < R; r++) {
		const float v = shape_eval(M, vs(rc.px(r), rc.py, rc.pz));
		sh[r * stride] = v;
		far = far && fabsf(v) > band;
	}
	return far;
}

// land, water, navigation of sample r with shape value sh (fields_of of the
// per-sample kernel); band > 0 and |sh| > band: every field is sh (narrow
// band of contouring); need_e false: no field needs the elevation
template<int EM> UP_HD void modes_run_fields(const ModesDesc &M, const RunCtx &rc, int r, float sh, bool need_e, float band,
	const float *tab, int stride, float v[3]) {
	v[0] = v[1] = v[2] = sh;
	if (!need_e || (band > 0.f && fabsf(sh) > band)) return;
	const NoiseRun<EM> nz{tab, r, stride};
	const float e = elevation_nz<float, NoiseRun<EM>, EM>(M, vs(rc.px(r), rc.py, rc.pz), nz) * 0.1f;
	v[0] = sh - e;
	v[2] = sh - s_max(e, 0.f);
}

} // namespace up
