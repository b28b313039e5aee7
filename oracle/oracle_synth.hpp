// Oracle: synthetic unit-scale planets (the benchmark programs) and their
// parameter vector theta. TEST INFRASTRUCTURE, parity unpinned (see
// oracle_core.hpp). Layout and semantics follow up_synth_program in
// include/up_abi.h; the smooth union is the reference's smoothMin
// (sources/math.cpp:28-33) and the "shape minus elevation" composition follows
// terrainSdfLand (sources/modesConfiguration.cpp:248-258) at unit scale.
#pragma once
#include "oracle_core.hpp"
#include "../include/up_abi.h"
#include <vector>

namespace orc {

inline int synth_theta_count(const up_synth_program &p) {
	int n = 0;
	for (int l = 0; l < p.n_layers; l++) n += 2 * p.layer[l].octaves;
	switch (p.base) {
		case UP_BASE_SPHERE: n += 1; break;
		case UP_BASE_TORUS: case UP_BASE_ROUNDED_BOX: n += 2; break;
		default: n += 2 + p.n_spheres + 1; break;
	}
	return n;
}

inline std::vector<double> synth_theta(const up_synth_program &p) {
	std::vector<double> t;
	for (int l = 0; l < p.n_layers; l++) {
		for (int i = 0; i < p.layer[l].octaves; i++) t.push_back(p.layer[l].amp[i]);
		for (int i = 0; i < p.layer[l].octaves; i++) t.push_back(p.layer[l].freq[i]);
	}
	switch (p.base) {
		case UP_BASE_SPHERE: t.push_back(p.param[0]); break;
		case UP_BASE_TORUS: case UP_BASE_ROUNDED_BOX: t.push_back(p.param[0]); t.push_back(p.param[1]); break;
		default:
			t.push_back(p.param[0]); t.push_back(p.param[1]);
			for (int s = 0; s < p.n_spheres; s++) t.push_back(p.sphere[s][3]);
			t.push_back(p.k);
	}
	return t;
}

// d(p; theta) for one synthetic program. theta has synth_theta_count entries.
template<class T>
T synth_eval(const up_synth_program &prog, const T *theta, const V3<T> &p) {
	int ti = 0;
	T elev = T(0.0);
	for (int l = 0; l < prog.n_layers; l++) {
		const up_noise_layer &L = prog.layer[l];
		const T *amp = theta + ti;
		const T *freq = theta + ti + L.octaves;
		ti += 2 * L.octaves;
		for (int i = 0; i < L.octaves; i++) {
			const V3<T> q(p.x * freq[i], p.y * freq[i], p.z * freq[i]);
			T n = noise_single(L.type, q, seed_key(L.seed + (uint32_t)i), L.distance, L.operation);
			if (L.fractal == UP_FRACTAL_RIDGED) n = 1.0 - 2.0 * abs(n);
			elev += amp[i] * n;
		}
	}
	T base;
	switch (prog.base) {
		case UP_BASE_SPHERE: base = length(p) - theta[ti]; break;
		case UP_BASE_TORUS: base = len2(len2(p.x, p.y) - theta[ti], p.z) - theta[ti + 1]; break;
		case UP_BASE_ROUNDED_BOX: {
			const T h = theta[ti], rr = theta[ti + 1];
			const V3<T> q = vabs(p) - V3<T>(h, h, h);
			base = length(vmax(q, 0.0)) + tmin(tmax(q.x, tmax(q.y, q.z)), T(0.0)) - rr;
			break;
		}
		default: {
			const T R = theta[ti], r = theta[ti + 1];
			const T k = theta[ti + 2 + prog.n_spheres];
			base = len2(len2(p.x, p.y) - R, p.z) - r;
			for (int s = 0; s < prog.n_spheres; s++) {
				const V3<T> c(T((double)prog.sphere[s][0]), T((double)prog.sphere[s][1]), T((double)prog.sphere[s][2]));
				const T sd = length(p - c) - theta[ti + 2 + s];
				base = smoothMin(base, sd, k);
			}
		}
	}
	return base - elev;
}

} // namespace orc
