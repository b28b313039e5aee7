// Test harness: compiles the CUDA path's device arithmetic headers as plain
// host C++ so the CPU test suite can compare them with the oracle without a
// GPU. It exercises arithmetic only; the kernels themselves run in the GPU
// tests. Built by tests/hostcheck/build_hostcheck.py into tests/hostcheck/_build.
#include "../../unnatural-planets_gb300/csrc/up_synth.cuh"

using namespace up;

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
uint32_t hc_corner_hash(int x, int y, int z, uint32_t key, int b) {
	Cell c; c.ix = x; c.iy = y; c.iz = z; c.fx = c.fy = c.fz = 0.f;
	return corner_hashes(c, key).h[b];
}
}
