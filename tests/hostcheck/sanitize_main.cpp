// Test harness: a sanitizer run of the host-compilable code. The oracle
// (oracle/oracle_capi.cpp), the device arithmetic headers compiled for the
// host (tests/hostcheck/device_math_host.cpp) and the mode tables
// (csrc/up_modes_host.cpp) are linked into one executable built with
// -fsanitize=address,undefined -fno-sanitize-recover=all, and every entry
// point is driven here on small inputs: any out-of-bounds access, leak, use
// after free or undefined behaviour ends the run with a report and a non-zero
// status. Replaces a device sanitizer, which is not available for the GPU
// kernels; the kernels' index arithmetic is the same source as the
// host-compiled helpers exercised here. Built and run by
// tests/test_sanitize_host.py.
#include "../../include/up_abi.h"

#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

extern "C" {
void orc_noise(int type, int fractal, int octaves, int dist, int op, double frequency, double lacunarity, double gain, uint32_t seed,
	const float *xyz, uint64_t n, int precision, double *out, double *grad);
uint64_t orc_synth_theta_count(const up_synth_program *p);
void orc_synth_theta(const up_synth_program *p, double *out);
void orc_synth_points(const up_synth_program *prog, const double *theta, const float *xyz, uint64_t n, int precision, double *out,
	double *grad, int threads);
int orc_synth_theta_grad(const up_synth_program *prog, const double *theta, const float *xyz, uint64_t n, const double *w,
	double *dtheta, int threads);
void orc_synth_count_ops(const up_synth_program *prog, const float *xyz, uint64_t n, double *counts5);
void orc_synth_grid_fp32(const up_synth_program *prog, const up_grid *grid, uint32_t z0, uint32_t z1, float *out, int threads);
void orc_synth_grid_fp32_cd(const up_synth_program *prog, const up_grid *grid, uint32_t z0, uint32_t z1, float h, float *out,
	float *grad, int threads);
void orc_grid_positions(const up_grid *grid, float *out);
void orc_grid_positions_at(const up_grid *grid, const uint64_t *idx, uint64_t n, float *out);
void *orc_contour_synth(const up_synth_program *prog, const up_grid *grid, const float *values);
void orc_mesh_counts(void *h, uint64_t *c4);
void orc_mesh_copy(void *h, uint64_t *cells, float *positions, float *normals, uint32_t *indices, uint64_t *edges);
void orc_mesh_free(void *h);
void *orc_planet_create(const char *shape, const char *elevation, const char *coloring, int poles, int flowers, uint32_t seed, char *err,
	int errn);
void orc_planet_free(void *p);
void orc_field_points(void *h, int field, const float *xyz, uint64_t n, int precision, double *out, double *grad, int threads);
void *orc_contour_planet(void *h, int field, const up_grid *grid, const float *values);
void orc_tiles(void *h, int purpose, const float *pos, const float *nrm, uint64_t n, double *out11, int32_t *biome_type, int threads);
void orc_texture(void *planet, const up_synth_program *prog, int purpose, const float *pos, const float *nrm, const float *uv,
	const uint32_t *idx, uint64_t nidx, uint32_t W, uint32_t H, int dilation, float *albedo_f, float *special_f, float *height_f,
	uint8_t *albedo8, uint8_t *special8, uint8_t *height8, int32_t *owner, int threads);
void orc_mesh_filter(uint32_t V, uint32_t T, const uint32_t *idx, const uint8_t *valid, uint8_t *keep_v, uint8_t *keep_t);

void hc_noise(int type, int dist, int op, uint32_t key, const float *xyz, uint64_t n, float *out, float *grad);
void hc_synth(const up_synth_program *P, const float *xyz, uint64_t n, float *out, float *grad);
int hc_synth_bwd(const up_synth_program *P, const float *xyz, uint64_t n, const float *w, double *dtheta);
void *hc_modes_create(const char *shape, const char *elevation, const char *coloring, int poles, int flowers, uint32_t seed);
void hc_modes_free(void *d);
void hc_modes_field(void *d, int field, const float *xyz, uint64_t n, float *out, float *grad);
void hc_tiles(void *d, int purpose, const float *pos, const float *nrm, uint64_t n, float *out11, int32_t *bt);
void hc_synth_texel(const up_synth_program *P, const float *pos, uint64_t n, float *out5);
void hc_grid_runs_band(const up_synth_program *P, const float *lo, const float *step, const uint32_t *n, float band, float *out);
void hc_grid_runs(const up_synth_program *P, const float *lo, const float *step, const uint32_t *n, float *out, float *grad);
int hc_modes_grid_runs(void *d, const float *lo, const float *step, const uint32_t *n, float band, float *o0, float *o1, float *o2);
float hc_task_band(const up_synth_program *P, const float *lo, const float *step, const uint32_t *n, float *task_val);
void hc_modes_task_band(void *d, const float *lo, const float *step, const uint32_t *n, float band, float *task_val);
void hc_row_signs(const uint64_t *p0, const uint32_t *m, uint64_t count, uint32_t *words);
void hc_fastdiv(uint32_t d, const uint32_t *n, uint64_t count, uint32_t *q);
}

static const char *SHAPES[] = {"asteroid", "belt", "bowl", "box", "bunny", "capsule", "cube", "disk", "doubletorus", "fibers", "gear",
	"h2o", "h3o", "h4o", "hemispheres", "hexagon", "hexagonalprism", "insidecube", "knot", "mandelbulb", "mobiusstrip", "monkeyhead",
	"octahedron", "pipe", "sphere", "square", "tetrahedron", "torus", "toruscross", "triangularprism", "tube", "twistedhexagonalprism",
	"twistedplane", "wormhole"};
static const char *ELEVATIONS[] = {"none", "simple", "legacy", "lakes", "islands", "craters"};
static const char *COLORINGS[] = {"default", "barren", "debug"};

static void layer(up_noise_layer &L, int type, int fractal, int octaves, float freq, float amp, uint32_t seed, int dist = 0, int op = 1) {
	L.type = type; L.fractal = fractal; L.octaves = octaves; L.distance = dist; L.operation = op; L.seed = seed;
	for (int i = 0; i < 8; i++) {
		L.amp[i] = i < octaves ? amp / (float)(1 << i) : 0.f;
		L.freq[i] = i < octaves ? freq * (float)(1 << i) : 0.f;
	}
}

static up_synth_program program(int which) {
	up_synth_program P = {};
	if (which == 0) {
		P.base = UP_BASE_SPHERE; P.param[0] = 1.f; P.n_layers = 1;
		layer(P.layer[0], UP_NOISE_SIMPLEX, UP_FRACTAL_FBM, 4, 2.f, 0.05f, 1337);
	} else {
		P.base = UP_BASE_TORUS_SPHERES; P.param[0] = 1.f; P.param[1] = 0.4f; P.n_spheres = 8; P.k = 0.1f; P.n_layers = 2;
		std::mt19937 r(42);
		std::uniform_real_distribution<float> U(-1.f, 1.f), Rr(0.1f, 0.3f);
		for (int s = 0; s < 8; s++) { P.sphere[s][0] = U(r); P.sphere[s][1] = U(r); P.sphere[s][2] = U(r); P.sphere[s][3] = Rr(r); }
		layer(P.layer[0], UP_NOISE_PERLIN, UP_FRACTAL_RIDGED, 6, 3.f, 0.04f, 42);
		layer(P.layer[1], UP_NOISE_CELLULAR, UP_FRACTAL_NONE, 1, 8.f, 0.02f, 50, UP_DIST_EUCLIDEAN, UP_OP_SUBTRACT);
	}
	return P;
}

int main() {
	std::mt19937 rng(7);
	auto pts = [&](int n, float lo, float hi) {
		std::uniform_real_distribution<float> U(lo, hi);
		std::vector<float> v(3 * (size_t)n);
		for (auto &x : v) x = U(rng);
		return v;
	};
	const int N = 96;
	std::vector<double> o(N), g(3 * N);
	std::vector<float> of(N), gf(3 * N);
	int calls = 0;

	// noise family: every type, fractal, metric and cellular operation
	auto xn = pts(N, -20.f, 20.f);
	for (int t = 0; t < 6; t++)
		for (int fr = 0; fr < 3; fr++)
			for (int d = 0; d < (t == 5 ? 3 : 1); d++)
				for (int op = 0; op < (t == 5 ? 7 : 1); op++)
					for (int prec = 0; prec < 2; prec++) {
						orc_noise(t, fr, 3, d, op, 0.7, 2.0, 0.5, 11, xn.data(), N, prec, o.data(), prec ? nullptr : g.data());
						hc_noise(t, d, op, 0x9E3779B9u, xn.data(), N, of.data(), gf.data());
						calls += 2;
					}

	// synthetic programs: values, gradients, adjoints, grids, contouring, texels
	for (int which = 0; which < 2; which++) {
		const up_synth_program P = program(which);
		auto x = pts(N, -1.6f, 1.6f);
		const uint64_t nt = orc_synth_theta_count(&P);
		std::vector<double> th(nt), dth(nt, 0.0), w(N, 1.0 / N), cnt(5);
		std::vector<float> wf(N, 1.f / N);
		orc_synth_theta(&P, th.data());
		for (int prec = 0; prec < 2; prec++) orc_synth_points(&P, th.data(), x.data(), N, prec, o.data(), g.data(), 2);
		orc_synth_theta_grad(&P, th.data(), x.data(), N, w.data(), dth.data(), 2);
		orc_synth_count_ops(&P, x.data(), N, cnt.data());
		hc_synth(&P, x.data(), N, of.data(), gf.data());
		hc_synth_bwd(&P, x.data(), N, wf.data(), dth.data());
		std::vector<float> tex(5 * N);
		hc_synth_texel(&P, x.data(), N, tex.data());
		const up_grid G = {{-1.6f, -1.6f, -1.6f}, {1.6f, 1.6f, 1.6f}, {23, 19, 17}};
		const size_t np = 23 * 19 * 17;
		std::vector<float> val(np), cd(np), cdg(3 * np), posg(3 * np);
		orc_synth_grid_fp32(&P, &G, 0, 17, val.data(), 2);
		orc_synth_grid_fp32_cd(&P, &G, 3, 9, 1e-3f, cd.data(), cdg.data(), 2);
		orc_grid_positions(&G, posg.data());
		const uint64_t some[4] = {0, 5, np / 2, np - 1};
		std::vector<float> pa(12);
		orc_grid_positions_at(&G, some, 4, pa.data());
		void *m = orc_contour_synth(&P, &G, val.data());
		uint64_t c4[4];
		orc_mesh_counts(m, c4);
		std::vector<uint64_t> cells(c4[0]), edges(c4[2]);
		std::vector<float> mp(3 * c4[0]), mn(3 * c4[0]);
		std::vector<uint32_t> mi(c4[1]);
		orc_mesh_copy(m, cells.data(), mp.data(), mn.data(), mi.data(), edges.data());
		orc_mesh_free(m);
		// mesh hygiene, water-style validity on every other vertex
		const uint32_t V = (uint32_t)c4[0], T = (uint32_t)(c4[1] / 3);
		std::vector<uint8_t> valid(V), kv(V), kt(T);
		for (uint32_t v = 0; v < V; v++) valid[v] = (uint8_t)(v & 1);
		orc_mesh_filter(V, T, mi.data(), nullptr, kv.data(), kt.data());
		orc_mesh_filter(V, T, mi.data(), valid.data(), kv.data(), kt.data());
		// texels of the first 64 triangles in a 40 x 24 atlas
		const uint32_t nidx = T < 64 ? 3 * T : 192;
		std::vector<float> uv(2 * (size_t)V);
		for (uint32_t v = 0; v < V; v++) { uv[2 * v] = (float)((v * 37) % 101) / 101.f; uv[2 * v + 1] = (float)((v * 53) % 97) / 97.f; }
		const uint32_t TW = 40, TH = 24;
		std::vector<float> af(TW * TH * 3), sf(TW * TH * 2), hf(TW * TH);
		std::vector<uint8_t> a8(TW * TH * 3), s8(TW * TH * 2), h8(TW * TH);
		std::vector<int32_t> own(TW * TH);
		orc_texture(nullptr, &P, 1, mp.data(), mn.data(), uv.data(), mi.data(), nidx, TW, TH, 7, af.data(), sf.data(), hf.data(), a8.data(),
			s8.data(), h8.data(), own.data(), 2);
		// the x-coherent run helpers on a ragged grid
		const float lo[3] = {-1.6f, -1.5f, -1.4f}, step[3] = {0.11f, 0.13f, 0.12f};
		const uint32_t n3[3] = {37, 9, 11};
		std::vector<float> r(37 * 9 * 11), rg(3 * 37 * 9 * 11), tv(4096);
		hc_grid_runs(&P, lo, step, n3, r.data(), rg.data());
		hc_grid_runs_band(&P, lo, step, n3, 0.3f, r.data());
		hc_task_band(&P, lo, step, n3, tv.data());
		calls += 20;
	}

	// reference modes: every shape and elevation, every field, tiles; contouring
	auto xm = pts(N, -2000.f, 2000.f);
	std::vector<float> nrm(3 * N);
	for (int i = 0; i < N; i++) {
		const float l = std::sqrt(xm[3 * i] * xm[3 * i] + xm[3 * i + 1] * xm[3 * i + 1] + xm[3 * i + 2] * xm[3 * i + 2]);
		for (int a = 0; a < 3; a++) nrm[3 * i + a] = xm[3 * i + a] / l;
	}
	char err[128];
	for (const char *s : SHAPES)
		for (const char *e : ELEVATIONS) {
			void *pl = orc_planet_create(s, e, "default", 1, 1, 3, err, sizeof(err));
			void *hd = hc_modes_create(s, e, "default", 1, 1, 3);
			if (!pl || !hd) { std::fprintf(stderr, "planet %s/%s: %s\n", s, e, err); return 2; }
			for (int f = 0; f < 5; f++) {
				orc_field_points(pl, f, xm.data(), N, 0, o.data(), g.data(), 1);
				hc_modes_field(hd, f, xm.data(), N, of.data(), gf.data());
			}
			orc_planet_free(pl);
			hc_modes_free(hd);
			calls += 12;
		}
	for (const char *c : COLORINGS) {
		void *pl = orc_planet_create("sphere", "lakes", c, 1, 1, 5, err, sizeof(err));
		void *hd = hc_modes_create("sphere", "lakes", c, 1, 1, 5);
		std::vector<double> t11(11 * N);
		std::vector<int32_t> bt(2 * N);
		std::vector<float> t11f(11 * N);
		for (int pu = 1; pu <= 3; pu++) {
			orc_tiles(pl, pu, xm.data(), nrm.data(), N, t11.data(), bt.data(), 2);
			hc_tiles(hd, pu, xm.data(), nrm.data(), N, t11f.data(), bt.data());
		}
		const up_grid G = {{-2000.f, -2000.f, -2000.f}, {2000.f, 2000.f, 2000.f}, {14, 13, 12}};
		std::vector<float> val(14 * 13 * 12);
		std::vector<double> vd(14 * 13 * 12);
		std::vector<float> gp(3 * 14 * 13 * 12);
		orc_grid_positions(&G, gp.data());
		orc_field_points(pl, 0, gp.data(), val.size(), 1, vd.data(), nullptr, 2);
		for (size_t i = 0; i < val.size(); i++) val[i] = (float)vd[i];
		void *m = orc_contour_planet(pl, 0, &G, val.data());
		orc_mesh_free(m);
		const float lo[3] = {-2000.f, -1900.f, -1800.f}, step[3] = {90.f, 130.f, 140.f};
		const uint32_t n3[3] = {45, 30, 27};
		std::vector<float> o0(45 * 30 * 27), o1(o0.size()), o2(o0.size()), tv(8192);
		hc_modes_grid_runs(hd, lo, step, n3, 0.f, o0.data(), o1.data(), o2.data());
		hc_modes_task_band(hd, lo, step, n3, 50.f, tv.data());
		orc_planet_free(pl);
		hc_modes_free(hd);
		calls += 10;
	}

	// word helpers
	std::vector<uint64_t> p0 = {0, 17, 40, 95};
	std::vector<uint32_t> msk = {0xFFFFu, 0x1234u, 0x8001u, 0x7u}, words(8, 0), q(1000), nn(1000);
	hc_row_signs(p0.data(), msk.data(), p0.size(), words.data());
	for (uint32_t i = 0; i < 1000; i++) nn[i] = i * 4099u;
	hc_fastdiv(191, nn.data(), 1000, q.data());
	std::printf("sanitized run: %d entry-point calls\n", calls);
	return 0;
}
