// C entry points of the oracle for the test suite (ctypes) and the CPU
// baseline of the benchmark. TEST INFRASTRUCTURE, parity unpinned (see
// oracle_core.hpp). Nothing in the product links this file.
#include "oracle_core.hpp"
#include "oracle_synth.hpp"
#include "oracle_contour.hpp"
#include "oracle_modes.hpp"
#include "oracle_coloring.hpp"

#include <atomic>
#include <cstdio>
#include <memory>
#include <thread>
#include <vector>

using namespace orc;

namespace {

template<class F>
void parallel_for(uint64_t n, int threads, F &&f) {
	if (threads <= 1 || n < 2) { for (uint64_t i = 0; i < n; i++) f(i); return; }
	std::atomic<uint64_t> next{0};
	std::vector<std::thread> ts;
	for (int t = 0; t < threads; t++)
		ts.emplace_back([&]() {
			for (;;) {
				const uint64_t i = next.fetch_add(1);
				if (i >= n) break;
				f(i);
			}
		});
	for (auto &t : ts) t.join();
}

template<class T>
std::vector<T> theta_as(const up_synth_program &p, const double *theta) {
	std::vector<double> t0 = synth_theta(p);
	std::vector<T> t(t0.size());
	for (size_t i = 0; i < t0.size(); i++) t[i] = T(theta ? theta[i] : t0[i]);
	return t;
}

} // namespace

extern "C" {

int orc_abi_version() { return 1; }

uint32_t orc_mix32(uint32_t x) { return mix32(x); }
uint32_t orc_lattice_hash(int32_t x, int32_t y, int32_t z, uint32_t key) { return lattice_hash(x, y, z, key); }
uint32_t orc_seed_key(uint32_t seed) { return seed_key(seed); }

// one noise function (NoiseCfg) at n points; precision 0 = FP64, 1 = FP32;
// grad (3 per point, FP64 dual numbers) when not null
void orc_noise(int type, int fractal, int octaves, int dist, int op, double frequency, double lacunarity, double gain,
	uint32_t seed, const float *xyz, uint64_t n, int precision, double *out, double *grad) {
	NoiseCfg c;
	c.type = type; c.fractal = fractal; c.octaves = octaves; c.dist = dist; c.op = op;
	c.frequency = frequency; c.lacunarity = lacunarity; c.gain = gain; c.seed = seed;
	const NoiseFn fn = make_noise(c);
	for (uint64_t i = 0; i < n; i++) {
		const float *q = xyz + 3 * i;
		if (grad) {
			V3<Dual<3>> p(Dual<3>::var(q[0], 0), Dual<3>::var(q[1], 1), Dual<3>::var(q[2], 2));
			Dual<3> v = noise_eval(fn, p);
			out[i] = v.v;
			for (int a = 0; a < 3; a++) grad[3 * i + a] = v.d[a];
		} else if (precision == 1) {
			out[i] = val(noise_eval(fn, V3<F32>(q[0], q[1], q[2])));
		} else {
			out[i] = noise_eval(fn, V3<double>(q[0], q[1], q[2]));
		}
	}
}

uint64_t orc_synth_theta_count(const up_synth_program *p) { return (uint64_t)synth_theta_count(*p); }
void orc_synth_theta(const up_synth_program *p, double *out) {
	auto t = synth_theta(*p);
	for (size_t i = 0; i < t.size(); i++) out[i] = t[i];
}

// d(p) of a synthetic program at n points; theta may be null (program's own)
void orc_synth_points(const up_synth_program *prog, const double *theta, const float *xyz, uint64_t n, int precision,
	double *out, double *grad, int threads) {
	const up_synth_program P = *prog;
	if (grad) {
		auto th = theta_as<Dual<3>>(P, theta);
		parallel_for(n, threads, [&](uint64_t i) {
			const float *q = xyz + 3 * i;
			V3<Dual<3>> p(Dual<3>::var(q[0], 0), Dual<3>::var(q[1], 1), Dual<3>::var(q[2], 2));
			Dual<3> v = synth_eval(P, th.data(), p);
			out[i] = v.v;
			for (int a = 0; a < 3; a++) grad[3 * i + a] = v.d[a];
		});
	} else if (precision == 1) {
		auto th = theta_as<F32>(P, theta);
		parallel_for(n, threads, [&](uint64_t i) {
			const float *q = xyz + 3 * i;
			out[i] = val(synth_eval(P, th.data(), V3<F32>(q[0], q[1], q[2])));
		});
	} else {
		auto th = theta_as<double>(P, theta);
		parallel_for(n, threads, [&](uint64_t i) {
			const float *q = xyz + 3 * i;
			out[i] = synth_eval(P, th.data(), V3<double>(q[0], q[1], q[2]));
		});
	}
}

// dtheta = sum_i w_i dd(p_i)/dtheta (FP64 forward-mode, up to 40 parameters)
int orc_synth_theta_grad(const up_synth_program *prog, const double *theta, const float *xyz, uint64_t n,
	const double *w, double *dtheta, int threads) {
	constexpr int K = 40;
	const up_synth_program P = *prog;
	const int nt = synth_theta_count(P);
	if (nt > K) return 1;
	std::vector<double> t0 = synth_theta(P);
	const int nth = std::max(threads, 1);
	std::vector<std::vector<double>> part(nth, std::vector<double>(nt, 0.0));
	const uint64_t chunk = (n + nth - 1) / nth;
	parallel_for((uint64_t)nth, nth, [&](uint64_t t) {
		std::vector<Dual<K>> th(nt);
		for (int j = 0; j < nt; j++) th[j] = Dual<K>::var(theta ? theta[j] : t0[j], j);
		for (uint64_t i = t * chunk; i < std::min(n, (t + 1) * chunk); i++) {
			const float *q = xyz + 3 * i;
			Dual<K> v = synth_eval(P, th.data(), V3<Dual<K>>(Dual<K>(q[0]), Dual<K>(q[1]), Dual<K>(q[2])));
			for (int j = 0; j < nt; j++) part[t][j] += w[i] * v.d[j];
		}
	});
	for (int j = 0; j < nt; j++) {
		double s = 0;
		for (int t = 0; t < nth; t++) s += part[t][j];
		dtheta[j] = s;
	}
	return 0;
}

// algorithmic operation counts per sample, averaged over n points
void orc_synth_count_ops(const up_synth_program *prog, const float *xyz, uint64_t n, double *counts5) {
	const up_synth_program P = *prog;
	auto th = theta_as<Counted>(P, nullptr);
	opcounts() = OpCounts();
	for (uint64_t i = 0; i < n; i++) {
		const float *q = xyz + 3 * i;
		(void)synth_eval(P, th.data(), V3<Counted>(q[0], q[1], q[2]));
	}
	const OpCounts c = opcounts();
	counts5[0] = (double)c.flop / n; counts5[1] = (double)c.div / n; counts5[2] = (double)c.sqrt / n;
	counts5[3] = (double)c.floor / n; counts5[4] = (double)c.transc / n;
}

// algorithmic operation counts per sample of the value together with its
// gradient dd/dp (sparse forward mode over the counting scalar, CDual),
// averaged over n points; same bins as orc_synth_count_ops
void orc_synth_count_ops_grad(const up_synth_program *prog, const float *xyz, uint64_t n, double *counts5) {
	const up_synth_program P = *prog;
	auto th = theta_as<CDual>(P, nullptr);
	opcounts() = OpCounts();
	for (uint64_t i = 0; i < n; i++) {
		const float *q = xyz + 3 * i;
		(void)synth_eval(P, th.data(), V3<CDual>(CDual::var(q[0], 0), CDual::var(q[1], 1), CDual::var(q[2], 2)));
	}
	const OpCounts c = opcounts();
	counts5[0] = (double)c.flop / n; counts5[1] = (double)c.div / n; counts5[2] = (double)c.sqrt / n;
	counts5[3] = (double)c.floor / n; counts5[4] = (double)c.transc / n;
}

// ---------------------------------------------------------------- CPU baseline
// The reference samples its SDF through a per-sample callback
// (Delegate<Real(const Vec3&)>, sources/meshGeneration.cpp:39). The baseline
// keeps that structure: an FP32 function pointer called once per sample,
// parallel over z-slabs on `threads` host threads.
namespace {
const up_synth_program *g_cb_prog = nullptr;
std::vector<F32> g_cb_theta;
float synth_callback(const float p[3]) { return (float)val(synth_eval(*g_cb_prog, g_cb_theta.data(), V3<F32>(p[0], p[1], p[2]))); }
}

// samples z-slabs [z0, z1) of the grid into out (nx*ny*(z1-z0) floats)
void orc_synth_grid_fp32(const up_synth_program *prog, const up_grid *grid, uint32_t z0, uint32_t z1, float *out, int threads) {
	g_cb_prog = prog;
	g_cb_theta = theta_as<F32>(*prog, nullptr);
	float (*const volatile fn)(const float *) = &synth_callback;
	const GridF g(*grid);
	const uint64_t nx = g.n[0], ny = g.n[1];
	parallel_for((uint64_t)(z1 - z0), threads, [&](uint64_t kz) {
		const uint32_t k = z0 + (uint32_t)kz;
		float p[3];
		p[2] = g.coord(2, k);
		for (uint64_t j = 0; j < ny; j++) {
			p[1] = g.coord(1, (uint32_t)j);
			for (uint64_t i = 0; i < nx; i++) {
				p[0] = g.coord(0, (uint32_t)i);
				out[(kz * ny + j) * nx + i] = fn(p);
			}
		}
	});
}

// Same, plus the gradient by 6-tap central differences (tap distance h):
// the reference-side way of obtaining contouring normals that the analytic
// gradient replaces. grad receives 3 planes of nx*ny*(z1-z0) floats.
void orc_synth_grid_fp32_cd(const up_synth_program *prog, const up_grid *grid, uint32_t z0, uint32_t z1, float h, float *out, float *grad,
	int threads) {
	g_cb_prog = prog;
	g_cb_theta = theta_as<F32>(*prog, nullptr);
	float (*const volatile fn)(const float *) = &synth_callback;
	const GridF g(*grid);
	const uint64_t nx = g.n[0], ny = g.n[1];
	const uint64_t plane = nx * ny * (uint64_t)(z1 - z0);
	const float inv = 0.5f / h;
	parallel_for((uint64_t)(z1 - z0), threads, [&](uint64_t kz) {
		const uint32_t k = z0 + (uint32_t)kz;
		float p[3], q[3];
		p[2] = g.coord(2, k);
		for (uint64_t j = 0; j < ny; j++) {
			p[1] = g.coord(1, (uint32_t)j);
			for (uint64_t i = 0; i < nx; i++) {
				p[0] = g.coord(0, (uint32_t)i);
				const uint64_t idx = (kz * ny + j) * nx + i;
				out[idx] = fn(p);
				for (int a = 0; a < 3; a++) {
					q[0] = p[0]; q[1] = p[1]; q[2] = p[2];
					q[a] = p[a] + h;
					const float fp = fn(q);
					q[a] = p[a] - h;
					const float fm = fn(q);
					grad[a * plane + idx] = (fp - fm) * inv;
				}
			}
		}
	});
}

// grid sample positions (3 floats per sample) exactly as the FP32 path forms them
void orc_grid_positions(const up_grid *grid, float *out) {
	const GridF g(*grid);
	uint64_t idx = 0;
	for (uint32_t k = 0; k < g.n[2]; k++)
		for (uint32_t j = 0; j < g.n[1]; j++)
			for (uint32_t i = 0; i < g.n[0]; i++) {
				out[3 * idx] = g.coord(0, i); out[3 * idx + 1] = g.coord(1, j); out[3 * idx + 2] = g.coord(2, k);
				idx++;
			}
}

// positions of the samples with linear indices idx[0..n) (x-fastest), the
// same FP32 formula as orc_grid_positions
void orc_grid_positions_at(const up_grid *grid, const uint64_t *idx, uint64_t n, float *out) {
	const GridF g(*grid);
	const uint64_t nx = g.n[0], ny = g.n[1];
	for (uint64_t q = 0; q < n; q++) {
		const uint64_t v = idx[q];
		out[3 * q] = g.coord(0, (uint32_t)(v % nx));
		out[3 * q + 1] = g.coord(1, (uint32_t)((v / nx) % ny));
		out[3 * q + 2] = g.coord(2, (uint32_t)(v / (nx * ny)));
	}
}

// ---------------------------------------------------------------- contour
struct OrcMesh { ContourResult r; };

static GradFn synth_gradfn(const up_synth_program *prog) {
	auto P = std::make_shared<up_synth_program>(*prog);
	auto th = std::make_shared<std::vector<Dual<3>>>(theta_as<Dual<3>>(*prog, nullptr));
	return [P, th](const double p[3], double g[3]) {
		V3<Dual<3>> q(Dual<3>::var(p[0], 0), Dual<3>::var(p[1], 1), Dual<3>::var(p[2], 2));
		Dual<3> v = synth_eval(*P, th->data(), q);
		for (int a = 0; a < 3; a++) g[a] = v.d[a];
	};
}

void *orc_contour_synth(const up_synth_program *prog, const up_grid *grid, const float *values) {
	auto *m = new OrcMesh();
	contour(*grid, values, synth_gradfn(prog), m->r);
	return m;
}

void orc_mesh_counts(void *h, uint64_t *c4) {
	auto *m = (OrcMesh *)h;
	c4[0] = m->r.cells.size(); c4[1] = m->r.indices.size(); c4[2] = m->r.edges.size(); c4[3] = 0;
}
void orc_mesh_copy(void *h, uint64_t *cells, float *positions, float *normals, uint32_t *indices, uint64_t *edges) {
	auto *m = (OrcMesh *)h;
	auto cp = [](auto &v, auto *dst) { if (dst) std::copy(v.begin(), v.end(), dst); };
	cp(m->r.cells, cells); cp(m->r.positions, positions); cp(m->r.normals, normals); cp(m->r.indices, indices); cp(m->r.edges, edges);
}
void orc_mesh_free(void *h) { delete (OrcMesh *)h; }


// ---------------------------------------------------------------- reference modes
void *orc_planet_create(const char *shape, const char *elevation, const char *coloring, int poles, int flowers, uint32_t seed, char *err, int errn) {
	auto *P = new Planet();
	const std::string e = make_planet(shape, elevation, coloring, poles != 0, flowers != 0, seed, *P);
	if (!e.empty()) {
		if (err && errn > 0) std::snprintf(err, errn, "%s", e.c_str());
		delete P;
		return nullptr;
	}
	return P;
}
void orc_planet_free(void *p) { delete (Planet *)p; }
int orc_planet_shape(void *p) { return ((Planet *)p)->shape; }

// field values at n points; precision 0 = FP64, 1 = FP32; grad (FP64 dual) when not null
void orc_field_points(void *h, int field, const float *xyz, uint64_t n, int precision, double *out, double *grad, int threads) {
	const Planet &P = *(Planet *)h;
	parallel_for(n, threads, [&](uint64_t i) {
		const float *q = xyz + 3 * i;
		if (grad) {
			V3<Dual<3>> p(Dual<3>::var(q[0], 0), Dual<3>::var(q[1], 1), Dual<3>::var(q[2], 2));
			const Dual<3> v = field_eval(P, field, p);
			out[i] = v.v;
			for (int a = 0; a < 3; a++) grad[3 * i + a] = v.d[a];
		} else if (precision == 1) {
			out[i] = val(field_eval(P, field, V3<F32>(q[0], q[1], q[2])));
		} else {
			out[i] = field_eval(P, field, V3<double>(q[0], q[1], q[2]));
		}
	});
}

static GradFn planet_gradfn(const Planet *P, int field) {
	return [P, field](const double p[3], double g[3]) {
		V3<Dual<3>> q(Dual<3>::var(p[0], 0), Dual<3>::var(p[1], 1), Dual<3>::var(p[2], 2));
		const Dual<3> v = field_eval(*P, field, q);
		for (int a = 0; a < 3; a++) g[a] = v.d[a];
	};
}
void *orc_contour_planet(void *h, int field, const up_grid *grid, const float *values) {
	auto *m = new OrcMesh();
	contour(*grid, values, planet_gradfn((Planet *)h, field), m->r);
	return m;
}

// per-point tiles: 11 floats per point out (albedo rgb, roughness, metallic,
// height, opacity, elevation, slope, temperature, precipitation) + biome, type
void orc_tiles(void *h, int purpose, const float *pos, const float *nrm, uint64_t n, double *out11, int32_t *biome_type, int threads) {
	const Planet &P = *(Planet *)h;
	Col<double> col(P);
	parallel_for(n, threads, [&](uint64_t i) {
		Tile<double> t;
		t.position = V3<double>(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
		t.normal = V3<double>(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
		t.purpose = purpose;
		col.run(t);
		double *o = out11 + 11 * i;
		o[0] = t.albedo.x; o[1] = t.albedo.y; o[2] = t.albedo.z; o[3] = t.roughness; o[4] = t.metallic; o[5] = t.height; o[6] = t.opacity;
		o[7] = t.elevation; o[8] = t.slope; o[9] = t.temperature; o[10] = t.precipitation;
		biome_type[2 * i] = t.biome;
		biome_type[2 * i + 1] = t.type;
	});
}

// texels: rasterise, color (planet or synthetic program), optional dilation,
// float images (NaN where uncovered) and 8-bit images. purpose 1 land (RGB),
// 2 water (RGBA). Either planet or prog is not null.
void orc_texture(void *planet, const up_synth_program *prog, int purpose, const float *pos, const float *nrm, const float *uv,
	const uint32_t *idx, uint64_t nidx, uint32_t W, uint32_t H, int dilation, float *albedo_f, float *special_f, float *height_f,
	uint8_t *albedo8, uint8_t *special8, uint8_t *height8, int32_t *owner, int threads) {
	Raster R;
	rasterize(uv, idx, nidx / 3, W, H, R);
	const int ach = purpose == PU_WATER ? 4 : 3;
	std::vector<float> A((size_t)W * H * ach, NAN), S((size_t)W * H * 2, NAN), Hh((size_t)W * H, NAN);
	parallel_for((uint64_t)H, threads, [&](uint64_t y) {
		for (uint32_t x = 0; x < W; x++) {
			const size_t q = (size_t)y * W + x;
			const int32_t t = R.owner[q];
			if (t < 0) continue;
			V3<double> p, nn;
			for (int k = 0; k < 3; k++) {
				const uint32_t v = idx[3 * (uint64_t)t + k];
				const double w = R.w[3 * q + k];
				p = p + V3<double>(pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]) * w;
				nn = nn + V3<double>(nrm[3 * v], nrm[3 * v + 1], nrm[3 * v + 2]) * w;
			}
			nn = normalize(nn);
			V3<double> alb;
			double rough, metal = 0, height, opacity = 1;
			if (planet) {
				Tile<double> tl;
				tl.position = p; tl.normal = nn; tl.purpose = purpose;
				Col<double>(*(Planet *)planet).run(tl);
				alb = tl.albedo; rough = tl.roughness; metal = tl.metallic; height = tl.height; opacity = tl.opacity;
			} else {
				synth_texel(*prog, p, alb, rough, height);
			}
			A[q * ach] = (float)alb.x; A[q * ach + 1] = (float)alb.y; A[q * ach + 2] = (float)alb.z;
			if (ach == 4) A[q * ach + 3] = (float)opacity;
			S[2 * q] = (float)rough; S[2 * q + 1] = (float)metal;
			Hh[q] = (float)height;
		}
	});
	if (dilation > 0) { dilate(A, W, H, ach, dilation); dilate(S, W, H, 2, dilation); dilate(Hh, W, H, 1, dilation); }
	if (albedo_f) std::copy(A.begin(), A.end(), albedo_f);
	if (special_f) std::copy(S.begin(), S.end(), special_f);
	if (height_f) std::copy(Hh.begin(), Hh.end(), height_f);
	for (size_t i = 0; albedo8 && i < A.size(); i++) albedo8[i] = to_u8(A[i]);
	for (size_t i = 0; special8 && i < S.size(); i++) special8[i] = to_u8(S[i]);
	for (size_t i = 0; height8 && i < Hh.size(); i++) height8[i] = to_u8(Hh[i]);
	if (owner) std::copy(R.owner.begin(), R.owner.end(), owner);
}

// Mesh hygiene of meshGenerateBase* (meshGeneration.cpp:41, 62-95), the
// project definitions restated sequentially: union-find over the vertex graph
// joined by triangles; kept component = most triangles, ties to the one
// holding the lowest vertex index; water (valid != NULL: the per-vertex test
// elevationRaw < 0.1, already evaluated): validity restricted to the kept
// component, two expansions over its triangles reading the previous pass,
// then triangles with an invalid vertex dropped. Outputs 0/1 keep flags.
void orc_mesh_filter(uint32_t V, uint32_t T, const uint32_t *idx, const uint8_t *valid, uint8_t *keep_v, uint8_t *keep_t) {
	std::vector<uint32_t> parent(V);
	for (uint32_t v = 0; v < V; v++) parent[v] = v;
	auto find = [&](uint32_t x) {
		while (parent[x] != x) {
			parent[x] = parent[parent[x]];
			x = parent[x];
		}
		return x;
	};
	auto unite = [&](uint32_t a, uint32_t b) {
		a = find(a);
		b = find(b);
		if (a == b) return;
		if (a < b) parent[b] = a;
		else parent[a] = b;
	};
	for (uint32_t t = 0; t < T; t++) {
		unite(idx[3 * t], idx[3 * t + 1]);
		unite(idx[3 * t], idx[3 * t + 2]);
	}
	std::vector<uint64_t> tri(V, 0);
	for (uint32_t t = 0; t < T; t++) tri[find(idx[3 * t])]++;
	uint32_t root = 0;
	uint64_t most = 0;
	bool any = false;
	for (uint32_t v = 0; v < V; v++) // roots are the lowest vertex of their component; ascending order breaks ties
		if (find(v) == v && (!any || tri[v] > most)) {
			root = v;
			most = tri[v];
			any = true;
		}
	std::vector<uint8_t> in(V);
	for (uint32_t v = 0; v < V; v++) in[v] = find(v) == root;
	if (!valid) {
		for (uint32_t v = 0; v < V; v++) keep_v[v] = in[v];
		for (uint32_t t = 0; t < T; t++) keep_t[t] = in[idx[3 * t]];
		return;
	}
	std::vector<uint8_t> ok(V), ok2;
	for (uint32_t v = 0; v < V; v++) ok[v] = in[v] && valid[v];
	for (int r = 0; r < 2; r++) {
		ok2 = ok;
		for (uint32_t t = 0; t < T; t++) {
			const uint32_t a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
			if (in[a] && (ok[a] || ok[b] || ok[c])) ok2[a] = ok2[b] = ok2[c] = 1;
		}
		ok.swap(ok2);
	}
	for (uint32_t v = 0; v < V; v++) keep_v[v] = ok[v];
	for (uint32_t t = 0; t < T; t++) keep_t[t] = ok[idx[3 * t]] && ok[idx[3 * t + 1]] && ok[idx[3 * t + 2]];
}

} // extern "C"
