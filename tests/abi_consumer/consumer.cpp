// A C++ consumer of include/up_abi.h written the way the reference would bind
// it (the binding a reference maintainer would write, as one program): mode selection by
// name, the per-point terrain callbacks called from several threads at once
// (generator.cpp:159,215,432-439 run the land, water and navmesh pipelines
// concurrently), the base land mesh with the capacity protocol, texels of a
// small chart and the image conversions. Exits 0 when every check passes.
// Test harness: built and run by tests/test_abi_consumer.py.
#include "up_abi.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

static int g_failures = 0;
#define CHECK(cond, ...)                                   \
	do {                                                   \
		if (!(cond)) {                                     \
			std::fprintf(stderr, "FAILED %s: ", #cond);    \
			std::fprintf(stderr, __VA_ARGS__);             \
			std::fprintf(stderr, "\n");                    \
			g_failures++;                                  \
		}                                                  \
	} while (0)

// the reference's TerrainFunctor shape: Real (*)(const Vec3 &)
using TerrainFunctor = float (*)(const float p[3]);

int main() {
	// terrainApplyConfig: names as on the command line (-s sphere -e lakes -c default)
	const up_modes bad = {"nosuchshape", "lakes", "default", 0, 0};
	up_context *none = nullptr;
	CHECK(up_context_create(&bad, nullptr, &none) == UP_ERR_INVALID_MODE, "unknown shape name must be rejected");
	const up_modes m = {"sphere", "lakes", "default", 0, 0};
	const up_seeds s = {7};
	up_context *planet = nullptr;
	int st = up_context_create(&m, &s, &planet);
	if (st != UP_OK) {
		std::fprintf(stderr, "up_context_create: %s\n", up_status_string(st));
		return st == UP_ERR_NO_DEVICE ? 3 : 1;
	}
	up_set_current_context(planet);

	// points of the reference's sampling box, one set per calling thread
	const int kThreads = 8, kPoints = 192;
	std::vector<std::vector<float>> pts(kThreads), got(kThreads);
	std::mt19937 rng(3);
	std::uniform_real_distribution<float> U(-2000.f, 2000.f);
	for (int t = 0; t < kThreads; t++) {
		pts[t].resize(3 * kPoints);
		for (auto &v : pts[t]) v = U(rng);
		got[t].assign(kPoints, NAN);
	}
	const TerrainFunctor fn[3] = {up_sdf_land, up_sdf_water, up_sdf_navigation};
	const int field_of[3] = {UP_FIELD_LAND, UP_FIELD_WATER, UP_FIELD_NAVIGATION};
	std::vector<std::thread> pool;
	for (int t = 0; t < kThreads; t++)
		pool.emplace_back([&, t]() {
			for (int i = 0; i < kPoints; i++) got[t][i] = fn[t % 3](&pts[t][3 * i]);
		});
	for (auto &th : pool) th.join();
	for (int t = 0; t < kThreads; t++) {
		std::vector<float> ref(kPoints);
		st = up_sdf_eval_points(planet, field_of[t % 3], pts[t].data(), kPoints, ref.data(), nullptr);
		CHECK(st == UP_OK, "up_sdf_eval_points: %s", up_last_error(planet));
		int diff = 0;
		for (int i = 0; i < kPoints; i++) diff += std::memcmp(&ref[i], &got[t][i], 4) != 0;
		CHECK(diff == 0, "thread %d: %d of %d callback values differ from the batched call", t, diff, kPoints);
	}

	// meshGenerateBaseLand: sizing call, then the real one
	const up_grid g = {{-2000.f, -2000.f, -2000.f}, {2000.f, 2000.f, 2000.f}, {64, 64, 64}};
	up_mesh_out mo;
	std::memset(&mo, 0, sizeof(mo));
	st = up_mesh_generate_base(planet, UP_FIELD_LAND, &g, nullptr, &mo);
	CHECK(st == UP_ERR_CAPACITY && mo.vertex_count > 0 && mo.index_count > 0, "sizing call: status %d", st);
	std::vector<float> pos(3 * mo.vertex_count), nrm(3 * mo.vertex_count);
	std::vector<uint32_t> idx(mo.index_count);
	mo.positions = pos.data();
	mo.normals = nrm.data();
	mo.indices = idx.data();
	mo.vertex_capacity = mo.vertex_count;
	mo.index_capacity = mo.index_count;
	st = up_mesh_generate_base(planet, UP_FIELD_LAND, &g, nullptr, &mo);
	CHECK(st == UP_OK, "up_mesh_generate_base: %s", up_last_error(planet));
	uint32_t bad_index = 0;
	for (uint32_t v : idx) bad_index += v >= mo.vertex_count;
	CHECK(bad_index == 0, "%u indices out of range", bad_index);

	// generateTexturesLand on one chart: the mesh's first triangle in a 32 x 32 atlas
	const uint32_t W = 32, H = 32;
	float cpos[9], cnrm[9];
	for (int c = 0; c < 3; c++)
		for (int a = 0; a < 3; a++) {
			cpos[3 * c + a] = pos[3 * idx[c] + a];
			cnrm[3 * c + a] = nrm[3 * idx[c] + a];
		}
	const float cuv[6] = {0.02f, 0.02f, 0.98f, 0.02f, 0.02f, 0.98f};
	const uint32_t cidx[3] = {0, 1, 2};
	const up_mesh_in in = {cpos, cnrm, cuv, cidx, 3, 3};
	std::vector<uint8_t> alb(W * H * 3), spc(W * H * 2), hgt(W * H), pbr(W * H * 3), nmap(W * H * 3);
	up_texture_out to = {alb.data(), spc.data(), hgt.data(), nullptr, nullptr, nullptr};
	st = up_texture(planet, UP_PURPOSE_LAND, &in, W, H, 7, &to);
	CHECK(st == UP_OK, "up_texture: %s", up_last_error(planet));
	// imageConvertSpecialToGltfPbr, imageConvertHeigthToNormal
	CHECK(up_image_special_to_gltf_pbr(planet, spc.data(), W, H, pbr.data()) == UP_OK, "pbr");
	CHECK(up_image_height_to_normal(planet, hgt.data(), W, H, 1.f, nmap.data()) == UP_OK, "normal map");
	int r255 = 0;
	for (uint32_t i = 0; i < W * H; i++) r255 += pbr[3 * i] == 255 && pbr[3 * i + 1] == spc[2 * i];
	CHECK(r255 == (int)(W * H), "pbr channel layout");

	up_set_current_context(nullptr);
	CHECK(std::isnan(up_sdf_land(pts[0].data())), "no installed context: the callback returns NaN");
	up_context_destroy(planet);
	std::printf("consumer: %d threads x %d callback values, base land mesh %llu vertices / %llu triangles, %ux%u texels, %d failures\n",
		kThreads, kPoints, (unsigned long long)mo.vertex_count, (unsigned long long)(mo.index_count / 3), W, H, g_failures);
	return g_failures ? 1 : 0;
}
