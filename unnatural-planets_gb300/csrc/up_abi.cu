// C ABI implementation: contexts, host/device buffer staging, error
// reporting, and the orchestration of the SDF, contouring, texel and batch
// kernels. Every entry point catches C++ exceptions and returns a status.
#include "up_internal.h"
#include "up_modes_desc.h"
#include "up_noise.cuh"
#include "up_ptr.h"
#include "up_synth.cuh"

#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

namespace up {
cudaError_t launch_synth_bwd_noalloc(const up_synth_program &P, const float *xyz, uint64_t n, const float *w, float *dtheta, float *scratch,
	cudaStream_t s);
cudaError_t noalloc_scratch_address(float **out);
int build_modes(const up_modes &m, uint32_t seed, ModesDesc &D, std::string &shape_name, bool &double_sided, std::string &err);
uint32_t instance_seed(uint32_t seed, uint32_t slot);
float modes_contour_band(const ModesDesc &D, int field, const float step[3]);
cudaError_t launch_modes_points(const ModesDesc *M, int field, const float *xyz, uint64_t n, float *d, float *grad, unsigned *nanflag,
	cudaStream_t s);
cudaError_t texture_run(const ModesDesc *M, const up_synth_program *synth, int purpose, const float *pos, const float *nrm, const float *uv,
	const uint32_t *idx, uint64_t nidx, uint32_t W, uint32_t H, int dilation, int *owner, double *tri_ia, float *img0, float *img1, uint8_t *a8, uint8_t *s8,
	uint8_t *h8, float *af, float *sf, float *hf, int *launches, cudaStream_t s);
cudaError_t tiles_run(const ModesDesc *M, int purpose, const float *pos, const float *nrm, uint64_t n, float *out11, uint8_t *bt, cudaStream_t s);
void batch_state_free(void *p);
cudaError_t batch_execute(void *&state, const up_synth_program *planets, size_t nplanets, const up_chunk *chunks, size_t nchunks,
	bool exact_values, uint32_t &ncells, uint32_t &nquads, std::vector<uint32_t> &chunk_cells, std::vector<uint32_t> &chunk_quads, const float *&dpos,
	const uint32_t *&didx, const float *&dvalues, uint64_t &nvalues, bool &nan, bool &replayed, unsigned &fault, cudaStream_t caller);
void batch_set_wait_limit(unsigned long long ns);
void batch_set_form(int form);
} // namespace up

using namespace up;

enum BufSlot {
	B_IN0, B_OUT0, B_OUT1, B_OUT2, B_GRAD, B_GRID, B_PARTIALS, B_W,
	B_DC_BLK, B_DC_TOT, B_DC_CMAP, B_DC_EMAP, B_DC_CLIST, B_DC_ELIST, B_DC_QLIST, B_DC_ET, B_DC_EN, B_DC_SIGNS, B_DC_FB, B_DC_FBF, B_TASKL,
	B_MESH_POS, B_MESH_NRM, B_MESH_IDX,
	B_TEX0, B_TEX1, B_TEX2, B_TEX3, B_TEX4, B_TEX5, B_TEX6, B_TEX7, B_TEX8, B_TEX9, B_TEXIA,
	B_BATCH0, B_BATCH1, B_BATCH2, B_BATCH3, B_BATCH4, B_BATCH5, B_BATCH6, B_BATCH7,
	B_BASE_POS, B_BASE_NRM, B_BASE_IDX, B_BASE_ELEV, B_BASE_PARENT, B_BASE_LABEL, B_BASE_CNT, B_BASE_NEWIDX, B_BASE_BLK, B_BASE_SMALL,
	B_BASE_KEEPV, B_BASE_VALID2, B_BASE_KEEPT, B_PIPE0, B_PIPE1,
	B_COUNT
};

struct up_context {
	int device = 0;
	cudaStream_t stream = nullptr;
	bool owns_stream = false; // per-thread copies of the shims create their own stream
	bool synthetic = false;
	up_synth_program prog{};
	ModesDesc modes{};
	ModesDesc *d_modes = nullptr; // device copy read by the mode kernels
	std::string shape_name;
	bool double_sided = false;
	std::string last_error;
	unsigned *d_flag = nullptr;
	float *noalloc_scratch = nullptr; // device address of the static scratch of up_sdf_param_backward_noalloc
	struct Buf { void *p = nullptr; size_t n = 0; } bufs[B_COUNT];
	void *batch = nullptr; // planned batch (up_batch.cu)
	// device-to-host pipeline of up_sdf_grid: copies of slab k overlap the
	// sampling of slab k + 1 (created on first use)
	cudaStream_t copy_stream = nullptr;
	cudaEvent_t ev_done[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
	cudaEvent_t ev_fork = nullptr, ev_join = nullptr; // contouring: FP64 QEF cells on copy_stream
};

namespace {

// The context installed for the per-point shims (up_set_current_context),
// and a generation number that changes whenever the installed context
// changes or is destroyed: a thread's copy of an older generation is stale.
std::mutex g_current_mu;
up_context *g_current = nullptr;
uint64_t g_current_gen = 0;

// Host-side fault injection: the next g_fail_allocs scratch allocations fail
// as if cudaMalloc had returned cudaErrorMemoryAllocation (no GPU involved).
std::atomic<uint32_t> g_fail_allocs{0};

// NVTX range around one entry point (shows in Nsight timelines; free when no
// tool is attached)
struct NvtxRange {
	explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
	~NvtxRange() { nvtxRangePop(); }
};

struct Fail {
	int code;
	std::string msg;
};

int fail(up_context *ctx, int code, const std::string &msg) {
	if (ctx) ctx->last_error = msg;
	return code;
}

void check(cudaError_t e, const char *what) {
	if (e == cudaSuccess) return;
	if (e == cudaErrorMemoryAllocation) throw Fail{UP_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e)};
	throw Fail{UP_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}

// the context's second stream and its events, created on first use: host
// copies of up_sdf_grid and the FP64 QEF cells of contouring run there
void side_stream(up_context *ctx) {
	if (ctx->copy_stream) return;
	check(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
	for (int b = 0; b < 2; b++) {
		check(cudaEventCreateWithFlags(&ctx->ev_done[b], cudaEventDisableTiming), "cudaEventCreate");
		check(cudaEventCreateWithFlags(&ctx->ev_copied[b], cudaEventDisableTiming), "cudaEventCreate");
	}
	check(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming), "cudaEventCreate");
	check(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming), "cudaEventCreate");
}

void *buf(up_context *ctx, int slot, size_t bytes) {
	auto &b = ctx->bufs[slot];
	if (bytes == 0) bytes = 16;
	if (b.n >= bytes) return b.p;
	if (b.p) check(cudaFree(b.p), "cudaFree");
	b.p = nullptr;
	b.n = 0;
	size_t want = bytes + bytes / 8;
	uint32_t f = g_fail_allocs.load();
	while (f > 0 && !g_fail_allocs.compare_exchange_weak(f, f - 1)) {}
	if (f > 0) throw Fail{UP_ERR_OOM, "cudaMalloc: out of memory (injected)"};
	check(cudaMalloc(&b.p, want), "cudaMalloc");
	b.n = want;
	return b.p;
}

// true when the kernels of ctx may read or write p in place: device memory
// of the context's own GPU, or managed memory. Host memory and memory of
// another GPU are copied through the context's scratch (cudaMemcpyDefault
// resolves either through unified addressing).
bool is_local(const up_context *ctx, const void *p) {
	if (!p) return false;
	cudaPointerAttributes a;
	const bool ok = cudaPointerGetAttributes(&a, p) == cudaSuccess;
	if (!ok) cudaGetLastError();
	return ptr_kind(ok, ok ? (int)a.type : 0, ok ? a.device : -1, ctx->device) == PTR_LOCAL;
}

// device view of a caller input: the pointer itself, or a staged copy
const void *stage_in(up_context *ctx, int slot, const void *p, size_t bytes) {
	if (is_local(ctx, p)) return p;
	void *d = buf(ctx, slot, bytes);
	check(cudaMemcpyAsync(d, p, bytes, cudaMemcpyDefault, ctx->stream), "cudaMemcpyAsync stage in");
	return d;
}
// device target for a caller output: the pointer itself, or scratch
void *stage_out(up_context *ctx, int slot, void *p, size_t bytes) {
	if (!p) return nullptr;
	if (is_local(ctx, p)) return p;
	return buf(ctx, slot, bytes);
}
void finish_out(up_context *ctx, void *dst, const void *dev, size_t bytes) {
	if (!dst || dst == dev) return;
	check(cudaMemcpyAsync(dst, dev, bytes, cudaMemcpyDefault, ctx->stream), "cudaMemcpyAsync stage out");
}

void set_device(up_context *ctx) { check(cudaSetDevice(ctx->device), "cudaSetDevice"); }

void reset_flag(up_context *ctx) { check(cudaMemsetAsync(ctx->d_flag, 0, sizeof(unsigned), ctx->stream), "cudaMemsetAsync"); }
unsigned read_flag(up_context *ctx) {
	unsigned f = 0;
	check(cudaMemcpyAsync(&f, ctx->d_flag, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync flag");
	check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
	return f;
}

const char *field_word(int field) {
	switch (field) {
		case UP_FIELD_LAND: return "land";
		case UP_FIELD_WATER: return "water";
		case UP_FIELD_NAVIGATION: return "navigation";
		case UP_FIELD_ELEVATION: return "elevation";
		default: return "elevation raw";
	}
}

int init_context(up_context *ctx) {
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
		cudaGetLastError();
		return UP_ERR_NO_DEVICE;
	}
	check(cudaGetDevice(&ctx->device), "cudaGetDevice");
	check(cudaMalloc(&ctx->d_flag, 16), "cudaMalloc flag");
	// the static scratch of up_sdf_param_backward_noalloc: its module is loaded
	// and its device address looked up now, at set-up, with the context's
	// device current, so the allocation-free entry point neither grows the
	// device footprint nor queries the runtime later (for example inside a
	// stream capture)
	check(noalloc_scratch_address(&ctx->noalloc_scratch), "cudaGetSymbolAddress (allocation-free scratch)");
	return UP_OK;
}

template<class F>
int guarded(up_context *ctx, const char *name, F &&f) {
	NvtxRange range(name);
	try {
		return f();
	} catch (const Fail &e) {
		return fail(ctx, e.code, e.msg);
	} catch (const std::bad_alloc &) {
		return fail(ctx, UP_ERR_OOM, "host allocation failed");
	} catch (const std::exception &e) {
		return fail(ctx, UP_ERR_CUDA, e.what());
	} catch (...) {
		return fail(ctx, UP_ERR_CUDA, "unknown error");
	}
}

bool valid_grid(const up_grid *g) {
	if (!g) return false;
	for (int a = 0; a < 3; a++) {
		if (g->n[a] < 2) return false;
		if (!(g->hi[a] > g->lo[a])) return false;
	}
	const uint64_t n = (uint64_t)g->n[0] * g->n[1] * g->n[2];
	return n < (1ull << 31);
}

bool valid_program(const up_synth_program &p) {
	if (p.base < 0 || p.base > 3 || p.n_layers < 0 || p.n_layers > 2 || p.n_spheres < 0 || p.n_spheres > 8) return false;
	for (int l = 0; l < p.n_layers; l++) {
		const up_noise_layer &L = p.layer[l];
		if (L.type < 0 || L.type > 5 || L.fractal < 0 || L.fractal > 2 || L.octaves < 1 || L.octaves > 8) return false;
		if (L.distance < 0 || L.distance > 2 || L.operation < 0 || L.operation > 6) return false;
	}
	return true;
}

// Contouring in two steps (shared by up_contour and up_mesh_generate_base):
// sampling (or staging the caller's values) and counting, then, once the
// caller has sized the outputs, emission and geometry into device pointers.
struct ContourRun {
	GridDev g;
	const float *d = nullptr;
	DcScratch S{};
	uint32_t ncells = 0, nedges = 0, nquads = 0;
};
int contour_count(up_context *ctx, int field, const up_grid *grid, const float *values, ContourRun &c) {
	c.g = make_grid(*grid);
	const size_t np = (size_t)grid->n[0] * grid->n[1] * grid->n[2];
	const size_t nc = (size_t)(grid->n[0] - 1) * (grid->n[1] - 1) * (grid->n[2] - 1);
	bool signs_ready = false; // the sampling launch wrote the sign words
	if (values) {
		c.d = (const float *)stage_in(ctx, B_GRID, values, np * 4);
	} else {
		float *gd = (float *)buf(ctx, B_GRID, np * 4);
		reset_flag(ctx);
		if (ctx->synthetic) {
			uint32_t *tl = (uint32_t *)buf(ctx, B_TASKL, runs_task_count(c.g) * 4);
			const float band = contour_band(ctx->prog, c.g);
			uint32_t *sg = nullptr;
			if (synth_grid_signs(ctx->prog, c.g, band)) {
				sg = (uint32_t *)buf(ctx, B_DC_SIGNS, dc_sign_words(c.g) * 4);
				signs_ready = true;
			}
			check(launch_synth_grid(ctx->prog, c.g, gd, nullptr, ctx->d_flag, ctx->stream, band, tl, sg), "sdf grid kernel");
		} else {
			float *o[3] = {nullptr, nullptr, nullptr};
			o[field] = gd;
			uint32_t *tl = (uint32_t *)buf(ctx, B_TASKL, runs_task_count(c.g) * 4);
			const float band = modes_contour_band(ctx->modes, field, c.g.step);
			uint32_t *sg = nullptr;
			if (modes_grid_signs(ctx->modes, 1u << field, c.g, band)) {
				sg = (uint32_t *)buf(ctx, B_DC_SIGNS, dc_sign_words(c.g) * 4);
				signs_ready = true;
			}
			check(launch_modes_grid(ctx->d_modes, ctx->modes, 1u << field, c.g, o[0], o[1], o[2], nullptr, ctx->d_flag, ctx->stream, band, tl, sg),
				"sdf grid kernel");
		}
		if (read_flag(ctx)) return fail(ctx, UP_ERR_NAN, std::string("invalid ") + field_word(field) + " sdf value");
		c.d = gd;
	}
	DcScratch &S = c.S;
	const uint32_t nb = dc_num_blocks(c.g);
	S.blk_counts = (uint32_t *)buf(ctx, B_DC_BLK, dc_scan_words(nb) * 4);
	S.totals = (uint32_t *)buf(ctx, B_DC_TOT, 16);
	S.cell_map = (uint32_t *)buf(ctx, B_DC_CMAP, nc * 4);
	S.edge_map = (uint32_t *)buf(ctx, B_DC_EMAP, np * 12);
	S.signs = (uint32_t *)buf(ctx, B_DC_SIGNS, dc_sign_words(c.g) * 4); // the same words when signs_ready
	check(dc_count(c.d, c.g, S, ctx->stream, signs_ready), "contour count");
	uint32_t tot[4] = {0, 0, 0, 0};
	check(cudaMemcpyAsync(tot, S.totals, 12, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync totals");
	check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
	c.ncells = tot[0];
	c.nedges = tot[1];
	c.nquads = tot[2];
	if (c.nquads == 0) return fail(ctx, UP_ERR_EMPTY_MESH, std::string("generated empty base ") + field_word(field) + " mesh");
	return UP_OK;
}
void contour_geometry(up_context *ctx, int field, ContourRun &c, float *pos, float *nrm, uint32_t *idx) {
	DcScratch &S = c.S;
	S.cell_list = (uint32_t *)buf(ctx, B_DC_CLIST, (size_t)c.ncells * 4);
	S.fb_list = (uint32_t *)buf(ctx, B_DC_FB, (size_t)c.ncells * 4);
	S.fb_flag = (uint8_t *)buf(ctx, B_DC_FBF, (size_t)c.ncells);
	side_stream(ctx);
	S.side = ctx->copy_stream;
	S.ev_fork = ctx->ev_fork;
	S.ev_join = ctx->ev_join;
	S.edge_list = (uint32_t *)buf(ctx, B_DC_ELIST, (size_t)c.nedges * 4);
	S.quad_list = (uint32_t *)buf(ctx, B_DC_QLIST, (size_t)c.nquads * 4);
	S.edge_t = (float *)buf(ctx, B_DC_ET, (size_t)c.nedges * 4);
	S.edge_n = (float *)buf(ctx, B_DC_EN, (size_t)c.nedges * 12);
	check(dc_emit(c.d, c.g, S, ctx->stream), "contour emit");
	if (ctx->synthetic) check(dc_geometry_synth(ctx->prog, c.d, c.g, S, c.ncells, c.nedges, c.nquads, pos, nrm, idx, ctx->stream), "contour geometry");
	else check(dc_geometry_modes(ctx->d_modes, field, c.d, c.g, S, c.ncells, c.nedges, c.nquads, pos, nrm, idx, ctx->stream), "contour geometry");
}

// up_sdf_grid into host memory, pipelined: the grid is sampled in z-slabs
// into two device staging buffers (fields then gradient planes of the slab);
// the copy stream moves slab k to the host while the caller's stream samples
// slab k + 1. Slab coordinates use the full grid's index (GridDev::k0), so
// values are bit-identical to the single launch.
constexpr size_t GRID_PIPE_MIN = (size_t)1 << 22; // samples
constexpr int GRID_PIPE_SLABS = 16;
int sdf_grid_pipelined(up_context *ctx, uint32_t mask, const GridDev &g, float *const out[3], float *grad) {
	side_stream(ctx);
	const uint32_t nz = g.n[2];
	const size_t plane = (size_t)g.n[0] * g.n[1];
	const size_t n = plane * nz;
	const uint32_t sz = (nz + GRID_PIPE_SLABS - 1) / GRID_PIPE_SLABS;
	int nf = 0;
	for (int f = 0; f < 3; f++) nf += (int)(mask >> f & 1u);
	const int nplanes = nf + (grad ? 3 : 0);
	float *stage[2];
	for (int b = 0; b < 2; b++) stage[b] = (float *)buf(ctx, B_PIPE0 + b, plane * sz * nplanes * 4);
	reset_flag(ctx);
	// the copy stream starts after work already queued on the caller's stream
	check(cudaEventRecord(ctx->ev_copied[0], ctx->stream), "cudaEventRecord");
	check(cudaEventRecord(ctx->ev_copied[1], ctx->stream), "cudaEventRecord");
	int slab = 0;
	for (uint32_t z0 = 0; z0 < nz; z0 += sz, slab++) {
		const int b = slab & 1;
		const uint32_t cz = nz - z0 < sz ? nz - z0 : sz;
		const size_t cn = plane * cz;
		GridDev gs = g;
		gs.n[2] = cz;
		gs.k0 = z0;
		// buffer b is free once its previous slab's copies are done
		check(cudaStreamWaitEvent(ctx->stream, ctx->ev_copied[b], 0), "cudaStreamWaitEvent");
		float *o[3] = {nullptr, nullptr, nullptr};
		int q = 0;
		for (int f = 0; f < 3; f++)
			if (mask >> f & 1u) o[f] = stage[b] + (size_t)(q++) * cn;
		float *dg = grad ? stage[b] + (size_t)nf * cn : nullptr;
		if (ctx->synthetic) check(launch_synth_grid(ctx->prog, gs, o[0], dg, ctx->d_flag, ctx->stream), "sdf grid kernel");
		else check(launch_modes_grid(ctx->d_modes, ctx->modes, mask, gs, o[0], o[1], o[2], dg, ctx->d_flag, ctx->stream), "sdf grid kernel");
		check(cudaEventRecord(ctx->ev_done[b], ctx->stream), "cudaEventRecord");
		check(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_done[b], 0), "cudaStreamWaitEvent");
		const size_t off = plane * z0;
		for (int f = 0; f < 3; f++)
			if (mask >> f & 1u)
				check(cudaMemcpyAsync(out[f] + off, o[f], cn * 4, cudaMemcpyDefault, ctx->copy_stream), "cudaMemcpyAsync D2H");
		for (int a = 0; grad && a < 3; a++)
			check(cudaMemcpyAsync(grad + (size_t)a * n + off, dg + (size_t)a * cn, cn * 4, cudaMemcpyDefault, ctx->copy_stream),
				"cudaMemcpyAsync D2H");
		check(cudaEventRecord(ctx->ev_copied[b], ctx->copy_stream), "cudaEventRecord");
	}
	// the call completes with the last copies
	check(cudaStreamWaitEvent(ctx->stream, ctx->ev_copied[(slab - 1) & 1], 0), "cudaStreamWaitEvent");
	if (read_flag(ctx)) {
		int f = 0;
		while (!(mask >> f & 1u)) f++;
		return fail(ctx, UP_ERR_NAN, std::string("invalid ") + field_word(f) + " sdf value");
	}
	return (int)UP_OK;
}

// frees everything a context holds (no lock: callers deal with the installed context)
void destroy_context(up_context *ctx) {
	cudaSetDevice(ctx->device);
	if (ctx->stream) cudaStreamSynchronize(ctx->stream);
	for (auto &b : ctx->bufs) if (b.p) cudaFree(b.p);
	if (ctx->d_flag) cudaFree(ctx->d_flag);
	if (ctx->d_modes) cudaFree(ctx->d_modes);
	if (ctx->batch) batch_state_free(ctx->batch);
	if (ctx->copy_stream) {
		cudaStreamSynchronize(ctx->copy_stream);
		cudaStreamDestroy(ctx->copy_stream);
	}
	for (int b = 0; b < 2; b++) {
		if (ctx->ev_done[b]) cudaEventDestroy(ctx->ev_done[b]);
		if (ctx->ev_copied[b]) cudaEventDestroy(ctx->ev_copied[b]);
	}
	if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
	if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
	if (ctx->owns_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
	delete ctx;
}

} // namespace

// ============================================================================
extern "C" {

const char *up_status_string(int s) {
	switch (s) {
		case UP_OK: return "ok";
		case UP_ERR_INVALID_ARGUMENT: return "invalid argument";
		case UP_ERR_INVALID_MODE: return "invalid mode";
		case UP_ERR_NAN: return "invalid sdf value";
		case UP_ERR_OOM: return "out of memory";
		case UP_ERR_CUDA: return "cuda error";
		case UP_ERR_CAPACITY: return "insufficient capacity";
		case UP_ERR_TIMEOUT: return "timeout";
		case UP_ERR_EMPTY_MESH: return "empty mesh";
		case UP_ERR_NO_DEVICE: return "no cuda device";
		default: return "unknown status";
	}
}

const char *up_last_error(const up_context *ctx) { return ctx ? ctx->last_error.c_str() : ""; }

uint32_t up_instance_seed(uint32_t seed, uint32_t slot) { return instance_seed(seed, slot); }

size_t up_synth_theta_count(const up_synth_program *p) {
	if (!p) return 0;
	size_t n = 0;
	for (int l = 0; l < p->n_layers && l < 2; l++) n += 2 * (size_t)p->layer[l].octaves;
	switch (p->base) {
		case UP_BASE_SPHERE: n += 1; break;
		case UP_BASE_TORUS: case UP_BASE_ROUNDED_BOX: n += 2; break;
		default: n += 3 + (size_t)p->n_spheres;
	}
	return n;
}

int up_context_create(const up_modes *modes, const up_seeds *seeds, up_context **out) {
	if (!modes || !out) return UP_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	up_context *ctx = new (std::nothrow) up_context();
	if (!ctx) return UP_ERR_OOM;
	std::string err;
	const int st = build_modes(*modes, seeds ? seeds->seed : 0u, ctx->modes, ctx->shape_name, ctx->double_sided, err);
	if (st != UP_OK) {
		delete ctx;
		return st;
	}
	const int r = guarded(ctx, "up_context_create", [&]() {
		const int st2 = init_context(ctx);
		if (st2 != UP_OK) return st2;
		check(cudaMalloc(&ctx->d_modes, sizeof(ModesDesc)), "cudaMalloc planet description");
		check(cudaMemcpy(ctx->d_modes, &ctx->modes, sizeof(ModesDesc), cudaMemcpyHostToDevice), "cudaMemcpy planet description");
		return (int)UP_OK;
	});
	if (r != UP_OK) {
		if (ctx->d_modes) cudaFree(ctx->d_modes);
		if (ctx->d_flag) cudaFree(ctx->d_flag);
		delete ctx;
		return r;
	}
	*out = ctx;
	return UP_OK;
}

int up_context_create_synthetic(const up_synth_program *program, up_context **out) {
	if (!program || !out) return UP_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	if (!valid_program(*program)) return UP_ERR_INVALID_ARGUMENT;
	up_context *ctx = new (std::nothrow) up_context();
	if (!ctx) return UP_ERR_OOM;
	ctx->synthetic = true;
	ctx->prog = *program;
	ctx->shape_name = "synthetic";
	const int r = guarded(ctx, "up_context_create_synthetic", [&]() { return init_context(ctx); });
	if (r != UP_OK) {
		delete ctx;
		return r;
	}
	*out = ctx;
	return UP_OK;
}

int up_context_destroy(up_context *ctx) {
	if (!ctx) return UP_ERR_INVALID_ARGUMENT;
	{
		std::lock_guard<std::mutex> lock(g_current_mu);
		if (g_current == ctx) {
			g_current = nullptr;
			g_current_gen++;
		}
	}
	destroy_context(ctx);
	return UP_OK;
}

size_t up_context_device_bytes(const up_context *ctx) {
	if (!ctx) return 0;
	size_t n = 0;
	for (const auto &b : ctx->bufs) n += b.n;
	return n;
}

void up_debug_fail_allocations(uint32_t count) { g_fail_allocs.store(count); }

void up_debug_set_wait_limit(uint64_t ns) { batch_set_wait_limit(ns); }

int up_debug_set_batch_form(int form) {
	if (form < 0 || form > 2) return UP_ERR_INVALID_ARGUMENT;
	batch_set_form(form);
	return UP_OK;
}

int up_context_set_stream(up_context *ctx, void *stream) {
	if (!ctx) return UP_ERR_INVALID_ARGUMENT;
	ctx->stream = (cudaStream_t)stream;
	return UP_OK;
}

int up_context_shape_name(const up_context *ctx, char *b, size_t n) {
	if (!ctx || !b || n == 0) return UP_ERR_INVALID_ARGUMENT;
	std::snprintf(b, n, "%s", ctx->shape_name.c_str());
	return ctx->shape_name.size() < n ? UP_OK : UP_ERR_CAPACITY;
}

int up_context_double_sided(const up_context *ctx) { return ctx && ctx->double_sided ? 1 : 0; }

int up_context_set_theta(up_context *ctx, const float *theta, size_t n) {
	if (!ctx || !theta || !ctx->synthetic) return UP_ERR_INVALID_ARGUMENT;
	up_synth_program &p = ctx->prog;
	if (n != up_synth_theta_count(&p)) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "theta size mismatch");
	size_t t = 0;
	for (int l = 0; l < p.n_layers; l++) {
		for (int i = 0; i < p.layer[l].octaves; i++) p.layer[l].amp[i] = theta[t++];
		for (int i = 0; i < p.layer[l].octaves; i++) p.layer[l].freq[i] = theta[t++];
	}
	switch (p.base) {
		case UP_BASE_SPHERE: p.param[0] = theta[t++]; break;
		case UP_BASE_TORUS: case UP_BASE_ROUNDED_BOX: p.param[0] = theta[t++]; p.param[1] = theta[t++]; break;
		default:
			p.param[0] = theta[t++]; p.param[1] = theta[t++];
			for (int s = 0; s < p.n_spheres; s++) p.sphere[s][3] = theta[t++];
			p.k = theta[t++];
	}
	std::lock_guard<std::mutex> lock(g_current_mu);
	if (g_current == ctx) g_current_gen++; // the shims' per-thread copies are stale
	return UP_OK;
}

int up_set_current_context(up_context *ctx) {
	std::lock_guard<std::mutex> lock(g_current_mu);
	g_current = ctx;
	g_current_gen++;
	return UP_OK;
}

int up_sdf_eval_points(up_context *ctx, int field, const float *xyz, size_t n, float *d, float *grad) {
	if (!ctx || !xyz || !d || n == 0) return UP_ERR_INVALID_ARGUMENT;
	if (field < 0 || field > 4) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "bad field");
	if (ctx->synthetic && field != UP_FIELD_LAND) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "synthetic programs have only the LAND field");
	return guarded(ctx, "up_sdf_eval_points", [&]() {
		set_device(ctx);
		const float *dx = (const float *)stage_in(ctx, B_IN0, xyz, n * 12);
		float *dd = (float *)stage_out(ctx, B_OUT0, d, n * 4);
		float *dg = (float *)stage_out(ctx, B_GRAD, grad, n * 12);
		reset_flag(ctx);
		if (ctx->synthetic) check(launch_synth_points(ctx->prog, dx, n, dd, dg, ctx->d_flag, ctx->stream), "sdf points kernel");
		else check(launch_modes_points(ctx->d_modes, field, dx, n, dd, dg, ctx->d_flag, ctx->stream), "sdf points kernel");
		finish_out(ctx, d, dd, n * 4);
		finish_out(ctx, grad, dg, n * 12);
		if (read_flag(ctx)) return fail(ctx, UP_ERR_NAN, std::string("invalid ") + field_word(field) + " sdf value");
		return (int)UP_OK;
	});
}

} // extern "C"

namespace {

// A copy of src for one host thread: the same planet description, its own
// stream, flag and scratch. Device memory of the copy is separate from src,
// so copies never share staging buffers, NaN flags or error messages.
up_context *clone_for_thread(const up_context *src) {
	up_context *c = new (std::nothrow) up_context();
	if (!c) return nullptr;
	c->synthetic = src->synthetic;
	c->prog = src->prog;
	c->modes = src->modes;
	c->shape_name = src->shape_name;
	c->double_sided = src->double_sided;
	const int r = guarded(c, "up_sdf_shim_context", [&]() {
		check(cudaSetDevice(src->device), "cudaSetDevice");
		const int st = init_context(c);
		if (st != UP_OK) return st;
		check(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
		c->owns_stream = true;
		if (!c->synthetic) {
			check(cudaMalloc(&c->d_modes, sizeof(ModesDesc)), "cudaMalloc planet description");
			check(cudaMemcpy(c->d_modes, &c->modes, sizeof(ModesDesc), cudaMemcpyHostToDevice), "cudaMemcpy planet description");
		}
		return (int)UP_OK;
	});
	if (r != UP_OK) {
		destroy_context(c);
		return nullptr;
	}
	return c;
}

// The calling thread's copy of the installed context, made on the thread's
// first shim call after up_set_current_context (or up_context_set_theta of
// the installed context) and destroyed when the thread exits.
struct ShimCopy {
	uint64_t gen = 0;
	up_context *ctx = nullptr;
	~ShimCopy() {
		if (ctx) destroy_context(ctx);
	}
};
thread_local ShimCopy t_shim;

up_context *shim_context() {
	std::lock_guard<std::mutex> lock(g_current_mu); // the installed context stays alive while it is copied
	if (!g_current) return nullptr;
	if (t_shim.ctx && t_shim.gen == g_current_gen) return t_shim.ctx;
	if (t_shim.ctx) {
		destroy_context(t_shim.ctx);
		t_shim.ctx = nullptr;
	}
	t_shim.ctx = clone_for_thread(g_current);
	t_shim.gen = g_current_gen;
	return t_shim.ctx;
}

float shim(int field, const float p[3]) {
	if (!p) return NAN;
	up_context *ctx = shim_context();
	if (!ctx) return NAN;
	float d = NAN;
	if (up_sdf_eval_points(ctx, field, p, 1, &d, nullptr) != UP_OK) return NAN;
	return d;
}

} // namespace

extern "C" {

float up_sdf_land(const float p[3]) { return shim(UP_FIELD_LAND, p); }
float up_sdf_water(const float p[3]) { return shim(UP_FIELD_WATER, p); }
float up_sdf_navigation(const float p[3]) { return shim(UP_FIELD_NAVIGATION, p); }

int up_sdf_grid(up_context *ctx, uint32_t mask, const up_grid *grid, float *const out[3], float *grad) {
	if (!ctx || !valid_grid(grid) || !out) return UP_ERR_INVALID_ARGUMENT;
	mask &= 7u;
	if (!mask) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "empty fields mask");
	if (ctx->synthetic && mask != 1u) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "synthetic programs have only the LAND field");
	for (int f = 0; f < 3; f++)
		if ((mask >> f & 1u) && !out[f]) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "missing output for a selected field");
	return guarded(ctx, "up_sdf_grid", [&]() {
		set_device(ctx);
		const GridDev g = make_grid(*grid);
		const size_t n = (size_t)grid->n[0] * grid->n[1] * grid->n[2];
		// no output on the context's GPU and a grid large enough: pipelined slabs
		bool host_only = n >= GRID_PIPE_MIN && !(grad && is_local(ctx, grad));
		for (int f = 0; f < 3; f++)
			if ((mask >> f & 1u) && is_local(ctx, out[f])) host_only = false;
		if (host_only) return sdf_grid_pipelined(ctx, mask, g, out, grad);
		float *o[3] = {nullptr, nullptr, nullptr};
		for (int f = 0; f < 3; f++)
			if (mask >> f & 1u) o[f] = (float *)stage_out(ctx, B_OUT0 + f, out[f], n * 4);
		float *dg = (float *)stage_out(ctx, B_GRAD, grad, n * 12);
		reset_flag(ctx);
		if (ctx->synthetic) check(launch_synth_grid(ctx->prog, g, o[0], dg, ctx->d_flag, ctx->stream), "sdf grid kernel");
		else check(launch_modes_grid(ctx->d_modes, ctx->modes, mask, g, o[0], o[1], o[2], dg, ctx->d_flag, ctx->stream), "sdf grid kernel");
		for (int f = 0; f < 3; f++)
			if (mask >> f & 1u) finish_out(ctx, out[f], o[f], n * 4);
		finish_out(ctx, grad, dg, n * 12);
		if (read_flag(ctx)) {
			int f = 0;
			while (!(mask >> f & 1u)) f++;
			return fail(ctx, UP_ERR_NAN, std::string("invalid ") + field_word(f) + " sdf value");
		}
		return (int)UP_OK;
	});
}

int up_contour(up_context *ctx, int field, const up_grid *grid, const float *values, up_mesh_out *mesh) {
	if (!ctx || !valid_grid(grid) || !mesh) return UP_ERR_INVALID_ARGUMENT;
	if (field < 0 || field > 2) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "contour field must be LAND, WATER or NAVIGATION");
	if (ctx->synthetic && field != UP_FIELD_LAND) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "synthetic programs have only the LAND field");
	return guarded(ctx, "up_contour", [&]() {
		set_device(ctx);
		ContourRun c;
		const int st = contour_count(ctx, field, grid, values, c);
		if (st != UP_OK) return st;
		mesh->vertex_count = c.ncells;
		mesh->index_count = 6ull * c.nquads;
		if (!mesh->positions || !mesh->indices || mesh->vertex_capacity < c.ncells || mesh->index_capacity < 6ull * c.nquads)
			return fail(ctx, UP_ERR_CAPACITY, "mesh buffers too small");
		float *pos = (float *)stage_out(ctx, B_MESH_POS, mesh->positions, (size_t)c.ncells * 12);
		float *nrm = (float *)stage_out(ctx, B_MESH_NRM, mesh->normals, (size_t)c.ncells * 12);
		uint32_t *idx = (uint32_t *)stage_out(ctx, B_MESH_IDX, mesh->indices, (size_t)c.nquads * 24);
		contour_geometry(ctx, field, c, pos, nrm, idx);
		finish_out(ctx, mesh->positions, pos, (size_t)c.ncells * 12);
		finish_out(ctx, mesh->normals, nrm, (size_t)c.ncells * 12);
		finish_out(ctx, mesh->indices, idx, (size_t)c.nquads * 24);
		check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
		return (int)UP_OK;
	});
}

int up_mesh_generate_base(up_context *ctx, int field, const up_grid *grid, const float *values, up_mesh_out *mesh) {
	if (!ctx || !valid_grid(grid) || !mesh) return UP_ERR_INVALID_ARGUMENT;
	if (field < 0 || field > 2) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "base mesh field must be LAND, WATER or NAVIGATION");
	if (ctx->synthetic && field != UP_FIELD_LAND) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "synthetic programs have only the LAND field");
	return guarded(ctx, "up_mesh_generate_base", [&]() {
		set_device(ctx);
		ContourRun c;
		const int st = contour_count(ctx, field, grid, values, c);
		if (st != UP_OK) return st;
		const uint32_t V = c.ncells, T = 2 * c.nquads;
		float *pos = (float *)buf(ctx, B_BASE_POS, (size_t)V * 12);
		float *nrm = mesh->normals ? (float *)buf(ctx, B_BASE_NRM, (size_t)V * 12) : nullptr;
		uint32_t *idx = (uint32_t *)buf(ctx, B_BASE_IDX, (size_t)T * 12);
		contour_geometry(ctx, field, c, pos, nrm, idx);
		MeshFilterArgs a{};
		a.V = V;
		a.T = T;
		a.pos = pos;
		a.nrm = nrm;
		a.idx = idx;
		if (field == UP_FIELD_WATER) {
			float *elev = (float *)buf(ctx, B_BASE_ELEV, (size_t)V * 4);
			// elevationRaw at the vertices; a NaN compares false and leaves the vertex invalid
			check(launch_modes_points(ctx->d_modes, UP_FIELD_ELEVATION_RAW, pos, V, elev, nullptr, ctx->d_flag, ctx->stream), "elevation kernel");
			a.elev = elev;
		}
		a.parent = (uint32_t *)buf(ctx, B_BASE_PARENT, (size_t)V * 4);
		a.label = (uint32_t *)buf(ctx, B_BASE_LABEL, (size_t)V * 4);
		a.cnt = (uint32_t *)buf(ctx, B_BASE_CNT, (size_t)V * 4);
		a.newidx = (uint32_t *)buf(ctx, B_BASE_NEWIDX, (size_t)V * 4);
		a.blk = (uint32_t *)buf(ctx, B_BASE_BLK, dc_scan_words(mesh_blocks(V, T)) * 4);
		uint32_t *small = (uint32_t *)buf(ctx, B_BASE_SMALL, 64);
		a.totals = small;
		a.err = small + 4;
		a.best = (unsigned long long *)(small + 8);
		a.keep_v = (uint8_t *)buf(ctx, B_BASE_KEEPV, V);
		a.valid2 = (uint8_t *)buf(ctx, B_BASE_VALID2, V);
		a.keep_t = (uint8_t *)buf(ctx, B_BASE_KEEPT, T);
		check(cudaMemsetAsync(a.err, 0, 4, ctx->stream), "cudaMemsetAsync");
		check(mesh_filter(a, ctx->stream), "mesh filter kernels");
		uint32_t tot[8] = {0, 0, 0, 0, 0, 0, 0, 0};
		check(cudaMemcpyAsync(tot, small, 32, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync totals");
		check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
		if (tot[4]) return fail(ctx, UP_ERR_CUDA, "connected components: iteration limit reached");
		const uint32_t nv = tot[0], nt = tot[1];
		mesh->vertex_count = nv;
		mesh->index_count = 3ull * nt;
		if (nt == 0) return fail(ctx, UP_ERR_EMPTY_MESH, std::string("generated empty base ") + field_word(field) + " mesh");
		if (!mesh->positions || !mesh->indices || mesh->vertex_capacity < nv || mesh->index_capacity < 3ull * nt)
			return fail(ctx, UP_ERR_CAPACITY, "mesh buffers too small");
		float *po = (float *)stage_out(ctx, B_MESH_POS, mesh->positions, (size_t)nv * 12);
		float *no = (float *)stage_out(ctx, B_MESH_NRM, mesh->normals, (size_t)nv * 12);
		uint32_t *io = (uint32_t *)stage_out(ctx, B_MESH_IDX, mesh->indices, (size_t)nt * 12);
		check(mesh_compact(a, po, no, io, ctx->stream), "mesh compaction kernels");
		finish_out(ctx, mesh->positions, po, (size_t)nv * 12);
		finish_out(ctx, mesh->normals, no, (size_t)nv * 12);
		finish_out(ctx, mesh->indices, io, (size_t)nt * 12);
		check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
		return (int)UP_OK;
	});
}

int up_image_special_to_gltf_pbr(up_context *ctx, const uint8_t *special, uint32_t width, uint32_t height, uint8_t *pbr) {
	if (!ctx || !special || !pbr || width == 0 || height == 0) return UP_ERR_INVALID_ARGUMENT;
	return guarded(ctx, "up_image_special_to_gltf_pbr", [&]() {
		set_device(ctx);
		const size_t n = (size_t)width * height;
		const uint8_t *si = (const uint8_t *)stage_in(ctx, B_IN0, special, n * 2);
		uint8_t *po = (uint8_t *)stage_out(ctx, B_OUT0, pbr, n * 3);
		check(image_pbr_run(si, width, height, po, ctx->stream), "pbr kernel");
		finish_out(ctx, pbr, po, n * 3);
		check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
		return (int)UP_OK;
	});
}

int up_image_height_to_normal(up_context *ctx, const uint8_t *height_map, uint32_t width, uint32_t height, float strength, uint8_t *normal) {
	if (!ctx || !height_map || !normal || width == 0 || height == 0 || !(strength == strength)) return UP_ERR_INVALID_ARGUMENT;
	return guarded(ctx, "up_image_height_to_normal", [&]() {
		set_device(ctx);
		const size_t n = (size_t)width * height;
		const uint8_t *hi = (const uint8_t *)stage_in(ctx, B_IN0, height_map, n);
		uint8_t *no = (uint8_t *)stage_out(ctx, B_OUT0, normal, n * 3);
		check(image_normal_run(hi, width, height, strength, no, ctx->stream), "normal-map kernel");
		finish_out(ctx, normal, no, n * 3);
		check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
		return (int)UP_OK;
	});
}

int up_sdf_param_backward(up_context *ctx, const float *points, size_t n, const float *dL_dd, float *dtheta) {
	if (!ctx || !points || !dL_dd || !dtheta || n == 0) return UP_ERR_INVALID_ARGUMENT;
	if (!ctx->synthetic) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "the parameter adjoint needs a synthetic context");
	return guarded(ctx, "up_sdf_param_backward", [&]() {
		set_device(ctx);
		const size_t nt = up_synth_theta_count(&ctx->prog);
		const float *dp = (const float *)stage_in(ctx, B_IN0, points, n * 12);
		const float *dw = (const float *)stage_in(ctx, B_W, dL_dd, n * 4);
		float *dt = (float *)stage_out(ctx, B_OUT0, dtheta, nt * 4);
		const int nb = synth_bwd_blocks(n);
		float *part = (float *)buf(ctx, B_PARTIALS, (size_t)nb * 43 * 4);
		check(launch_synth_bwd(ctx->prog, dp, n, dw, part, nb, dt, ctx->stream), "adjoint kernel");
		finish_out(ctx, dtheta, dt, nt * 4);
		check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
		return (int)UP_OK;
	});
}

// Allocation-free adjoint (see include/up_abi.h): device buffers only, no
// staging, scratch in a static device array of up_sdf.cu.
int up_sdf_param_backward_noalloc(up_context *ctx, const float *points, size_t n, const float *dL_dd, float *dtheta) {
	if (!ctx || !points || !dL_dd || !dtheta || n == 0) return UP_ERR_INVALID_ARGUMENT;
	if (!ctx->synthetic) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "the parameter adjoint needs a synthetic context");
	return guarded(ctx, "up_sdf_param_backward_noalloc", [&]() {
		set_device(ctx);
		if (!is_local(ctx, points) || !is_local(ctx, dL_dd) || !is_local(ctx, dtheta))
			return fail(ctx, UP_ERR_INVALID_ARGUMENT,
				"up_sdf_param_backward_noalloc needs device buffers of the context's GPU: it allocates nothing, so it cannot stage "
				"host memory or memory of another GPU");
		if (up_synth_theta_count(&ctx->prog) > 43)
			return fail(ctx, UP_ERR_INVALID_ARGUMENT, "parameter vector longer than the 43-entry scratch row");
		check(launch_synth_bwd_noalloc(ctx->prog, points, n, dL_dd, dtheta, ctx->noalloc_scratch, ctx->stream), "adjoint kernel (no allocation)");
		check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
		return (int)UP_OK;
	});
}

int up_texture(up_context *ctx, int purpose, const up_mesh_in *mesh, uint32_t width, uint32_t height, int dilation, up_texture_out *out) {
	if (!ctx || !mesh || !out || width == 0 || height == 0 || dilation < 0) return UP_ERR_INVALID_ARGUMENT;
	if (purpose != UP_PURPOSE_LAND && purpose != UP_PURPOSE_WATER) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "purpose must be LAND or WATER");
	if (!mesh->positions || !mesh->normals || !mesh->uvs || !mesh->indices || mesh->index_count % 3 != 0)
		return fail(ctx, UP_ERR_INVALID_ARGUMENT, "mesh needs positions, normals, uvs and a multiple of 3 indices");
	if ((uint64_t)width * height >= (1ull << 31)) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "atlas too large");
	return guarded(ctx, "up_texture", [&]() {
		set_device(ctx);
		const uint64_t V = mesh->vertex_count, I = mesh->index_count, n = (uint64_t)width * height;
		const int ach = purpose == UP_PURPOSE_WATER ? 4 : 3;
		const float *pos = (const float *)stage_in(ctx, B_TEX0, mesh->positions, V * 12);
		const float *nrm = (const float *)stage_in(ctx, B_TEX1, mesh->normals, V * 12);
		const float *uv = (const float *)stage_in(ctx, B_TEX2, mesh->uvs, V * 8);
		const uint32_t *idx = (const uint32_t *)stage_in(ctx, B_TEX3, mesh->indices, I * 4);
		int *owner = (int *)buf(ctx, B_TEX4, n * 4);
		double *tri_ia = (double *)buf(ctx, B_TEXIA, (I / 3) * 8);
		float *img0 = (float *)buf(ctx, B_TEX5, n * (ach + 3) * 4);
		float *img1 = dilation > 0 ? (float *)buf(ctx, B_TEX6, n * (ach + 3) * 4) : nullptr;
		uint8_t *a8 = (uint8_t *)stage_out(ctx, B_TEX7, out->albedo, n * ach);
		uint8_t *s8 = (uint8_t *)stage_out(ctx, B_TEX8, out->special, n * 2);
		uint8_t *h8 = (uint8_t *)stage_out(ctx, B_TEX9, out->height, n);
		float *af = (float *)stage_out(ctx, B_BATCH0, out->albedo_f32, n * ach * 4);
		float *sf = (float *)stage_out(ctx, B_BATCH1, out->special_f32, n * 8);
		float *hf = (float *)stage_out(ctx, B_BATCH2, out->height_f32, n * 4);
		check(texture_run(ctx->synthetic ? nullptr : ctx->d_modes, ctx->synthetic ? &ctx->prog : nullptr, purpose, pos, nrm, uv, idx, I,
			width, height, dilation, owner, tri_ia, img0, img1, a8, s8, h8, af, sf, hf, nullptr, ctx->stream), "texture kernels");
		finish_out(ctx, out->albedo, a8, n * ach);
		finish_out(ctx, out->special, s8, n * 2);
		finish_out(ctx, out->height, h8, n);
		finish_out(ctx, out->albedo_f32, af, n * ach * 4);
		finish_out(ctx, out->special_f32, sf, n * 8);
		finish_out(ctx, out->height_f32, hf, n * 4);
		check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
		return (int)UP_OK;
	});
}

int up_tiles(up_context *ctx, int purpose, const float *positions, const float *normals, size_t n, up_tile_out *out) {
	if (!ctx || !positions || !normals || !out || n == 0) return UP_ERR_INVALID_ARGUMENT;
	if (ctx->synthetic) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "tiles need a reference-mode context");
	if (purpose < UP_PURPOSE_LAND || purpose > UP_PURPOSE_NAVIGATION) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "bad purpose");
	return guarded(ctx, "up_tiles", [&]() {
		set_device(ctx);
		const float *p = (const float *)stage_in(ctx, B_IN0, positions, n * 12);
		const float *q = (const float *)stage_in(ctx, B_GRAD, normals, n * 12);
		float *o11 = (float *)buf(ctx, B_OUT0, n * 44);
		uint8_t *bt = (uint8_t *)buf(ctx, B_OUT1, n * 2);
		check(tiles_run(ctx->d_modes, purpose, p, q, n, o11, bt, ctx->stream), "tiles kernel");
		// one plane per field; destinations may be host or device memory
		float *dst[9] = {out->roughness, out->metallic, out->height, out->opacity, out->elevation, out->slope, out->temperature,
			out->precipitation, nullptr};
		for (int c = 0; out->albedo && c < 3; c++) // plane c -> every third float
			check(cudaMemcpy2DAsync(out->albedo + c, 3 * sizeof(float), o11 + (size_t)c * n, sizeof(float), sizeof(float), n, cudaMemcpyDefault,
				ctx->stream), "cudaMemcpy2DAsync albedo");
		for (int k = 0; k < 8; k++)
			if (dst[k]) check(cudaMemcpyAsync(dst[k], o11 + (size_t)(3 + k) * n, n * 4, cudaMemcpyDefault, ctx->stream), "cudaMemcpyAsync tiles");
		if (out->biome) check(cudaMemcpyAsync(out->biome, bt, n, cudaMemcpyDefault, ctx->stream), "cudaMemcpyAsync biome");
		if (out->type) check(cudaMemcpyAsync(out->type, bt + n, n, cudaMemcpyDefault, ctx->stream), "cudaMemcpyAsync type");
		check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
		return (int)UP_OK;
	});
}

int up_batch_run(up_context *ctx, const up_synth_program *planets, size_t nplanets, const up_chunk *chunks, size_t nchunks, up_batch_out *out) {
	if (!ctx || !planets || !chunks || !out || nplanets == 0 || nchunks == 0) return UP_ERR_INVALID_ARGUMENT;
	for (size_t i = 0; i < nplanets; i++)
		if (!valid_program(planets[i])) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "invalid planet program");
	for (size_t c = 0; c < nchunks; c++)
		if (chunks[c].planet >= nplanets || !valid_grid(&chunks[c].grid)) return fail(ctx, UP_ERR_INVALID_ARGUMENT, "invalid chunk");
	return guarded(ctx, "up_batch_run", [&]() {
		set_device(ctx);
		uint32_t ncells = 0, nquads = 0;
		std::vector<uint32_t> cc, cq;
		const float *dpos = nullptr, *dval = nullptr;
		const uint32_t *didx = nullptr;
		uint64_t nval = 0;
		bool nan = false, replayed = false;
		unsigned fault = 0;
		check(batch_execute(ctx->batch, planets, nplanets, chunks, nchunks, out->values != nullptr, ncells, nquads, cc, cq, dpos, didx, dval, nval,
			nan, replayed, fault, ctx->stream), "batch kernels");
		if (fault & 1u) return fail(ctx, UP_ERR_TIMEOUT, "batch: a grid barrier wait of the persistent launch ran out; the outputs are not valid");
		if (fault) return fail(ctx, UP_ERR_CUDA, "batch: the persistent launch's counts differ from the plan; the outputs are not valid");
		if (nan) return fail(ctx, UP_ERR_NAN, "invalid land sdf value");
		out->vertex_count = ncells;
		out->index_count = 6ull * nquads;
		if (out->chunk_vertex_offset)
			for (size_t c = 0; c <= nchunks; c++) out->chunk_vertex_offset[c] = cc[c];
		if (out->chunk_index_offset)
			for (size_t c = 0; c <= nchunks; c++) out->chunk_index_offset[c] = 6ull * cq[c];
		if (!out->positions || !out->indices || out->vertex_capacity < ncells || out->index_capacity < 6ull * nquads)
			return fail(ctx, UP_ERR_CAPACITY, "batch output buffers too small");
		if (out->values && out->values_capacity < nval) return fail(ctx, UP_ERR_CAPACITY, "batch values buffer too small");
		// host, this GPU or another GPU: unified addressing resolves the direction
		check(cudaMemcpyAsync(out->positions, dpos, (size_t)ncells * 12, cudaMemcpyDefault, ctx->stream), "cudaMemcpyAsync batch positions");
		check(cudaMemcpyAsync(out->indices, didx, (size_t)nquads * 24, cudaMemcpyDefault, ctx->stream), "cudaMemcpyAsync batch indices");
		if (out->values)
			check(cudaMemcpyAsync(out->values, dval, (size_t)nval * 4, cudaMemcpyDefault, ctx->stream), "cudaMemcpyAsync batch values");
		check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
		return (int)UP_OK;
	});
}

} // extern "C"
