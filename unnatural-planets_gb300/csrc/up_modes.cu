// Kernels of the reference modes (the planet description is read from device
// memory, uploaded once per context): grid sampling of up to three fields in one
// pass (land, water, navigation share the shape and elevation evaluation),
// scattered points with optional analytic gradient, and the contouring
// Hermite/QEF instantiation.
//
// Replaces the three MarchingCubes::updateByPosition passes per planet
// (sources/meshGeneration.cpp:39, called at :50, :60 and :103) and the
// per-point terrainSdf* callbacks (sources/modesConfiguration.cpp:230-279).
#include "up_contour.cuh"
#include "up_modes.cuh"

namespace up {

__device__ __forceinline__ float mgrid_coord(const GridDev &g, int a, uint32_t i) {
	return __fadd_rn(__fmul_rn((float)i, g.step[a]), g.lo[a]);
}

// land = s - e/10, water = s, navigation = s - max(e/10, 0)
template<class S>
__device__ __forceinline__ void fields_of(const ModesDesc &M, uint32_t mask, V3S<S> p, S out[3]) {
	const S s = shape_eval(M, p);
	S e = mk<S>(0.f);
	if (mask & 5u) e = elevation_eval(M, p) * 0.1f;
	out[0] = s - e;
	out[1] = s;
	out[2] = s - s_max(e, mk<S>(0.f));
}

// band > 0 (one field, no gradient): samples with |shape| > band take the
// shape value (narrow band of contouring, modes_contour_band)
template<bool GRAD>
__global__ void __launch_bounds__(128) modes_grid_kernel(const ModesDesc *__restrict__ Mp, uint32_t mask, const GridDev g, float *__restrict__ o0,
	float *__restrict__ o1, float *__restrict__ o2, float *__restrict__ grad, unsigned *__restrict__ nanflag, float band) {
	const uint32_t nx = g.n[0], ny = g.n[1];
	const uint64_t plane = (uint64_t)nx * ny * g.n[2];
	const uint32_t total = (uint32_t)plane;
	const ModesDesc &M = *Mp;
	const int gf = (mask & 1u) ? 0 : ((mask & 2u) ? 1 : 2); // gradient of the lowest selected field
	bool bad = false;
	for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
		const uint32_t i = idx % nx, r = idx / nx, j = r % ny, k = r / ny;
		const V3f p = v3(mgrid_coord(g, 0, i), mgrid_coord(g, 1, j), mgrid_coord(g, 2, k + g.k0));
		float v[3];
		if (GRAD) {
			Df f[3];
			fields_of(M, mask, dual_point(p), f);
			v[0] = f[0].v; v[1] = f[1].v; v[2] = f[2].v;
			grad[idx] = f[gf].d.x;
			grad[plane + idx] = f[gf].d.y;
			grad[2 * plane + idx] = f[gf].d.z;
		} else {
			const float sh = band > 0.f ? shape_eval(M, vs(p.x, p.y, p.z)) : 0.f;
			if (band > 0.f && fabsf(sh) > band) v[0] = v[1] = v[2] = sh;
			else fields_of(M, mask, vs(p.x, p.y, p.z), v);
		}
		if (mask & 1u) { o0[idx] = v[0]; bad |= isnan(v[0]); }
		if (mask & 2u) { o1[idx] = v[1]; bad |= isnan(v[1]); }
		if (mask & 4u) { o2[idx] = v[2]; bad |= isnan(v[2]); }
	}
	if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(nanflag, 1u);
}

template<bool GRAD>
__global__ void __launch_bounds__(128) modes_points_kernel(const ModesDesc *__restrict__ Mp, int field, const float *__restrict__ xyz, uint64_t n,
	float *__restrict__ out, float *__restrict__ grad, unsigned *__restrict__ nanflag) {
	const ModesDesc &M = *Mp;
	bool bad = false;
	for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (uint64_t)gridDim.x * blockDim.x) {
		const V3f p = v3(xyz[3 * idx], xyz[3 * idx + 1], xyz[3 * idx + 2]);
		float v;
		if (GRAD) {
			const Df f = field_eval(M, field, dual_point(p));
			v = f.v;
			grad[3 * idx] = f.d.x;
			grad[3 * idx + 1] = f.d.y;
			grad[3 * idx + 2] = f.d.z;
		} else {
			v = field_eval(M, field, vs(p.x, p.y, p.z));
		}
		out[idx] = v;
		bad |= isnan(v);
	}
	if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(nanflag, 1u);
}

template<class K, class... A>
static cudaError_t launch_p(K kernel, uint64_t work, cudaStream_t s, A... args) {
	const int threads = 128;
	int blocks = persistent_blocks((const void *)kernel, threads);
	const uint64_t need = (work + threads - 1) / threads;
	if ((uint64_t)blocks > need) blocks = (int)(need > 0 ? need : 1);
	kernel<<<blocks, threads, 0, s>>>(args...);
	return cudaGetLastError();
}

cudaError_t launch_modes_grid(const ModesDesc *M, uint32_t mask, const GridDev &g, float *o0, float *o1, float *o2, float *grad, unsigned *nanflag,
	cudaStream_t s, float band) {
	const uint64_t n = (uint64_t)g.n[0] * g.n[1] * g.n[2];
	if (grad) return launch_p(modes_grid_kernel<true>, n, s, M, mask, g, o0, o1, o2, grad, nanflag, 0.f);
	return launch_p(modes_grid_kernel<false>, n, s, M, mask, g, o0, o1, o2, grad, nanflag, band);
}

cudaError_t launch_modes_points(const ModesDesc *M, int field, const float *xyz, uint64_t n, float *d, float *grad, unsigned *nanflag, cudaStream_t s) {
	if (grad) return launch_p(modes_points_kernel<true>, n, s, M, field, xyz, n, d, grad, nanflag);
	return launch_p(modes_points_kernel<false>, n, s, M, field, xyz, n, d, grad, nanflag);
}

struct ModesEvalF {
	const ModesDesc *M;
	int field;
	__device__ __forceinline__ NG operator()(V3f p) const {
		const Df f = field_eval(*M, field, dual_point(p));
		return ng(f.v, f.d);
	}
};

cudaError_t dc_geometry_modes(const ModesDesc *M, int field, const float *d, const GridDev &g, DcScratch &S, uint32_t ncells, uint32_t nedges,
	uint32_t nquads, float *pos, float *nrm, uint32_t *idx, cudaStream_t s) {
	ModesEvalF ev{M, field};
	return dc_geometry_t(ev, d, g, S, ncells, nedges, nquads, pos, nrm, idx, s);
}

} // namespace up
