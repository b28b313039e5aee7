// Texture post-processing after up_texture, as the reference's generator does
// before saving (sources/generator.cpp:135-139):
//   imageConvertSpecialToGltfPbr: special (roughness, metallic) -> RGB8
//     (255, roughness, metallic), the glTF metallicRoughness convention
//     (G = roughness, B = metalness; R left at 255, no occlusion);
//   imageConvertHeigthToNormal(height, strength): h = height / 255,
//     n = normalize(-s dh/dx, -s dh/dy, 1) with central differences in texels
//     (one-sided at the image border), stored (n + 1) / 2 as RGB8.
// Both are byte stencils bound by HBM: one thread per texel, coalesced rows.
#include "up_internal.h"

namespace up {

__global__ void img_pbr_kernel(const uint8_t *__restrict__ special, uint64_t n, uint8_t *__restrict__ pbr) {
	for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
		pbr[3 * i] = 255;
		pbr[3 * i + 1] = special[2 * i];
		pbr[3 * i + 2] = special[2 * i + 1];
	}
}

__device__ __forceinline__ uint8_t unit_to_u8(float v) {
	const float c = fminf(fmaxf(v, 0.f), 1.f);
	return (uint8_t)(c * 255.f + 0.5f);
}

__global__ void img_normal_kernel(const uint8_t *__restrict__ h, uint32_t W, uint32_t H, float strength, uint8_t *__restrict__ out) {
	const uint64_t n = (uint64_t)W * H;
	for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
		const uint32_t y = (uint32_t)(i / W), x = (uint32_t)(i - (uint64_t)y * W);
		const uint8_t *row = h + (uint64_t)y * W;
		float dx = 0.f, dy = 0.f;
		if (W > 1) {
			if (x == 0) dx = (float)row[1] - (float)row[0];
			else if (x == W - 1) dx = (float)row[W - 1] - (float)row[W - 2];
			else dx = 0.5f * ((float)row[x + 1] - (float)row[x - 1]);
		}
		if (H > 1) {
			if (y == 0) dy = (float)h[W + x] - (float)h[x];
			else if (y == H - 1) dy = (float)h[(uint64_t)(H - 1) * W + x] - (float)h[(uint64_t)(H - 2) * W + x];
			else dy = 0.5f * ((float)h[(uint64_t)(y + 1) * W + x] - (float)h[(uint64_t)(y - 1) * W + x]);
		}
		const float nx = -strength * dx * (1.f / 255.f), ny = -strength * dy * (1.f / 255.f);
		const float il = 1.f / sqrtf(nx * nx + ny * ny + 1.f);
		out[3 * i] = unit_to_u8(nx * il * 0.5f + 0.5f);
		out[3 * i + 1] = unit_to_u8(ny * il * 0.5f + 0.5f);
		out[3 * i + 2] = unit_to_u8(il * 0.5f + 0.5f);
	}
}

static unsigned img_grid(const void *k, uint64_t n) {
	const int b = persistent_blocks(k, 256);
	const uint64_t need = (n + 255) / 256;
	return (unsigned)(need < (uint64_t)b ? (need ? need : 1) : (uint64_t)b);
}

cudaError_t image_pbr_run(const uint8_t *special, uint32_t W, uint32_t H, uint8_t *pbr, cudaStream_t s) {
	const uint64_t n = (uint64_t)W * H;
	img_pbr_kernel<<<img_grid((const void *)img_pbr_kernel, n), 256, 0, s>>>(special, n, pbr);
	return cudaGetLastError();
}

cudaError_t image_normal_run(const uint8_t *height, uint32_t W, uint32_t H, float strength, uint8_t *normal, cudaStream_t s) {
	const uint64_t n = (uint64_t)W * H;
	img_normal_kernel<<<img_grid((const void *)img_normal_kernel, n), 256, 0, s>>>(height, W, H, strength, normal);
	return cudaGetLastError();
}

} // namespace up
