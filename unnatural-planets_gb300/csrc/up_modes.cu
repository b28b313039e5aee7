// Reference-mode SDF evaluation (shapes x elevation modes).
#include "up_internal.h"
#include "up_modes_desc.h"

namespace up {

cudaError_t launch_modes_grid(const ModesDesc &, uint32_t, const GridDev &, float *, float *, float *, float *, unsigned *, cudaStream_t) {
	return cudaErrorNotSupported;
}
cudaError_t launch_modes_points(const ModesDesc &, int, const float *, uint64_t, float *, float *, unsigned *, cudaStream_t) {
	return cudaErrorNotSupported;
}
cudaError_t dc_geometry_modes(const ModesDesc &, int, const float *, const GridDev &, DcScratch &, uint32_t, uint32_t, uint32_t, float *,
	float *, uint32_t *, cudaStream_t) {
	return cudaErrorNotSupported;
}

} // namespace up
