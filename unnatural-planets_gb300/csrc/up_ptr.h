// Where a caller's buffer lives, relative to the GPU of a context. Pure
// logic on the fields of cudaPointerAttributes, kept free of CUDA headers so
// that the host tests can check it without a GPU.
#pragma once

namespace up {

enum PtrKind {
	PTR_HOST = 0,         // pageable or page-locked host memory: copied through scratch
	PTR_LOCAL = 1,        // device memory of the context's GPU, or managed memory: used in place
	PTR_OTHER_DEVICE = 2  // device memory of another GPU: copied through scratch (never read
	                      // by a kernel of this context, which would be a peer access)
};

// attr_type: cudaPointerAttributes::type (0 unregistered, 1 host, 2 device,
// 3 managed); attr_device: cudaPointerAttributes::device; ctx_device: the
// context's GPU. query_ok: cudaPointerGetAttributes succeeded.
inline PtrKind ptr_kind(bool query_ok, int attr_type, int attr_device, int ctx_device) {
	if (!query_ok) return PTR_HOST;
	if (attr_type == 3) return PTR_LOCAL;
	if (attr_type == 2) return attr_device == ctx_device ? PTR_LOCAL : PTR_OTHER_DEVICE;
	return PTR_HOST;
}

} // namespace up
