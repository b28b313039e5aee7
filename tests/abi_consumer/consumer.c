/* A C99 consumer of include/up_abi.h: the header compiles as C and the
 * library links from C. Evaluates a synthetic sphere at a few points and
 * checks the values against |p| - R (no noise layer). Exits 0 on success,
 * 3 when no CUDA device is present. Test harness: built and run by
 * tests/test_abi_consumer.py. */
#include "up_abi.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

int main(void) {
	up_synth_program p;
	up_context *ctx = NULL;
	float xyz[12] = {2.f, 0.f, 0.f, 0.f, 0.5f, 0.f, 0.f, 0.f, -1.25f, 0.3f, 0.4f, 0.f};
	float d[4];
	int st, i, bad = 0;
	memset(&p, 0, sizeof(p));
	p.base = UP_BASE_SPHERE;
	p.param[0] = 1.0f;
	p.n_layers = 0;
	st = up_context_create_synthetic(&p, &ctx);
	if (st != UP_OK) {
		fprintf(stderr, "up_context_create_synthetic: %s\n", up_status_string(st));
		return st == UP_ERR_NO_DEVICE ? 3 : 1;
	}
	st = up_sdf_eval_points(ctx, UP_FIELD_LAND, xyz, 4, d, NULL);
	for (i = 0; i < 4; i++) {
		const float r = sqrtf(xyz[3 * i] * xyz[3 * i] + xyz[3 * i + 1] * xyz[3 * i + 1] + xyz[3 * i + 2] * xyz[3 * i + 2]);
		bad += fabsf(d[i] - (r - 1.0f)) > 1e-6f;
	}
	up_context_destroy(ctx);
	printf("c consumer: status %d, %d mismatches\n", st, bad);
	return st == UP_OK && bad == 0 ? 0 : 1;
}
