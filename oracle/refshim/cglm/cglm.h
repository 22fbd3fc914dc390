/*
 * Minimal stand-in for the cglm header the reference includes. Only
 * glm_vec_distance is used on the hot path (src/chunkset/edit.c:221); it is
 * the Euclidean distance computed in float with sqrtf, as in cglm.
 * TEST INFRASTRUCTURE ONLY: used to compile the reference as the oracle.
 */
#ifndef VP_REFSHIM_CGLM_H
#define VP_REFSHIM_CGLM_H
#include <math.h>
static inline float glm_vec_distance(float *a, float *b)
{
	float d0 = b[0] - a[0], d1 = b[1] - a[1], d2 = b[2] - a[2];
	return sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
}
#endif
