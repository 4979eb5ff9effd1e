/* svo_trig.h — the engine's float restatements of sin, cos, atan and acos, as plain C (TEST
 * INFRASTRUCTURE ONLY: the oracle's copy of the rule the CUDA kernels follow, also used by the reference
 * harness when it is built to evaluate GLSL's transcendental built-ins with that rule).  Every operation
 * is a separately rounded binary32 operation: compile with -ffp-contract=off.
 *
 *   sincos_2pi(u): sin and cos of 2 pi u, u in [0, 1]: quadrant split, then the Taylor polynomials of
 *                  sin (to a^13) and cos (to a^12) on [0, pi/2) in Horner form;
 *   svo_sincos(x): sin and cos of x radians via u = frac(x / (2 pi));
 *   svo_atan2:     two half-angle reductions z / (1 + sqrt(1 + z^2)), then the Taylor series of atan to
 *                  z^15, with the octant identities; 0 for (0, 0);
 *   svo_acos(x):   atan2(sqrt((1 - x)(1 + x)), x) on x clamped to [-1, 1]. */
#ifndef SVO_TRIG_H
#define SVO_TRIG_H

#ifdef __cplusplus
#include <cmath>
#define SVO_FLOORF std::floor
#define SVO_SQRTF std::sqrt
#define SVO_FABSF std::fabs
#define SVO_FMINF std::fmin
#define SVO_FMAXF std::fmax
#else
#include <math.h>
#define SVO_FLOORF floorf
#define SVO_SQRTF sqrtf
#define SVO_FABSF fabsf
#define SVO_FMINF fminf
#define SVO_FMAXF fmaxf
#endif

static inline void sincos_2pi(float u, float *s_out, float *c_out) {
	float q4 = u * 4.0f;
	int q = (int)q4;
	float r = q4 - (float)q;
	float a = r * 1.57079632679489662f;
	float a2 = a * a;
	float s = 1.0f / 6227020800.0f;
	s = s * a2 + -1.0f / 39916800.0f;
	s = s * a2 + 1.0f / 362880.0f;
	s = s * a2 + -1.0f / 5040.0f;
	s = s * a2 + 1.0f / 120.0f;
	s = s * a2 + -1.0f / 6.0f;
	s = s * a2 + 1.0f;
	s = s * a;
	float c = 1.0f / 479001600.0f;
	c = c * a2 + -1.0f / 3628800.0f;
	c = c * a2 + 1.0f / 40320.0f;
	c = c * a2 + -1.0f / 720.0f;
	c = c * a2 + 1.0f / 24.0f;
	c = c * a2 + -0.5f;
	c = c * a2 + 1.0f;
	switch (q & 3) {
	case 0: *s_out = s; *c_out = c; break;
	case 1: *s_out = c; *c_out = -s; break;
	case 2: *s_out = -s; *c_out = -c; break;
	default: *s_out = -c; *c_out = s; break;
	}
}

static inline void svo_sincos(float x, float *s_out, float *c_out) {
	float u = x * 0.159154943091895336f; /* 1 / (2 pi) */
	u = u - SVO_FLOORF(u);
	sincos_2pi(u, s_out, c_out);
}

static inline float svo_atan_unit(float z) {
	z = z / (1.0f + SVO_SQRTF(1.0f + z * z));
	z = z / (1.0f + SVO_SQRTF(1.0f + z * z));
	float z2 = z * z;
	float p = -1.0f / 15.0f;
	p = p * z2 + 1.0f / 13.0f;
	p = p * z2 + -1.0f / 11.0f;
	p = p * z2 + 1.0f / 9.0f;
	p = p * z2 + -1.0f / 7.0f;
	p = p * z2 + 1.0f / 5.0f;
	p = p * z2 + -1.0f / 3.0f;
	p = p * z2 + 1.0f;
	return 4.0f * (z * p);
}

static inline float svo_atan2(float y, float x) {
	float ax = SVO_FABSF(x), ay = SVO_FABSF(y);
	if (ax == 0.0f && ay == 0.0f)
		return 0.0f;
	float a = ay <= ax ? svo_atan_unit(ay / ax) : 1.57079632679489662f - svo_atan_unit(ax / ay);
	if (x < 0.0f)
		a = 3.14159265358979323846f - a;
	return y < 0.0f ? -a : a;
}

static inline float svo_acos(float x) {
	x = SVO_FMINF(SVO_FMAXF(x, -1.0f), 1.0f);
	return svo_atan2(SVO_SQRTF((1.0f - x) * (1.0f + x)), x);
}

#endif
