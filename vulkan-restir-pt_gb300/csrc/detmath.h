/*
 * detmath.h — deterministic sin / cos / tan (binary32) and exp (binary64) for grisrt.
 *
 * The shaders of the reference call GLSL sin/cos/tan (toConcentricDisk,
 * src/shader/math.glsl:23-39; pinholeCameraSampleRay, src/shader/camera.glsl:28-42),
 * whose results are implementation-defined. grisrt defines them once, by a published
 * method, so the CUDA kernels, the host and any CPU checker that follows the same
 * definition agree bit for bit:
 *   Cody-Waite reduction by pi/2 (Cody & Waite, "Software Manual for the Elementary
 *   Functions", 1980; pi/2 split into P1, P2 of 12 significant bits and P3) followed by
 *   the Taylor polynomials of sin (to r^11) and cos (to r^10) on |r| <= pi/4 in Horner form.
 * Each step is one IEEE-754 operation: device code is compiled with --fmad=false and host
 * code with -ffp-contract=off, so no multiply-add is fused.
 *
 * gris_det_exp (binary64, host only) serves the scene generators: reduction by ln 2
 * (two-part constant) and a degree-13 Taylor polynomial, so generated scenes are
 * bit-identical on x86-64 and aarch64 hosts.
 */
#ifndef GRISRT_DETMATH_H
#define GRISRT_DETMATH_H

#ifdef __CUDACC__
#define GRIS_DM_HD __host__ __device__ __forceinline__
#else
#define GRIS_DM_HD static inline
#endif

GRIS_DM_HD void gris_det_sincosf(float x, float* s, float* c) {
#ifdef __CUDA_ARCH__
    float kf = rintf(x * 0.636619746685028076f);
#else
    float kf = __builtin_rintf(x * 0.636619746685028076f);
#endif
    float r = x - kf * 1.5703125f;
    r = r - kf * 4.837512969970703125e-4f;
    r = r - kf * 7.549790126404332e-8f;
    float r2 = r * r;
    float ps = -2.50521079e-8f;
    ps = ps * r2 + 2.75573188e-6f;
    ps = ps * r2 - 1.98412701e-4f;
    ps = ps * r2 + 8.33333377e-3f;
    ps = ps * r2 - 0.166666672f;
    float sn = r + (r * r2) * ps;
    float pc = -2.75573200e-7f;
    pc = pc * r2 + 2.48015876e-5f;
    pc = pc * r2 - 1.38888892e-3f;
    pc = pc * r2 + 4.16666679e-2f;
    pc = pc * r2 - 0.5f;
    float cs = 1.0f + r2 * pc;
    int q = ((int)kf) & 3;
    if (q == 0) { *s = sn; *c = cs; }
    else if (q == 1) { *s = cs; *c = -sn; }
    else if (q == 2) { *s = -sn; *c = -cs; }
    else { *s = -cs; *c = sn; }
}
GRIS_DM_HD float gris_det_sinf(float x) { float s, c; gris_det_sincosf(x, &s, &c); return s; }
GRIS_DM_HD float gris_det_cosf(float x) { float s, c; gris_det_sincosf(x, &s, &c); return c; }
GRIS_DM_HD float gris_det_tanf(float x) { float s, c; gris_det_sincosf(x, &s, &c); return s / c; }

#ifndef __CUDA_ARCH__
static inline double gris_det_exp(double x) {
    double k = __builtin_rint(x * 1.4426950408889634);
    double r = (x - k * 0.693145751953125) - k * 1.4286068203094172321e-6;
    double p = 1.0 / 6227020800.0;
    const double inv_fact[13] = {1.0 / 479001600.0, 1.0 / 39916800.0, 1.0 / 3628800.0, 1.0 / 362880.0,
                                 1.0 / 40320.0, 1.0 / 5040.0, 1.0 / 720.0, 1.0 / 120.0, 1.0 / 24.0,
                                 1.0 / 6.0, 0.5, 1.0, 1.0};
    for (int i = 0; i < 13; i++) p = p * r + inv_fact[i];
    return __builtin_ldexp(p, (int)k);
}
#endif

#endif
