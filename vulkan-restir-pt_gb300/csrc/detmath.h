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
 * gris_det_powf (binary32) serves the gamma correction of the post-processing pass (GLSL pow,
 * post_proc.frag:40-42): x^y = 2^(y log2 x) with log2 from the atanh series
 * ln m = 2 (t + t^3/3 + ... + t^9/9), t = (m - 1) / (m + 1), m in [sqrt(1/2), sqrt(2)), and 2^f
 * (|f| <= 1/2) from the Taylor series of e^(f ln 2) to degree 7; the exponent split and scaling
 * are exact bit operations. Negative or NaN x gives NaN, x = 0 gives 0 (y > 0).
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

GRIS_DM_HD unsigned gris_dm_bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    unsigned u; __builtin_memcpy(&u, &x, 4); return u;
#endif
}
GRIS_DM_HD float gris_dm_float(unsigned u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x; __builtin_memcpy(&x, &u, 4); return x;
#endif
}
/* 2^n for n in [-126, 127] (exact); the caller keeps n in range */
GRIS_DM_HD float gris_dm_pow2i(int n) { return gris_dm_float((unsigned)(n + 127) << 23); }

GRIS_DM_HD float gris_det_powf(float x, float y) {
    if (!(x >= 0.0f)) return gris_dm_float(0x7fc00000u);   /* negative or NaN */
    if (x == 0.0f) return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : gris_dm_float(0x7f800000u));
    if (x > 3.4028235e38f) return y > 0.0f ? x : (y == 0.0f ? 1.0f : 0.0f);
    int e = 0;
    if (x < 1.17549435e-38f) { x = x * 16777216.0f; e = -24; }   /* subnormal: scale by 2^24 (exact) */
    unsigned b = gris_dm_bits(x);
    e += (int)((b >> 23) & 0xffu) - 126;
    float m = gris_dm_float((b & 0x007fffffu) | 0x3f000000u);   /* [0.5, 1) */
    if (m < 0.707106769f) { m = m * 2.0f; e -= 1; }
    float t = (m - 1.0f) / (m + 1.0f);
    float t2 = t * t;
    float p = 0.111111112f;
    p = p * t2 + 0.142857149f;
    p = p * t2 + 0.200000003f;
    p = p * t2 + 0.333333343f;
    p = p * t2 + 1.0f;
    float l2 = (float)e + ((2.0f * t) * p) * 1.44269502f;   /* log2 x */
    float z = y * l2;
    if (z > 128.0f) return gris_dm_float(0x7f800000u);
    if (z < -150.0f) return 0.0f;
#ifdef __CUDA_ARCH__
    float n = rintf(z);
#else
    float n = __builtin_rintf(z);
#endif
    float r = (z - n) * 0.693147182f;
    float q = 1.98412701e-4f;
    q = q * r + 1.38888892e-3f;
    q = q * r + 8.33333377e-3f;
    q = q * r + 4.16666679e-2f;
    q = q * r + 0.166666672f;
    q = q * r + 0.5f;
    q = q * r + 1.0f;
    q = q * r + 1.0f;
    int k = (int)n;
    if (k > 127) return q * gris_dm_pow2i(127) * gris_dm_pow2i(k - 127);
    if (k < -126) return q * gris_dm_pow2i(-126) * gris_dm_pow2i(k + 126);
    return q * gris_dm_pow2i(k);
}

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
