/*
 * detmath.h — deterministic single-precision sin / cos / tan for the CPU oracle.
 *
 * TEST INFRASTRUCTURE: this header belongs to the oracle (the CPU checker). Only
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may use
 * anything under oracle/.
 *
 * The reference calls GLSL sin/cos/tan in toConcentricDisk (src/shader/math.glsl:23-39)
 * and pinholeCameraSampleRay (src/shader/camera.glsl:28-42). Their results are
 * implementation-defined, so this project defines them once, by a published method,
 * and every implementation (compiled reference, oracle restatement, CUDA kernels)
 * evaluates exactly the same float operations:
 *   - Cody-Waite argument reduction by pi/2 (Cody & Waite, "Software Manual for the
 *     Elementary Functions", 1980) with pi/2 split into three parts: P1 and P2 carry
 *     12 significant bits each, so k*P1 and k*P2 are exact for the small quadrant
 *     counts that occur (|k| < 2^11), and P3 is the float nearest the remainder.
 *   - Taylor polynomials of sin (to r^11) and cos (to r^10) on |r| <= pi/4, evaluated
 *     by Horner's rule. Coefficients are the floats nearest +-1/k!.
 * Every operation is a separate IEEE-754 binary32 multiply or add (the oracle is built
 * with -ffp-contract=off; the CUDA kernels with --fmad=false), so results are
 * bit-identical on x86-64, aarch64 and sm_103a. Accuracy is about 1-2 ulp on the
 * ranges used here (|x| <= 3*pi/4).
 */
#ifndef GRIS_ORACLE_DETMATH_H
#define GRIS_ORACLE_DETMATH_H

static inline float oracle_det_rint(float x) { return __builtin_rintf(x); }

static inline void oracle_det_sincosf(float x, float* s, float* c) {
    float kf = oracle_det_rint(x * 0.636619746685028076f);
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

static inline float oracle_det_sinf(float x) { float s, c; oracle_det_sincosf(x, &s, &c); return s; }
static inline float oracle_det_cosf(float x) { float s, c; oracle_det_sincosf(x, &s, &c); return c; }
static inline float oracle_det_tanf(float x) { float s, c; oracle_det_sincosf(x, &s, &c); return s / c; }

/* x^y as the library's gris_det_powf (vulkan-restir-pt_gb300/csrc/detmath.h): 2^(y log2 x) with
 * log2 from the atanh series of the mantissa in [sqrt(1/2), sqrt(2)) and 2^f from the Taylor
 * series of e^(f ln 2); restated here so the oracle stays independent of the product's headers. */
static inline unsigned oracle_dm_bits(float x) { unsigned u; __builtin_memcpy(&u, &x, 4); return u; }
static inline float oracle_dm_float(unsigned u) { float x; __builtin_memcpy(&x, &u, 4); return x; }
static inline float oracle_dm_pow2i(int n) { return oracle_dm_float((unsigned)(n + 127) << 23); }
static inline float oracle_det_powf(float x, float y) {
    if (!(x >= 0.0f)) return oracle_dm_float(0x7fc00000u);
    if (x == 0.0f) return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : oracle_dm_float(0x7f800000u));
    if (x > 3.4028235e38f) return y > 0.0f ? x : (y == 0.0f ? 1.0f : 0.0f);
    int e = 0;
    if (x < 1.17549435e-38f) { x = x * 16777216.0f; e = -24; }
    unsigned b = oracle_dm_bits(x);
    e += (int)((b >> 23) & 0xffu) - 126;
    float m = oracle_dm_float((b & 0x007fffffu) | 0x3f000000u);
    if (m < 0.707106769f) { m = m * 2.0f; e -= 1; }
    float t = (m - 1.0f) / (m + 1.0f), t2 = t * t;
    float p = 0.111111112f;
    p = p * t2 + 0.142857149f;
    p = p * t2 + 0.200000003f;
    p = p * t2 + 0.333333343f;
    p = p * t2 + 1.0f;
    float z = y * ((float)e + ((2.0f * t) * p) * 1.44269502f);
    if (z > 128.0f) return oracle_dm_float(0x7f800000u);
    if (z < -150.0f) return 0.0f;
    float n = __builtin_rintf(z);
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
    if (k > 127) return q * oracle_dm_pow2i(127) * oracle_dm_pow2i(k - 127);
    if (k < -126) return q * oracle_dm_pow2i(-126) * oracle_dm_pow2i(k + 126);
    return q * oracle_dm_pow2i(k);
}

#endif
