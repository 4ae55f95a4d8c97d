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

#endif
