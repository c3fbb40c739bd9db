/*
 * Scalar stand-in for the handful of AArch64 NEON intrinsics that the reference's CPU
 * kernels use, so that those kernels compile unmodified on an x86_64 host (test
 * infrastructure only: the oracle and the golden-vector generator use it; nothing on the
 * product path includes it).
 *
 * Semantics follow the Arm C Language Extensions definitions lane by lane:
 *   vfmaq_n_f32 / vfmaq_laneq_f32 : fused multiply-add per lane (one rounding)  -> fmaf
 *   vmlaq_f32                      : a + b*c per lane; like GCC's own header this is
 *                                    written as a plain expression, so -ffp-contract
 *                                    decides whether it is fused, exactly as on Arm.
 *   vadd_f32 / vpadd_f32           : lane-wise add / pairwise add
 * Used by: SDMM.cpp (vld1q_f32, vst1q_f32, vfmaq_n_f32, vfmaq_laneq_f32),
 *          SpMV.cpp (vdupq_n_f32, vmlaq_f32, vget_high/low_f32, vadd_f32, vpadd_f32,
 *                    vget_lane_f32), gcn/pytorch-custom/spmm.cpp (vld1q_f32, vfmaq_n_f32).
 */
#ifndef ARMSPARSE_ORACLE_NEON_SHIM_H
#define ARMSPARSE_ORACLE_NEON_SHIM_H

#include <math.h>

typedef float float32_t;
typedef struct { float v[4]; } float32x4_t;
typedef struct { float v[2]; } float32x2_t;

static inline float32x4_t vld1q_f32(const float32_t *p) {
    float32x4_t r; r.v[0] = p[0]; r.v[1] = p[1]; r.v[2] = p[2]; r.v[3] = p[3]; return r;
}
static inline void vst1q_f32(float32_t *p, float32x4_t a) {
    p[0] = a.v[0]; p[1] = a.v[1]; p[2] = a.v[2]; p[3] = a.v[3];
}
static inline float32x4_t vdupq_n_f32(float32_t x) {
    float32x4_t r; r.v[0] = r.v[1] = r.v[2] = r.v[3] = x; return r;
}
static inline float32x4_t vmovq_n_f32(float32_t x) { return vdupq_n_f32(x); }
/* a + b * n, fused per lane */
static inline float32x4_t vfmaq_n_f32(float32x4_t a, float32x4_t b, float32_t n) {
    float32x4_t r;
    for (int i = 0; i < 4; ++i) r.v[i] = fmaf(b.v[i], n, a.v[i]);
    return r;
}
/* a + b * v[lane], fused per lane */
static inline float32x4_t vfmaq_laneq_f32(float32x4_t a, float32x4_t b, float32x4_t v, int lane) {
    return vfmaq_n_f32(a, b, v.v[lane]);
}
/* a + b * c per lane, written as an expression (contraction decided by the compiler) */
static inline float32x4_t vmlaq_f32(float32x4_t a, float32x4_t b, float32x4_t c) {
    float32x4_t r;
    for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] + b.v[i] * c.v[i];
    return r;
}
static inline float32x4_t vmulq_n_f32(float32x4_t a, float32_t n) {
    float32x4_t r;
    for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] * n;
    return r;
}
static inline float32x2_t vget_high_f32(float32x4_t a) {
    float32x2_t r; r.v[0] = a.v[2]; r.v[1] = a.v[3]; return r;
}
static inline float32x2_t vget_low_f32(float32x4_t a) {
    float32x2_t r; r.v[0] = a.v[0]; r.v[1] = a.v[1]; return r;
}
static inline float32x2_t vadd_f32(float32x2_t a, float32x2_t b) {
    float32x2_t r; r.v[0] = a.v[0] + b.v[0]; r.v[1] = a.v[1] + b.v[1]; return r;
}
static inline float32x2_t vpadd_f32(float32x2_t a, float32x2_t b) {
    float32x2_t r; r.v[0] = a.v[0] + a.v[1]; r.v[1] = b.v[0] + b.v[1]; return r;
}
static inline float32_t vget_lane_f32(float32x2_t a, int lane) { return a.v[lane]; }

#endif
