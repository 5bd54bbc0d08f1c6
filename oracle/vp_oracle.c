/*
 * TEST INFRASTRUCTURE ONLY — the oracle.  Nothing in the voxelproj_gb300
 * package loads or calls this file; only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg do, as the reference for parity or as the
 * timed CPU baseline.
 *
 * CPU restatement of the reference voxelproj exact-trapezoid projector pair,
 * written from its mathematics:
 *   - per-angle constants a, b, h = 1/(a+b)     sp_backward_z0.cuh:45-58,
 *                                               sp_forward_z0.cuh:136-149
 *   - trapezoid CDF (FP64 form)                 projection_common.cuh:61-85
 *   - trapezoid CDF (FP32 form)                 projection_common.cuh:139-166
 *   - detector coordinate and 3-bin rule        sp_backward_z0.cuh:24-26, 71-95
 *   - index maps z_order 0                      sp_forward_z0.cuh:127, sp_backward_z0.cuh:97
 *   - index maps z_order 2                      sp_forward_z2.cuh:115, sp_backward_z2.cuh:98
 *   - accumulate into the output                sp_forward_z0.cuh:167, sp_backward_z0.cuh:98
 * Both directions are voxel-driven (scatter for A, gather for A^T), so the
 * FP64 A is by construction the exact transpose of the FP64 A^T.
 *
 * FP64 operator (accuracy reference): float32 inputs and angles promoted to
 * double, outputs in double into a compact array laid out (n_h, n_ang, PX)
 * for A and (n_h, SY, SX) for A^T, for the heights listed in h_list (all
 * heights 0..H-1 when h_list is NULL).  The output is accumulated into.
 *
 * FP32 operator (timed CPU baseline): the same operator in float with libm
 * trig, OpenMP over angles (A) or volume rows (A^T), accumulated in place into
 * arrays in the caller's z_order layout.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define VPO_API __attribute__((visibility("default")))

/* ---------------------------------------------------------------- FP64 --- */

typedef struct {
  double c, s, a, b, ymax;
} ang64;

static ang64 angle_params64(float phi) {
  ang64 k;
  k.c = cos((double)phi);
  k.s = sin((double)phi);
  const double cms = fabs(0.5 * (k.c - k.s));
  const double cps = fabs(0.5 * (k.c + k.s));
  k.a = cms < cps ? cms : cps;
  k.b = cms < cps ? cps : cms;
  k.ymax = 1.0 / (k.a + k.b);
  return k;
}

/* projection_common.cuh:61-85 (dpiece_wise_integrated). */
static double cdf64(double x, double a, double b, double ymax) {
  const double coeff = 0.5 * ymax;
  if (x <= -b) return 0.0;
  if (x < -a) return coeff * (x + b) * (x + b) / (b - a);
  if (x < a) return coeff * (b + a) + ymax * x;
  if (x < b) return coeff * (b - x) * (b - x) / (a - b) + 1.0;
  return 1.0;
}

/* sp_backward_z0.cuh:84-91 in FP64: r = round-half-even(xp), weights of
 * bins r-1, r, r+1. */
static void weights64(double xp, const ang64* k, int* r, double w[3]) {
  const double rr = nearbyint(xp);
  const double xv = rr - xp;
  const double v1 = cdf64(xv - 0.5, k->a, k->b, k->ymax);
  const double v2 = cdf64(xv + 0.5, k->a, k->b, k->ymax);
  *r = (int)rr;
  w[0] = v1;
  w[1] = v2 - v1;
  w[2] = 1.0 - v2;
}

static inline size_t xidx(int z_order, int SY, int SX, int Hx, int yi, int xi, int h) {
  return z_order == 0 ? ((size_t)yi * SX + xi) * Hx + h : ((size_t)h * SY + yi) * SX + xi;
}
static inline size_t yidx(int z_order, int n_ang, int PX, int Hy, int a, int p, int h) {
  return z_order == 0 ? ((size_t)a * PX + p) * Hy + h : ((size_t)h * n_ang + a) * PX + p;
}

VPO_API void vpo_angle_params_f64(float phi, double out[5]) {
  const ang64 k = angle_params64(phi);
  out[0] = k.c;
  out[1] = k.s;
  out[2] = k.a;
  out[3] = k.b;
  out[4] = k.ymax;
}

/* Weights of one voxel at detector coordinate xp for angle phi. */
VPO_API int vpo_weights_f64(float phi, double xp, double w[3]) {
  const ang64 k = angle_params64(phi);
  int r;
  weights64(xp, &k, &r, w);
  return r;
}

/* y_out (n_h, n_ang, PX) += A x for the listed heights (FP64).
 * x is float32 in z_order layout: z0 (SY, SX, Hx), z2 (Hx, SY, SX). */
VPO_API void vpo_forward_f64(const float* x, int z_order, int SY, int SX, int Hx,
                             const float* angles, int n_ang, int PX, const int* h_list, int n_h,
                             double* y_out) {
  const double xc = 0.5 * (SX - 1), yc = 0.5 * (SY - 1), pc = 0.5 * (PX - 1);
#pragma omp parallel for schedule(dynamic, 1)
  for (int a = 0; a < n_ang; ++a) {
    const ang64 k = angle_params64(angles[a]);
    for (int yi = 0; yi < SY; ++yi) {
      for (int xi = 0; xi < SX; ++xi) {
        const double xp = (xi - xc) * k.c + (yi - yc) * k.s + pc;
        int r;
        double w[3];
        weights64(xp, &k, &r, w);
        for (int t = 0; t < 3; ++t) {
          const int p = r - 1 + t;
          if (p < 0 || p >= PX || w[t] == 0.0) continue;
          for (int hh = 0; hh < n_h; ++hh) {
            const int h = h_list ? h_list[hh] : hh;
            y_out[((size_t)hh * n_ang + a) * PX + p] +=
                w[t] * (double)x[xidx(z_order, SY, SX, Hx, yi, xi, h)];
          }
        }
      }
    }
  }
}

/* x_out (n_h, SY, SX) += A^T y for the listed heights (FP64).
 * y is float32 in z_order layout: z0 (n_ang, PX, Hy), z2 (Hy, n_ang, PX). */
VPO_API void vpo_backward_f64(const float* y, int z_order, int n_ang, int PX, int Hy,
                              const float* angles, int SY, int SX, const int* h_list, int n_h,
                              double* x_out) {
  const double xc = 0.5 * (SX - 1), yc = 0.5 * (SY - 1), pc = 0.5 * (PX - 1);
#pragma omp parallel for schedule(dynamic, 1)
  for (int yi = 0; yi < SY; ++yi) {
    for (int a = 0; a < n_ang; ++a) {
      const ang64 k = angle_params64(angles[a]);
      for (int xi = 0; xi < SX; ++xi) {
        const double xp = (xi - xc) * k.c + (yi - yc) * k.s + pc;
        int r;
        double w[3];
        weights64(xp, &k, &r, w);
        for (int t = 0; t < 3; ++t) {
          const int p = r - 1 + t;
          if (p < 0 || p >= PX || w[t] == 0.0) continue;
          for (int hh = 0; hh < n_h; ++hh) {
            const int h = h_list ? h_list[hh] : hh;
            x_out[((size_t)hh * SY + yi) * SX + xi] +=
                w[t] * (double)y[yidx(z_order, n_ang, PX, Hy, a, p, h)];
          }
        }
      }
    }
  }
}

/* ---------------------------------------------------------------- FP32 --- */

typedef struct {
  float c, s, a, b, coeff, cd;
} ang32;

static ang32 angle_params32(float phi) {
  ang32 k;
  k.c = cosf(phi);
  k.s = sinf(phi);
  const float cms = fabsf(0.5f * (k.c - k.s));
  const float cps = fabsf(0.5f * (k.c + k.s));
  k.a = cms < cps ? cms : cps;
  k.b = cms < cps ? cps : cms;
  k.coeff = 0.5f / ((k.b - k.a) + 2.0f * k.a);
  k.cd = k.b > k.a ? k.coeff / (k.b - k.a) : 0.0f;
  return k;
}

/* projection_common.cuh:139-166 (spiece_wise_integrated_precalc). */
static inline float cdf32(float x, const ang32* k) {
  if (x <= -k->b) return 0.0f;
  if (x < -k->a) return k->cd * (x + k->b) * (x + k->b);
  if (x < k->a) return k->coeff * (k->b + k->a) + 2.0f * k->coeff * x;
  if (x < k->b) return 1.0f - k->cd * (k->b - x) * (k->b - x);
  return 1.0f;
}

static inline void weights32(float xp, const ang32* k, int* r, float w[3]) {
  const float rr = nearbyintf(xp);
  const float xv = rr - xp;
  const float v1 = cdf32(xv - 0.5f, k);
  const float v2 = cdf32(xv + 0.5f, k);
  *r = (int)rr;
  w[0] = v1;
  w[1] = v2 - v1;
  w[2] = 1.0f - v2;
}

VPO_API int vpo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* y += A x in float, in place, caller's layout; angles [a_lo, a_hi) only. */
VPO_API void vpo_forward_f32(const float* x, float* y, int z_order, int SY, int SX, int n_ang,
                             int PX, int H, const float* angles, int a_lo, int a_hi) {
  const float xc = 0.5f * (SX - 1), yc = 0.5f * (SY - 1), pc = 0.5f * (PX - 1);
#pragma omp parallel for schedule(dynamic, 1)
  for (int a = a_lo; a < a_hi; ++a) {
    const ang32 k = angle_params32(angles[a]);
    for (int yi = 0; yi < SY; ++yi) {
      for (int xi = 0; xi < SX; ++xi) {
        const float xp = (xi - xc) * k.c + (yi - yc) * k.s + pc;
        int r;
        float w[3];
        weights32(xp, &k, &r, w);
        for (int t = 0; t < 3; ++t) {
          const int p = r - 1 + t;
          if (p < 0 || p >= PX) continue;
          const float wt = w[t];
          if (z_order == 0) {
            const float* xs = x + ((size_t)yi * SX + xi) * H;
            float* yd = y + ((size_t)a * PX + p) * H;
            for (int h = 0; h < H; ++h) yd[h] += wt * xs[h];
          } else {
            for (int h = 0; h < H; ++h)
              y[((size_t)h * n_ang + a) * PX + p] += wt * x[((size_t)h * SY + yi) * SX + xi];
          }
        }
      }
    }
  }
}

/* x += A^T y in float, in place, caller's layout; angles [a_lo, a_hi) only. */
VPO_API void vpo_backward_f32(const float* y, float* x, int z_order, int SY, int SX, int n_ang,
                              int PX, int H, const float* angles, int a_lo, int a_hi) {
  const float xc = 0.5f * (SX - 1), yc = 0.5f * (SY - 1), pc = 0.5f * (PX - 1);
#pragma omp parallel for schedule(dynamic, 1)
  for (int yi = 0; yi < SY; ++yi) {
    for (int a = a_lo; a < a_hi; ++a) {
      const ang32 k = angle_params32(angles[a]);
      for (int xi = 0; xi < SX; ++xi) {
        const float xp = (xi - xc) * k.c + (yi - yc) * k.s + pc;
        int r;
        float w[3];
        weights32(xp, &k, &r, w);
        for (int t = 0; t < 3; ++t) {
          const int p = r - 1 + t;
          if (p < 0 || p >= PX) continue;
          const float wt = w[t];
          if (z_order == 0) {
            const float* ys = y + ((size_t)a * PX + p) * H;
            float* xd = x + ((size_t)yi * SX + xi) * H;
            for (int h = 0; h < H; ++h) xd[h] += wt * ys[h];
          } else {
            for (int h = 0; h < H; ++h)
              x[((size_t)h * SY + yi) * SX + xi] += wt * y[((size_t)h * n_ang + a) * PX + p];
          }
        }
      }
    }
  }
}
