// Shared device helpers for the finite-volume kernels: status codes, launch helpers and the
// forward-mode dual number used by the Jacobian-vector product.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "../../include/fvgb.h"

#define FV_HD __host__ __device__ __forceinline__

// ------------------------------------------------------------------------------------------------
// Forward-mode dual number.  ``Dual`` carries one tangent; the kernels are templates over the
// scalar type, so the residual pipeline evaluated with ``Dual`` is exactly the JVP of the residual
// pipeline evaluated with ``double``.
//
// max / min follow JAX's convention at a tie (each argument gets half the tangent), so that the
// JVP at a state with ties (e.g. the zero state, where every mass flux is exactly 0) equals the
// reference's ``jax.jvp``.
// ------------------------------------------------------------------------------------------------
struct Dual {
  double v, d;
};

FV_HD Dual mk(double v, double d) { return Dual{v, d}; }
FV_HD double val(double x) { return x; }
FV_HD double val(const Dual& x) { return x.v; }
FV_HD double tan(const Dual& x) { return x.d; }

FV_HD Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
FV_HD Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
FV_HD Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
FV_HD Dual operator/(Dual a, Dual b) {
  double r = 1.0 / b.v;  // one fp64 division per dual division
  double q = a.v * r;
  return {q, (a.d - q * b.d) * r};
}
FV_HD Dual operator-(Dual a) { return {-a.v, -a.d}; }
FV_HD Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
FV_HD Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
FV_HD Dual operator-(Dual a, double b) { return {a.v - b, a.d}; }
FV_HD Dual operator-(double a, Dual b) { return {a - b.v, -b.d}; }
FV_HD Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
FV_HD Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
FV_HD Dual operator/(Dual a, double b) {
  double r = 1.0 / b;
  return {a.v * r, a.d * r};
}
FV_HD Dual operator/(double a, Dual b) {
  double r = 1.0 / b.v;
  double q = a * r;
  return {q, -q * b.d * r};
}
FV_HD Dual& operator+=(Dual& a, Dual b) { a = a + b; return a; }
FV_HD Dual& operator-=(Dual& a, Dual b) { a = a - b; return a; }

// a + g (b - a): the linear owner / neighbour blend (1 - g) a + g b with one multiply-add.
FV_HD double lerp(double a, double b, double g) { return fma(g, b - a, a); }
FV_HD Dual lerp(Dual a, Dual b, double g) { return {fma(g, b.v - a.v, a.v), fma(g, b.d - a.d, a.d)}; }
FV_HD Dual lerp(Dual a, Dual b, Dual g) {
  return {fma(g.v, b.v - a.v, a.v), fma(g.v, b.d - a.d, a.d) + g.d * (b.v - a.v)};
}

// Scalar-generic elementary functions.
FV_HD double cst(double x, double) { return x; }
FV_HD Dual cst(double x, Dual) { return {x, 0.0}; }

FV_HD double fv_max(double a, double b) { return a > b ? a : b; }
FV_HD double fv_min(double a, double b) { return a < b ? a : b; }
FV_HD Dual fv_max(Dual a, Dual b) {
  if (a.v > b.v) return a;
  if (a.v < b.v) return b;
  return {a.v, 0.5 * (a.d + b.d)};
}
FV_HD Dual fv_min(Dual a, Dual b) {
  if (a.v < b.v) return a;
  if (a.v > b.v) return b;
  return {a.v, 0.5 * (a.d + b.d)};
}
FV_HD Dual fv_max(Dual a, double b) { return fv_max(a, Dual{b, 0.0}); }
FV_HD Dual fv_min(Dual a, double b) { return fv_min(a, Dual{b, 0.0}); }

FV_HD double fv_abs(double x) { return fabs(x); }
FV_HD Dual fv_abs(Dual x) { return {fabs(x.v), x.v > 0.0 ? x.d : (x.v < 0.0 ? -x.d : 0.0)}; }
FV_HD double fv_sqrt(double x) { return sqrt(x); }
FV_HD Dual fv_sqrt(Dual x) {
  double s = sqrt(x.v);
  return {s, 0.5 * x.d / s};
}
FV_HD double fv_tanh(double x) { return tanh(x); }
FV_HD Dual fv_tanh(Dual x) {
  double t = tanh(x.v);
  return {t, (1.0 - t * t) * x.d};
}
FV_HD double fv_log(double x) { return log(x); }
FV_HD Dual fv_log(Dual x) { return {log(x.v), x.d / x.v}; }

// ------------------------------------------------------------------------------------------------
// Single-precision dual number.  The same templates evaluated with ``DualF`` give the residual's
// directional derivative in fp32 arithmetic: GB300 has ~64x the fp32 throughput of its fp64 pipe,
// and the preconditioner's Jacobian (and the Krylov operator of a mixed-precision Newton, whose
// defect stays fp64) needs no more than fp32 accuracy.  Double operands are rounded to float at
// the operation; the JAX tie rule of max / min is kept.
// ------------------------------------------------------------------------------------------------
struct DualF {
  float v, d;
};

FV_HD float val(const DualF& x) { return x.v; }
FV_HD DualF operator+(DualF a, DualF b) { return {a.v + b.v, a.d + b.d}; }
FV_HD DualF operator-(DualF a, DualF b) { return {a.v - b.v, a.d - b.d}; }
FV_HD DualF operator*(DualF a, DualF b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
FV_HD DualF operator/(DualF a, DualF b) {
  const float r = 1.0f / b.v;
  const float q = a.v * r;
  return {q, (a.d - q * b.d) * r};
}
FV_HD DualF operator-(DualF a) { return {-a.v, -a.d}; }
FV_HD DualF operator+(DualF a, double b) { return {a.v + (float)b, a.d}; }
FV_HD DualF operator+(double a, DualF b) { return {(float)a + b.v, b.d}; }
FV_HD DualF operator-(DualF a, double b) { return {a.v - (float)b, a.d}; }
FV_HD DualF operator-(double a, DualF b) { return {(float)a - b.v, -b.d}; }
FV_HD DualF operator*(DualF a, double b) { return {a.v * (float)b, a.d * (float)b}; }
FV_HD DualF operator*(double a, DualF b) { return {(float)a * b.v, (float)a * b.d}; }
FV_HD DualF operator/(DualF a, double b) {
  const float r = 1.0f / (float)b;
  return {a.v * r, a.d * r};
}
FV_HD DualF operator/(double a, DualF b) {
  const float r = 1.0f / b.v;
  const float q = (float)a * r;
  return {q, -q * b.d * r};
}
FV_HD DualF operator+(DualF a, float b) { return {a.v + b, a.d}; }
FV_HD DualF operator+(float a, DualF b) { return {a + b.v, b.d}; }
FV_HD DualF operator-(DualF a, float b) { return {a.v - b, a.d}; }
FV_HD DualF operator-(float a, DualF b) { return {a - b.v, -b.d}; }
FV_HD DualF operator*(DualF a, float b) { return {a.v * b, a.d * b}; }
FV_HD DualF operator*(float a, DualF b) { return {a * b.v, a * b.d}; }
FV_HD DualF operator/(DualF a, float b) {
  const float r = 1.0f / b;
  return {a.v * r, a.d * r};
}
FV_HD DualF operator/(float a, DualF b) {
  const float r = 1.0f / b.v;
  const float q = a * r;
  return {q, -q * b.d * r};
}
FV_HD DualF& operator+=(DualF& a, DualF b) { a = a + b; return a; }
FV_HD DualF& operator-=(DualF& a, DualF b) { a = a - b; return a; }
FV_HD DualF lerp(DualF a, DualF b, double g) {
  const float gf = (float)g;
  return {fmaf(gf, b.v - a.v, a.v), fmaf(gf, b.d - a.d, a.d)};
}
FV_HD DualF lerp(DualF a, DualF b, float g) {
  return {fmaf(g, b.v - a.v, a.v), fmaf(g, b.d - a.d, a.d)};
}
FV_HD DualF lerp(DualF a, DualF b, DualF g) {
  return {fmaf(g.v, b.v - a.v, a.v), fmaf(g.v, b.d - a.d, a.d) + g.d * (b.v - a.v)};
}
FV_HD DualF cst(double x, DualF) { return {(float)x, 0.0f}; }
FV_HD DualF fv_max(DualF a, DualF b) {
  if (a.v > b.v) return a;
  if (a.v < b.v) return b;
  return {a.v, 0.5f * (a.d + b.d)};
}
FV_HD DualF fv_min(DualF a, DualF b) {
  if (a.v < b.v) return a;
  if (a.v > b.v) return b;
  return {a.v, 0.5f * (a.d + b.d)};
}
FV_HD DualF fv_max(DualF a, double b) { return fv_max(a, DualF{(float)b, 0.0f}); }
FV_HD DualF fv_min(DualF a, double b) { return fv_min(a, DualF{(float)b, 0.0f}); }
FV_HD DualF fv_abs(DualF x) { return {fabsf(x.v), x.v > 0.0f ? x.d : (x.v < 0.0f ? -x.d : 0.0f)}; }
FV_HD DualF fv_sqrt(DualF x) {
  const float s = sqrtf(x.v);
  return {s, 0.5f * x.d / s};
}
FV_HD DualF fv_tanh(DualF x) {
  const float t = tanhf(x.v);
  return {t, (1.0f - t * t) * x.d};
}
FV_HD DualF fv_log(DualF x) { return {logf(x.v), x.d / x.v}; }

// sqrt with the reference's guard (``aquaflux/turbulence/strain.py:32-43``): 0 (and a zero
// tangent) for a non-positive argument.
template <class T>
FV_HD T safe_sqrt(T x) {
  return val(x) > 0.0 ? fv_sqrt(x) : cst(0.0, x);
}
// max(x, 0) with the JAX tie rule.
template <class T>
FV_HD T pos(T x) {
  return fv_max(x, cst(0.0, x));
}

// ------------------------------------------------------------------------------------------------
// Launch helpers.
// ------------------------------------------------------------------------------------------------
static inline int fv_blocks(long n, int threads) { return (int)((n + threads - 1) / threads); }

#define FV_CUDA_TRY(expr)                                    \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) {                                 \
      fv_set_error("%s: %s", #expr, cudaGetErrorString(_e)); \
      return FV_ERR_CUDA;                                    \
    }                                                        \
  } while (0)

// Records a formatted message returned by ``fv_last_error``.
void fv_set_error(const char* fmt, ...);

// A CSR offset list of n rows (host): it starts at 0 and never decreases; otherwise records
// "<who>: indptr is not a non-decreasing offset list from 0" and returns false.
inline bool fv_offsets_ok(const char* who, int n, const int* indptr) {
  bool ok = indptr[0] == 0;
  for (int i = 0; ok && i < n; ++i) ok = indptr[i] <= indptr[i + 1];
  if (!ok) fv_set_error("%s: indptr is not a non-decreasing offset list from 0", who);
  return ok;
}
