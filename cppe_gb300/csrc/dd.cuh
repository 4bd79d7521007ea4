// Double-float ("DD") arithmetic on the FP32 pipe: a value is the unevaluated
// sum h + l of two floats (about 48 significant bits).  Products take the
// rounding error of h*h' from an FMA; sums carry the error of the high parts
// from Knuth's two-sum (Dekker 1971, "A floating-point technique for extending
// the available precision").  Results are not always renormalised: |l| stays
// a few ulps of h, which the next operation absorbs.
#pragma once

namespace cg {

struct dd {
  float h, l;
};

__device__ __forceinline__ dd dd_from(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double dd_to(dd a) { return (double)a.h + (double)a.l; }

// s + e = a + b exactly (any magnitudes)
__device__ __forceinline__ dd dd_two_sum(float a, float b) {
  const float s  = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
// s + e = a + b exactly, |a| >= |b|
__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ dd dd_add(dd a, dd b) {
  dd s = dd_two_sum(a.h, b.h);
  return dd_fast_two_sum(s.h, s.l + (a.l + b.l));
}
__device__ __forceinline__ dd dd_neg(dd a) { return {-a.h, -a.l}; }
__device__ __forceinline__ dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }
// a + b without the final renormalisation (inputs of similar scale)
__device__ __forceinline__ dd dd_add_lazy(dd a, dd b) {
  dd s = dd_two_sum(a.h, b.h);
  return {s.h, s.l + (a.l + b.l)};
}
__device__ __forceinline__ dd dd_mul(dd a, dd b) {
  const float p = a.h * b.h;
  float e       = fmaf(a.h, b.h, -p);
  e             = fmaf(a.h, b.l, e);
  e             = fmaf(a.l, b.h, e);
  return {p, e};
}
__device__ __forceinline__ dd dd_sqr(dd a) {
  const float p = a.h * a.h;
  float e       = fmaf(a.h, a.h, -p);
  e             = fmaf(2.f * a.h, a.l, e);
  return {p, e};
}
// a^2 including the l^2 term (for pairs whose high parts may be zero)
__device__ __forceinline__ dd dd_sqr_full(dd a) {
  const float p = a.h * a.h;
  float e       = fmaf(a.h, a.h, -p);
  e             = fmaf(2.f * a.h, a.l, e);
  e             = fmaf(a.l, a.l, e);
  return {p, e};
}
__device__ __forceinline__ dd dd_mul_f(dd a, float b) {
  const float p = a.h * b;
  return {p, fmaf(a.l, b, fmaf(a.h, b, -p))};
}
// a * 2^k for a power-of-two float scale (exact)
__device__ __forceinline__ dd dd_scale(dd a, float pow2) { return {a.h * pow2, a.l * pow2}; }

// 1/sqrt(a) for a > 0: FP32 estimate y corrected by the series
// (1 + h)^(-1/2) = 1 - h/2 + 3h^2/8 - ... in h = a y^2 - 1 (|h| ~ 1e-7, formed
// with y^2 split by an FMA); the truncation error is ~(5/16) |h|^3.
__device__ __forceinline__ dd dd_rsqrt(dd a) {
  const float y  = rsqrtf(a.h);
  const float q  = y * y;
  const float qe = fmaf(y, y, -q);
  float h        = fmaf(a.h, q, -1.f);  // a.h*q - 1, |.| ~ 1e-7, one rounding
  h              = fmaf(a.h, qe, fmaf(a.l, q, h));
  return {y, y * h * fmaf(0.375f, h, -0.5f)};
}

// e^-v for 0 <= v < 20 to about 1e-13 relative: v = k/16 + t with |t| <= 1/32,
// e^-v = E[k] e^-t with E[k] = e^-(k/16) tabulated in DD (`tab`, k = 0..320)
// and e^-t from its Taylor series (terms through t^6; t^7/7! < 7e-15).  The
// series keeps 1 - t + t^2/2 in DD and the t^3..t^6 tail in FP32.
constexpr int DD_EXP_TAB = 321;
// 1/6 = DD(1.f/6.f, DD_SIXTH_LO)
constexpr float DD_SIXTH_LO = (float)(1.0 / 6.0 - (double)(1.f / 6.f));
__device__ __forceinline__ dd dd_exp_neg(dd v, const float2* tab) {
  const int k    = __float2int_rn(v.h * 16.f);
  const float th = v.h - (float)k * 0.0625f;  // exact (Sterbenz)
  const dd t     = dd_two_sum(th, v.l);
  const dd t2    = dd_sqr(t);
  float c        = fmaf(t.h, 1.f / 720.f, -1.f / 120.f);
  c              = fmaf(t.h, c, 1.f / 24.f);
  c              = fmaf(t.h, c, -1.f / 6.f);
  const float r3 = t2.h * t.h * c;
  const dd s     = dd_fast_two_sum(1.f, -t.h);
  const dd s2    = dd_fast_two_sum(s.h, 0.5f * t2.h);
  const dd et    = {s2.h, s.l + s2.l - t.l + 0.5f * t2.l + r3};
  const float2 e = tab[k];
  return dd_mul({e.x, e.y}, et);
}

// ---------------------------------------------------------------------------
// A value type over dd for generic code (the generated M2L translations):
// +, -, * with dd accuracy, division by a Newton-corrected quotient.
// ---------------------------------------------------------------------------
struct ddv {
  float h, l;
  __device__ __forceinline__ ddv() : h(0.f), l(0.f) {}
  __device__ __forceinline__ explicit ddv(int v) : h((float)v), l(0.f) {}
  __device__ __forceinline__ ddv(float hh, float ll) : h(hh), l(ll) {}
  __device__ __forceinline__ ddv(dd a) : h(a.h), l(a.l) {}
  __device__ __forceinline__ operator dd() const { return dd{h, l}; }
};
__device__ __forceinline__ ddv operator+(ddv a, ddv b) { return dd_add(a, b); }
__device__ __forceinline__ ddv operator-(ddv a) { return ddv(-a.h, -a.l); }
__device__ __forceinline__ ddv operator-(ddv a, ddv b) { return dd_add(a, ddv(-b.h, -b.l)); }
__device__ __forceinline__ ddv operator*(ddv a, ddv b) { return dd_mul(a, b); }
__device__ __forceinline__ ddv fma(ddv a, ddv b, ddv c) { return dd_add(dd_mul(a, b), c); }
// (the float and double overloads, visible next to the ddv one inside cg)
__device__ __forceinline__ float fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
__device__ __forceinline__ ddv operator/(ddv a, ddv b) {
  const float q1 = a.h / b.h;
  const dd r     = dd_add(a, dd_neg(dd_mul(b, dd{q1, 0.f})));
  return dd_fast_two_sum(q1, r.h / b.h);
}
__device__ __forceinline__ ddv rsqrt_t(ddv a) { return dd_rsqrt(a); }

// 1/o for a small positive integer o, in the precision of T (constant-folded)
template <typename T>
__device__ __forceinline__ T cinv(int o);
template <>
__device__ __forceinline__ float cinv<float>(int o) {
  return 1.f / (float)o;
}
template <>
__device__ __forceinline__ double cinv<double>(int o) {
  return 1.0 / (double)o;
}
template <>
__device__ __forceinline__ ddv cinv<ddv>(int o) {
  const double v = 1.0 / (double)o;
  const float hh = (float)v;
  return ddv(hh, (float)(v - (double)hh));
}

}  // namespace cg
