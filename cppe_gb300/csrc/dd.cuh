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
// a * b + c with c a lazily renormalised accumulator: the rounding error of
// the high parts' sum is carried into c.l without a final renormalisation
// (sums of many products; 12 FP32 operations)
__device__ __forceinline__ dd dd_fma_lazy(dd a, dd b, dd c) {
  const float p  = a.h * b.h;
  float e        = fmaf(a.h, b.h, -p);
  e              = fmaf(a.h, b.l, e);
  e              = fmaf(a.l, b.h, e);
  const float s  = c.h + p;
  const float bb = s - c.h;
  const float f  = (c.h - (s - bb)) + (p - bb);
  return {s, c.l + (f + e)};
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
// Packed double-float: two independent dd values in the halves of float2
// registers, so that one FFMA2/FMUL2/FADD2 (sm_100 and later) advances both.
// Same algorithms as the scalar functions above.
// ---------------------------------------------------------------------------
struct dd2 {
  float2 h, l;
};
__device__ __forceinline__ float2 p2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 pneg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __fadd2_rn(a, pneg(b)); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 psel(bool cx, bool cy, float2 a, float2 b) {
  return make_float2(cx ? a.x : b.x, cy ? a.y : b.y);
}
__device__ __forceinline__ dd2 dd2_sel(bool cx, bool cy, dd2 a, dd2 b) {
  return {psel(cx, cy, a.h, b.h), psel(cx, cy, a.l, b.l)};
}
__device__ __forceinline__ dd2 dd2_two_sum(float2 a, float2 b) {
  const float2 s  = padd(a, b);
  const float2 bb = psub(s, a);
  return {s, padd(psub(a, psub(s, bb)), psub(b, bb))};
}
__device__ __forceinline__ dd2 dd2_fast_two_sum(float2 a, float2 b) {
  const float2 s = padd(a, b);
  return {s, psub(b, psub(s, a))};
}
__device__ __forceinline__ dd2 dd2_add(dd2 a, dd2 b) {
  const dd2 s = dd2_two_sum(a.h, b.h);
  return dd2_fast_two_sum(s.h, padd(s.l, padd(a.l, b.l)));
}
__device__ __forceinline__ dd2 dd2_add_lazy(dd2 a, dd2 b) {
  const dd2 s = dd2_two_sum(a.h, b.h);
  return {s.h, padd(s.l, padd(a.l, b.l))};
}
__device__ __forceinline__ dd2 dd2_neg(dd2 a) { return {pneg(a.h), pneg(a.l)}; }
__device__ __forceinline__ dd2 dd2_mul(dd2 a, dd2 b) {
  const float2 p = pmul(a.h, b.h);
  float2 e       = pfma(a.h, b.h, pneg(p));
  e              = pfma(a.h, b.l, e);
  e              = pfma(a.l, b.h, e);
  return {p, e};
}
__device__ __forceinline__ dd2 dd2_sqr(dd2 a) {
  const float2 p = pmul(a.h, a.h);
  float2 e       = pfma(a.h, a.h, pneg(p));
  e              = pfma(padd(a.h, a.h), a.l, e);
  return {p, e};
}
__device__ __forceinline__ dd2 dd2_sqr_full(dd2 a) {
  const float2 p = pmul(a.h, a.h);
  float2 e       = pfma(a.h, a.h, pneg(p));
  e              = pfma(padd(a.h, a.h), a.l, e);
  e              = pfma(a.l, a.l, e);
  return {p, e};
}
__device__ __forceinline__ dd2 dd2_mul_f(dd2 a, float2 b) {
  const float2 p = pmul(a.h, b);
  return {p, pfma(a.l, b, pfma(a.h, b, pneg(p)))};
}
// 1/sqrt(a) for a > 0 (as dd_rsqrt); the estimate is one MUFU operation per
// half (`rsqrt.approx.ftz`: the inputs are squared distances, never subnormal)
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ dd2 dd2_rsqrt(dd2 a) {
  const float2 y  = make_float2(rsqrt_ftz(a.h.x), rsqrt_ftz(a.h.y));
  const float2 q  = pmul(y, y);
  const float2 qe = pfma(y, y, pneg(q));
  float2 h        = pfma(a.h, q, p2(-1.f));
  h               = pfma(a.h, qe, pfma(a.l, q, h));
  return {y, pmul(pmul(y, h), pfma(p2(0.375f), h, p2(-0.5f)))};
}
// e^-v as dd_exp_neg, each half with its own table entry; v.h < 20 (callers
// clamp the halves they do not use)
__device__ __forceinline__ dd2 dd2_exp_neg(dd2 v, const float* tab_h, const float* tab_l) {
  const int kx    = __float2int_rn(v.h.x * 16.f), ky = __float2int_rn(v.h.y * 16.f);
  const float2 th = pfma(make_float2((float)kx, (float)ky), p2(-0.0625f), v.h);
  const dd2 t     = dd2_two_sum(th, v.l);
  const dd2 t2    = dd2_sqr(t);
  float2 c        = pfma(t.h, p2(1.f / 720.f), p2(-1.f / 120.f));
  c               = pfma(t.h, c, p2(1.f / 24.f));
  c               = pfma(t.h, c, p2(-1.f / 6.f));
  const float2 r3 = pmul(pmul(t2.h, t.h), c);
  const dd2 s     = dd2_fast_two_sum(p2(1.f), pneg(t.h));
  const dd2 s2    = dd2_fast_two_sum(s.h, pmul(p2(0.5f), t2.h));
  const float2 el = padd(pfma(p2(0.5f), t2.l, psub(padd(s.l, s2.l), t.l)), r3);
  const dd2 e     = {make_float2(tab_h[kx], tab_h[ky]), make_float2(tab_l[kx], tab_l[ky])};
  return dd2_mul(e, {s2.h, el});
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
