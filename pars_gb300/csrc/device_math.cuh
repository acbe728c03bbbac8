// Device-side field sampling and integrator steps for the tracing kernels.
//
// The FROZEN path reproduces the reference's FP32 arithmetic operation by
// operation, with every operation separately rounded (explicit __f*_rn
// intrinsics, never contracted into FMAs), so that it gives the reference's
// bits:
//   vector_field::contains     pa/source/math/vector_field.cpp:12-21
//   vector_field::interpolate  pa/source/math/vector_field.cpp:22-48
//   linear_interpolate         pa/include/pa/math/linear_interpolate.hpp:6-10
//   isZero                     Eigen default precision 1e-5f
//   frozen-velocity step       pa/source/stages/particle_tracer.cpp:315-334
// The RESAMPLED paths (stages sampled where they fall) carry a particle in
// local cell coordinates -- its cell, the offset in the cell and a
// compensation term (local_position, compensated_add) -- sample with FMA
// lerps on the register-cached corners of the cell, and end a curve when the
// cell leaves the grid (local_inside).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pars
{
// A block of a vector field, resident as float4 (x, y, z, 0) per vertex,
// [X][Y][Z] in C order (z fastest), like pa::vector_field::data.
struct field_view
{
  const float4* data;
  int           nx, ny, nz;
  float         ox, oy, oz;        // offset
  float         hx, hy, hz;        // spacing
  float         maxx, maxy, maxz;  // offset + size (block-exit face tests)
  float         inv_hx, inv_hy, inv_hz;  // 1 / spacing (re-sampled path)
};

// The termination and invalid vertices (integral_curves.hpp:18-19).
__device__ __forceinline__ float4 termination_vertex() { return make_float4(-2.0f, -2.0f, -2.0f, 0.0f); }
__device__ __forceinline__ bool   is_invalid_vertex(const float4& v)
{
  return v.x == -1.0f && v.y == -1.0f && v.z == -1.0f && v.w == 0.0f;
}
__device__ __forceinline__ bool   is_termination_vertex(const float4& v)
{
  return v.x == -2.0f && v.y == -2.0f && v.z == -2.0f && v.w == 0.0f;
}

// Per-axis cell search of vector_field::contains / interpolate.
// s = floor((p - o) / h) (IEEE division, as the reference); the weight is
// fmod(p - o, h) / h.  fmod is computed exactly without a loop: with
// q = trunc(d / h) rounded, q is the true truncated quotient or one more (the
// division can round up onto the next integer), and d - q h is exactly
// representable when q is the true quotient, so one FMA gives it exactly; a
// negative FMA result (for d >= 0) means q was one too large.
struct axis_cell
{
  float s;   // floor((p - o) / h)
  float w;   // fmod(p - o, h) / h
};
__device__ __forceinline__ axis_cell cell_of(float p, float o, float h)
{
  const float d = __fsub_rn(p, o);
  const float s = floorf(__fdiv_rn(d, h));
  float r = __fmaf_rn(-s, h, d);
  // For d < 0, fmod truncates toward zero (remainder has the sign of d).  The
  // only d < 0 that pass contains() have d / h rounding to -0 (s = -0), where
  // the FMA already returns d itself.
  if (d >= 0.0f) { if (r < 0.0f) r = __fmaf_rn(-(s - 1.0f), h, d); }
  else           { if (r > 0.0f) r = __fmaf_rn(-(s + 1.0f), h, d); }
  return axis_cell{s, __fdiv_rn(r, h)};
}

__device__ __forceinline__ bool cell_inside(float s, int n) { return s >= 0.0f && s <= float(n - 2); }

// (1 - w) a + w b with each operation rounded separately.
__device__ __forceinline__ float lerp_exact(float a, float b, float w, float one_minus_w)
{
  return __fadd_rn(__fmul_rn(one_minus_w, a), __fmul_rn(w, b));
}

__device__ __forceinline__ float3 blend8(const float4& c000, const float4& c001, const float4& c010, const float4& c011,
                                         const float4& c100, const float4& c101, const float4& c110, const float4& c111,
                                         float wx, float wy, float wz)
{
  const float mx = __fsub_rn(1.0f, wx), my = __fsub_rn(1.0f, wy), mz = __fsub_rn(1.0f, wz);
  float3 out;
  {
    const float c00 = lerp_exact(c000.x, c001.x, wz, mz), c01 = lerp_exact(c010.x, c011.x, wz, mz);
    const float c10 = lerp_exact(c100.x, c101.x, wz, mz), c11 = lerp_exact(c110.x, c111.x, wz, mz);
    out.x = lerp_exact(lerp_exact(c00, c01, wy, my), lerp_exact(c10, c11, wy, my), wx, mx);
  }
  {
    const float c00 = lerp_exact(c000.y, c001.y, wz, mz), c01 = lerp_exact(c010.y, c011.y, wz, mz);
    const float c10 = lerp_exact(c100.y, c101.y, wz, mz), c11 = lerp_exact(c110.y, c111.y, wz, mz);
    out.y = lerp_exact(lerp_exact(c00, c01, wy, my), lerp_exact(c10, c11, wy, my), wx, mx);
  }
  {
    const float c00 = lerp_exact(c000.z, c001.z, wz, mz), c01 = lerp_exact(c010.z, c011.z, wz, mz);
    const float c10 = lerp_exact(c100.z, c101.z, wz, mz), c11 = lerp_exact(c110.z, c111.z, wz, mz);
    out.z = lerp_exact(lerp_exact(c00, c01, wy, my), lerp_exact(c10, c11, wy, my), wx, mx);
  }
  return out;
}

// Eight 16-byte corner loads through the read-only path.
__device__ __forceinline__ float3 gather_blend(const field_view& f, int ix, int iy, int iz, float wx, float wy, float wz)
{
  const long long syz = (long long)f.ny * f.nz;
  const float4* base = f.data + ((long long)ix * f.ny + iy) * f.nz + iz;
  const float4 c000 = __ldg(base);
  const float4 c001 = __ldg(base + 1);
  const float4 c010 = __ldg(base + f.nz);
  const float4 c011 = __ldg(base + f.nz + 1);
  const float4 c100 = __ldg(base + syz);
  const float4 c101 = __ldg(base + syz + 1);
  const float4 c110 = __ldg(base + syz + f.nz);
  const float4 c111 = __ldg(base + syz + f.nz + 1);
  return blend8(c000, c001, c010, c011, c100, c101, c110, c111, wx, wy, wz);
}

// contains() followed by interpolate() at p: returns false when p is outside.
__device__ __forceinline__ bool sample_inside(const field_view& f, const float4& p, float3& v)
{
  const axis_cell cx = cell_of(p.x, f.ox, f.hx);
  const axis_cell cy = cell_of(p.y, f.oy, f.hy);
  const axis_cell cz = cell_of(p.z, f.oz, f.hz);
  if (!(cell_inside(cx.s, f.nx) && cell_inside(cy.s, f.ny) && cell_inside(cz.s, f.nz))) return false;
  v = gather_blend(f, int(cx.s), int(cy.s), int(cz.s), cx.w, cy.w, cz.w);
  return true;
}

// ---- RESAMPLED-mode sampling ------------------------------------------------
// The reference takes the cell index from the ROUNDED quotient floor(d / h)
// but the weight from the EXACT remainder fmod(d, h): when d / h rounds up
// onto an integer the two disagree and the sample lands a whole cell away
// (weight ~1 in the next cell).  In FP32 this happens for many positions on
// or next to grid planes (every flow-map seed sits on a grid vertex).  The
// frozen path keeps that behaviour for bit-exact parity; the re-sampled path
// uses a consistent pair: s is corrected until r = d - s h lies in [0, h),
// then w = r / h.  The quotient estimate uses a reciprocal multiply (the FMA
// correction makes the pair exact whatever the estimate).
__device__ __forceinline__ axis_cell cell_consistent(float p, float o, float h, float inv_h)
{
  const float d = p - o;
  float s = floorf(d * inv_h);
  float r = fmaf(-s, h, d);
  if (r < 0.0f)   { s -= 1.0f; r = fmaf(-s, h, d); }
  else if (r >= h) { s += 1.0f; r = fmaf(-s, h, d); }
  return axis_cell{s, r * inv_h};
}

// Lerp with one FMA (re-sampled path; not bit-exact with the reference).
__device__ __forceinline__ float lerp_fast(float a, float b, float w) { return fmaf(w, b - a, a); }

// ---- Register-cached cell (re-sampled path) ----------------------------------
// A particle moves up to about a cell per RK4 step, so most stage samples fall
// into the cell sampled last.  The lane keeps that cell's eight corners in
// registers, and only a change of cell issues the eight 16-byte corner loads.
// Within a warp some lane changes cell at almost every sample, so whatever
// runs only for the lanes that change cell costs the whole warp nearly every
// sample: that part is kept to the loads, and the interpolation (lerps along
// z, then y, then x) runs once for all lanes together.
struct corner_cache
{
  int    ix = -1, iy = -1, iz = -1;
  float3 c000, c001, c010, c011, c100, c101, c110, c111;
};

__device__ __forceinline__ float3 xyz_of(const float4& v) { return make_float3(v.x, v.y, v.z); }

__device__ __forceinline__ void corner_load(const field_view& f, corner_cache& k, int ix, int iy, int iz)
{
  const long long syz = (long long)f.ny * f.nz;
  const float4* base = f.data + ((long long)ix * f.ny + iy) * f.nz + iz;
  k.ix = ix; k.iy = iy; k.iz = iz;
  k.c000 = xyz_of(__ldg(base));
  k.c001 = xyz_of(__ldg(base + 1));
  k.c010 = xyz_of(__ldg(base + f.nz));
  k.c011 = xyz_of(__ldg(base + f.nz + 1));
  k.c100 = xyz_of(__ldg(base + syz));
  k.c101 = xyz_of(__ldg(base + syz + 1));
  k.c110 = xyz_of(__ldg(base + syz + f.nz));
  k.c111 = xyz_of(__ldg(base + syz + f.nz + 1));
}

__device__ __forceinline__ float corner_eval1(float c000, float c001, float c010, float c011, float c100, float c101,
                                              float c110, float c111, float wx, float wy, float wz)
{
  const float c00 = lerp_fast(c000, c001, wz), c01 = lerp_fast(c010, c011, wz);
  const float c10 = lerp_fast(c100, c101, wz), c11 = lerp_fast(c110, c111, wz);
  return lerp_fast(lerp_fast(c00, c01, wy), lerp_fast(c10, c11, wy), wx);
}

// The reference's blend (lerp_exact along z, then y, then x) of a cached cell:
// the same arithmetic as blend8, so the frozen path stays bit-exact.
__device__ __forceinline__ float3 blend8_cached(const corner_cache& k, float wx, float wy, float wz)
{
  const float4 c000 = make_float4(k.c000.x, k.c000.y, k.c000.z, 0.f), c001 = make_float4(k.c001.x, k.c001.y, k.c001.z, 0.f);
  const float4 c010 = make_float4(k.c010.x, k.c010.y, k.c010.z, 0.f), c011 = make_float4(k.c011.x, k.c011.y, k.c011.z, 0.f);
  const float4 c100 = make_float4(k.c100.x, k.c100.y, k.c100.z, 0.f), c101 = make_float4(k.c101.x, k.c101.y, k.c101.z, 0.f);
  const float4 c110 = make_float4(k.c110.x, k.c110.y, k.c110.z, 0.f), c111 = make_float4(k.c111.x, k.c111.y, k.c111.z, 0.f);
  return blend8(c000, c001, c010, c011, c100, c101, c110, c111, wx, wy, wz);
}

// contains() followed by interpolate() at p (the reference's cell search and
// blend), the cell's corners kept in the lane's cache between steps.
__device__ __forceinline__ bool sample_inside_cached(const field_view& f, corner_cache& k, const float4& p, float3& v)
{
  const axis_cell cx = cell_of(p.x, f.ox, f.hx);
  const axis_cell cy = cell_of(p.y, f.oy, f.hy);
  const axis_cell cz = cell_of(p.z, f.oz, f.hz);
  if (!(cell_inside(cx.s, f.nx) && cell_inside(cy.s, f.ny) && cell_inside(cz.s, f.nz))) return false;
  const int ix = int(cx.s), iy = int(cy.s), iz = int(cz.s);
  if (ix != k.ix || iy != k.iy || iz != k.iz) corner_load(f, k, ix, iy, iz);
  v = blend8_cached(k, cx.w, cy.w, cz.w);
  return true;
}

// lerp_fast on a pair of components with the packed FP32x2 instructions
// (FADD2 / FFMA2, round-to-nearest per component): the difference feeds an
// explicit FMA, so nothing can be folded into it, and each component is
// bit-identical to lerp_fast (the 256^3 flow map's end points were).
__device__ __forceinline__ float2 lerp_fast2(float2 a, float2 b, float2 w)
{
  return __ffma2_rn(w, __fadd2_rn(b, make_float2(-a.x, -a.y)), a);
}

// The trilinear blend of a cached cell with lerp_fast along z, then y, then x:
// x and y components through the packed pair (7 paired lerps instead of 14
// scalar ones), z through the scalar blend.  Measured on the 256^3 FTLE
// workload: 4.4 % less kernel time than three scalar blends, same end points.
__device__ __forceinline__ float3 corner_eval(const corner_cache& k, float wx, float wy, float wz)
{
  const float2 Wz = make_float2(wz, wz), Wy = make_float2(wy, wy), Wx = make_float2(wx, wx);
  const float2 c00 = lerp_fast2(make_float2(k.c000.x, k.c000.y), make_float2(k.c001.x, k.c001.y), Wz);
  const float2 c01 = lerp_fast2(make_float2(k.c010.x, k.c010.y), make_float2(k.c011.x, k.c011.y), Wz);
  const float2 c10 = lerp_fast2(make_float2(k.c100.x, k.c100.y), make_float2(k.c101.x, k.c101.y), Wz);
  const float2 c11 = lerp_fast2(make_float2(k.c110.x, k.c110.y), make_float2(k.c111.x, k.c111.y), Wz);
  const float2 xy = lerp_fast2(lerp_fast2(c00, c01, Wy), lerp_fast2(c10, c11, Wy), Wx);
  return make_float3(xy.x, xy.y,
                     corner_eval1(k.c000.z, k.c001.z, k.c010.z, k.c011.z, k.c100.z, k.c101.z, k.c110.z, k.c111.z, wx, wy, wz));
}

// Eigen isZero() with its default precision (NumTraits<float>::dummy_precision).
__device__ __forceinline__ bool is_zero(const float3& v)
{
  const float precision = 1e-5f;
  return fabsf(v.x) <= precision && fabsf(v.y) <= precision && fabsf(v.z) <= precision;
}

// Integrator parameters.  RESAMPLED: classical RK4 (or Euler) with a sample
// at each stage point.  FROZEN (the reference's scheme: every stage sees the
// velocity v sampled at the step start), by method:
//  * weighted sum (Euler, RK4, Cash-Karp 5(4), Dormand-Prince 5, Fehlberg 7(8),
//    Adams-Bashforth-Moulton 2): out = 1*x + c_0 v + ... + c_{k-1} v with
//    c_i = b_i * h (b_i in FP32), accumulated left to right, zero weights
//    included;
//  * modified midpoint (two substeps, H = h/2): z1 = x + c_0 v, z2 = x + c_1 v,
//    out = 0.5 z2 + 0.5 z1 + c_2 v (c_0 = H, c_1 = 2H, c_2 = 0.5H);
//  * Adams-Bashforth 2: the particle's first step is the weighted sum (RK4
//    weights), later ones out = x + c_4 v_n + c_5 v_{n-1} (c_4 = 1.5 h,
//    c_5 = -0.5 h), with the previous step's velocity kept per particle.
enum frozen_method { frozen_weighted_sum = 0, frozen_midpoint = 1, frozen_multistep = 2 };

// Re-sampled stages of the other integrators ("true form"): explicit RK
// tableaux (modified midpoint as a 3-stage scheme, Cash-Karp 5(4) and
// Dormand-Prince 5 with their 5th-order weights, Fehlberg 7(8) with its
// 8th-order weights -- the orders odeint's steppers propagate) and the
// two-step Adams-Bashforth / Adams-Bashforth-Moulton schemes (RK4 for a
// particle's first step).
enum resampled_scheme { scheme_classic = 0, scheme_tableau = 1, scheme_adams_bashforth = 2, scheme_adams_moulton = 3 };

struct step_rule
{
  int   frozen;      // 1 = frozen velocity, 0 = resampled stages
  int   rk4;         // resampled classic scheme: 1 = RK4, 0 = Euler
  int   count;       // frozen weighted sum: number of coefficients
  int   method;      // frozen_method
  float c[16];       // frozen coefficients
  float h;           // step size
  int   scheme;      // resampled_scheme
  int   tableau;     // scheme_tableau: index into rk_tableaux
};

// The multistep scheme's per-particle history.
struct frozen_history
{
  float3 v = make_float3(0.f, 0.f, 0.f);
  int    started = 0;
};

__device__ __forceinline__ float midpoint_component(const step_rule& r, float x, float v)
{
  const float z1 = __fadd_rn(x, __fmul_rn(r.c[0], v));
  const float z2 = __fadd_rn(x, __fmul_rn(r.c[1], v));
  return __fadd_rn(__fadd_rn(__fmul_rn(0.5f, z2), __fmul_rn(0.5f, z1)), __fmul_rn(r.c[2], v));
}

__device__ __forceinline__ float multistep_component(const step_rule& r, float x, float v, float previous)
{
  return __fadd_rn(__fadd_rn(x, __fmul_rn(r.c[4], v)), __fmul_rn(r.c[5], previous));
}

// FROZEN step from x with the velocity v = v(x): the reference's operation order.
__device__ __forceinline__ float4 frozen_step(const step_rule& r, const float4& x, const float3& v, frozen_history& hist)
{
  float4 out;
  if (r.method == frozen_midpoint)
    out = make_float4(midpoint_component(r, x.x, v.x), midpoint_component(r, x.y, v.y), midpoint_component(r, x.z, v.z),
                      midpoint_component(r, x.w, 0.0f));
  else if (r.method == frozen_multistep && hist.started)
    out = make_float4(multistep_component(r, x.x, v.x, hist.v.x), multistep_component(r, x.y, v.y, hist.v.y),
                      multistep_component(r, x.z, v.z, hist.v.z), multistep_component(r, x.w, 0.0f, 0.0f));
  else
  {
    // each component: 1 * x (exact) + c_0 v + c_1 v + ..., left to right
    out = x;
    for (int i = 0; i < r.count; ++i)
    {
      const float c = r.c[i];
      out.x = __fadd_rn(out.x, __fmul_rn(c, v.x));
      out.y = __fadd_rn(out.y, __fmul_rn(c, v.y));
      out.z = __fadd_rn(out.z, __fmul_rn(c, v.z));
      out.w = __fadd_rn(out.w, __fmul_rn(c, 0.0f));
    }
  }
  if (r.method == frozen_multistep) { hist.v = v; hist.started = 1; }
  return out;
}

// Adds delta to the compensated position (hi, lo) with Knuth's error-free
// TwoSum: hi receives the rounded sum, lo the exact rounding error, so that
// hi + lo carries the position to about twice FP32 precision.  Small steps
// added to positions of order one otherwise lose a correlated fraction of an
// ulp every step.
__device__ __forceinline__ void compensated_add(float& hi, float& lo, float delta)
{
  const float d = delta + lo;
  const float s = hi + d;
  const float bp = s - hi;
  lo = (hi - (s - bp)) + (d - bp);
  hi = s;
}

// Knuth's error-free TwoSum: s = RN(a + b) and e = (a + b) - s exactly.
// Written with round-to-nearest intrinsics, which the compiler never fuses
// with a neighbouring multiply: the proof needs s to be the rounded sum of
// the rounded operands.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// u (with its compensation term l) += h6 (k1 + 2 k2 + 2 k3 + k4): the RK4
// weighted sum is formed with TwoSums and the product with its exact FMA
// error, and both errors go into the compensation term, so the only rounding
// left is that of the (tiny) compensation term itself.  A plain FP32 sum and
// product lose about two ulps of the increment per step, which the flow's
// stretching amplifies: on the 256^3 ABC workload this halves the largest
// end-point errors against an FP64 integration.  Every operation of this
// scalar form is an explicit round-to-nearest one, never contracted.  The
// packed pair form (rk4_update2) is not contraction-proof: the compiler folds
// a packed product into the packed sum that consumes it (a sum of two packed
// products differed from two roundings in 43 % of random cases, with the
// intrinsics, with explicit-rounding PTX and with --fmad=false alike), so its
// x and y can differ from this form in the last bits; both meet the
// end-point bar against FP64.
__device__ __forceinline__ void rk4_update(float& u, float& l, float h6, float k1, float k2, float k3, float k4)
{
  float a, ea, b, eb, t, et;
  two_sum(k1, k4, a, ea);
  two_sum(k2, k3, b, eb);
  two_sum(a, __fmul_rn(2.0f, b), t, et);
  const float e = __fadd_rn(fmaf(2.0f, eb, ea), et);
  const float p = __fmul_rn(h6, t);
  l = __fadd_rn(l, fmaf(h6, e, fmaf(h6, t, -p)));
  compensated_add(u, l, p);
}

// ---- Packed pairs (FP32x2) ----------------------------------------------------
// The x and y components of the re-sampled RK4 step go through the packed
// FP32x2 instructions (FADD2 / FMUL2 / FFMA2: two round-to-nearest operations
// in one instruction), z through the scalar forms above.  A packed product
// that feeds a packed sum may be folded into one FFMA2 (see rk4_update), so
// these forms are not bit-identical to the scalar ones; the frozen scheme,
// which must give the reference's bits, stays scalar.
__device__ __forceinline__ float2 pair(float v) { return make_float2(v, v); }

// a - b as FMA(b, -1, a): one rounding, one instruction.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, pair(-1.0f), a); }

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e)
{
  s = __fadd2_rn(a, b);
  const float2 bp = sub2(s, a);
  e = __fadd2_rn(sub2(a, sub2(s, bp)), sub2(b, bp));
}

__device__ __forceinline__ void compensated_add2(float2& hi, float2& lo, float2 delta)
{
  const float2 d = __fadd2_rn(delta, lo);
  const float2 s = __fadd2_rn(hi, d);
  const float2 bp = sub2(s, hi);
  lo = __fadd2_rn(sub2(hi, sub2(s, bp)), sub2(d, bp));
  hi = s;
}

__device__ __forceinline__ void rk4_update2(float2& u, float2& l, float h6, float2 k1, float2 k2, float2 k3, float2 k4)
{
  float2 a, ea, b, eb, t, et;
  two_sum2(k1, k4, a, ea);
  two_sum2(k2, k3, b, eb);
  two_sum2(a, __fmul2_rn(pair(2.0f), b), t, et);
  const float2 e = __fadd2_rn(__ffma2_rn(pair(2.0f), eb, ea), et);
  const float2 p = __fmul2_rn(pair(h6), t);
  l = __fadd2_rn(l, __ffma2_rn(pair(h6), e, __ffma2_rn(pair(h6), t, make_float2(-p.x, -p.y))));
  compensated_add2(u, l, p);
}

// Butcher tableaux of the re-sampled general schemes (stage matrix a, weights
// b), FP32 quotients of the published fractions.
struct rk_tableau
{
  int   stages;
  float a[13][13];
  float b[13];
};

struct rk_entry { int i, j, p, q; };

template <int NA, int NB>
constexpr rk_tableau make_tableau(int stages, const rk_entry (&a)[NA], const rk_entry (&b)[NB])
{
  rk_tableau t {};
  t.stages = stages;
  for (int k = 0; k < NA; ++k) t.a[a[k].i][a[k].j] = float(a[k].p) / float(a[k].q);
  for (int k = 0; k < NB; ++k) t.b[b[k].i] = float(b[k].p) / float(b[k].q);
  return t;
}

// Gragg's modified midpoint with two substeps (odeint's modified_midpoint):
// z1 = x + (h/2) f(x), z2 = x + h f(z1), out = (z2 + z1 + (h/2) f(z2)) / 2.
constexpr rk_entry midpoint_a[] = {{1, 0, 1, 2}, {2, 1, 1, 1}};
constexpr rk_entry midpoint_b[] = {{0, 0, 1, 4}, {1, 0, 1, 2}, {2, 0, 1, 4}};
constexpr rk_entry cash_karp_a[] = {
  {1, 0, 1, 5}, {2, 0, 3, 40}, {2, 1, 9, 40}, {3, 0, 3, 10}, {3, 1, -9, 10}, {3, 2, 6, 5},
  {4, 0, -11, 54}, {4, 1, 5, 2}, {4, 2, -70, 27}, {4, 3, 35, 27},
  {5, 0, 1631, 55296}, {5, 1, 175, 512}, {5, 2, 575, 13824}, {5, 3, 44275, 110592}, {5, 4, 253, 4096}};
constexpr rk_entry cash_karp_b[] = {{0, 0, 37, 378}, {2, 0, 250, 621}, {3, 0, 125, 594}, {5, 0, 512, 1771}};
constexpr rk_entry dormand_prince_a[] = {
  {1, 0, 1, 5}, {2, 0, 3, 40}, {2, 1, 9, 40}, {3, 0, 44, 45}, {3, 1, -56, 15}, {3, 2, 32, 9},
  {4, 0, 19372, 6561}, {4, 1, -25360, 2187}, {4, 2, 64448, 6561}, {4, 3, -212, 729},
  {5, 0, 9017, 3168}, {5, 1, -355, 33}, {5, 2, 46732, 5247}, {5, 3, 49, 176}, {5, 4, -5103, 18656}};
constexpr rk_entry dormand_prince_b[] = {{0, 0, 35, 384}, {2, 0, 500, 1113}, {3, 0, 125, 192}, {4, 0, -2187, 6784}, {5, 0, 11, 84}};
constexpr rk_entry fehlberg_a[] = {
  {1, 0, 2, 27}, {2, 0, 1, 36}, {2, 1, 1, 12}, {3, 0, 1, 24}, {3, 2, 1, 8},
  {4, 0, 5, 12}, {4, 2, -25, 16}, {4, 3, 25, 16}, {5, 0, 1, 20}, {5, 3, 1, 4}, {5, 4, 1, 5},
  {6, 0, -25, 108}, {6, 3, 125, 108}, {6, 4, -65, 27}, {6, 5, 125, 54},
  {7, 0, 31, 300}, {7, 4, 61, 225}, {7, 5, -2, 9}, {7, 6, 13, 900},
  {8, 0, 2, 1}, {8, 3, -53, 6}, {8, 4, 704, 45}, {8, 5, -107, 9}, {8, 6, 67, 90}, {8, 7, 3, 1},
  {9, 0, -91, 108}, {9, 3, 23, 108}, {9, 4, -976, 135}, {9, 5, 311, 54}, {9, 6, -19, 60}, {9, 7, 17, 6}, {9, 8, -1, 12},
  {10, 0, 2383, 4100}, {10, 3, -341, 164}, {10, 4, 4496, 1025}, {10, 5, -301, 82}, {10, 6, 2133, 4100}, {10, 7, 45, 82},
  {10, 8, 45, 164}, {10, 9, 18, 41},
  {11, 0, 3, 205}, {11, 5, -6, 41}, {11, 6, -3, 205}, {11, 7, -3, 41}, {11, 8, 3, 41}, {11, 9, 6, 41},
  {12, 0, -1777, 4100}, {12, 3, -341, 164}, {12, 4, 4496, 1025}, {12, 5, -289, 82}, {12, 6, 2193, 4100}, {12, 7, 51, 82},
  {12, 8, 33, 164}, {12, 9, 12, 41}, {12, 11, 1, 1}};
constexpr rk_entry fehlberg_b[] = {{5, 0, 34, 105}, {6, 0, 9, 35}, {7, 0, 9, 35}, {8, 0, 9, 280}, {9, 0, 9, 280},
                                   {11, 0, 41, 840}, {12, 0, 41, 840}};

enum rk_tableau_index { tableau_midpoint = 0, tableau_cash_karp = 1, tableau_dormand_prince = 2, tableau_fehlberg = 3 };

__constant__ const rk_tableau rk_tableaux[4] = {
  make_tableau(3, midpoint_a, midpoint_b),
  make_tableau(6, cash_karp_a, cash_karp_b),
  make_tableau(6, dormand_prince_a, dormand_prince_b),
  make_tableau(13, fehlberg_a, fehlberg_b)};

// ---- Unsteady fields (pathlines) ----------------------------------------------
// An unsteady field is a sequence of `nt` slices of one grid, slice k holding
// the velocity at time t0 + k * slice_dt; between slices the velocity is
// linear in time.  Time is carried as the slice coordinate s = (t - t0) /
// slice_dt.  Step n of a job starting at time t_b samples s at
// s_b + (n + c) * D (c = 0, 1/2, 1; D = h / slice_dt): computed from n every
// step (no accumulated rounding) as an unevaluated pair of floats (hi + lo,
// about 44 bits), which keeps the arithmetic on the FP32 pipes (a GB300 SM
// issues FP64 at 1/64 of its FP32 rate); the time weight enters the FP32
// blend.
struct time_axis
{
  int       nt;              // number of slices (1 = steady)
  long long slice_stride;    // float4 elements per slice
  double    t0;              // time of slice 0
  double    inv_slice_dt;    // 1 / slice spacing in time
};

// A job's clock: s_b and D as float pairs (set on the host from FP64 values).
struct slice_clock
{
  float s_hi = 0.0f, s_lo = 0.0f;   // slice coordinate at the job's start time
  float d_hi = 0.0f, d_lo = 0.0f;   // slice coordinate per step
};

inline slice_clock make_slice_clock(const time_axis& ta, double time_begin, float h)
{
  slice_clock c;
  const double s = (time_begin - ta.t0) * ta.inv_slice_dt, d = double(h) * ta.inv_slice_dt;
  c.s_hi = float(s); c.s_lo = float(s - double(c.s_hi));
  c.d_hi = float(d); c.d_lo = float(d - double(c.d_hi));
  return c;
}

struct slice_time { float hi, lo; };

// Knuth's TwoSum: a + b = s + e exactly.
__device__ __forceinline__ void two_sum_rn(float a, float b, float& s, float& e)
{
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// s_b + n * D.  n is split into a high part (multiple of 4096) and a low part
// so that both convert to float exactly for any int n >= 0; their products
// with d_hi are split into rounded value and exact error by an FMA.
__device__ __forceinline__ slice_time step_time(const slice_clock& c, int n)
{
  const float nh = __int2float_rn(n & ~0xfff), nl = __int2float_rn(n & 0xfff);
  const float p1 = __fmul_rn(nh, c.d_hi), e1 = fmaf(nh, c.d_hi, -p1);
  const float p2 = __fmul_rn(nl, c.d_hi), e2 = fmaf(nl, c.d_hi, -p2);
  float a, b, a2, b2;
  two_sum_rn(c.s_hi, p1, a, b);
  two_sum_rn(a, p2, a2, b2);
  const float lo = (b + b2) + (e1 + e2) + fmaf(__int2float_rn(n), c.d_lo, c.s_lo);
  return {a2, lo};
}

// t + c * D for c = 1/2 or 1 (c * d_hi and c * d_lo are exact).
__device__ __forceinline__ slice_time advance_time(const slice_time& t, const slice_clock& c, float frac)
{
  float a, b;
  two_sum_rn(t.hi, __fmul_rn(frac, c.d_hi), a, b);
  return {a, b + (t.lo + __fmul_rn(frac, c.d_lo))};
}

// The slice pair around time t and the weight of the later slice: floor(s)
// and s - floor(s) of s = hi + lo; before slice 0 the first slice, after the
// last one the last slice.
__device__ __forceinline__ void slice_of(const time_axis& ta, const slice_time& t, int& slice, float& wt)
{
  if (ta.nt <= 1) { slice = 0; wt = 0.0f; return; }
  float fs = floorf(t.hi);
  float w = __fadd_rn(__fsub_rn(t.hi, fs), t.lo);   // hi - floor(hi) is exact
  if (w < 0.0f) { fs -= 1.0f; w = __fadd_rn(w, 1.0f); }
  else if (w >= 1.0f) { fs += 1.0f; w = __fsub_rn(w, 1.0f); }
  if (!(fs >= 0.0f)) { slice = 0; wt = 0.0f; }
  else if (fs >= float(ta.nt - 1)) { slice = ta.nt - 2; wt = 1.0f; }
  else { slice = int(fs); wt = w; }
}

// The corners of one cell in the two slices around the current time;
// reloaded when the cell or the slice pair changes.
struct corner_cache2
{
  int          slice = -1;
  corner_cache c0, c1;
};

// ---- Local cell coordinates (batched engine) -----------------------------------
// A particle is carried as its cell (ix, iy, iz) and its offset u in [0, 1)^3
// within that cell, in units of the cell; position = offset + (i + u) * h.
// Samples return the velocity in cells per unit time (scaled by 1/h per
// component), so a stage point is u + c * h * k.  A sample inside the current
// cell needs no floor, division or conversion; the offset keeps 24 bits of
// precision within its cell however far the cell is from the origin.  A
// compensation term (lx, ly, lz) carries what the rounding of each step's
// update dropped from the offset (as compensated_add does for absolute
// positions), so rounding does not accumulate over the steps.
//
// The lane caches the eight corners of the cell it last sampled.  Within a
// warp some lane changes cell at almost every sample, so whatever runs only
// for the lanes that change cell costs the whole warp nearly every sample:
// that part is kept to the eight loads (and, for a stage point outside the
// particle's cell, the floor and clamp), and the interpolation itself runs
// once for all lanes together.
struct local_position
{
  int   ix, iy, iz;
  float ux, uy, uz;
  float lx, ly, lz;
};

// Whether an offset lies in [0, 1): the bit patterns of the floats in [0, 1)
// are exactly the unsigned values below that of 1.0f (negative values, -0,
// infinities and NaNs all compare above), so one unsigned compare per axis —
// or one for the largest of three — does the two-sided test.
__device__ __forceinline__ bool in_unit(float u) { return __float_as_uint(u) < 0x3f800000u; }
__device__ __forceinline__ bool in_unit_cube(float ux, float uy, float uz)
{
  return max(max(__float_as_uint(ux), __float_as_uint(uy)), __float_as_uint(uz)) < 0x3f800000u;
}

// Velocity (cells per unit time) at cell (cx, cy, cz) + (ux, uy, uz), where
// (cx, cy, cz) is the particle's own cell (inside the grid).  The offset may
// lie outside [0, 1) (a stage point that left the cell); the cell it falls in
// is then clamped to the grid (weight 0 or 1).
__device__ __forceinline__ float3 sample_local(const field_view& f, corner_cache& k, int cx, int cy, int cz, float ux, float uy, float uz)
{
  int ix = cx, iy = cy, iz = cz;
  float wx = ux, wy = uy, wz = uz;
  if (!in_unit_cube(ux, uy, uz))
  {
    const float fx = floorf(ux), fy = floorf(uy), fz = floorf(uz);
    ix += int(fx); iy += int(fy); iz += int(fz);
    wx -= fx; wy -= fy; wz -= fz;
    if (ix < 0) { ix = 0; wx = 0.0f; } else if (ix > f.nx - 2) { ix = f.nx - 2; wx = 1.0f; }
    if (iy < 0) { iy = 0; wy = 0.0f; } else if (iy > f.ny - 2) { iy = f.ny - 2; wy = 1.0f; }
    if (iz < 0) { iz = 0; wz = 0.0f; } else if (iz > f.nz - 2) { iz = f.nz - 2; wz = 1.0f; }
  }
  if (ix != k.ix || iy != k.iy || iz != k.iz) corner_load(f, k, ix, iy, iz);
  const float3 v = corner_eval(k, wx, wy, wz);
  const float2 vxy = __fmul2_rn(make_float2(f.inv_hx, f.inv_hy), make_float2(v.x, v.y));
  return make_float3(vxy.x, vxy.y, __fmul_rn(f.inv_hz, v.z));
}

// Moves the offset back into [0, 1) and the cell accordingly.  For an offset
// >= 1 the subtraction of its floor is exact; for a negative offset u, 1 + u
// rounds to within 2^-25 and may give exactly 1 (the same point as offset 0
// of the next cell).
__device__ __forceinline__ void renormalize(local_position& p)
{
  if (!in_unit(p.ux)) { const float fl = floorf(p.ux); p.ix += int(fl); p.ux -= fl; }
  if (!in_unit(p.uy)) { const float fl = floorf(p.uy); p.iy += int(fl); p.uy -= fl; }
  if (!in_unit(p.uz)) { const float fl = floorf(p.uz); p.iz += int(fl); p.uz -= fl; }
}

__device__ __forceinline__ local_position to_local(const field_view& f, const float4& p)
{
  local_position q;
  const axis_cell cx = cell_consistent(p.x, f.ox, f.hx, f.inv_hx);
  const axis_cell cy = cell_consistent(p.y, f.oy, f.hy, f.inv_hy);
  const axis_cell cz = cell_consistent(p.z, f.oz, f.hz, f.inv_hz);
  q.ix = int(cx.s); q.iy = int(cy.s); q.iz = int(cz.s);
  q.ux = cx.w; q.uy = cy.w; q.uz = cz.w;
  q.lx = q.ly = q.lz = 0.0f;
  renormalize(q);   // w can round up to exactly 1
  return q;
}

__device__ __forceinline__ float4 to_absolute(const field_view& f, const local_position& q, float w)
{
  return make_float4(fmaf(float(q.ix) + q.ux, f.hx, f.ox), fmaf(float(q.iy) + q.uy, f.hy, f.oy),
                     fmaf(float(q.iz) + q.uz, f.hz, f.oz), w);
}

// ---- Flow-map positions with sub-ulp residuals ---------------------------------
// An FTLE is a difference quotient of neighbouring flow-map positions, so the
// FP32 rounding of the stored positions (half an ulp: about 1e-5 cells at
// |x| ~ 6 on a 256^3 grid of [0, 2 pi]^3) bounds its accuracy where the FTLE is
// small.  The re-sampled advection kernels therefore store each end position
// as its correctly rounded FP32 coordinates plus, in the otherwise unused w
// lane, the rounding residual of each coordinate as a signed 10-bit code:
// coordinate = x + code / 1022 * ulp(x) (bits 0-9: x, 10-19: y, 20-29: z; the
// top two bits are zero, so w reads as an ordinary float in [0, 2)).  That
// carries each coordinate to about 34 bits.  Frozen-scheme flow maps, the
// reference's FP32 state, store w = 0 (no residual).

// ulp of a normal FP32 x with |x| >= 2^-103; 0 for smaller x (no residual).
__device__ __forceinline__ float residual_ulp(float x)
{
  const unsigned e = __float_as_uint(x) & 0x7f800000u;
  return e > (23u << 23) ? __uint_as_float(e - (23u << 23)) : 0.0f;
}

// 1 / ulp(x) for a normal x with |x| >= 2^-103 (a power of two, so scaling
// by it is exact).
__device__ __forceinline__ float residual_inverse_ulp(float x)
{
  const unsigned e = __float_as_uint(x) & 0x7f800000u;
  return __uint_as_float((277u << 23) - e);
}

// The residual of x coded in w's bits [shift, shift + 10).
__device__ __forceinline__ float residual_value(float x, unsigned w, int shift)
{
  const int q = int(w << (22 - shift)) >> 22;
  return float(q) * (residual_ulp(x) * (1.0f / 1022.0f));
}

// One coordinate o + (i + u + l) h of a local position as its correctly
// rounded FP32 value and residual code, in FP32 error-free arithmetic (the
// FP64 pipe of a GB300 SM runs at 1/64 of the FP32 rate, and a retiring lane
// would run it for its whole warp): TwoSum for i + u, the exact FMA error of
// the product with h, TwoSum for the addition of o.
__device__ __forceinline__ float coordinate_with_residual(int i, float u, float l, float h, float o, unsigned& code)
{
  float s, e1;
  two_sum(float(i), u, s, e1);
  const float p = s * h;
  const float lo1 = fmaf(e1 + l, h, fmaf(s, h, -p));
  float t, e2;
  two_sum(o, p, t, e2);
  const float lo = lo1 + e2;
  const float x = t + lo;                       // RN(t + lo): the correctly rounded coordinate
  const float r = (t - x) + lo;                 // what the rounding dropped
  const unsigned exponent = __float_as_uint(x) & 0x7f800000u;
  if (exponent <= (23u << 23)) { code = 0u; return x; }
  const int q = __float2int_rn(r * residual_inverse_ulp(x) * 1022.0f);
  code = unsigned(max(-511, min(511, q))) & 0x3ffu;
  return x;
}

// The end position of a particle carried in local coordinates, with the
// residual codes in w.
__device__ __forceinline__ float4 flow_position(const field_view& f, const local_position& q)
{
  unsigned cx, cy, cz;
  const float x = coordinate_with_residual(q.ix, q.ux, q.lx, f.hx, f.ox, cx);
  const float y = coordinate_with_residual(q.iy, q.uy, q.ly, f.hy, f.oy, cy);
  const float z = coordinate_with_residual(q.iz, q.uz, q.lz, f.hz, f.oz, cz);
  return make_float4(x, y, z, __uint_as_float(cx | (cy << 10) | (cz << 20)));
}

__device__ __forceinline__ bool local_inside(const field_view& f, const local_position& q)
{
  // 0 <= i < n - 1 as one unsigned compare per axis (false for every i when n = 1)
  return unsigned(q.ix) < unsigned(f.nx - 1) && unsigned(q.iy) < unsigned(f.ny - 1) && unsigned(q.iz) < unsigned(f.nz - 1);
}

// |v_i| <= 1e-5 with v in cells per unit time: |v_i| <= 1e-5 / h_i.
__device__ __forceinline__ bool is_zero_local(const field_view& f, const float3& v)
{
  return fabsf(v.x) <= 1e-5f * f.inv_hx && fabsf(v.y) <= 1e-5f * f.inv_hy && fabsf(v.z) <= 1e-5f * f.inv_hz;
}

// One classical RK4 (or Euler) step in local coordinates with k1 sampled at q.
__device__ __forceinline__ void local_step(const field_view& f, corner_cache& k, int rk4, float h, local_position& q, const float3& k1)
{
  if (!rk4)
  {
    compensated_add(q.ux, q.lx, h * k1.x);
    compensated_add(q.uy, q.ly, h * k1.y);
    compensated_add(q.uz, q.lz, h * k1.z);
    renormalize(q);
    return;
  }
  // x and y as packed pairs, z scalar
  const float hh = 0.5f * h;
  float2 u = make_float2(q.ux, q.uy), l = make_float2(q.lx, q.ly);
  const float2 k1xy = make_float2(k1.x, k1.y);
  const float2 s2 = __ffma2_rn(pair(hh), k1xy, u);
  const float3 k2 = sample_local(f, k, q.ix, q.iy, q.iz, s2.x, s2.y, fmaf(hh, k1.z, q.uz));
  const float2 k2xy = make_float2(k2.x, k2.y);
  const float2 s3 = __ffma2_rn(pair(hh), k2xy, u);
  const float3 k3 = sample_local(f, k, q.ix, q.iy, q.iz, s3.x, s3.y, fmaf(hh, k2.z, q.uz));
  const float2 k3xy = make_float2(k3.x, k3.y);
  const float2 s4 = __ffma2_rn(pair(h), k3xy, u);
  const float3 k4 = sample_local(f, k, q.ix, q.iy, q.iz, s4.x, s4.y, fmaf(h, k3.z, q.uz));
  const float h6 = h * (1.0f / 6.0f);
  rk4_update2(u, l, h6, k1xy, k2xy, k3xy, make_float2(k4.x, k4.y));
  q.ux = u.x; q.uy = u.y; q.lx = l.x; q.ly = l.y;
  rk4_update(q.uz, q.lz, h6, k1.z, k2.z, k3.z, k4.z);
  renormalize(q);
}

// Unsteady sample in local coordinates: the two slices around time t, blended
// linearly in time; velocity in cells per unit time.
__device__ __forceinline__ float3 sample_local_unsteady(const field_view& f, const time_axis& ta, corner_cache2& k, int cx, int cy,
                                                        int cz, float ux, float uy, float uz, const slice_time& t)
{
  int ix = cx, iy = cy, iz = cz;
  float wx = ux, wy = uy, wz = uz;
  if (!in_unit_cube(ux, uy, uz))
  {
    const float fx = floorf(ux), fy = floorf(uy), fz = floorf(uz);
    ix += int(fx); iy += int(fy); iz += int(fz);
    wx -= fx; wy -= fy; wz -= fz;
    if (ix < 0) { ix = 0; wx = 0.0f; } else if (ix > f.nx - 2) { ix = f.nx - 2; wx = 1.0f; }
    if (iy < 0) { iy = 0; wy = 0.0f; } else if (iy > f.ny - 2) { iy = f.ny - 2; wy = 1.0f; }
    if (iz < 0) { iz = 0; wz = 0.0f; } else if (iz > f.nz - 2) { iz = f.nz - 2; wz = 1.0f; }
  }
  int slice;
  float wt;
  slice_of(ta, t, slice, wt);
  if (slice != k.slice || ix != k.c0.ix || iy != k.c0.iy || iz != k.c0.iz)
  {
    field_view s0 = f, s1 = f;
    s0.data = f.data + (long long)slice * ta.slice_stride;
    s1.data = f.data + (long long)(ta.nt > 1 ? slice + 1 : slice) * ta.slice_stride;
    corner_load(s0, k.c0, ix, iy, iz);
    corner_load(s1, k.c1, ix, iy, iz);
    k.slice = slice;
  }
  float3 v = corner_eval(k.c0, wx, wy, wz);
  if (wt != 0.0f)
  {
    const float3 v1 = corner_eval(k.c1, wx, wy, wz);
    v = make_float3(fmaf(wt, v1.x - v.x, v.x), fmaf(wt, v1.y - v.y, v.y), fmaf(wt, v1.z - v.z, v.z));
  }
  return make_float3(f.inv_hx * v.x, f.inv_hy * v.y, f.inv_hz * v.z);
}

// One pathline step in local coordinates: classical RK4 in space-time (stages
// at t, t + h/2, t + h/2, t + h) or Euler, k1 sampled at (q, t).
__device__ __forceinline__ void local_unsteady_step(const field_view& f, const time_axis& ta, const slice_clock& clock,
                                                    corner_cache2& k, int rk4, float h, local_position& q, const float3& k1,
                                                    const slice_time& t)
{
  if (!rk4)
  {
    compensated_add(q.ux, q.lx, h * k1.x);
    compensated_add(q.uy, q.ly, h * k1.y);
    compensated_add(q.uz, q.lz, h * k1.z);
    renormalize(q);
    return;
  }
  const float hh = 0.5f * h;
  const slice_time th = advance_time(t, clock, 0.5f), t1 = advance_time(t, clock, 1.0f);
  const float3 k2 = sample_local_unsteady(f, ta, k, q.ix, q.iy, q.iz, fmaf(hh, k1.x, q.ux), fmaf(hh, k1.y, q.uy), fmaf(hh, k1.z, q.uz), th);
  const float3 k3 = sample_local_unsteady(f, ta, k, q.ix, q.iy, q.iz, fmaf(hh, k2.x, q.ux), fmaf(hh, k2.y, q.uy), fmaf(hh, k2.z, q.uz), th);
  const float3 k4 = sample_local_unsteady(f, ta, k, q.ix, q.iy, q.iz, fmaf(h, k3.x, q.ux), fmaf(h, k3.y, q.uy), fmaf(h, k3.z, q.uz), t1);
  const float h6 = h * (1.0f / 6.0f);
  compensated_add(q.ux, q.lx, h6 * (k1.x + 2.0f * (k2.x + k3.x) + k4.x));
  compensated_add(q.uy, q.ly, h6 * (k1.y + 2.0f * (k2.y + k3.y) + k4.y));
  compensated_add(q.uz, q.lz, h6 * (k1.z + 2.0f * (k2.z + k3.z) + k4.z));
  renormalize(q);
}

// RESAMPLED step of any scheme in local coordinates (k1 sampled at q, in cells
// per unit time): the classic step above, an explicit tableau (stage s at
// u + h sum_j a_sj k_j), or a two-step Adams scheme whose history (the
// previous step's k1) is kept per particle; offsets accumulate compensated.
__device__ __forceinline__ void general_step_local(const field_view& f, corner_cache& cache, const step_rule& r, local_position& q,
                                                   const float3& k1, frozen_history& hist)
{
  if (r.scheme == scheme_classic) { local_step(f, cache, r.rk4, r.h, q, k1); return; }
  float3 delta;
  if (r.scheme == scheme_tableau)
  {
    const rk_tableau& T = rk_tableaux[r.tableau];
    float3 k[13];
    k[0] = k1;
    for (int s = 1; s < T.stages; ++s)
    {
      float3 acc = make_float3(0.f, 0.f, 0.f);
      for (int j = 0; j < s; ++j)
      {
        const float a = T.a[s][j];
        if (a != 0.0f) acc = make_float3(fmaf(a, k[j].x, acc.x), fmaf(a, k[j].y, acc.y), fmaf(a, k[j].z, acc.z));
      }
      k[s] = sample_local(f, cache, q.ix, q.iy, q.iz, fmaf(r.h, acc.x, q.ux), fmaf(r.h, acc.y, q.uy), fmaf(r.h, acc.z, q.uz));
    }
    float3 sum = make_float3(0.f, 0.f, 0.f);
    for (int s = 0; s < T.stages; ++s)
    {
      const float b = T.b[s];
      if (b != 0.0f) sum = make_float3(fmaf(b, k[s].x, sum.x), fmaf(b, k[s].y, sum.y), fmaf(b, k[s].z, sum.z));
    }
    delta = make_float3(r.h * sum.x, r.h * sum.y, r.h * sum.z);
  }
  else
  {
    // Adams-Bashforth 2: u + h (3/2 k_n - 1/2 k_{n-1}); a particle's first
    // step is RK4.  Adams-Bashforth-Moulton 2: that prediction u*, then the
    // trapezoid u + h/2 (k_n + f(u*)).
    local_position predicted = q;
    if (hist.started)
    {
      compensated_add(predicted.ux, predicted.lx, r.h * fmaf(1.5f, k1.x, -0.5f * hist.v.x));
      compensated_add(predicted.uy, predicted.ly, r.h * fmaf(1.5f, k1.y, -0.5f * hist.v.y));
      compensated_add(predicted.uz, predicted.lz, r.h * fmaf(1.5f, k1.z, -0.5f * hist.v.z));
      renormalize(predicted);
    }
    else
      local_step(f, cache, 1, r.h, predicted, k1);
    hist.v = k1;
    hist.started = 1;
    if (r.scheme == scheme_adams_bashforth) { q = predicted; return; }
    // f(u*) relative to the particle's own cell, which is inside the grid:
    // the predictor's cell may not be, and sample_local clamps only offsets
    // that leave the given cell (the cell differences are small integers, so
    // the shifted offsets are exact).
    const float3 kp = sample_local(f, cache, q.ix, q.iy, q.iz, predicted.ux + float(predicted.ix - q.ix),
                                   predicted.uy + float(predicted.iy - q.iy), predicted.uz + float(predicted.iz - q.iz));
    const float hh = 0.5f * r.h;
    delta = make_float3(hh * (k1.x + kp.x), hh * (k1.y + kp.y), hh * (k1.z + kp.z));
  }
  compensated_add(q.ux, q.lx, delta.x);
  compensated_add(q.uy, q.ly, delta.y);
  compensated_add(q.uz, q.lz, delta.z);
  renormalize(q);
}

// Face crossed by a particle leaving its block: the reference's else-if ladder
// (particle_tracer.cpp:288-293) — the first face, in order -x,+x,-y,+y,-z,+z,
// whose strict bound test holds and whose neighbour exists; -1 if none.
__device__ __forceinline__ int exit_face(const field_view& f, const float4& p, const int* neighbor)
{
  if (p.x < f.ox   && neighbor[0] >= 0) return 0;
  if (p.x > f.maxx && neighbor[1] >= 0) return 1;
  if (p.y < f.oy   && neighbor[2] >= 0) return 2;
  if (p.y > f.maxy && neighbor[3] >= 0) return 3;
  if (p.z < f.oz   && neighbor[4] >= 0) return 4;
  if (p.z > f.maxz && neighbor[5] >= 0) return 5;
  return -1;
}
}
