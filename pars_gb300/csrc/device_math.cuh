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
// The RESAMPLED path (classical RK4 with four samples per step) keeps the
// reference's contains() test for termination but samples with a consistent
// cell/weight pair, FMA lerps, and accumulates positions with a compensation
// term (see cell_consistent and compensated_add).
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

// Outside the grid the cell index is clamped to [0, n-2] and the weight to 0
// or 1 (constant extension of the boundary values).
__device__ __forceinline__ void clamp_cell(axis_cell& c, int n)
{
  if (!(c.s >= 0.0f)) { c.s = 0.0f; c.w = 0.0f; }
  else if (c.s > float(n - 2)) { c.s = float(n - 2); c.w = 1.0f; }
}

// Trilinear blend with FMAs (re-sampled path; not bit-exact with the reference).
__device__ __forceinline__ float lerp_fast(float a, float b, float w) { return fmaf(w, b - a, a); }
__device__ __forceinline__ float3 gather_blend_fast(const field_view& f, int ix, int iy, int iz, float wx, float wy, float wz)
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
  float3 out;
  out.x = lerp_fast(lerp_fast(lerp_fast(c000.x, c001.x, wz), lerp_fast(c010.x, c011.x, wz), wy),
                    lerp_fast(lerp_fast(c100.x, c101.x, wz), lerp_fast(c110.x, c111.x, wz), wy), wx);
  out.y = lerp_fast(lerp_fast(lerp_fast(c000.y, c001.y, wz), lerp_fast(c010.y, c011.y, wz), wy),
                    lerp_fast(lerp_fast(c100.y, c101.y, wz), lerp_fast(c110.y, c111.y, wz), wy), wx);
  out.z = lerp_fast(lerp_fast(lerp_fast(c000.z, c001.z, wz), lerp_fast(c010.z, c011.z, wz), wy),
                    lerp_fast(lerp_fast(c100.z, c101.z, wz), lerp_fast(c110.z, c111.z, wz), wy), wx);
  return out;
}

__device__ __forceinline__ float3 sample_clamped(const field_view& f, float px, float py, float pz)
{
  axis_cell cx = cell_consistent(px, f.ox, f.hx, f.inv_hx), cy = cell_consistent(py, f.oy, f.hy, f.inv_hy),
            cz = cell_consistent(pz, f.oz, f.hz, f.inv_hz);
  clamp_cell(cx, f.nx); clamp_cell(cy, f.ny); clamp_cell(cz, f.nz);
  return gather_blend_fast(f, int(cx.s), int(cy.s), int(cz.s), cx.w, cy.w, cz.w);
}

// First stage of a re-sampled step: the reference's contains() decides
// termination (floor of the IEEE quotient, as vector_field.cpp:16-17), and the
// velocity comes from the consistent sampler.
__device__ __forceinline__ bool sample_inside_resampled(const field_view& f, const float4& p, float3& v)
{
  const float sx = floorf(__fdiv_rn(__fsub_rn(p.x, f.ox), f.hx));
  const float sy = floorf(__fdiv_rn(__fsub_rn(p.y, f.oy), f.hy));
  const float sz = floorf(__fdiv_rn(__fsub_rn(p.z, f.oz), f.hz));
  if (!(cell_inside(sx, f.nx) && cell_inside(sy, f.ny) && cell_inside(sz, f.nz))) return false;
  v = sample_clamped(f, p.x, p.y, p.z);
  return true;
}

// Eigen isZero() with its default precision (NumTraits<float>::dummy_precision).
__device__ __forceinline__ bool is_zero(const float3& v)
{
  const float precision = 1e-5f;
  return fabsf(v.x) <= precision && fabsf(v.y) <= precision && fabsf(v.z) <= precision;
}

// Integrator parameters.  FROZEN: out = 1*x + c_0 v + ... + c_{k-1} v with
// c_i = b_i * h (b_i in FP32), accumulated left to right.  RESAMPLED: classical
// RK4 (or Euler) with a sample at each stage point.
struct step_rule
{
  int   frozen;      // 1 = frozen velocity, 0 = resampled stages
  int   rk4;         // 1 = RK4, 0 = Euler
  int   count;       // number of frozen coefficients
  float c[4];        // frozen coefficients b_i * h
  float h;           // step size
};

__device__ __forceinline__ float frozen_component(const step_rule& r, float x, float v)
{
  float acc = x;   // 1 * x is exact
  #pragma unroll
  for (int i = 0; i < 4; ++i)
    if (i < r.count) acc = __fadd_rn(acc, __fmul_rn(r.c[i], v));
  return acc;
}

// FROZEN step from x with the velocity v = v(x): the reference's operation order.
__device__ __forceinline__ float4 frozen_step(const step_rule& r, const float4& x, const float3& v)
{
  return make_float4(frozen_component(r, x.x, v.x), frozen_component(r, x.y, v.y),
                     frozen_component(r, x.z, v.z), frozen_component(r, x.w, 0.0f));
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

// RESAMPLED step: classical RK4 (or Euler) with the first-stage velocity k1
// already sampled at x; stage points are sampled with sample_clamped.
__device__ __forceinline__ void resampled_step(const field_view& f, const step_rule& r, float4& x, float3& lo, const float3& k1)
{
  if (!r.rk4)
  {
    compensated_add(x.x, lo.x, r.h * k1.x);
    compensated_add(x.y, lo.y, r.h * k1.y);
    compensated_add(x.z, lo.z, r.h * k1.z);
    return;
  }
  const float hh = 0.5f * r.h;
  const float3 k2 = sample_clamped(f, fmaf(hh, k1.x, x.x), fmaf(hh, k1.y, x.y), fmaf(hh, k1.z, x.z));
  const float3 k3 = sample_clamped(f, fmaf(hh, k2.x, x.x), fmaf(hh, k2.y, x.y), fmaf(hh, k2.z, x.z));
  const float3 k4 = sample_clamped(f, fmaf(r.h, k3.x, x.x), fmaf(r.h, k3.y, x.y), fmaf(r.h, k3.z, x.z));
  const float h6 = r.h * (1.0f / 6.0f);
  compensated_add(x.x, lo.x, h6 * (k1.x + 2.0f * (k2.x + k3.x) + k4.x));
  compensated_add(x.y, lo.y, h6 * (k1.y + 2.0f * (k2.y + k3.y) + k4.y));
  compensated_add(x.z, lo.z, h6 * (k1.z + 2.0f * (k2.z + k3.z) + k4.z));
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
