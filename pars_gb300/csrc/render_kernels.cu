// Ray tracing of integral curves and a scalar volume on the GPU: the
// counterpart of pars::ray_tracer (pars/source/stages/ray_tracer.cpp:7-253),
// which hands the same scene to OSPRay on the CPU.
//
// Scene (ray_tracer.cpp:28-44, 156-211): every line index i of a batch is a
// capsule -- a cylinder of the streamline radius around the segment
// (vertex[i], vertex[i+1]) with spheres of that radius at both ends -- coloured
// with vertex colour[i] (the colour the reference always writes for an index,
// color_generator.cpp:30-37); a structured scalar volume (ray_tracer.cpp:
// 130-163) with the piecewise-linear transfer function of :46-54 (colour black
// -> white, opacity 0.0001 -> 0.0255 over values 0 -> 1).
// Camera (:62-66, 213-229): perspective, fovy 68 degrees, aspect = width /
// height, image rows from the top (imageStart (0, 1), imageEnd (1, 0)).
// Lights (:68-91): ambient intensity 1; two distant lights travelling along
// (1, 1, -0.5) and (-1, 0, 0.5), colour (1, 1, 0.8).  Material (:158-161):
// diffuse 0.8 times the vertex colour, specular 0.7 with exponent 10, lit on
// the side facing the light only; no shadows, no ambient occlusion (aoSamples
// 0), background (0, 0, 0, 1), one sample per pixel per frame, frames
// accumulated (OSP_FB_ACCUM) until the camera, image size or scene changes.
//
// OSPRay is not part of this library; the shading above is this library's own
// definition of that configuration (the CPU restatement in the oracle follows
// it operation by operation).  Output: sRGB-encoded RGBA8 (OSP_FB_SRGBA).
//
// GPU design: one thread per pixel in 8 x 8 tiles (coherent primary rays);
// the curves' capsules sit in a linear BVH (Karras, "Maximizing parallelism in
// the construction of BVHs, octrees, and k-d trees", HPG 2012) built on the
// device from 30-bit Morton codes in a handful of launches; a node holds both
// children's boxes (one 64-byte fetch tests two boxes).  The closest hit is
// the smallest (distance, segment) pair, so it does not depend on the order in
// which the tree is walked.  This file is compiled without FMA contraction, so
// every operation rounds as the CPU restatement's does.
#include "context.hpp"

#include <climits>
#include <cmath>
#include <cstring>

namespace pars
{
namespace
{
constexpr int render_tile = 8;
constexpr int stack_depth = 64;
// A BVH leaf holds a run of up to K consecutive segments of one curve (a new
// leaf starts at a curve break and where the segment's start vertex crosses a
// multiple of K), packed as the run's first start vertex | (segments - 1) <<
// 56.  K = 2 from 2 M segments up, 1 below: on the served stream's scenes (up
// to 32 M segments) pairs made the builds 2.4 times faster for 10 % more
// render time per frame (+6.5 % requests/s with one lane, +8 % with two;
// runs of 4 and 8: -1 % and -34 %), while on a 520 k-segment scene single
// segments render 16 % faster.
constexpr long long leaf_vertex_mask = (1LL << 56) - 1;
constexpr long long leaf_pairs_from = 2LL << 20;
int leaf_segments_for(long long segments) { return segments >= leaf_pairs_from ? 2 : 1; }

unsigned int blocks_for(long long work, int threads)
{
  const long long b = (work + threads - 1) / threads;
  return (unsigned int)(b < 1 ? 1 : b);
}

__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 scale3(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float  dot3(float3 a, float3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float3 normalize3(float3 a)
{
  const float l = sqrtf(dot3(a, a));
  return make_float3(a.x / l, a.y / l, a.z / l);
}
__device__ __forceinline__ float3 xyz(float4 a) { return make_float3(a.x, a.y, a.z); }

// Order-preserving map of a float to an unsigned integer (for atomicMin/Max).
__device__ __forceinline__ unsigned int float_key(float f)
{
  const unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(unsigned int k)
{
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// ---- BVH build ------------------------------------------------------------------
// bounds[0..2]: min of the segment centres, [3..5]: their max, [6]: max
// |coordinate|.  Grid-stride over the prims, reduced per block (shuffles, then
// shared memory), so the seven global atomics are taken once per block.
constexpr int bounds_threads = 256;

__global__ void __launch_bounds__(bounds_threads) scene_bounds_kernel(const float4* __restrict__ vertices,
                                                                      const long long* __restrict__ prim_vertex, long long prims,
                                                                      unsigned int* __restrict__ bounds)
{
  float v[7] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY, 0.0f};
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < prims; k += (long long)gridDim.x * blockDim.x)
  {
    const long long g = prim_vertex[k];
    const float4 a = vertices[g], b = vertices[g + 1];
    const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
    for (int i = 0; i < 3; ++i) { v[i] = fminf(v[i], c[i]); v[3 + i] = fmaxf(v[3 + i], c[i]); }
    v[6] = fmaxf(v[6], fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fmaxf(fabsf(a.z), fabsf(b.x))), fmaxf(fabsf(b.y), fabsf(b.z))));
  }
  for (int off = 16; off > 0; off >>= 1)
    for (int i = 0; i < 7; ++i)
    {
      const float o = __shfl_down_sync(0xffffffffu, v[i], off);
      v[i] = i < 3 ? fminf(v[i], o) : fmaxf(v[i], o);
    }
  __shared__ float partial[bounds_threads / 32][7];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int i = 0; i < 7; ++i) partial[warp][i] = v[i];
  __syncthreads();
  if (threadIdx.x < 7)
  {
    const int i = threadIdx.x;
    float r = partial[0][i];
    for (int w = 1; w < bounds_threads / 32; ++w) r = i < 3 ? fminf(r, partial[w][i]) : fmaxf(r, partial[w][i]);
    if (i < 3) atomicMin(bounds + i, float_key(r));
    else atomicMax(bounds + i, float_key(r));
  }
}

__device__ __forceinline__ unsigned int spread_bits(unsigned int v)
{
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__device__ __forceinline__ unsigned int quantize(float x, float lo, float hi)
{
  const float extent = hi - lo;
  float u = extent > 0.0f ? (x - lo) / extent : 0.0f;
  u = fminf(fmaxf(u * 1024.0f, 0.0f), 1023.0f);
  return (unsigned int)u;
}

// 1 where segment k starts a leaf: the first segment, a segment that does
// not continue its predecessor's curve, or one whose start vertex enters the
// next block of `segments` vertices.
__global__ void leaf_start_kernel(const long long* __restrict__ prim_vertex, long long prims, int segments, int* __restrict__ flags)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= prims) return;
  int start = 1;
  if (k > 0)
  {
    const long long g = prim_vertex[k], p = prim_vertex[k - 1];
    start = (g != p + 1 || g / segments != p / segments) ? 1 : 0;
  }
  flags[k] = start;
}

// first[l] = the first segment of leaf l.
__global__ void leaf_first_kernel(const int* __restrict__ flags, const long long* __restrict__ index, long long prims,
                                  long long* __restrict__ first)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < prims && flags[k]) first[index[k]] = k;
}

// Leaf boxes (the union of the leaf's capsule boxes, padded so that a hit
// computed in FP32 lies strictly inside it) and Morton keys of the box
// centres; run[l] = the leaf's packed first start vertex and segment count.
__global__ void leaf_kernel(const float4* __restrict__ vertices, const long long* __restrict__ prim_vertex, long long prims,
                            const long long* __restrict__ first, long long leaves, float radius,
                            const unsigned int* __restrict__ bounds, float4* __restrict__ leaf_lo, float4* __restrict__ leaf_hi,
                            long long* __restrict__ run, unsigned long long* __restrict__ keys, unsigned int* __restrict__ values)
{
  const long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= leaves) return;
  // first == nullptr: one segment per leaf
  const long long f = first ? first[l] : l;
  const long long count = first ? (l + 1 < leaves ? first[l + 1] : prims) - f : 1;
  const long long g = prim_vertex[f];
  float4 v = vertices[g];
  float3 lo = make_float3(v.x, v.y, v.z), hi = lo;
  for (long long s = 1; s <= count; ++s)
  {
    v = vertices[g + s];
    lo = make_float3(fminf(lo.x, v.x), fminf(lo.y, v.y), fminf(lo.z, v.z));
    hi = make_float3(fmaxf(hi.x, v.x), fmaxf(hi.y, v.y), fmaxf(hi.z, v.z));
  }
  const float pad = radius + (radius + key_float(bounds[6])) * (1.0f / 65536.0f);
  leaf_lo[l] = make_float4(lo.x - pad, lo.y - pad, lo.z - pad, 0.0f);
  leaf_hi[l] = make_float4(hi.x + pad, hi.y + pad, hi.z + pad, 0.0f);
  run[l] = g | ((count - 1) << 56);
  const unsigned int mx = quantize((lo.x + hi.x) * 0.5f, key_float(bounds[0]), key_float(bounds[3]));
  const unsigned int my = quantize((lo.y + hi.y) * 0.5f, key_float(bounds[1]), key_float(bounds[4]));
  const unsigned int mz = quantize((lo.z + hi.z) * 0.5f, key_float(bounds[2]), key_float(bounds[5]));
  keys[l] = (unsigned long long)((spread_bits(mx) << 2) | (spread_bits(my) << 1) | spread_bits(mz));
  values[l] = (unsigned int)l;
}

// Leaves in key order: their boxes, packed runs and parent (set later).
__global__ void leaf_order_kernel(const unsigned int* __restrict__ order, long long leaves, const long long* __restrict__ run,
                                  const float4* __restrict__ leaf_lo, const float4* __restrict__ leaf_hi,
                                  float4* __restrict__ sorted_lo, float4* __restrict__ sorted_hi, long long* __restrict__ sorted_run)
{
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= leaves) return;
  const unsigned int k = order[j];
  sorted_lo[j] = leaf_lo[k];
  sorted_hi[j] = leaf_hi[k];
  sorted_run[j] = run[k];
}

// Common prefix length of keys i and j (ties broken by position); -1 outside.
__device__ __forceinline__ int prefix(const unsigned long long* __restrict__ keys, long long n, long long i, long long j)
{
  if (j < 0 || j >= n) return -1;
  const unsigned long long a = keys[i], b = keys[j];
  if (a != b) return __clzll(a ^ b);
  return 64 + __clzll((unsigned long long)(i ^ j));
}

struct __align__(16) bvh_node
{
  float4 a;   // left.lo.xyz, left.hi.x
  float4 b;   // left.hi.yz, right.lo.xy
  float4 c;   // right.lo.z, right.hi.xyz
  int4   d;   // left, right (>= 0 node, < 0 leaf ~j)
};

// Karras' construction: internal node i covers a key range with i at one end;
// its split is where the common prefix of the range ends.
__global__ void internal_nodes_kernel(const unsigned long long* __restrict__ keys, long long n, bvh_node* __restrict__ nodes,
                                      int* __restrict__ node_parent, int* __restrict__ leaf_parent)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = prefix(keys, n, i, i + 1) - prefix(keys, n, i, i - 1) >= 0 ? 1 : -1;
  const int minimum = prefix(keys, n, i, i - d);
  long long span = 2;
  while (prefix(keys, n, i, i + span * d) > minimum) span *= 2;
  long long length = 0;
  for (long long t = span / 2; t >= 1; t /= 2)
    if (prefix(keys, n, i, i + (length + t) * d) > minimum) length += t;
  const long long j = i + length * d;
  const int node_prefix = prefix(keys, n, i, j);
  long long split = 0, t = length;
  do
  {
    t = (t + 1) >> 1;
    if (prefix(keys, n, i, i + (split + t) * d) > node_prefix) split += t;
  } while (t > 1);
  const long long gamma = i + split * d + (d < 0 ? -1 : 0);
  const long long first = d > 0 ? i : j, last = d > 0 ? j : i;
  int left, right;
  if (first == gamma) { left = ~int(gamma); leaf_parent[gamma] = int(i); }
  else { left = int(gamma); node_parent[gamma] = int(i); }
  if (last == gamma + 1) { right = ~int(gamma + 1); leaf_parent[gamma + 1] = int(i); }
  else { right = int(gamma + 1); node_parent[gamma + 1] = int(i); }
  nodes[i].d = make_int4(left, right, 0, 0);
  if (i == 0) node_parent[0] = -1;
}

// Bottom-up boxes: each leaf walks towards the root; the second child to
// reach a node computes the node's box (the first stops there).
__global__ void refit_kernel(long long n, const float4* __restrict__ sorted_lo, const float4* __restrict__ sorted_hi,
                             const int* __restrict__ leaf_parent, const int* __restrict__ node_parent, bvh_node* nodes,
                             int* __restrict__ arrivals, int* __restrict__ status)
{
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  float3 lo = xyz(sorted_lo[j]), hi = xyz(sorted_hi[j]);
  int child = ~int(j);
  int p = leaf_parent[j];
  // a Karras tree over at most 2^31 keys of 30 bits is at most 62 levels deep
  for (int level = 0; p >= 0; ++level)
  {
    if (level >= 128) { atomicOr(status, 2); return; }
    bvh_node* node = nodes + p;
    const int4 d = __ldcg(&node->d);
    if (d.x == child)
    {
      __stcg(&node->a, make_float4(lo.x, lo.y, lo.z, hi.x));
      __stcg(&node->b.x, hi.y);
      __stcg(&node->b.y, hi.z);
    }
    else
    {
      __stcg(&node->b.z, lo.x);
      __stcg(&node->b.w, lo.y);
      __stcg(&node->c, make_float4(lo.z, hi.x, hi.y, hi.z));
    }
    __threadfence();
    if (atomicAdd(arrivals + p, 1) == 0) return;
    __threadfence();
    const float4 a = __ldcg(&node->a), b = __ldcg(&node->b), c = __ldcg(&node->c);
    lo = make_float3(fminf(a.x, b.z), fminf(a.y, b.w), fminf(a.z, c.x));
    hi = make_float3(fmaxf(a.w, c.y), fmaxf(b.x, c.z), fmaxf(b.y, c.w));
    child = p;
    p = node_parent[p];
  }
}

// ---- rendering ---------------------------------------------------------------------
struct render_args
{
  int          width, height;
  float3       origin, corner, du, dv;     // ray(sx, sy) = normalize(corner + sx du + sy dv)
  float3       light[2];                   // unit vectors towards the lights
  float3       light_color[2];
  float        ambient, kd, ks;
  // curves
  const bvh_node*  nodes;
  const float4*    leaf_lo;                // root box when the tree is one leaf
  const float4*    leaf_hi;
  const long long* leaf_vertex;            // each leaf's run: first start vertex | (segments - 1) << 56
  long long        leaves;
  const unsigned int* bounds;              // scene bounds of the build (the leaf padding)
  const float4*    vertices;
  const float4*    colors;                 // nullptr: white
  float            radius;
  // volume
  const float*     volume;                 // [x][y][z] or nullptr
  int              vx, vy, vz;
  float3           vo, vh, vhi;
  float            dt;
  // frames
  const float2*    jitter;
  int              frames;
  float4*          accum;
  int*             status;                 // bit 0: traversal stack overflow
};

struct hit_record
{
  float     t;
  long long g;        // segment start vertex (LLONG_MAX: no hit)
  int       part;     // 0 body, 1 sphere at the start, 2 sphere at the end
};

// Slab test of a box against [0, t_max]; NaNs from 0 * inf are ignored.
__device__ __forceinline__ bool box_hit(float3 o, float3 inv, float lx, float ly, float lz, float hx, float hy, float hz,
                                        float t_max, float& t_near)
{
  const float tx0 = (lx - o.x) * inv.x, tx1 = (hx - o.x) * inv.x;
  const float ty0 = (ly - o.y) * inv.y, ty1 = (hy - o.y) * inv.y;
  const float tz0 = (lz - o.z) * inv.z, tz1 = (hz - o.z) * inv.z;
  const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
  const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), t_max));
  t_near = tn;
  return tn <= tf;
}

// Nearest entry (> 0) of the ray into sphere c of radius r, origin shifted to
// o (the ray's closest approach to the segment start); INFINITY if none.
__device__ __forceinline__ float sphere_entry(float3 o, float3 d, float3 c, float r)
{
  const float3 oc = sub3(o, c);
  const float b = dot3(d, oc);
  const float h = b * b - (dot3(oc, oc) - r * r);
  if (h < 0.0f) return INFINITY;
  return -b - sqrtf(h);
}

// Capsule test for segment (a, b): updates `best` when this segment's nearest
// entry beats it (smaller distance, or equal distance and smaller vertex).
__device__ __forceinline__ void capsule_test(float3 o, float3 d, float4 a4, float4 b4, float r, long long g, hit_record& best)
{
  const float3 a = xyz(a4), b = xyz(b4);
  // shift the origin to the point of the ray nearest to a: the quadratics
  // below then work with distances of the segment's own size
  const float tc = dot3(sub3(a, o), d);
  const float3 s = add3(o, scale3(d, tc));
  float t = INFINITY;
  int part = -1;
  const float3 ba = sub3(b, a), sa = sub3(s, a);
  const float baba = dot3(ba, ba);
  if (baba > 0.0f)
  {
    const float bard = dot3(ba, d), baoa = dot3(ba, sa), rdoa = dot3(d, sa), oaoa = dot3(sa, sa);
    const float qa = baba - bard * bard;
    if (qa > 0.0f)
    {
      const float qb = baba * rdoa - baoa * bard;
      const float qc = baba * oaoa - baoa * baoa - r * r * baba;
      const float h = qb * qb - qa * qc;
      if (h >= 0.0f)
      {
        const float u = (-qb - sqrtf(h)) / qa;
        const float y = baoa + u * bard;
        if (y > 0.0f && y < baba && tc + u > 0.0f) { t = tc + u; part = 0; }
      }
    }
  }
  const float ea = tc + sphere_entry(s, d, a, r);
  if (ea > 0.0f && ea < t) { t = ea; part = 1; }
  const float eb = tc + sphere_entry(s, d, b, r);
  if (eb > 0.0f && eb < t) { t = eb; part = 2; }
  if (part >= 0 && (t < best.t || (t == best.t && g < best.g))) { best.t = t; best.g = g; best.part = part; }
}

// The capsules of one leaf's run of consecutive segments.  In a run of more
// than one, each segment's own padded box (the box its one-segment leaf would
// have) is tested before its capsule, as the tree's bottom levels would.
// RUNS false: every leaf is one segment (scenes below leaf_pairs_from).
template <bool RUNS>
__device__ __forceinline__ void leaf_test(const render_args& A, float3 o, float3 d, float3 inv, long long packed, hit_record& best)
{
  const long long g = packed & leaf_vertex_mask;
  const int count = RUNS ? int(packed >> 56) + 1 : 1;
  float4 a = A.vertices[g];
  if (count == 1) { capsule_test(o, d, a, A.vertices[g + 1], A.radius, g, best); return; }
  const float pad = A.radius + (A.radius + key_float(A.bounds[6])) * (1.0f / 65536.0f);
  for (int s = 0; s < count; ++s)
  {
    const float4 b = A.vertices[g + s + 1];
    float tn;
    if (box_hit(o, inv, fminf(a.x, b.x) - pad, fminf(a.y, b.y) - pad, fminf(a.z, b.z) - pad, fmaxf(a.x, b.x) + pad,
                fmaxf(a.y, b.y) + pad, fmaxf(a.z, b.z) + pad, best.t, tn))
      capsule_test(o, d, a, b, A.radius, g + s, best);
    a = b;
  }
}

template <bool RUNS>
__device__ hit_record closest_hit(const render_args& A, float3 o, float3 d, float3 inv)
{
  hit_record best {INFINITY, LLONG_MAX, -1};
  if (A.leaves <= 0) return best;
  if (A.leaves == 1)
  {
    float tn;
    const float4 lo = A.leaf_lo[0], hi = A.leaf_hi[0];
    if (box_hit(o, inv, lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, INFINITY, tn)) leaf_test<RUNS>(A, o, d, inv, A.leaf_vertex[0], best);
    return best;
  }
  int stack[stack_depth];
  int sp = 0;
  int ref = 0;
  // each node is visited at most once; the bound only guards a malformed tree
  for (long long visits = 0;; ++visits)
  {
    if (visits > A.leaves) { atomicOr(A.status, 4); break; }
    const bvh_node* node = A.nodes + ref;
    const float4 na = __ldg(&node->a), nb = __ldg(&node->b), nc = __ldg(&node->c);
    const int4 nd = __ldg(&node->d);
    float tl, tr;
    const bool hl = box_hit(o, inv, na.x, na.y, na.z, na.w, nb.x, nb.y, best.t, tl);
    const bool hr = box_hit(o, inv, nb.z, nb.w, nc.x, nc.y, nc.z, nc.w, best.t, tr);
    int next[2];
    int count = 0;
    // leaves are tested at once; internal children are visited nearest first
    if (hl)
    {
      if (nd.x < 0) leaf_test<RUNS>(A, o, d, inv, A.leaf_vertex[~nd.x], best);
      else next[count++] = nd.x;
    }
    if (hr)
    {
      if (nd.y < 0) leaf_test<RUNS>(A, o, d, inv, A.leaf_vertex[~nd.y], best);
      else next[count++] = nd.y;
    }
    if (count == 2)
    {
      const bool swap = tr < tl;
      ref = swap ? next[1] : next[0];
      if (sp < stack_depth) stack[sp++] = swap ? next[0] : next[1];
      else atomicOr(A.status, 1);
      continue;
    }
    if (count == 1) { ref = next[0]; continue; }
    if (sp == 0) break;
    ref = stack[--sp];
  }
  return best;
}

__device__ __forceinline__ float lerp_volume(float a, float b, float w) { return a + w * (b - a); }

// Trilinear sample of the volume at p (cell by floor of the IEEE quotient,
// clamped to the grid; lerp along z, then y, then x).
__device__ float volume_sample(const render_args& A, float3 p)
{
  const float qx = (p.x - A.vo.x) / A.vh.x, qy = (p.y - A.vo.y) / A.vh.y, qz = (p.z - A.vo.z) / A.vh.z;
  const float fx = fminf(fmaxf(floorf(qx), 0.0f), float(A.vx - 2));
  const float fy = fminf(fmaxf(floorf(qy), 0.0f), float(A.vy - 2));
  const float fz = fminf(fmaxf(floorf(qz), 0.0f), float(A.vz - 2));
  const float wx = fminf(fmaxf(qx - fx, 0.0f), 1.0f), wy = fminf(fmaxf(qy - fy, 0.0f), 1.0f), wz = fminf(fmaxf(qz - fz, 0.0f), 1.0f);
  const long long ix = (long long)fx, iy = (long long)fy, iz = (long long)fz;
  const long long sy = A.vz, sx = (long long)A.vy * A.vz;
  const float* c = A.volume + ix * sx + iy * sy + iz;
  const float c000 = __ldg(c), c001 = __ldg(c + 1), c010 = __ldg(c + sy), c011 = __ldg(c + sy + 1);
  const float c100 = __ldg(c + sx), c101 = __ldg(c + sx + 1), c110 = __ldg(c + sx + sy), c111 = __ldg(c + sx + sy + 1);
  const float c00 = lerp_volume(c000, c001, wz), c01 = lerp_volume(c010, c011, wz);
  const float c10 = lerp_volume(c100, c101, wz), c11 = lerp_volume(c110, c111, wz);
  const float c0 = lerp_volume(c00, c01, wy), c1 = lerp_volume(c10, c11, wy);
  return lerp_volume(c0, c1, wx);
}

// Linear RGB of the surface hit: ambient + two distant lights, diffuse and
// specular (x^10), lit only where the normal faces the light.
__device__ float3 shade(const render_args& A, float3 o, float3 d, const hit_record& h)
{
  const float4 a4 = A.vertices[h.g], b4 = A.vertices[h.g + 1];
  const float3 a = xyz(a4), b = xyz(b4);
  const float3 p = add3(o, scale3(d, h.t));
  float3 n;
  if (h.part == 1) n = sub3(p, a);
  else if (h.part == 2) n = sub3(p, b);
  else
  {
    const float3 ba = sub3(b, a), pa = sub3(p, a);
    n = sub3(pa, scale3(ba, dot3(pa, ba) / dot3(ba, ba)));
  }
  n = normalize3(n);
  const float3 v = make_float3(-d.x, -d.y, -d.z);
  float3 base = make_float3(A.kd, A.kd, A.kd);
  if (A.colors)
  {
    const float4 c = A.colors[h.g];
    base = make_float3(A.kd * c.x, A.kd * c.y, A.kd * c.z);
  }
  float3 out = scale3(base, A.ambient);
  for (int l = 0; l < 2; ++l)
  {
    const float ndl = dot3(n, A.light[l]);
    if (ndl <= 0.0f) continue;
    const float3 lc = A.light_color[l];
    out = add3(out, make_float3(base.x * ndl * lc.x, base.y * ndl * lc.y, base.z * ndl * lc.z));
    const float ndh = dot3(n, normalize3(add3(A.light[l], v)));
    if (ndh > 0.0f)
    {
      const float x2 = ndh * ndh, x4 = x2 * x2, x8 = x4 * x4, s = A.ks * (x8 * x2);
      out = add3(out, make_float3(s * lc.x, s * lc.y, s * lc.z));
    }
  }
  return out;
}

template <bool RUNS>
__global__ void __launch_bounds__(render_tile * render_tile) render_kernel(render_args A)
{
  const int px = blockIdx.x * render_tile + threadIdx.x, py = blockIdx.y * render_tile + threadIdx.y;
  if (px >= A.width || py >= A.height) return;
  const long long pixel = (long long)py * A.width + px;
  float4 acc = A.accum[pixel];
  for (int f = 0; f < A.frames; ++f)
  {
    const float2 j = A.jitter[f];
    const float sx = (float(px) + j.x) / float(A.width);
    const float sy = 1.0f - (float(py) + j.y) / float(A.height);
    const float3 r = make_float3(A.corner.x + sx * A.du.x + sy * A.dv.x, A.corner.y + sx * A.du.y + sy * A.dv.y,
                                 A.corner.z + sx * A.du.z + sy * A.dv.z);
    const float3 d = normalize3(r);
    const float3 inv = make_float3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    const float3 o = A.origin;
    const hit_record h = closest_hit<RUNS>(A, o, d, inv);
    float cr = 0.0f, cg = 0.0f, cb = 0.0f, alpha = 0.0f;
    if (A.volume)
    {
      float t_enter;
      if (box_hit(o, inv, A.vo.x, A.vo.y, A.vo.z, A.vhi.x, A.vhi.y, A.vhi.z, INFINITY, t_enter))
      {
        // far end of the box
        const float tx = fmaxf((A.vo.x - o.x) * inv.x, (A.vhi.x - o.x) * inv.x);
        const float ty = fmaxf((A.vo.y - o.y) * inv.y, (A.vhi.y - o.y) * inv.y);
        const float tz = fmaxf((A.vo.z - o.z) * inv.z, (A.vhi.z - o.z) * inv.z);
        const float t_exit = fminf(fminf(fminf(tx, ty), tz), h.t);
        for (int k = 0; k < (1 << 22); ++k)
        {
          const float t = t_enter + (float(k) + 0.5f) * A.dt;
          if (!(t < t_exit)) break;
          const float value = fminf(fmaxf(volume_sample(A, add3(o, scale3(d, t))), 0.0f), 1.0f);
          const float opacity = 0.0001f + value * 0.0254f;
          const float a = 1.0f - sqrtf(1.0f - opacity);   // two samples per cell
          const float w = (1.0f - alpha) * a;
          cr = cr + w * value; cg = cg + w * value; cb = cb + w * value;
          alpha = alpha + w;
        }
      }
    }
    if (h.part >= 0)
    {
      const float3 s = shade(A, o, d, h);
      const float w = 1.0f - alpha;
      cr = cr + w * s.x; cg = cg + w * s.y; cb = cb + w * s.z;
    }
    acc.x = acc.x + fminf(fmaxf(cr, 0.0f), 1.0f);
    acc.y = acc.y + fminf(fmaxf(cg, 0.0f), 1.0f);
    acc.z = acc.z + fminf(fmaxf(cb, 0.0f), 1.0f);
    acc.w = acc.w + 1.0f;
  }
  A.accum[pixel] = acc;
}

// sRGB8 of the average: the byte q is the count of thresholds (linear values
// where the rounded sRGB code steps up) at or below the value.
__device__ __forceinline__ unsigned int srgb_byte(float c, const float* __restrict__ thresholds)
{
  unsigned int lo = 0, hi = 255;       // answer in [lo, hi]
  while (lo < hi)
  {
    const unsigned int mid = (lo + hi + 1) >> 1;
    if (c >= thresholds[mid - 1]) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void encode_kernel(const float4* __restrict__ accum, long long pixels, float frames, const float* __restrict__ thresholds,
                              uchar4* __restrict__ out)
{
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= pixels) return;
  const float4 a = accum[p];
  out[p] = make_uchar4((unsigned char)srgb_byte(a.x / frames, thresholds), (unsigned char)srgb_byte(a.y / frames, thresholds),
                       (unsigned char)srgb_byte(a.z / frames, thresholds), 255);
}

__global__ void span_prims_kernel(const int* __restrict__ indices, long long vertex_offset, long long count, long long* __restrict__ out)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count) out[k] = vertex_offset + indices[k];
}

__global__ void curve_prims_kernel(const int* __restrict__ indices, const long long* __restrict__ vbounds,
                                   const long long* __restrict__ ibounds, int batches, long long total, long long* __restrict__ out)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  int lo = 0, hi = batches - 1;
  while (lo < hi)
  {
    const int mid = (lo + hi + 1) >> 1;
    if (ibounds[mid] <= k) lo = mid;
    else hi = mid - 1;
  }
  out[k] = vbounds[lo] + indices[k];
}
}  // namespace

// ---- host side ----------------------------------------------------------------------
render_state::render_state()
{
  // sRGB thresholds: the linear value at which the rounded 8-bit sRGB code
  // reaches q + 1, q = 0..254 (IEC 61966-2-1 transfer function, in double)
  for (int q = 0; q < 255; ++q)
  {
    const double s = (q + 0.5) / 255.0;
    srgb_thresholds[q] = float(s <= 0.04045 ? s / 12.92 : std::pow((s + 0.055) / 1.055, 2.4));
  }
}

void render_jitter(long long frame, float& jx, float& jy)
{
  if (frame == 0) { jx = 0.5f; jy = 0.5f; return; }
  // Halton points in bases 2 and 3 (radical inverses of the frame number)
  double x = 0.0, f = 0.5;
  for (long long i = frame; i > 0; i /= 2, f *= 0.5) x += f * double(i % 2);
  double y = 0.0, g = 1.0 / 3.0;
  for (long long i = frame; i > 0; i /= 3, g /= 3.0) y += g * double(i % 3);
  jx = float(x);
  jy = float(y);
}

void render_camera(const float position[3], const float forward[3], const float up[3], int width, int height,
                   float corner[3], float du[3], float dv[3])
{
  const double pi = 3.14159265358979323846;
  double f[3] = {forward[0], forward[1], forward[2]};
  const double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  for (auto& x : f) x /= fl;
  double u[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
  const double ul = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  for (auto& x : u) x /= ul;
  const double v[3] = {u[1] * f[2] - u[2] * f[1], u[2] * f[0] - u[0] * f[2], u[0] * f[1] - u[1] * f[0]};
  const double size_y = 2.0 * std::tan(68.0 * pi / 360.0);
  const double size_x = size_y * double(width) / double(height);
  for (int i = 0; i < 3; ++i)
  {
    corner[i] = float(f[i] - 0.5 * size_x * u[i] - 0.5 * size_y * v[i]);
    du[i] = float(size_x * u[i]);
    dv[i] = float(size_y * v[i]);
  }
}

void render_clear(render_state& r)
{
  r.frames = 0;
  r.accum_valid = false;
}

// Builds the BVH over r.prim_vertex (r.prims segments of r.vertices): leaves
// are runs of up to leaf_segments_for(r.prims) consecutive segments of one
// curve.
void render_build(pars_gpu_context& ctx, render_state& r)
{
  r.tree_valid = false;
  r.leaves = 0;
  const long long prims = r.prims;
  if (prims <= 0) { r.tree_valid = true; return; }
  PARS_REQUIRE(prims < (1LL << 31) - 1, "too many curve segments for one scene");
  // the leaves of runs of two: start flags, their exclusive sum (leaf
  // numbers; one host read of the count) and each leaf's first segment
  long long n = prims;
  const long long* first = nullptr;
  if (leaf_segments_for(prims) > 1)
  {
    r.leaf_flags.reserve(sizeof(int) * prims);
    r.leaf_index.reserve(sizeof(long long) * (prims + 1));
    leaf_start_kernel<<<blocks_for(prims, 256), 256, 0, ctx.stream>>>(r.prim_vertex.as<long long>(), prims, leaf_segments_for(prims),
                                                                      r.leaf_flags.as<int>());
    PARS_CUDA(cudaGetLastError());
    exclusive_sum(ctx, r.leaf_flags.as<int>(), r.leaf_index.as<long long>(), prims);
    PARS_CUDA(cudaMemcpyAsync(&n, r.leaf_index.as<long long>() + prims, sizeof(long long), cudaMemcpyDeviceToHost, ctx.stream));
    PARS_CUDA(cudaStreamSynchronize(ctx.stream));
    PARS_REQUIRE(n >= 1 && n <= prims, "leaf count out of range");
    r.leaf_first.reserve(sizeof(long long) * n);
    leaf_first_kernel<<<blocks_for(prims, 256), 256, 0, ctx.stream>>>(r.leaf_flags.as<int>(), r.leaf_index.as<long long>(), prims,
                                                                      r.leaf_first.as<long long>());
    first = r.leaf_first.as<const long long>();
  }
  launch_scope scope(ctx, "bvh_build");
  r.status.reserve(sizeof(int));
  PARS_CUDA(cudaMemsetAsync(r.status.get(), 0, sizeof(int), ctx.stream));
  r.bounds.reserve(sizeof(unsigned int) * 8);
  unsigned int init[8] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u, 0u, 0u};
  PARS_CUDA(cudaMemcpyAsync(r.bounds.get(), init, sizeof(init), cudaMemcpyHostToDevice, ctx.stream));
  const unsigned int blocks = blocks_for(n, 256);
  if (ctx.sm_count <= 0) PARS_CUDA(cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, ctx.device));
  const unsigned int bound_blocks = std::min<unsigned int>(blocks_for(prims, bounds_threads), unsigned(std::max(ctx.sm_count, 1)) * 4);
  scene_bounds_kernel<<<bound_blocks, bounds_threads, 0, ctx.stream>>>(r.vertices, r.prim_vertex.as<long long>(), prims,
                                                                       r.bounds.as<unsigned int>());
  r.leaf_lo_unsorted.reserve(sizeof(float4) * n);
  r.leaf_hi_unsorted.reserve(sizeof(float4) * n);
  r.leaf_run.reserve(sizeof(long long) * n);
  r.keys.reserve(sizeof(unsigned long long) * n * 2);
  r.values.reserve(sizeof(unsigned int) * n * 2);
  auto* keys = r.keys.as<unsigned long long>();
  auto* values = r.values.as<unsigned int>();
  leaf_kernel<<<blocks, 256, 0, ctx.stream>>>(r.vertices, r.prim_vertex.as<long long>(), prims, first, n,
                                              r.radius, r.bounds.as<unsigned int>(), r.leaf_lo_unsorted.as<float4>(),
                                              r.leaf_hi_unsorted.as<float4>(), r.leaf_run.as<long long>(), keys, values);
  PARS_CUDA(cudaGetLastError());
  sort_pairs(ctx, keys, keys + n, values, values + n, n, 30);
  r.leaf_lo.reserve(sizeof(float4) * n);
  r.leaf_hi.reserve(sizeof(float4) * n);
  r.leaf_vertex.reserve(sizeof(long long) * n);
  leaf_order_kernel<<<blocks, 256, 0, ctx.stream>>>(values + n, n, r.leaf_run.as<long long>(), r.leaf_lo_unsorted.as<float4>(),
                                                    r.leaf_hi_unsorted.as<float4>(), r.leaf_lo.as<float4>(), r.leaf_hi.as<float4>(),
                                                    r.leaf_vertex.as<long long>());
  if (n > 1)
  {
    r.nodes.reserve(sizeof(bvh_node) * (n - 1));
    r.node_parent.reserve(sizeof(int) * (n - 1));
    r.leaf_parent.reserve(sizeof(int) * n);
    r.arrivals.reserve(sizeof(int) * (n - 1));
    PARS_CUDA(cudaMemsetAsync(r.arrivals.get(), 0, sizeof(int) * (n - 1), ctx.stream));
    internal_nodes_kernel<<<blocks_for(n - 1, 256), 256, 0, ctx.stream>>>(keys + n, n, r.nodes.as<bvh_node>(), r.node_parent.as<int>(),
                                                                           r.leaf_parent.as<int>());
    refit_kernel<<<blocks, 256, 0, ctx.stream>>>(n, r.leaf_lo.as<float4>(), r.leaf_hi.as<float4>(), r.leaf_parent.as<int>(),
                                                 r.node_parent.as<int>(), r.nodes.as<bvh_node>(), r.arrivals.as<int>(),
                                                 r.status.as<int>());
  }
  PARS_CUDA(cudaGetLastError());
  r.leaves = n;
  r.tree_valid = true;
  r.status_pending = true;    // the build's status is read with the next frames
}

// Prims of the context's curves (indexed): one per packed line index.
void render_use_context_curves(pars_gpu_context& ctx, render_state& r)
{
  auto& c = ctx.curves;
  if (!c.indexed) throw error(PARS_ERR_STATE, "curves must be indexed before they are rendered");
  r.prims = c.index_total;
  r.vertices = c.vertices.as<const float4>();
  r.colors = c.colored ? c.colors.as<const float4>() : nullptr;
  r.prim_vertex.reserve(sizeof(long long) * std::max<long long>(r.prims, 1));
  const int batches = int(c.batches.size());
  if (r.prims > 0)
  {
    std::vector<long long> bounds(2 * (batches + 1));
    for (int b = 0; b < batches; ++b) { bounds[b] = c.batches[b].vertex_offset; bounds[batches + 1 + b] = c.batches[b].index_offset; }
    bounds[batches] = c.vertex_total;
    bounds[2 * batches + 1] = c.index_total;
    r.batch_bounds.reserve(sizeof(long long) * bounds.size());
    PARS_CUDA(cudaMemcpyAsync(r.batch_bounds.get(), bounds.data(), sizeof(long long) * bounds.size(), cudaMemcpyHostToDevice, ctx.stream));
    const long long* vb = r.batch_bounds.as<long long>();
    curve_prims_kernel<<<blocks_for(r.prims, 256), 256, 0, ctx.stream>>>(c.indices.as<const int>(), vb, vb + batches + 1, batches,
                                                                        r.prims, r.prim_vertex.as<long long>());
    PARS_CUDA(cudaGetLastError());
    // the host copy of the bounds must outlive the asynchronous copy
    PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  }
}

void render_use_spans(pars_gpu_context& ctx, render_state& r, const float4* vertices, const float4* colors, const int* indices,
                      const std::vector<std::array<long long, 3>>& spans)
{
  long long total = 0;
  for (const auto& s : spans) total += s[2];
  r.prims = total;
  r.vertices = vertices;
  r.colors = colors;
  r.prim_vertex.reserve(sizeof(long long) * std::max<long long>(total, 1));
  long long first = 0;
  for (const auto& s : spans)
  {
    if (s[2] <= 0) continue;
    span_prims_kernel<<<blocks_for(s[2], 256), 256, 0, ctx.stream>>>(indices + s[1], s[0], s[2], r.prim_vertex.as<long long>() + first);
    first += s[2];
  }
  PARS_CUDA(cudaGetLastError());
  r.curves_generation = -1;
  r.tree_valid = false;
  render_clear(r);
}

void render_set_view(render_state& r, const float position[3], const float forward[3], const float up[3], int width, int height)
{
  for (int i = 0; i < 3; ++i) { r.position[i] = position[i]; r.forward[i] = forward[i]; r.up[i] = up[i]; }
  r.camera_set = true;
  r.width = width;
  r.height = height;
  render_camera(r.position, r.forward, r.up, r.width, r.height, r.corner, r.du, r.dv);
  render_clear(r);
}

void render_frames(pars_gpu_context& ctx, render_state& r, int iterations)
{
  PARS_REQUIRE(r.width > 0 && r.height > 0, "image size not set");
  PARS_REQUIRE(r.camera_set, "camera not set");
  PARS_REQUIRE(iterations >= 0, "iterations must be >= 0");
  if (!r.tree_valid) render_build(ctx, r);
  const long long pixels = (long long)r.width * r.height;
  if (!r.accum_valid)
  {
    r.accum.reserve(sizeof(float4) * pixels);
    PARS_CUDA(cudaMemsetAsync(r.accum.get(), 0, sizeof(float4) * pixels, ctx.stream));
    r.frames = 0;
    r.accum_valid = true;
  }
  if (iterations == 0) return;
  std::vector<float2> jitter(iterations);
  for (int i = 0; i < iterations; ++i) render_jitter(r.frames + i, jitter[i].x, jitter[i].y);
  r.jitter.reserve(sizeof(float2) * iterations);
  PARS_CUDA(cudaMemcpyAsync(r.jitter.get(), jitter.data(), sizeof(float2) * iterations, cudaMemcpyHostToDevice, ctx.stream));
  r.status.reserve(sizeof(int));
  if (r.tree_valid && !r.status_pending) PARS_CUDA(cudaMemsetAsync(r.status.get(), 0, sizeof(int), ctx.stream));
  r.status_pending = false;

  render_args A {};
  A.width = r.width; A.height = r.height;
  A.origin = make_float3(r.position[0], r.position[1], r.position[2]);
  A.corner = make_float3(r.corner[0], r.corner[1], r.corner[2]);
  A.du = make_float3(r.du[0], r.du[1], r.du[2]);
  A.dv = make_float3(r.dv[0], r.dv[1], r.dv[2]);
  const double directions[2][3] = {{1.0, 1.0, -0.5}, {-1.0, 0.0, 0.5}};
  for (int l = 0; l < 2; ++l)
  {
    const double* dl = directions[l];
    const double len = std::sqrt(dl[0] * dl[0] + dl[1] * dl[1] + dl[2] * dl[2]);
    A.light[l] = make_float3(float(-dl[0] / len), float(-dl[1] / len), float(-dl[2] / len));
    A.light_color[l] = make_float3(1.0f, 1.0f, 0.8f);
  }
  A.ambient = 1.0f; A.kd = 0.8f; A.ks = 0.7f;
  A.nodes = r.nodes.as<const bvh_node>();
  A.leaf_lo = r.leaf_lo.as<const float4>();
  A.leaf_hi = r.leaf_hi.as<const float4>();
  A.leaf_vertex = r.leaf_vertex.as<const long long>();
  A.leaves = r.leaves;
  A.vertices = r.vertices;
  A.colors = r.colors;
  A.radius = r.radius;
  if (r.has_volume)
  {
    A.volume = r.volume_data;
    A.vx = r.volume_shape[0]; A.vy = r.volume_shape[1]; A.vz = r.volume_shape[2];
    A.vo = make_float3(r.volume_offset[0], r.volume_offset[1], r.volume_offset[2]);
    A.vh = make_float3(r.volume_spacing[0], r.volume_spacing[1], r.volume_spacing[2]);
    A.vhi = make_float3(r.volume_offset[0] + float(r.volume_shape[0] - 1) * r.volume_spacing[0],
                        r.volume_offset[1] + float(r.volume_shape[1] - 1) * r.volume_spacing[1],
                        r.volume_offset[2] + float(r.volume_shape[2] - 1) * r.volume_spacing[2]);
    A.dt = 0.5f * std::min(r.volume_spacing[0], std::min(r.volume_spacing[1], r.volume_spacing[2]));
  }
  A.jitter = r.jitter.as<const float2>();
  A.frames = iterations;
  A.accum = r.accum.as<float4>();
  A.status = r.status.as<int>();
  A.bounds = r.bounds.as<const unsigned int>();
  const dim3 block(render_tile, render_tile);
  const dim3 grid((r.width + render_tile - 1) / render_tile, (r.height + render_tile - 1) / render_tile);
  {
    launch_scope scope(ctx, "render");
    if (r.leaves < r.prims) render_kernel<true><<<grid, block, 0, ctx.stream>>>(A);
    else render_kernel<false><<<grid, block, 0, ctx.stream>>>(A);
  }
  PARS_CUDA(cudaGetLastError());
  int status = 0;
  PARS_CUDA(cudaMemcpyAsync(&status, r.status.get(), sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  if (status) throw error(PARS_ERR_STATE, (status & 1) ? "BVH traversal stack overflow" : "malformed BVH");
  r.frames += iterations;
}

void render_encode(pars_gpu_context& ctx, render_state& r, uint8_t* host_rgba)
{
  PARS_REQUIRE(r.width > 0 && r.height > 0, "image size not set");
  const long long pixels = (long long)r.width * r.height;
  r.image.reserve(sizeof(uchar4) * pixels);
  r.thresholds.reserve(sizeof(float) * 255);
  PARS_CUDA(cudaMemcpyAsync(r.thresholds.get(), r.srgb_thresholds, sizeof(float) * 255, cudaMemcpyHostToDevice, ctx.stream));
  if (!r.accum_valid || r.frames == 0)
  {
    // nothing traced yet: the background
    for (long long p = 0; p < pixels; ++p)
    {
      host_rgba[4 * p] = host_rgba[4 * p + 1] = host_rgba[4 * p + 2] = 0;
      host_rgba[4 * p + 3] = 255;
    }
    return;
  }
  {
    launch_scope scope(ctx, "render_encode");
    encode_kernel<<<blocks_for(pixels, 256), 256, 0, ctx.stream>>>(r.accum.as<const float4>(), pixels, float(r.frames),
                                                                  r.thresholds.as<const float>(), r.image.as<uchar4>());
  }
  PARS_CUDA(cudaGetLastError());
  PARS_CUDA(cudaMemcpyAsync(host_rgba, r.image.get(), sizeof(uchar4) * pixels, cudaMemcpyDeviceToHost, ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
}
}  // namespace pars

// ---- C ABI: the ray tracer of a context (ray_tracer.hpp:27-34) ----------------------
using pars::error;
using pars::render_state;

namespace
{
render_state& tracer_of(pars_gpu_context* ctx)
{
  if (!ctx->render) ctx->render = std::make_unique<render_state>();
  return *ctx->render;
}

void check_volume_args(const int32_t shape[3], const float offset[3], const float spacing[3])
{
  PARS_REQUIRE(shape && offset && spacing, "shape, offset and spacing are required");
  for (int i = 0; i < 3; ++i)
  {
    PARS_REQUIRE(shape[i] >= 2, "every volume extent must be >= 2");
    PARS_REQUIRE(spacing[i] > 0.0f, "volume spacing must be positive");
  }
}

void set_volume(pars_gpu_context* ctx, const float* values, bool device, const int32_t shape[3], const float offset[3], const float spacing[3])
{
  check_volume_args(shape, offset, spacing);
  PARS_REQUIRE(values, "volume values are required");
  auto& r = tracer_of(ctx);
  const std::size_t bytes = sizeof(float) * (std::size_t)shape[0] * shape[1] * shape[2];
  r.volume.reserve(bytes);
  PARS_CUDA(cudaMemcpyAsync(r.volume.get(), values, bytes, device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
  PARS_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int i = 0; i < 3; ++i)
  {
    r.volume_shape[i] = shape[i];
    r.volume_offset[i] = offset[i];
    r.volume_spacing[i] = spacing[i];
  }
  r.has_volume = true;
  r.volume_data = r.volume.as<const float>();
  pars::render_clear(r);
}
}

// The library is built with hidden visibility; only the C ABI is exported.
#pragma GCC visibility push(default)
extern "C" {

int32_t pars_gpu_ray_tracer_set_volume(pars_gpu_context* ctx, const float* values, const int32_t shape[3], const float offset[3],
                                       const float spacing[3])
{
  return pars::run_guarded(ctx, [&] { set_volume(ctx, values, false, shape, offset, spacing); });
}

int32_t pars_gpu_ray_tracer_set_volume_device(pars_gpu_context* ctx, const float* device_values, const int32_t shape[3],
                                              const float offset[3], const float spacing[3])
{
  return pars::run_guarded(ctx, [&] { set_volume(ctx, device_values, true, shape, offset, spacing); });
}

int32_t pars_gpu_ray_tracer_clear_volume(pars_gpu_context* ctx)
{
  return pars::run_guarded(ctx, [&] {
    auto& r = tracer_of(ctx);
    r.has_volume = false;
    r.volume_data = nullptr;
    r.volume.release();
    pars::render_clear(r);
  });
}

int32_t pars_gpu_ray_tracer_set_integral_curves(pars_gpu_context* ctx, float radius)
{
  return pars::run_guarded(ctx, [&] {
    PARS_REQUIRE(radius > 0.0f, "radius must be positive");
    auto& r = tracer_of(ctx);
    r.radius = radius;
    pars::render_use_context_curves(*ctx, r);
    r.curves_generation = ctx->curves.generation;
    r.tree_valid = false;
    pars::render_clear(r);
  });
}

int32_t pars_gpu_ray_tracer_set_integral_curves_host(pars_gpu_context* ctx, int64_t batches, const int64_t* vertex_counts,
                                                     const float* const* vertices, const float* const* colors,
                                                     const int64_t* index_counts, const int32_t* const* indices, float radius)
{
  return pars::run_guarded(ctx, [&] {
    PARS_REQUIRE(radius > 0.0f, "radius must be positive");
    PARS_REQUIRE(batches >= 0 && (batches == 0 || (vertex_counts && vertices && index_counts && indices)), "curve arrays are required");
    auto& r = tracer_of(ctx);
    long long total_vertices = 0, total_indices = 0;
    bool with_colors = colors != nullptr;
    for (int64_t b = 0; b < batches; ++b)
    {
      PARS_REQUIRE(vertex_counts[b] >= 0 && index_counts[b] >= 0, "negative counts");
      if (index_counts[b] == 0) continue;
      total_vertices += vertex_counts[b];
      total_indices += index_counts[b];
      if (colors && !colors[b]) with_colors = false;
    }
    r.own_vertices.reserve(sizeof(float4) * std::max<long long>(total_vertices, 1));
    if (with_colors) r.own_colors.reserve(sizeof(float4) * std::max<long long>(total_vertices, 1));
    std::vector<long long> prims;
    prims.reserve(total_indices);
    long long offset = 0;
    for (int64_t b = 0; b < batches; ++b)
    {
      if (index_counts[b] == 0) continue;   // batches without indices are not rendered (ray_tracer.cpp:183-184)
      const long long nv = vertex_counts[b];
      for (int64_t k = 0; k < index_counts[b]; ++k)
      {
        const int32_t i = indices[b][k];
        PARS_REQUIRE(i >= 0 && (long long)i + 1 < nv, "line index out of range");
        prims.push_back(offset + i);
      }
      PARS_CUDA(cudaMemcpyAsync(r.own_vertices.as<float4>() + offset, vertices[b], sizeof(float4) * nv, cudaMemcpyHostToDevice, ctx->stream));
      if (with_colors)
        PARS_CUDA(cudaMemcpyAsync(r.own_colors.as<float4>() + offset, colors[b], sizeof(float4) * nv, cudaMemcpyHostToDevice, ctx->stream));
      offset += nv;
    }
    r.prims = (long long)prims.size();
    r.prim_vertex.reserve(sizeof(long long) * std::max<long long>(r.prims, 1));
    if (r.prims)
      PARS_CUDA(cudaMemcpyAsync(r.prim_vertex.get(), prims.data(), sizeof(long long) * r.prims, cudaMemcpyHostToDevice, ctx->stream));
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    r.vertices = r.own_vertices.as<const float4>();
    r.colors = with_colors ? r.own_colors.as<const float4>() : nullptr;
    r.radius = radius;
    r.curves_generation = -1;
    r.tree_valid = false;
    pars::render_clear(r);
  });
}

int32_t pars_gpu_ray_tracer_set_camera(pars_gpu_context* ctx, const float position[3], const float forward[3], const float up[3])
{
  return pars::run_guarded(ctx, [&] {
    PARS_REQUIRE(position && forward && up, "position, forward and up are required");
    auto& r = tracer_of(ctx);
    for (int i = 0; i < 3; ++i) { r.position[i] = position[i]; r.forward[i] = forward[i]; r.up[i] = up[i]; }
    r.camera_set = true;
    if (r.width > 0) pars::render_camera(r.position, r.forward, r.up, r.width, r.height, r.corner, r.du, r.dv);
    pars::render_clear(r);
  });
}

int32_t pars_gpu_ray_tracer_set_image_size(pars_gpu_context* ctx, int32_t width, int32_t height)
{
  return pars::run_guarded(ctx, [&] {
    PARS_REQUIRE(width > 0 && height > 0 && (long long)width * height <= (1LL << 28), "image size out of range");
    auto& r = tracer_of(ctx);
    r.width = width;
    r.height = height;
    if (r.camera_set) pars::render_camera(r.position, r.forward, r.up, r.width, r.height, r.corner, r.du, r.dv);
    pars::render_clear(r);
  });
}

int32_t pars_gpu_ray_tracer_trace(pars_gpu_context* ctx, int32_t iterations)
{
  return pars::run_guarded(ctx, [&] {
    auto& r = tracer_of(ctx);
    if (r.curves_generation >= 0 && r.curves_generation != ctx->curves.generation)
      throw error(PARS_ERR_STATE, "the context's curves changed after set_integral_curves");
    pars::render_frames(*ctx, r, iterations);
  });
}

int32_t pars_gpu_ray_tracer_serialize(pars_gpu_context* ctx, uint8_t* rgba, int32_t size[2])
{
  return pars::run_guarded(ctx, [&] {
    auto& r = tracer_of(ctx);
    PARS_REQUIRE(r.width > 0 && r.height > 0, "image size not set");
    if (size) { size[0] = r.width; size[1] = r.height; }
    if (rgba) pars::render_encode(*ctx, r, rgba);
  });
}

// The `image` message (pars/proto/image.proto): size = 1 (repeated int32,
// packed as proto3 writes it), data = 2 (bytes); fields in number order.
int32_t pars_gpu_image_encode(const int32_t size[2], const uint8_t* data, int64_t data_bytes, uint8_t* out, int64_t capacity,
                              int64_t* length)
{
  if (!size || !length || data_bytes < 0 || (data_bytes > 0 && !data)) return PARS_ERR_INVALID_ARGUMENT;
  auto varint_size = [](uint64_t v) { int64_t n = 1; while (v >= 0x80) { v >>= 7; ++n; } return n; };
  auto put_varint = [](uint8_t*& p, uint64_t v) { while (v >= 0x80) { *p++ = uint8_t(v | 0x80); v >>= 7; } *p++ = uint8_t(v); };
  // int32 values are sign-extended to 64 bits on the wire
  const uint64_t w = (uint64_t)(int64_t)size[0], h = (uint64_t)(int64_t)size[1];
  const int64_t packed = varint_size(w) + varint_size(h);
  int64_t total = 1 + varint_size((uint64_t)packed) + packed;
  if (data_bytes > 0) total += 1 + varint_size((uint64_t)data_bytes) + data_bytes;
  *length = total;
  if (!out) return PARS_OK;
  if (capacity < total) return PARS_ERR_INVALID_ARGUMENT;
  uint8_t* p = out;
  *p++ = 0x0A;
  put_varint(p, (uint64_t)packed);
  put_varint(p, w);
  put_varint(p, h);
  if (data_bytes > 0)
  {
    *p++ = 0x12;
    put_varint(p, (uint64_t)data_bytes);
    std::memcpy(p, data, (std::size_t)data_bytes);
  }
  return PARS_OK;
}

int32_t pars_gpu_ray_tracer_frames(pars_gpu_context* ctx, int64_t* frames)
{
  return pars::run_guarded(ctx, [&] {
    PARS_REQUIRE(frames, "frames is required");
    *frames = ctx->render ? ctx->render->frames : 0;
  });
}

}  // extern "C"
#pragma GCC visibility pop
