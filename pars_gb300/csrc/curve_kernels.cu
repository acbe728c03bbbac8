// Index and colour generation on device-resident curve batches.
//
// index_generator::generate (pa/source/stages/index_generator.cpp:10-24):
//   indices = [ i for i in 0..n-2 if v[i] != termination and v[i+1] != termination ]
//   in increasing order — a stream compaction, done here in two passes over
//   tiles (count, scan of tile counts, write).
// color_generator::generate (pa/source/stages/color_generator.cpp:16-98): one
//   thread per index; the FP32 operations follow the reference one by one with
//   explicit round-to-nearest intrinsics (no FMA contraction).  The tangent's
//   squared norm is reduced in the order of Eigen's SSE packet reduction,
//   (d0^2 + d2^2) + (d1^2 + d3^2).  atan2 and acos are FP32 functions on both
//   sides (the host libm's there, CUDA's here), so hue / saturation colours
//   agree to a few FP32 ulps rather than bit for bit.
#include <cub/cub.cuh>

#include "context.hpp"

namespace pars
{
namespace
{
constexpr int index_threads = 256;
constexpr int index_items   = 8;
constexpr int index_tile    = index_threads * index_items;

__device__ __forceinline__ bool index_flag(const float4* __restrict__ v, long long i, long long n)
{
  return i + 1 < n && !is_termination_vertex(v[i]) && !is_termination_vertex(v[i + 1]);
}

__global__ void __launch_bounds__(index_threads) index_count_kernel(const float4* __restrict__ v, long long n, int* __restrict__ tile_counts)
{
  using reduce = cub::BlockReduce<int, index_threads>;
  __shared__ typename reduce::TempStorage storage;
  const long long first = (long long)blockIdx.x * index_tile + (long long)threadIdx.x * index_items;
  int count = 0;
  #pragma unroll
  for (int k = 0; k < index_items; ++k) count += index_flag(v, first + k, n) ? 1 : 0;
  const int total = reduce(storage).Sum(count);
  if (threadIdx.x == 0) tile_counts[blockIdx.x] = total;
}

__global__ void __launch_bounds__(index_threads) index_write_kernel(const float4* __restrict__ v, long long n,
                                                                    const long long* __restrict__ tile_offsets, int* __restrict__ indices)
{
  using scan = cub::BlockScan<int, index_threads>;
  __shared__ typename scan::TempStorage storage;
  const long long first = (long long)blockIdx.x * index_tile + (long long)threadIdx.x * index_items;
  bool flags[index_items];
  int count = 0;
  #pragma unroll
  for (int k = 0; k < index_items; ++k) { flags[k] = index_flag(v, first + k, n); count += flags[k] ? 1 : 0; }
  int prefix = 0;
  scan(storage).ExclusiveSum(count, prefix);
  long long out = tile_offsets[blockIdx.x] + prefix;
  #pragma unroll
  for (int k = 0; k < index_items; ++k)
    if (flags[k]) indices[out++] = int(first + k);
}

// ---- colours ----------------------------------------------------------------
__device__ __forceinline__ float clamp01(float x) { return x < 0.0f ? 0.0f : (1.0f < x ? 1.0f : x); }

__device__ __forceinline__ float4 hue_to_rgba(float hue)
{
  const float six_h = __fmul_rn(6.0f, hue);
  return make_float4(clamp01(__fsub_rn(fabsf(__fsub_rn(six_h, 3.0f)), 1.0f)),
                     clamp01(__fsub_rn(2.0f, fabsf(__fsub_rn(six_h, 2.0f)))),
                     clamp01(__fsub_rn(2.0f, fabsf(__fsub_rn(six_h, 4.0f)))),
                     1.0f);
}

// Error-free sum (Knuth's TwoSum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// float(sqrt(double(x)^2 + double(y)^2 + double(z)^2)) — the reference's
// radius (coordinates.hpp:8-16: std::pow(float, int) promotes to double) — in
// FP32 arithmetic: each square as an exact pair (product + FMA remainder), the
// six terms summed error-free into hi + lo, then the correctly rounded square
// root of hi + lo, decided against the rounding midpoints of sqrtf(hi) with the
// exact remainder hi - r0^2.  It can differ from the double evaluation only
// where the root lies within about 2^-46 of a float midpoint (no case in
// 300,000 random and axis-aligned tangents).
__device__ __forceinline__ float reference_radius(float x, float y, float z)
{
  const float px = __fmul_rn(x, x), py = __fmul_rn(y, y), pz = __fmul_rn(z, z);
  const float ex = __fmaf_rn(x, x, -px), ey = __fmaf_rn(y, y, -py), ez = __fmaf_rn(z, z, -pz);
  float s1, t1, s2, t2;
  two_sum(px, py, s1, t1);
  two_sum(s1, pz, s2, t2);
  float lo = __fadd_rn(__fadd_rn(__fadd_rn(t1, t2), __fadd_rn(ex, ey)), ez);
  const float hi = __fadd_rn(s2, lo);
  lo = __fsub_rn(lo, __fsub_rn(hi, s2));
  const float r0 = __fsqrt_rn(hi);
  const float rho = __fadd_rn(__fmaf_rn(-r0, r0, hi), lo);          // (hi + lo) - r0^2
  const float up = __int_as_float(__float_as_int(r0) + 1), dn = __int_as_float(__float_as_int(r0) - 1);
  const float u = __fsub_rn(up, r0), ud = __fsub_rn(r0, dn);       // ulps above and below r0
  // (r0 + u/2)^2 - r0^2 = r0 u + u^2/4, (r0 - ud/2)^2 - r0^2 = -r0 ud + ud^2/4
  if (rho > __fadd_rn(__fmul_rn(r0, u), __fmul_rn(__fmul_rn(u, u), 0.25f))) return up;
  if (rho < __fadd_rn(__fmul_rn(-r0, ud), __fmul_rn(__fmul_rn(ud, ud), 0.25f))) return dn;
  return r0;
}

__device__ float4 color_of(const float4& a, const float4& b, int mode, float parameter)
{
  // (b - a).normalized() as Eigen evaluates it for Vector4f.
  float4 d = make_float4(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y), __fsub_rn(b.z, a.z), __fsub_rn(b.w, a.w));
  const float z = __fadd_rn(__fadd_rn(__fmul_rn(d.x, d.x), __fmul_rn(d.z, d.z)), __fadd_rn(__fmul_rn(d.y, d.y), __fmul_rn(d.w, d.w)));
  if (z > 0.0f)
  {
    const float r = __fsqrt_rn(z);
    d = make_float4(__fdiv_rn(d.x, r), __fdiv_rn(d.y, r), __fdiv_rn(d.z, r), __fdiv_rn(d.w, r));
  }
  if (mode == PARS_COLOR_RGB) return make_float4(fabsf(d.x), fabsf(d.z), fabsf(d.y), 1.0f);

  // to_spherical (coordinates.hpp:8-16): the radius as the reference rounds
  // it (acos near +-1 would magnify any difference in it); atan2 and acos are
  // the FP32 functions, as the reference calls them (the host libm's atan2f /
  // acosf there, CUDA's here: within 3 and 2 ulp).
  const float radius = reference_radius(d.x, d.y, d.z);
  float s1 = atan2f(d.y, d.x);
  float s2 = acosf(__fdiv_rn(d.z, radius));
  // correct_range (color_generator.cpp:41-54).
  const float pi = float(3.14159265358979323846);
  if (s1 <  0.0f) s1 = __fadd_rn(s1, pi);
  if (s1 >= pi)   s1 = __fsub_rn(s1, pi);
  s1 = __fsub_rn(pi, s1);
  if (s2 <  0.0f) s2 = fabsf(s2);
  if (s2 >= float(3.14159265358979323846 / 2.0)) s2 = __fsub_rn(pi, s2);
  // s / M_PI and s / (M_PI / 2): the reference divides in double and rounds to
  // float; an FP32 multiply by the rounded reciprocal is within one ulp of
  // that (hue and saturation are already a few ulps apart from the reference
  // through atan2f / acosf).
  const float hue    = __fmul_rn(s1, float(1.0 / 3.14159265358979323846));
  const float second = __fmul_rn(s2, float(2.0 / 3.14159265358979323846));

  const bool constant_first = (mode == PARS_COLOR_HSL_CONSTANT_S || mode == PARS_COLOR_HSV_CONSTANT_S);
  const float sat   = constant_first ? parameter : second;
  const float third = constant_first ? second : parameter;
  float4 c = hue_to_rgba(hue);
  if (mode == PARS_COLOR_HSL_CONSTANT_S || mode == PARS_COLOR_HSL_CONSTANT_L)
  {
    // hsl_to_rgba (color_generator.cpp:65-72)
    const float pre = __fmul_rn(__fsub_rn(1.0f, fabsf(__fsub_rn(__fmul_rn(2.0f, third), 1.0f))), sat);
    c.x = __fadd_rn(__fmul_rn(__fsub_rn(c.x, 0.5f), pre), third);
    c.y = __fadd_rn(__fmul_rn(__fsub_rn(c.y, 0.5f), pre), third);
    c.z = __fadd_rn(__fmul_rn(__fsub_rn(c.z, 0.5f), pre), third);
  }
  else
  {
    // hsv_to_rgba (color_generator.cpp:73-79)
    c.x = __fmul_rn(__fadd_rn(__fmul_rn(__fsub_rn(c.x, 1.0f), sat), 1.0f), third);
    c.y = __fmul_rn(__fadd_rn(__fmul_rn(__fsub_rn(c.y, 1.0f), sat), 1.0f), third);
    c.z = __fmul_rn(__fadd_rn(__fmul_rn(__fsub_rn(c.z, 1.0f), sat), 1.0f), third);
  }
  c.w = 1.0f;
  return c;
}

__global__ void __launch_bounds__(256) color_kernel(const float4* __restrict__ v, const int* __restrict__ indices, long long m,
                                                    int mode, float parameter, float4* __restrict__ colors)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int index = indices[i];
  const float4 c = color_of(v[index], v[index + 1], mode, parameter);
  colors[index] = c;
  // The last vertex of a run copies its colour (color_generator.cpp:36-37).
  if (i != m - 1 && indices[i + 1] != index + 1) colors[index + 1] = c;
}

// ---- every batch of a curves store at once ------------------------------------
// The batches are consecutive ranges of one vertex buffer (bounds[b] ..
// bounds[b + 1]).  Index generation runs over the whole buffer with each
// vertex's flag confined to its batch; one scan gives every flagged vertex its
// position in the packed index buffer, which holds the batches' indices one
// after the other (each index relative to its batch, as the reference's).

// The last segment s in [0, segments) with bounds[s] <= x.
__device__ __forceinline__ int segment_of(const long long* __restrict__ bounds, int segments, long long x)
{
  int lo = 0, hi = segments - 1;
  while (lo < hi)
  {
    const int mid = (lo + hi + 1) >> 1;
    if (bounds[mid] <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Flags of a thread's items: bit k set when vertex first + k is indexed.
__device__ __forceinline__ unsigned batch_flags(const float4* __restrict__ v, const long long* __restrict__ vbounds, int batches,
                                                long long first, int& b)
{
  const long long n = vbounds[batches];
  unsigned flags = 0;
  if (first >= n) return 0;
  b = segment_of(vbounds, batches, first);
  long long end = vbounds[b + 1];
  bool term_i = is_termination_vertex(v[first]);
  #pragma unroll
  for (int k = 0; k < index_items; ++k)
  {
    const long long i = first + k;
    if (i >= n) break;
    while (i >= end) { ++b; end = vbounds[b + 1]; }
    const bool has_next = i + 1 < end;
    const bool term_next = i + 1 < n ? is_termination_vertex(v[i + 1]) : true;
    if (has_next && !term_i && !term_next) flags |= 1u << k;
    term_i = term_next;
  }
  return flags;
}

__global__ void __launch_bounds__(index_threads) batch_index_count_kernel(const float4* __restrict__ v, const long long* __restrict__ vbounds,
                                                                          int batches, int* __restrict__ tile_counts)
{
  using reduce = cub::BlockReduce<int, index_threads>;
  __shared__ typename reduce::TempStorage storage;
  const long long first = (long long)blockIdx.x * index_tile + (long long)threadIdx.x * index_items;
  int b = 0;
  const int count = __popc(batch_flags(v, vbounds, batches, first, b));
  const int total = reduce(storage).Sum(count);
  if (threadIdx.x == 0) tile_counts[blockIdx.x] = total;
}

// Writes the packed indices and, for every batch starting at one of the
// thread's vertices, the batch's first position in the packed buffer.
__global__ void __launch_bounds__(index_threads) batch_index_write_kernel(const float4* __restrict__ v, const long long* __restrict__ vbounds,
                                                                          int batches, const long long* __restrict__ tile_offsets,
                                                                          int* __restrict__ indices, long long* __restrict__ ibounds)
{
  using scan = cub::BlockScan<int, index_threads>;
  __shared__ typename scan::TempStorage storage;
  const long long first = (long long)blockIdx.x * index_tile + (long long)threadIdx.x * index_items;
  const long long n = vbounds[batches];
  int b = 0;
  const unsigned flags = batch_flags(v, vbounds, batches, first, b);
  int prefix = 0;
  scan(storage).ExclusiveSum(__popc(flags), prefix);
  if (first >= n) return;
  long long out = tile_offsets[blockIdx.x] + prefix;
  b = segment_of(vbounds, batches, first);
  // batches that start inside this thread's range (several when some are empty)
  int s = b;
  while (s > 0 && vbounds[s] == first) --s;       // the first batch starting at `first`
  if (vbounds[s] < first) ++s;
  #pragma unroll
  for (int k = 0; k < index_items; ++k)
  {
    const long long i = first + k;
    if (i >= n) break;
    while (s < batches && vbounds[s] == i) { ibounds[s] = out; ++s; }
    while (i >= vbounds[b + 1]) ++b;
    if (flags & (1u << k)) indices[out++] = int(i - vbounds[b]);
  }
}

__global__ void __launch_bounds__(256) batch_color_kernel(const float4* __restrict__ v, const int* __restrict__ indices,
                                                          const long long* __restrict__ vbounds, const long long* __restrict__ ibounds,
                                                          int batches, const color_spec* __restrict__ specs, float4* __restrict__ colors)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ibounds[batches]) return;
  const int b = segment_of(ibounds, batches, k);
  const int index = indices[k];
  const long long g = vbounds[b] + index;
  const color_spec spec = specs[b];
  const float4 c = color_of(v[g], v[g + 1], spec.mode, spec.parameter);
  colors[g] = c;
  // The last vertex of a run copies its colour (color_generator.cpp:36-37);
  // the last vertex of a batch keeps none.
  if (k + 1 < ibounds[b + 1] && indices[k + 1] != index + 1) colors[g + 1] = c;
}
}

void index_batches(pars_gpu_context& ctx, curves_store& c)
{
  const int batches = int(c.batches.size());
  std::vector<long long> vbounds(batches + 1), ibounds(batches + 1, 0);
  for (int b = 0; b < batches; ++b) vbounds[b] = c.batches[b].vertex_offset;
  vbounds[batches] = c.vertex_total;
  for (int b = 0; b < batches; ++b)
    PARS_REQUIRE(c.batches[b].vertex_offset + c.batches[b].vertex_count == vbounds[b + 1], "curve batches are not consecutive");
  c.indices.reserve(sizeof(int) * (std::size_t)std::max<long long>(c.vertex_total, 1));
  ctx.curve_bounds.reserve(sizeof(long long) * 2 * (batches + 1));
  long long* d_vbounds = ctx.curve_bounds.as<long long>();
  long long* d_ibounds = d_vbounds + batches + 1;
  const long long n = c.vertex_total;
  if (batches > 0 && n > 0)
  {
    PARS_CUDA(cudaMemcpyAsync(d_vbounds, vbounds.data(), sizeof(long long) * (batches + 1), cudaMemcpyHostToDevice, ctx.stream));
    const long long tiles = (n + index_tile - 1) / index_tile;
    ctx.tile_counts.reserve(sizeof(int) * tiles);
    ctx.tile_offsets.reserve(sizeof(long long) * (tiles + 1));
    {
      launch_scope scope(ctx, "index_count");
      batch_index_count_kernel<<<(unsigned)tiles, index_threads, 0, ctx.stream>>>(c.vertices.as<const float4>(), d_vbounds, batches,
                                                                                  ctx.tile_counts.as<int>());
    }
    exclusive_sum(ctx, ctx.tile_counts.as<int>(), ctx.tile_offsets.as<long long>(), tiles);
    {
      launch_scope scope(ctx, "index_write");
      batch_index_write_kernel<<<(unsigned)tiles, index_threads, 0, ctx.stream>>>(c.vertices.as<const float4>(), d_vbounds, batches,
                                                                                  ctx.tile_offsets.as<const long long>(),
                                                                                  c.indices.as<int>(), d_ibounds);
    }
    long long total = 0;
    PARS_CUDA(cudaMemcpyAsync(ibounds.data(), d_ibounds, sizeof(long long) * batches, cudaMemcpyDeviceToHost, ctx.stream));
    PARS_CUDA(cudaMemcpyAsync(&total, ctx.tile_offsets.as<long long>() + tiles, sizeof(long long), cudaMemcpyDeviceToHost, ctx.stream));
    PARS_CUDA(cudaStreamSynchronize(ctx.stream));
    ibounds[batches] = total;
    // batches starting at the very end (empty) were not seen by any thread
    for (int b = batches - 1; b >= 0; --b) if (vbounds[b] == n) ibounds[b] = total;
    PARS_CUDA(cudaMemcpyAsync(d_ibounds, ibounds.data(), sizeof(long long) * (batches + 1), cudaMemcpyHostToDevice, ctx.stream));
  }
  else if (batches > 0)
  {
    PARS_CUDA(cudaMemcpyAsync(d_vbounds, vbounds.data(), sizeof(long long) * (batches + 1), cudaMemcpyHostToDevice, ctx.stream));
    PARS_CUDA(cudaMemcpyAsync(d_ibounds, ibounds.data(), sizeof(long long) * (batches + 1), cudaMemcpyHostToDevice, ctx.stream));
  }
  for (int b = 0; b < batches; ++b)
  {
    c.batches[b].index_offset = ibounds[b];
    c.batches[b].index_count = ibounds[b + 1] - ibounds[b];
  }
  c.index_total = ibounds[batches];
}

void color_batches(pars_gpu_context& ctx, curves_store& c, const std::vector<color_spec>& specs)
{
  const int batches = int(c.batches.size());
  PARS_REQUIRE(specs.size() == std::size_t(batches), "one colour spec per batch");
  c.colors.reserve(sizeof(float4) * (std::size_t)std::max<long long>(c.vertex_total, 1));
  if (c.vertex_total > 0) PARS_CUDA(cudaMemsetAsync(c.colors.get(), 0, sizeof(float4) * c.vertex_total, ctx.stream));
  if (batches == 0 || c.index_total == 0) return;
  ctx.color_specs.reserve(sizeof(color_spec) * batches);
  PARS_CUDA(cudaMemcpyAsync(ctx.color_specs.get(), specs.data(), sizeof(color_spec) * batches, cudaMemcpyHostToDevice, ctx.stream));
  const long long* d_vbounds = ctx.curve_bounds.as<const long long>();
  const long long* d_ibounds = d_vbounds + batches + 1;
  launch_scope scope(ctx, "color_generate");
  batch_color_kernel<<<(unsigned)((c.index_total + 255) / 256), 256, 0, ctx.stream>>>(
    c.vertices.as<const float4>(), c.indices.as<const int>(), d_vbounds, d_ibounds, batches, ctx.color_specs.as<const color_spec>(),
    c.colors.as<float4>());
}

long long launch_index_generate(pars_gpu_context& ctx, const float4* vertices, long long n, int* indices)
{
  if (n < 2) return 0;
  const long long tiles = (n + index_tile - 1) / index_tile;
  ctx.tile_counts.reserve(sizeof(int) * tiles);
  ctx.tile_offsets.reserve(sizeof(long long) * (tiles + 1));
  {
    launch_scope scope(ctx, "index_count");
    index_count_kernel<<<(unsigned)tiles, index_threads, 0, ctx.stream>>>(vertices, n, ctx.tile_counts.as<int>());
  }
  exclusive_sum(ctx, ctx.tile_counts.as<int>(), ctx.tile_offsets.as<long long>(), tiles);
  {
    launch_scope scope(ctx, "index_write");
    index_write_kernel<<<(unsigned)tiles, index_threads, 0, ctx.stream>>>(vertices, n, ctx.tile_offsets.as<long long>(), indices);
  }
  long long total = 0;
  PARS_CUDA(cudaMemcpyAsync(&total, ctx.tile_offsets.as<long long>() + tiles, sizeof(long long), cudaMemcpyDeviceToHost, ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  return total;
}

void launch_color_generate(pars_gpu_context& ctx, const float4* vertices, const int* indices, long long index_count,
                           int mode, float parameter, float4* colors)
{
  if (index_count <= 0) return;
  launch_scope scope(ctx, "color_generate");
  color_kernel<<<(unsigned)((index_count + 255) / 256), 256, 0, ctx.stream>>>(vertices, indices, index_count, mode, parameter, colors);
}
}
