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
//   (d0^2 + d2^2) + (d1^2 + d3^2).  atan2 and acos are evaluated in FP64 and
//   rounded to FP32 (the reference calls the host libm's FP32 versions).
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

  // to_spherical (coordinates.hpp:8-16): std::pow(float, int) promotes to double.
  const double tx = d.x, ty = d.y, tz = d.z;
  const float radius = __double2float_rn(__dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(tx, tx), __dmul_rn(ty, ty)), __dmul_rn(tz, tz))));
  float s1 = __double2float_rn(atan2(ty, tx));
  float s2 = __double2float_rn(acos(double(__fdiv_rn(d.z, radius))));
  // correct_range (color_generator.cpp:41-54).
  const float pi = float(3.14159265358979323846);
  if (s1 <  0.0f) s1 = __fadd_rn(s1, pi);
  if (s1 >= pi)   s1 = __fsub_rn(s1, pi);
  s1 = __fsub_rn(pi, s1);
  if (s2 <  0.0f) s2 = fabsf(s2);
  if (s2 >= float(3.14159265358979323846 / 2.0)) s2 = __fsub_rn(pi, s2);
  const float hue    = __double2float_rn(__ddiv_rn(double(s1), 3.14159265358979323846));
  const float second = __double2float_rn(__ddiv_rn(double(s2), 3.14159265358979323846 / 2.0));

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
