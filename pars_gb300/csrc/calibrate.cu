// Gather-bandwidth calibration: the measured ceilings the advection kernels'
// corner gathers are judged against.
//
// The advection kernels read a field through 16-byte non-coherent loads
// (ld.global.nc.v4.f32, one per cell corner).  Which memory level serves them
// depends on the working set, so the ceiling is measured per level on the
// device itself, with the same load instruction:
//   coalesced: each warp request reads 512 contiguous bytes (four 128-byte
//              lines) at a random 512-byte-aligned offset: the most useful
//              bytes the L1 data pipe can deliver per wavefront;
//   random:    each lane reads 16 bytes at its own random 16-byte-aligned
//              offset (a sector per lane);
//   cells:     each lane loads the eight corners of a random cell of a cube
//              float4 field — the reload of an uncached trilinear sample.
// A buffer of 32 KB stays in every SM's L1; 64 MB stays in L2 (129 MB) but
// not in L1; anything far above L2 streams from HBM.  Bytes delivered per
// second = threads x loads x 16 B / kernel time (CUDA events on the
// context's stream, after a warm-up launch).
#include "context.hpp"

namespace pars
{
namespace
{
constexpr int calibrate_threads = 256;
constexpr int calibrate_unroll = 8;

struct calibrate_args
{
  const float4* data;
  long long     mask;      // buffer size in float4 - 1 (a power of two)
  int           edge;      // cells pattern: cube edge in vertices
  int           iterations;
  int           pattern;
  float*        sink;
};

__device__ __forceinline__ unsigned int next_random(unsigned int& s)
{
  // xorshift32 (Marsaglia 2003)
  s ^= s << 13;
  s ^= s >> 17;
  s ^= s << 5;
  return s;
}

__global__ void __launch_bounds__(calibrate_threads) gather_calibrate_kernel(const __grid_constant__ calibrate_args a)
{
  const unsigned int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned int lane = threadIdx.x & 31;
  // coalesced: every lane of a warp draws the same sequence (warp-uniform seed)
  unsigned int s = a.pattern == 0 ? (tid >> 5) * 2654435761u + 12345u : tid * 2654435761u + 12345u;
  if (s == 0) s = 1;
  float acc = 0.0f;
  if (a.pattern == 2)
  {
    const int cells = a.edge - 1;
    const long long syz = (long long)a.edge * a.edge;
    for (int it = 0; it < a.iterations; ++it)
    {
      const int ix = int(__umulhi(next_random(s), unsigned(cells)));
      const int iy = int(__umulhi(next_random(s), unsigned(cells)));
      const int iz = int(__umulhi(next_random(s), unsigned(cells)));
      const float4* base = a.data + ix * syz + (long long)iy * a.edge + iz;
      const float4 c0 = __ldg(base), c1 = __ldg(base + 1), c2 = __ldg(base + a.edge), c3 = __ldg(base + a.edge + 1);
      const float4 c4 = __ldg(base + syz), c5 = __ldg(base + syz + 1), c6 = __ldg(base + syz + a.edge);
      const float4 c7 = __ldg(base + syz + a.edge + 1);
      acc += (c0.x + c1.x) + (c2.x + c3.x) + (c4.x + c5.x) + (c6.x + c7.x);
    }
  }
  else
  {
    const unsigned int groups = unsigned((a.mask + 1) >> 5) - 1u;   // 512-byte groups - 1 (a power of two - 1)
    for (int it = 0; it < a.iterations; ++it)
    {
      long long offset[calibrate_unroll];
      if (a.pattern == 0)
      {
        // one draw per iteration; the other groups of the iteration follow
        // at odd multiples of the golden-ratio constant (masked: in range)
        const unsigned int r = next_random(s);
#pragma unroll
        for (int u = 0; u < calibrate_unroll; ++u)
          offset[u] = (long long)((r + unsigned(u) * 0x9E3779B9u) & groups) * 32 + lane;
      }
      else
      {
#pragma unroll
        for (int u = 0; u < calibrate_unroll; ++u) offset[u] = (long long)(next_random(s) & unsigned(a.mask));
      }
      float4 v[calibrate_unroll];
#pragma unroll
      for (int u = 0; u < calibrate_unroll; ++u) v[u] = __ldg(a.data + offset[u]);
#pragma unroll
      for (int u = 0; u < calibrate_unroll; ++u) acc += v[u].x + v[u].w;
    }
  }
  // The buffer holds zeros: the store never happens, but the loads cannot be
  // removed because the condition depends on them.
  if (acc == 1.2345f) a.sink[tid] = acc;
}
}
}

using namespace pars;

#pragma GCC visibility push(default)
extern "C" int32_t pars_gpu_gather_peak(pars_gpu_context* ctx, int64_t buffer_bytes, int32_t pattern, double* bytes_per_second)
{
  return run_guarded(ctx, [&] {
    PARS_REQUIRE(bytes_per_second, "bytes_per_second is required");
    PARS_REQUIRE(pattern >= 0 && pattern <= 2, "pattern must be 0 (coalesced), 1 (random) or 2 (cells)");
    PARS_REQUIRE(buffer_bytes >= 4096 && buffer_bytes <= (int64_t(1) << 36), "buffer_bytes must lie in [4 KiB, 64 GiB]");
    // the largest power of two of float4s within buffer_bytes
    long long count = 1;
    while (count * 2 * 16 <= buffer_bytes) count *= 2;
    int edge = 2;
    while ((long long)(edge + 1) * (edge + 1) * (edge + 1) <= count) ++edge;
    device_buffer data = acquire_buffer(*ctx, sizeof(float4) * count);
    PARS_CUDA(cudaMemsetAsync(data.get(), 0, sizeof(float4) * count, ctx->stream));
    if (ctx->sm_count <= 0) PARS_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device));
    int per_sm = 0;
    PARS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gather_calibrate_kernel, calibrate_threads, 0));
    const unsigned int blocks = unsigned(std::max(per_sm, 1) * ctx->sm_count);
    const long long threads = (long long)blocks * calibrate_threads;
    device_buffer sink;
    sink.reserve(sizeof(float) * threads);
    calibrate_args a;
    a.data = data.as<const float4>();
    a.mask = count - 1;
    a.edge = edge;
    a.pattern = pattern;
    a.sink = sink.as<float>();
    const int loads_per_iteration = pattern == 2 ? 8 : calibrate_unroll;
    // warm-up (fills the caches), then a launch of about 2^32 loads timed
    a.iterations = 16;
    {
      launch_scope scope(*ctx, "gather_calibrate");
      gather_calibrate_kernel<<<blocks, calibrate_threads, 0, ctx->stream>>>(a);
    }
    a.iterations = int(std::max<long long>(16, (1LL << 32) / (threads * loads_per_iteration)));
    cudaEvent_t start, stop;
    PARS_CUDA(cudaEventCreate(&start));
    PARS_CUDA(cudaEventCreate(&stop));
    PARS_CUDA(cudaEventRecord(start, ctx->stream));
    {
      launch_scope scope(*ctx, "gather_calibrate");
      gather_calibrate_kernel<<<blocks, calibrate_threads, 0, ctx->stream>>>(a);
    }
    PARS_CUDA(cudaEventRecord(stop, ctx->stream));
    PARS_CUDA(cudaEventSynchronize(stop));
    float ms = 0.0f;
    PARS_CUDA(cudaEventElapsedTime(&ms, start, stop));
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    recycle_buffer(*ctx, std::move(data));
    *bytes_per_second = double(threads) * a.iterations * loads_per_iteration * 16.0 / (double(ms) * 1e-3);
  });
}
#pragma GCC visibility pop
