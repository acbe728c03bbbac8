// Batched advection: many jobs (seed sets on steady or unsteady fields of
// different sizes) in ONE persistent launch.
//
// The grid holds as many CTAs as fit on the GPU at once.  Each CTA repeatedly
// takes the next chunk of seeds from a device counter (one atomic per chunk),
// finds the chunk's job by binary search over the jobs' chunk prefixes, and
// advects one seed per thread with the flow-map rules of particle_advector
// (particle_advector.cpp:74-139): stop when the particle leaves the grid,
// meets a zero velocity, or has taken max_steps steps; its last position is
// written to the job's output.  Uneven jobs balance themselves: a CTA that
// finishes early takes the next chunk, whatever job it belongs to.
#include "context.hpp"

namespace pars
{
namespace
{
__device__ __forceinline__ int find_job(const batch_job_device* __restrict__ jobs, int njobs, long long chunk)
{
  int lo = 0, hi = njobs - 1;
  while (lo < hi)
  {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].first_chunk <= chunk) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// UNSTEADY = false: every job is on a steady field (one slice).
// UNSTEADY = true: jobs may have several time slices (a steady job works too).
template <int THREADS, int MIN_BLOCKS, bool UNSTEADY>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS)
batch_advect_kernel(const batch_job_device* __restrict__ jobs, int njobs, long long total_chunks,
                    unsigned long long* __restrict__ chunk_counter)
{
  __shared__ long long s_chunk;
  __shared__ int s_job;
  for (;;)
  {
    if (threadIdx.x == 0)
    {
      const long long c = (long long)atomicAdd(chunk_counter, 1ULL);
      s_chunk = c;
      s_job = c < total_chunks ? find_job(jobs, njobs, c) : 0;
    }
    __syncthreads();
    const long long chunk = s_chunk;
    const int j = s_job;
    __syncthreads();
    if (chunk >= total_chunks) return;

    const batch_job_device& job = jobs[j];
    const long long seed = (chunk - job.first_chunk) * THREADS + threadIdx.x;
    unsigned int steps = 0;
    if (seed < job.seed_count)
    {
      float4 pos;
      if (job.seeds) pos = job.seeds[seed];
      else
      {
        // lattice seed (seed_generator.cpp:14-19), C order
        const int iz = int(seed % job.pz);
        const int iy = int((seed / job.pz) % job.py);
        const int ix = int(seed / ((long long)job.pz * job.py));
        pos = make_float4(__fadd_rn(job.ox, __fmul_rn(job.sx, float(ix))), __fadd_rn(job.oy, __fmul_rn(job.sy, float(iy))),
                          __fadd_rn(job.oz, __fmul_rn(job.sz, float(iz))), 0.0f);
      }
      const field_view f = job.field;
      const step_rule rule = job.rule;
      float3 lo = make_float3(0.0f, 0.0f, 0.0f);
      if (!UNSTEADY)
      {
        cell_cache cache;
        for (int it = 0; it < job.max_steps; ++it)
        {
          if (!contains_reference(f, pos)) break;
          const float3 v = sample_cached(f, cache, pos.x, pos.y, pos.z);
          if (is_zero(v)) break;
          resampled_step_cached(f, cache, rule, pos, lo, v);
          ++steps;
        }
      }
      else
      {
        cell_cache2 cache;
        for (int it = 0; it < job.max_steps; ++it)
        {
          if (!contains_reference(f, pos)) break;
          // FP64 time of this step: start + n h (no accumulated rounding)
          const double t = job.time_begin + double(it) * double(rule.h);
          const float3 v = sample_unsteady_cached(f, job.time, cache, pos.x, pos.y, pos.z, t);
          if (is_zero(v)) break;
          unsteady_step(f, job.time, cache, rule, pos, lo, v, t);
          ++steps;
        }
      }
      if (job.end_positions) job.end_positions[seed] = pos;
      if (job.end_steps) job.end_steps[seed] = int(steps);
    }
    const unsigned int warp_steps = __reduce_add_sync(0xffffffffu, steps);
    if ((threadIdx.x & 31) == 0 && warp_steps) atomicAdd(job.steps, (unsigned long long)warp_steps);
  }
}

struct variant
{
  int threads, min_blocks;
  const void* kernel;
};

// Launch shapes the autotuner chooses from, per job class: threads per CTA
// (= seeds per chunk) and the minimum resident CTAs per SM the register
// allocation must allow.
const variant variants[2][4] = {
  {{64, 1, (const void*)batch_advect_kernel<64, 1, false>},
   {128, 1, (const void*)batch_advect_kernel<128, 1, false>},
   {128, 4, (const void*)batch_advect_kernel<128, 4, false>},
   {256, 1, (const void*)batch_advect_kernel<256, 1, false>}},
  {{64, 1, (const void*)batch_advect_kernel<64, 1, true>},
   {128, 1, (const void*)batch_advect_kernel<128, 1, true>},
   {128, 3, (const void*)batch_advect_kernel<128, 3, true>},
   {256, 1, (const void*)batch_advect_kernel<256, 1, true>}},
};
}

int batch_variant_count() { return 4; }
int batch_variant_threads(int v) { return variants[0][v].threads; }

void launch_batch_advect(pars_gpu_context& ctx, int job_class, int v, const batch_job_device* jobs, int njobs,
                         long long total_chunks, unsigned long long* counter)
{
  if (total_chunks <= 0) return;
  const variant& var = variants[job_class][v];
  int per_sm = 0, sms = 0;
  PARS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, var.kernel, var.threads, 0));
  PARS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
  const long long persistent = (long long)std::max(per_sm, 1) * sms;
  const unsigned grid = (unsigned)std::min<long long>(persistent, total_chunks);
  launch_scope scope(ctx, "batch_advect");
  void* args[] = {(void*)&jobs, (void*)&njobs, (void*)&total_chunks, (void*)&counter};
  PARS_CUDA(cudaLaunchKernel(var.kernel, grid, var.threads, args, 0, ctx.stream));
}
}
