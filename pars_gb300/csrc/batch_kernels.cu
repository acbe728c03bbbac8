// Batched advection: many jobs (seed sets on steady or unsteady fields of
// different sizes) in ONE persistent launch that drains a device work queue.
//
// The grid holds as many CTAs as fit on the GPU at once.  Work is a queue of
// pools (POOL consecutive seeds of one job); a warp takes pools with one
// atomic and hands their seeds to its lanes.  A lane whose particle retires
// takes the next seed of the pool at once (warp ballot + prefix), so lanes do
// not idle while the rest of the warp finishes long particles.  All lanes of a
// warp work on the same job; a warp moves to another job only when its lanes
// have drained, so job parameters stay warp-uniform.
//
// Each particle follows the flow-map rules of particle_advector
// (particle_advector.cpp:74-139): before every step it stops when it has
// taken max_steps steps, left the grid or meets a zero velocity
// (|v_i| <= 1e-5); its last position (and optionally its step count) is
// written to the job's output.  Re-sampled jobs (steady and unsteady alike)
// carry particles in local cell coordinates and test their cell index, which
// differs from the reference's contains() (floor of the IEEE quotient) only
// within an ulp of the grid's last face.  Frozen jobs (the reference's
// scheme, any of the eight integrators) keep absolute positions and the
// reference's arithmetic bit for bit, as flow_map_kernel<true> does, one
// field sample per step on the lane's cached corners.
#include "context.hpp"

namespace pars
{
namespace
{
constexpr unsigned full_mask = 0xffffffffu;
constexpr int pool_seeds = 256;

__device__ __forceinline__ int find_job(const batch_job_device* __restrict__ jobs, int njobs, long long pool)
{
  int lo = 0, hi = njobs - 1;
  while (lo < hi)
  {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].first_pool <= pool) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <int CLASS>
struct lane_cache { corner_cache k; };
template <> struct lane_cache<batch_unsteady> { corner_cache2 k; };

// CLASS batch_steady: re-sampled stages, every job on a steady field (one
// slice).  batch_unsteady: re-sampled stages, jobs may have several time
// slices (a steady job works too).  batch_frozen: the frozen scheme.
template <int THREADS, int MIN_BLOCKS, int CLASS>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS)
batch_advect_kernel(const batch_job_device* __restrict__ jobs, int njobs, long long total_pools,
                    unsigned long long* __restrict__ pool_counter)
{
  const int lane = threadIdx.x & 31;
  const unsigned lanes_below = (1u << lane) - 1u;

  // warp-uniform work state
  int job = -1;
  long long pool_next = 0, pool_end = 0, pending = -1;
  bool exhausted = false;
  unsigned int job_steps = 0;       // this lane's steps on the current job
  // lane state
  bool alive = false;
  long long seed = 0;
  int steps = 0;
  float4 pos = make_float4(0.f, 0.f, 0.f, 0.f);   // seed / end position
  local_position local {0, 0, 0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // cell + offset
  frozen_history hist;                                            // frozen multistep scheme
  lane_cache<CLASS> cache;
  // current job's parameters (warp-uniform)
  field_view f {};
  time_axis ta {};
  float h = 0.0f;
  int rk4 = 1, max_steps = 0;
  slice_clock clock {};
  const step_rule* rule = nullptr;   // frozen jobs: the coefficients, read where they lie

  for (;;)
  {
    // ---- refill idle lanes ---------------------------------------------------
    unsigned need = __ballot_sync(full_mask, !alive);
    while (need)
    {
      if (pool_next < pool_end)
      {
        const long long s = pool_next + __popc(need & lanes_below);
        if (!alive && s < pool_end)
        {
          const batch_job_device& J = jobs[job];
          seed = s;
          if (J.seeds) pos = J.seeds[s];
          else
          {
            const int iz = int(s % J.pz);
            const int iy = int((s / J.pz) % J.py);
            const int ix = int(s / ((long long)J.pz * J.py));
            pos = make_float4(__fadd_rn(J.ox, __fmul_rn(J.sx, float(ix))), __fadd_rn(J.oy, __fmul_rn(J.sy, float(iy))),
                              __fadd_rn(J.oz, __fmul_rn(J.sz, float(iz))), 0.0f);
          }
          if constexpr (CLASS == batch_frozen) hist = frozen_history();
          else local = to_local(f, pos);
          steps = 0;
          alive = true;
        }
        pool_next = min(pool_end, pool_next + (long long)__popc(need));
        need = __ballot_sync(full_mask, !alive);
        continue;
      }
      if (exhausted) break;
      long long p = pending;
      if (p < 0)
      {
        if (lane == 0) p = (long long)atomicAdd(pool_counter, 1ULL);
        p = __shfl_sync(full_mask, p, 0);
      }
      if (p >= total_pools) { exhausted = true; break; }
      const int pj = find_job(jobs, njobs, p);
      if (pj != job)
      {
        if (__any_sync(full_mask, alive)) { pending = p; break; }   // drain the current job first
        // switch job: flush this lane's step count, load the new parameters
        if (job >= 0)
        {
          const unsigned int total = __reduce_add_sync(full_mask, job_steps);
          if (lane == 0 && total) atomicAdd(jobs[job].steps, (unsigned long long)total);
        }
        job_steps = 0;
        job = pj;
        const batch_job_device& J = jobs[job];
        f = J.field; ta = J.time; h = J.rule.h; rk4 = J.rule.rk4; max_steps = J.max_steps; clock = J.clock;
        rule = &J.rule;
        cache = lane_cache<CLASS>();
      }
      pending = -1;
      pool_next = (p - jobs[job].first_pool) * pool_seeds;
      pool_end = min(pool_next + pool_seeds, jobs[job].seed_count);
    }
    if (!__any_sync(full_mask, alive))
    {
      if (exhausted) break;
      continue;   // switch to the pending job
    }

    // ---- one step of every live lane -------------------------------------------
    if (alive)
    {
      bool retire = steps >= max_steps;
      if constexpr (CLASS == batch_frozen)
      {
        // contains() + interpolate() at the step start, then the frozen step
        if (!retire)
        {
          float3 v;
          if (!sample_inside_cached(f, cache.k, pos, v) || is_zero(v)) retire = true;
          else { pos = frozen_step(*rule, pos, v, hist); ++steps; ++job_steps; }
        }
      }
      else if constexpr (CLASS == batch_unsteady)
      {
        // local coordinates as for steady jobs, with the time of this step
        // (start + n h, from n: no accumulated rounding)
        if (!retire) retire = !local_inside(f, local);
        if (!retire)
        {
          const slice_time t = step_time(clock, steps);
          const float3 k1 = sample_local_unsteady(f, ta, cache.k, local.ix, local.iy, local.iz, local.ux, local.uy, local.uz, t);
          if (is_zero_local(f, k1)) retire = true;
          else { local_unsteady_step(f, ta, clock, cache.k, rk4, h, local, k1, t); ++steps; ++job_steps; }
        }
        if (retire) pos = flow_position(f, local);
      }
      else
      {
        // the step-start test: the particle's cell inside the grid
        if (!retire) retire = !local_inside(f, local);
        if (!retire)
        {
          const float3 k1 = sample_local(f, cache.k, local.ix, local.iy, local.iz, local.ux, local.uy, local.uz);
          if (is_zero_local(f, k1)) retire = true;
          else { local_step(f, cache.k, rk4, h, local, k1); ++steps; ++job_steps; }
        }
        if (retire) pos = flow_position(f, local);
      }
      if (retire)
      {
        const batch_job_device& J = jobs[job];
        if (J.end_positions)
        {
          long long out = seed;
          bool write = true;
          if (!J.seeds && J.ux > 0)
          {
            // lattice seed -> output voxel of the flow map's own shape
            const int iz = int(seed % J.pz), iy = int((seed / J.pz) % J.py), ix = int(seed / ((long long)J.pz * J.py));
            write = ix < J.ux && iy < J.uy && iz < J.uz;
            out = ((long long)ix * J.uy + iy) * J.uz + iz;
          }
          if (write) J.end_positions[out] = pos;
        }
        if (J.end_steps) J.end_steps[seed] = steps;
        alive = false;
      }
    }
  }
  if (job >= 0)
  {
    const unsigned int total = __reduce_add_sync(full_mask, job_steps);
    if (lane == 0 && total) atomicAdd(jobs[job].steps, (unsigned long long)total);
  }
}

struct variant
{
  int threads, min_blocks;
  const void* kernel;
};

// Launch shapes the autotuner chooses from, per job class: threads per CTA and
// the minimum resident CTAs per SM that the register allocation must allow.
const variant variants[batch_classes][4] = {
  {{64, 1, (const void*)batch_advect_kernel<64, 1, batch_steady>},
   {128, 1, (const void*)batch_advect_kernel<128, 1, batch_steady>},
   {128, 5, (const void*)batch_advect_kernel<128, 5, batch_steady>},
   {256, 1, (const void*)batch_advect_kernel<256, 1, batch_steady>}},
  {{64, 1, (const void*)batch_advect_kernel<64, 1, batch_unsteady>},
   {128, 1, (const void*)batch_advect_kernel<128, 1, batch_unsteady>},
   {128, 3, (const void*)batch_advect_kernel<128, 3, batch_unsteady>},
   {256, 1, (const void*)batch_advect_kernel<256, 1, batch_unsteady>}},
  {{64, 1, (const void*)batch_advect_kernel<64, 1, batch_frozen>},
   {128, 1, (const void*)batch_advect_kernel<128, 1, batch_frozen>},
   {128, 6, (const void*)batch_advect_kernel<128, 6, batch_frozen>},
   {256, 1, (const void*)batch_advect_kernel<256, 1, batch_frozen>}},
};
}

int batch_variant_count() { return 4; }

int batch_resident_warps(pars_gpu_context& ctx, int job_class, int v)
{
  const variant& var = variants[job_class][v];
  int& per_sm = ctx.batch_ctas_per_sm[job_class][v];
  if (per_sm < 0) PARS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, var.kernel, var.threads, 0));
  return per_sm * var.threads / 32;
}
int batch_variant_threads(int v) { return variants[0][v].threads; }
int batch_pool_seeds() { return pool_seeds; }

void launch_batch_advect(pars_gpu_context& ctx, int job_class, int v, const batch_job_device* jobs, int njobs,
                         long long total_pools, unsigned long long* counter)
{
  if (total_pools <= 0) return;
  const variant& var = variants[job_class][v];
  int& per_sm = ctx.batch_ctas_per_sm[job_class][v];
  if (per_sm < 0) PARS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, var.kernel, var.threads, 0));
  if (ctx.sm_count <= 0) PARS_CUDA(cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, ctx.device));
  const long long persistent = (long long)std::max(per_sm, 1) * ctx.sm_count;
  const long long warps_needed = total_pools;   // at least one pool per warp
  const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>(persistent, (warps_needed * 32 + var.threads - 1) / var.threads));
  launch_scope scope(ctx, "batch_advect");
  void* args[] = {(void*)&jobs, (void*)&njobs, (void*)&total_pools, (void*)&counter};
  PARS_CUDA(cudaLaunchKernel(var.kernel, grid, var.threads, args, 0, ctx.stream));
}
}
