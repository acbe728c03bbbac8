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
//
// Horizon launches (HORIZON = true) bound a launch's length so that a host can
// append jobs between launches (continuous admission): a warp that has taken
// `iterations` steps parks its state -- its job, its live particles, the
// unconsumed seeds of its pool and a pool it has taken but not begun -- as one
// group and leaves (and raises a flag that makes every other warp park within
// 16 steps); the next launch's warps resume the parked groups first (one
// each) and then take pools from the same counter.  A particle's
// arithmetic does not depend on where it runs, so a job's results are the
// same bits however its work is split into launches.
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

// Device-scope relaxed accesses to the horizon launch's stop flag (PTX
// ld.relaxed.gpu / st.relaxed.gpu: they bypass the SM's L1, so a flag raised on
// one SM is seen on the others).
__device__ __forceinline__ unsigned int load_relaxed(const unsigned int* p)
{
  unsigned int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void store_relaxed(unsigned int* p, unsigned int v)
{
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

template <int CLASS>
struct lane_cache { corner_cache k; };
template <> struct lane_cache<batch_unsteady> { corner_cache2 k; };

// CLASS batch_steady: re-sampled stages, every job on a steady field (one
// slice).  batch_unsteady: re-sampled stages, jobs may have several time
// slices (a steady job works too).  batch_frozen: the frozen scheme.
template <int THREADS, int MIN_BLOCKS, int CLASS, bool HORIZON = false>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS)
batch_advect_kernel(const batch_job_device* __restrict__ jobs, int njobs, long long total_pools,
                    unsigned long long* __restrict__ pool_counter, const __grid_constant__ batch_horizon_args hz)
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
  // horizon launches: steps this warp has taken
  int iteration = 0;

  if constexpr (HORIZON)
  {
    // resume one parked group (the host launches at least as many warps as
    // there are groups)
    unsigned int g = 0;
    if (lane == 0) g = atomicAdd(hz.in_counter, 1u);
    g = __shfl_sync(full_mask, g, 0);
    if (g < unsigned(hz.in_count))
    {
      const batch_parked_group G = hz.in_groups[g];
      job = G.job;
      const batch_job_device& J = jobs[job];
      f = J.field; ta = J.time; h = J.rule.h; rk4 = J.rule.rk4; max_steps = J.max_steps; clock = J.clock;
      rule = &J.rule;
      pool_next = G.pool_next;
      pool_end = G.pool_end;
      pending = G.pending;
      if (lane < G.count)
      {
        const batch_parked_lane& P = hz.in_lanes[(long long)g * 32 + lane];
        seed = P.seed;
        steps = P.steps;
        if constexpr (CLASS == batch_frozen)
        {
          pos = P.pos;
          hist.v = P.hist_v;
          hist.started = P.started;
        }
        else local = local_position {P.ix, P.iy, P.iz, P.ux, P.uy, P.uz, P.lx, P.ly, P.lz};
        alive = true;
      }
    }
  }

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

    if constexpr (HORIZON)
    {
      // The first warp to reach the horizon raises the launch's stop flag;
      // the others see it within 16 steps, so the launch ends with every SM
      // busy to the end instead of waiting for its slowest warp.
      ++iteration;
      bool stop = iteration > hz.iterations;
      if (!stop && (iteration & 15) == 0)
      {
        unsigned int flag = 0;
        if (lane == 0) flag = load_relaxed(hz.stop);
        stop = __shfl_sync(full_mask, flag, 0) != 0u;
      }
      if (stop)
      {
        if (lane == 0 && iteration > hz.iterations) store_relaxed(hz.stop, 1u);
        // park: the group record, then the live lanes' particles in lane order
        const unsigned live = __ballot_sync(full_mask, alive);
        unsigned int g = 0;
        if (lane == 0) g = atomicAdd(hz.out_count, 1u);
        g = __shfl_sync(full_mask, g, 0);
        if (alive)
        {
          // each class parks only the state it carries
          batch_parked_lane& P = hz.out_lanes[(long long)g * 32 + __popc(live & lanes_below)];
          P.seed = seed;
          P.steps = steps;
          if constexpr (CLASS == batch_frozen)
          {
            P.pos = pos;
            P.hist_v = hist.v;
            P.started = hist.started;
          }
          else
          {
            P.ix = local.ix; P.iy = local.iy; P.iz = local.iz;
            P.ux = local.ux; P.uy = local.uy; P.uz = local.uz;
            P.lx = local.lx; P.ly = local.ly; P.lz = local.lz;
          }
        }
        if (lane == 0) hz.out_groups[g] = batch_parked_group {job, __popc(live), pool_next, pool_end, pending};
        break;
      }
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
  const void* horizon_kernel;
};
#define PARS_BATCH_VARIANT(T, M, C) {T, M, (const void*)batch_advect_kernel<T, M, C>, (const void*)batch_advect_kernel<T, M, C, true>}

// Launch shapes the autotuner chooses from, per job class: threads per CTA and
// the minimum resident CTAs per SM that the register allocation must allow.
const variant variants[batch_classes][4] = {
  {PARS_BATCH_VARIANT(64, 1, batch_steady), PARS_BATCH_VARIANT(128, 1, batch_steady),
   PARS_BATCH_VARIANT(128, 5, batch_steady), PARS_BATCH_VARIANT(256, 1, batch_steady)},
  {PARS_BATCH_VARIANT(64, 1, batch_unsteady), PARS_BATCH_VARIANT(128, 1, batch_unsteady),
   PARS_BATCH_VARIANT(128, 3, batch_unsteady), PARS_BATCH_VARIANT(256, 1, batch_unsteady)},
  {PARS_BATCH_VARIANT(64, 1, batch_frozen), PARS_BATCH_VARIANT(128, 1, batch_frozen),
   PARS_BATCH_VARIANT(128, 6, batch_frozen), PARS_BATCH_VARIANT(256, 1, batch_frozen)},
};
#undef PARS_BATCH_VARIANT
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
  const batch_horizon_args none {};
  launch_scope scope(ctx, "batch_advect");
  void* args[] = {(void*)&jobs, (void*)&njobs, (void*)&total_pools, (void*)&counter, (void*)&none};
  PARS_CUDA(cudaLaunchKernel(var.kernel, grid, var.threads, args, 0, ctx.stream));
}

long long batch_horizon_warps(pars_gpu_context& ctx, int job_class, int v)
{
  const variant& var = variants[job_class][v];
  int& per_sm = ctx.horizon_ctas_per_sm[job_class][v];
  if (per_sm < 0) PARS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, var.horizon_kernel, var.threads, 0));
  if (ctx.sm_count <= 0) PARS_CUDA(cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, ctx.device));
  return (long long)std::max(per_sm, 1) * ctx.sm_count * (var.threads / 32);
}

void launch_batch_advect_horizon(pars_gpu_context& ctx, int job_class, int v, const batch_job_device* jobs, int njobs,
                                 long long total_pools, unsigned long long* counter, const batch_horizon_args& hz, long long warps)
{
  const variant& var = variants[job_class][v];
  const long long resident = batch_horizon_warps(ctx, job_class, v);
  const long long want = std::min(resident, std::max<long long>({warps, (long long)hz.in_count, 1}));
  const unsigned grid = (unsigned)((want * 32 + var.threads - 1) / var.threads);
  // every parked group needs a warp of its own to resume it
  PARS_REQUIRE((long long)grid * (var.threads / 32) >= hz.in_count, "more parked groups than warps");
  launch_scope scope(ctx, "batch_advect_horizon");
  void* args[] = {(void*)&jobs, (void*)&njobs, (void*)&total_pools, (void*)&counter, (void*)&hz};
  PARS_CUDA(cudaLaunchKernel(var.horizon_kernel, grid, var.threads, args, 0, ctx.stream));
}
}
