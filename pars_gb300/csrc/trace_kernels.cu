// Streamline tracing kernels: a lane at a time runs the reference's
// per-particle loop (particle_tracer.cpp:258-336) for one particle and writes
// its slot range of the padded vertex layout; a warp per particle then prunes
// invalid vertices (particle_tracer.cpp:402-409) into the packed curve buffer.
// Particles that leave their block are pushed onto a device exit queue (one
// atomic per exiting particle), then stably sorted by (destination block,
// source order) to form the next round's per-block particle lists
// (particle_tracer.cpp:376-393).
#include <algorithm>

#include <cub/cub.cuh>

#include "context.hpp"

namespace pars
{
namespace
{
constexpr unsigned full_mask = 0xffffffffu;

// One persistent launch per round.  Warps take pools of particles from a
// device counter; a lane whose particle has ended takes the next particle of
// the pool at once (warp ballot + prefix), so lanes do not idle while the rest
// of the warp finishes longer curves.  Every particle writes only its own slot
// range, its counts and (when it leaves the block) an exit-queue entry keyed
// by its index, so the result does not depend on which lane traced it.
// FROZEN = true: the reference's scheme and FP32 operation order (bit-exact).
// FROZEN = false: re-sampled stages, consistent cell weights, compensated
// position accumulation.
template <bool FROZEN>
__global__ void __launch_bounds__(128) trace_kernel(const trace_launch a, int pool_size)
{
  const int lane = threadIdx.x & 31;
  const unsigned lanes_below = (1u << lane) - 1u;
  const float4 term = termination_vertex();
  // warp-uniform pool state
  long long pool_next = 0, pool_end = 0;
  bool exhausted = false;
  unsigned int steps = 0;            // this lane's steps, all particles
  // the lane's particle
  bool alive = false;
  long long i = 0;
  int it = 0, N = 0, written = 0, kept = 0, block = 0;
  float4 last = make_float4(0.f, 0.f, 0.f, 0.f);
  float3 lo = make_float3(0.f, 0.f, 0.f);
  corner_cache cache;
  field_view f {};
  step_rule rule {};
  float4* out = nullptr;

  for (;;)
  {
    unsigned need = __ballot_sync(full_mask, !alive);
    if (need && !exhausted)
    {
      // ---- refill idle lanes ---------------------------------------------------
      while (need)
      {
        if (pool_next < pool_end)
        {
          const long long s = pool_next + __popc(need & lanes_below);
          if (!alive && s < pool_end)
          {
            i = s;
            block = a.block_of ? a.block_of[i] : 0;
            f = a.blocks[block].field;
            rule = a.block_rules ? a.block_rules[block] : a.rule;
            const float4* record = reinterpret_cast<const float4*>(a.particles + i);
            last = record[0];
            N = __float_as_int(record[1].x);   // remaining_iterations
            const slot_layout L = a.block_slots[block];
            out = a.slots + L.origin + i * L.stride;
            out[0] = last;
            written = 1;
            kept = is_invalid_vertex(last) ? 0 : 1;
            lo = make_float3(0.f, 0.f, 0.f);
            cache = corner_cache();
            it = 1;
            alive = true;
          }
          pool_next = min(pool_end, pool_next + (long long)__popc(need));
          need = __ballot_sync(full_mask, !alive);
          continue;
        }
        long long p = 0;
        if (lane == 0) p = (long long)atomicAdd(a.next, (unsigned long long)pool_size);
        p = __shfl_sync(full_mask, p, 0);
        if (p >= a.count) { exhausted = true; break; }
        pool_next = p;
        pool_end = min(p + pool_size, a.count);
      }
    }
    if (need == full_mask) break;   // every lane idle, and the pools are exhausted

    // ---- one iteration of the reference's per-particle loop -------------------
    if (alive)
    {
      bool finish = false;
      if (it >= N) finish = true;                                   // remaining_iterations <= 1
      else if (it == N - 1) { out[it] = term; ++written; ++kept; finish = true; }
      else
      {
        float3 v;
        bool inside;
        if (FROZEN) inside = sample_inside(f, last, v);
        else        inside = sample_start(f, cache, last, v);
        if (!inside)
        {
          out[it] = term; ++written; ++kept; finish = true;
          if (a.route_exits)
          {
            const int face = exit_face(f, last, a.blocks[block].neighbor);
            if (face >= 0)
            {
              // the exit queue is sorted by (destination, source index)
              // afterwards, so its slots may be taken in any order
              const unsigned int slot = atomicAdd(a.exit_count, 1u);
              pars_particle p;
              p.position[0] = last.x; p.position[1] = last.y; p.position[2] = last.z; p.position[3] = last.w;
              p.remaining_iterations = N - it;
              p.vector_field_index = -1;
              p.original_rank = 0;
              p.original_voxel[0] = p.original_voxel[1] = p.original_voxel[2] = 0;
              p.padding[0] = p.padding[1] = 0;
              const int destination = a.blocks[block].neighbor[face];
              a.exit_particles[slot] = p;
              a.exit_keys[slot] = ((unsigned long long)destination << 40) | (unsigned long long)i;
            }
          }
        }
        else if (is_zero(v)) { out[it] = term; ++written; ++kept; finish = true; }
        else
        {
          float4 next;
          if (FROZEN) next = frozen_step(rule, last, v);
          else { next = last; resampled_step_cached(f, cache, rule, next, lo, v); }
          out[it] = next;
          ++written;
          kept += is_invalid_vertex(next) ? 0 : 1;
          last = next;
          ++steps;
          ++it;
        }
      }
      if (finish)
      {
        a.written[i] = written;
        a.kept[i] = kept;
        alive = false;
      }
    }
  }

  // Warp-aggregated step count.
  const unsigned int warp_steps = __reduce_add_sync(full_mask, steps);
  if (lane == 0 && warp_steps) atomicAdd(a.steps, (unsigned long long)warp_steps);
}

// One warp per particle: copy its written slots, minus invalid vertices, to
// the packed output at its offset.
__global__ void __launch_bounds__(256) compact_kernel(const float4* __restrict__ slots, const slot_layout* __restrict__ block_slots,
                                                      const int* __restrict__ block_of, const int* __restrict__ written,
                                                      const long long* __restrict__ offsets, long long count,
                                                      float4* __restrict__ out)
{
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= count) return;
  const int n = written[warp];
  long long dst = offsets[warp];
  const slot_layout L = block_slots[block_of ? block_of[warp] : 0];
  const float4* src = slots + L.origin + warp * L.stride;
  for (int j0 = 0; j0 < n; j0 += 32)
  {
    const int j = j0 + lane;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    bool keep = false;
    if (j < n) { v = src[j]; keep = !is_invalid_vertex(v); }
    const unsigned mask = __ballot_sync(full_mask, keep);
    if (keep) out[dst + __popc(mask & ((1u << lane) - 1u))] = v;
    dst += __popc(mask);
  }
}

__global__ void widen_kernel(const int* __restrict__ in, long long* __restrict__ out, long long count)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = in[i];
  else if (i == count) out[i] = 0;
}

__global__ void gather_exits_kernel(const pars_particle* __restrict__ exits, const unsigned int* __restrict__ order,
                                    const unsigned long long* __restrict__ keys, long long count,
                                    pars_particle* __restrict__ out, int* __restrict__ block_of, int* __restrict__ block_max,
                                    int* __restrict__ block_count)
{
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= count) return;
  const pars_particle p = exits[order[j]];
  const int block = int(keys[j] >> 40);
  out[j] = p;
  block_of[j] = block;
  atomicMax(block_max + block, p.remaining_iterations);
  atomicAdd(block_count + block, 1);
}

__global__ void iota_kernel(unsigned int* __restrict__ out, long long count)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = (unsigned int)i;
}

__global__ void gather_offsets_kernel(const long long* __restrict__ offsets, const long long* __restrict__ positions, long long n,
                                      long long* __restrict__ out)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = offsets[positions[k]];
}

__global__ void particle_stats_kernel(const pars_particle* __restrict__ particles, const int* __restrict__ block_of, long long count,
                                      int* __restrict__ block_max)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int block = block_of ? block_of[i] : 0;
  atomicMax(block_max + block, particles[i].remaining_iterations);
}

__global__ void extract_block_kernel(const float* __restrict__ domain, int dy, int dz, int ox, int oy, int oz,
                                     int sx, int sy, int sz, float4* __restrict__ out)
{
  const long long total = (long long)sx * sy * sz;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int z = int(i % sz);
  const int y = int((i / sz) % sy);
  const int x = int(i / ((long long)sz * sy));
  const long long g = ((long long)(ox + x) * dy + (oy + y)) * dz + (oz + z);
  out[i] = make_float4(domain[3 * g], domain[3 * g + 1], domain[3 * g + 2], 0.0f);
}

unsigned int grid_for(long long work, int threads)
{
  return (unsigned int)((work + threads - 1) / threads);
}
}

void launch_trace(pars_gpu_context& ctx, const trace_launch& a)
{
  if (a.count <= 0) return;
  const void* kernel = a.rule.frozen ? (const void*)trace_kernel<true> : (const void*)trace_kernel<false>;
  int& per_sm = ctx.trace_ctas_per_sm[a.rule.frozen ? 0 : 1];
  if (ctx.sm_count <= 0) PARS_CUDA(cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, ctx.device));
  if (per_sm < 0) PARS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0));
  const int sms = ctx.sm_count;
  const long long resident_warps = (long long)std::max(per_sm, 1) * sms * 4;
  // Pools of 256 particles when every resident warp gets several; otherwise
  // one particle per lane, spread over as many SMs as possible (narrow CTAs)
  // because small launches are latency-bound.
  const int pool = a.count >= resident_warps * 256 * 2 ? 256 : 32;
  const long long warps = std::min(resident_warps, (a.count + pool - 1) / pool);
  const int threads = warps >= 4LL * sms ? 128 : 32;
  const unsigned grid = (unsigned)((warps * 32 + threads - 1) / threads);
  launch_scope scope(ctx, "trace_streamlines");
  int pool_size = pool;
  void* args[] = {(void*)&a, (void*)&pool_size};
  PARS_CUDA(cudaLaunchKernel(kernel, grid, threads, args, 0, ctx.stream));
}

void launch_compact_vertices(pars_gpu_context& ctx, const float4* slots, const slot_layout* block_slots, const int* block_of,
                             const int* written, const long long* offsets, long long count, float4* out)
{
  if (count <= 0) return;
  launch_scope scope(ctx, "prune_compact");
  compact_kernel<<<grid_for(count * 32, 256), 256, 0, ctx.stream>>>(slots, block_slots, block_of, written, offsets, count, out);
}

void exclusive_sum(pars_gpu_context& ctx, const int* in, long long* out, long long count)
{
  // Widen to int64 with a trailing zero, so that the exclusive scan over
  // count + 1 entries leaves the total in out[count].
  ctx.scan_input.reserve(sizeof(long long) * (count + 1));
  long long* wide = ctx.scan_input.as<long long>();
  {
    launch_scope scope(ctx, "scan_widen");
    widen_kernel<<<grid_for(count + 1, 256), 256, 0, ctx.stream>>>(in, wide, count);
  }
  std::size_t bytes = 0;
  PARS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, bytes, wide, out, count + 1, ctx.stream));
  ctx.cub_temp.reserve(bytes);
  launch_scope scope(ctx, "scan");
  PARS_CUDA(cub::DeviceScan::ExclusiveSum(ctx.cub_temp.get(), bytes, wide, out, count + 1, ctx.stream));
}

void sort_pairs(pars_gpu_context& ctx, const unsigned long long* keys_in, unsigned long long* keys_out,
                const unsigned int* values_in, unsigned int* values_out, long long count, int bits)
{
  if (count <= 0) return;
  std::size_t bytes = 0;
  PARS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, keys_in, keys_out, values_in, values_out, count, 0, bits, ctx.stream));
  ctx.cub_temp.reserve(bytes);
  launch_scope scope(ctx, "exit_sort");
  PARS_CUDA(cub::DeviceRadixSort::SortPairs(ctx.cub_temp.get(), bytes, keys_in, keys_out, values_in, values_out, count, 0, bits, ctx.stream));
}

void launch_gather_exits(pars_gpu_context& ctx, const pars_particle* exits, const unsigned int* order,
                         const unsigned long long* keys, long long count, pars_particle* out, int* block_of,
                         int* block_max, int* block_count)
{
  if (count <= 0) return;
  launch_scope scope(ctx, "exit_gather");
  gather_exits_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(exits, order, keys, count, out, block_of, block_max, block_count);
}

void launch_iota(pars_gpu_context& ctx, unsigned int* out, long long count)
{
  if (count <= 0) return;
  launch_scope scope(ctx, "iota");
  iota_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(out, count);
}

void launch_gather_offsets(pars_gpu_context& ctx, const long long* offsets, const long long* positions, long long n, long long* out)
{
  if (n <= 0) return;
  launch_scope scope(ctx, "gather_offsets");
  gather_offsets_kernel<<<grid_for(n, 256), 256, 0, ctx.stream>>>(offsets, positions, n, out);
}

void launch_particle_stats(pars_gpu_context& ctx, const pars_particle* particles, const int* block_of, long long count, int* block_max)
{
  if (count <= 0) return;
  launch_scope scope(ctx, "particle_stats");
  particle_stats_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(particles, block_of, count, block_max);
}

void launch_extract_block(pars_gpu_context& ctx, const float* domain_xyz, const int32_t domain[3], const int32_t offset[3],
                          const int shape[3], float4* out)
{
  const long long total = (long long)shape[0] * shape[1] * shape[2];
  if (total <= 0) return;
  launch_scope scope(ctx, "extract_block");
  extract_block_kernel<<<grid_for(total, 256), 256, 0, ctx.stream>>>(domain_xyz, domain[1], domain[2], offset[0], offset[1], offset[2],
                                                                    shape[0], shape[1], shape[2], out);
}
}
