// Streamline tracing kernels: one thread per particle runs the reference's
// per-particle loop (particle_tracer.cpp:258-336) and writes its slot range of
// the padded vertex layout; a warp per particle then prunes invalid vertices
// (particle_tracer.cpp:402-409) into the packed curve buffer.  Particles that
// leave their block are pushed onto a device exit queue (warp ballot + one
// atomic per warp), then stably sorted by (destination block, source order) to
// form the next round's per-block particle lists (particle_tracer.cpp:376-393).
#include <cub/cub.cuh>

#include "context.hpp"

namespace pars
{
namespace
{
constexpr unsigned full_mask = 0xffffffffu;

// FROZEN = true: the reference's scheme and FP32 operation order (bit-exact).
// FROZEN = false: re-sampled stages, consistent cell weights, compensated
// position accumulation.
template <bool FROZEN>
__global__ void __launch_bounds__(256) trace_kernel(const trace_launch a)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < a.count;
  unsigned int steps = 0;
  bool exits = false;
  float4 exit_position = make_float4(0.f, 0.f, 0.f, 0.f);
  int exit_remaining = 0, exit_block = 0;

  if (active)
  {
    const int block = a.block_of ? a.block_of[i] : 0;
    const field_view f = a.blocks[block].field;
    const step_rule rule = a.block_rules ? a.block_rules[block] : a.rule;
    const float4* record = reinterpret_cast<const float4*>(a.particles + i);
    float4 last = record[0];
    const int N = __float_as_int(record[1].x);   // remaining_iterations
    const slot_layout L = a.block_slots[block];
    float4* out = a.slots + L.origin + i * L.stride;
    out[0] = last;
    int written = 1;
    int kept = is_invalid_vertex(last) ? 0 : 1;
    const float4 term = termination_vertex();
    float3 lo = make_float3(0.0f, 0.0f, 0.0f);
    corner_cache cache;
    for (int it = 1; it < N; ++it)
    {
      if (it == N - 1) { out[it] = term; ++written; ++kept; break; }
      float3 v;
      bool inside;
      if (FROZEN) inside = sample_inside(f, last, v);
      else        inside = sample_start(f, cache, last, v);
      if (!inside)
      {
        out[it] = term; ++written; ++kept;
        if (a.route_exits)
        {
          const int face = exit_face(f, last, a.blocks[block].neighbor);
          if (face >= 0)
          {
            exits = true;
            exit_position = last;
            exit_remaining = N - it;
            exit_block = a.blocks[block].neighbor[face];
          }
        }
        break;
      }
      if (is_zero(v)) { out[it] = term; ++written; ++kept; break; }
      float4 next;
      if (FROZEN) next = frozen_step(rule, last, v);
      else { next = last; resampled_step_cached(f, cache, rule, next, lo, v); }
      out[it] = next;
      ++written;
      kept += is_invalid_vertex(next) ? 0 : 1;
      last = next;
      ++steps;
    }
    a.written[i] = written;
    a.kept[i] = kept;
  }

  // Warp-aggregated step count.
  const unsigned int warp_steps = __reduce_add_sync(full_mask, steps);
  const int lane = threadIdx.x & 31;
  if (lane == 0 && warp_steps) atomicAdd(a.steps, (unsigned long long)warp_steps);

  // Warp ballot + prefix: one atomic reserves the warp's exit slots.
  const unsigned mask = __ballot_sync(full_mask, exits);
  if (mask)
  {
    unsigned int base = 0;
    const int leader = __ffs(mask) - 1;
    if (lane == leader) base = atomicAdd(a.exit_count, (unsigned int)__popc(mask));
    base = __shfl_sync(full_mask, base, leader);
    if (exits)
    {
      const unsigned int slot = base + __popc(mask & ((1u << lane) - 1u));
      pars_particle p;
      p.position[0] = exit_position.x; p.position[1] = exit_position.y;
      p.position[2] = exit_position.z; p.position[3] = exit_position.w;
      p.remaining_iterations = exit_remaining;
      p.vector_field_index = -1;
      p.original_rank = 0;
      p.original_voxel[0] = p.original_voxel[1] = p.original_voxel[2] = 0;
      p.padding[0] = p.padding[1] = 0;
      a.exit_particles[slot] = p;
      a.exit_keys[slot] = ((unsigned long long)exit_block << 40) | (unsigned long long)i;
    }
  }
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
  // Small particle counts: narrow blocks so that the work spreads over all SMs.
  int threads = 128;
  if (a.count <= 152LL * 128) threads = 32;
  else if (a.count <= 152LL * 256) threads = 64;
  launch_scope scope(ctx, "trace_streamlines");
  if (a.rule.frozen) trace_kernel<true><<<grid_for(a.count, threads), threads, 0, ctx.stream>>>(a);
  else               trace_kernel<false><<<grid_for(a.count, threads), threads, 0, ctx.stream>>>(a);
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
