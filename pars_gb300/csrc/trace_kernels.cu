// Streamline tracing kernels: a lane runs the reference's per-particle loop
// (particle_tracer.cpp:258-336) for one particle at a time and writes its slot
// range of the padded vertex layout; a warp per particle then prunes
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
enum trace_mode { trace_frozen = 0, trace_classic = 1, trace_general = 2 };

// The particle a lane traces.
struct lane_particle
{
  long long    i = 0;
  int          it = 0, N = 0, written = 0, kept = 0, block = 0;
  float4       last = make_float4(0.f, 0.f, 0.f, 0.f);   // the last vertex written
  local_position q {0, 0, 0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};   // re-sampled RK4 / Euler: cell + offset
  corner_cache cache;
  field_view   f {};
  step_rule    rule {};                      // re-sampled stages: the rule's h and scheme
  const step_rule* frozen_rule = nullptr;    // frozen scheme: the rule in parameter / global memory
  frozen_history   hist;                     // frozen multistep scheme: the previous step's velocity
  float4*      out = nullptr;
};

// Loads particle i and writes its seed vertex (slot 0).
template <int MODE>
__device__ __forceinline__ void particle_start(const trace_launch& a, lane_particle& p, long long i)
{
  p.i = i;
  p.block = a.block_of ? a.block_of[i] : 0;
  p.f = a.blocks[p.block].field;
  p.rule = a.block_rules ? a.block_rules[p.block] : a.rule;
  p.frozen_rule = a.block_rules ? a.block_rules + p.block : &a.rule;
  p.hist = frozen_history();
  const float4* record = reinterpret_cast<const float4*>(a.particles + i);
  p.last = record[0];
  p.N = __float_as_int(record[1].x);   // remaining_iterations
  const slot_layout L = a.block_slots[p.block];
  p.out = a.slots + L.origin + i * L.stride;
  p.out[0] = p.last;
  p.written = 1;
  p.kept = is_invalid_vertex(p.last) ? 0 : 1;
  if constexpr (MODE != trace_frozen) p.q = to_local(p.f, p.last);
  p.cache = corner_cache();
  p.it = 1;
}

// One iteration of the reference's per-particle loop (particle_tracer.cpp:
// 266-335); returns true when the particle has ended (its counts are then
// stored, and a particle that left its block through a face with a neighbour
// is pushed onto the exit queue with one atomic — the queue is sorted by
// (destination, source index) afterwards, so slots may be taken in any order).
// MODE trace_frozen: the reference's scheme and FP32 operation order
// (bit-exact).  MODE trace_classic: re-sampled stages of RK4 / Euler carried
// in local cell coordinates (cell + offset + compensation, as the batched
// engine does; the step-start test is the cell index, which differs from
// contains() only within an ulp of the block's last face), each vertex
// written as offset + (cell + u) h.  MODE trace_general: the same for any
// re-sampled scheme (general_step_local).
template <int MODE>
__device__ __forceinline__ bool particle_iteration(const trace_launch& a, lane_particle& p, unsigned int& steps)
{
  const float4 term = termination_vertex();
  bool finish = false;
  if (p.it >= p.N) finish = true;                                     // remaining_iterations <= 1
  else if (p.it == p.N - 1) { p.out[p.it] = term; ++p.written; ++p.kept; finish = true; }
  else
  {
    float3 v;
    bool inside;
    if constexpr (MODE == trace_frozen) inside = sample_inside_cached(p.f, p.cache, p.last, v);
    else
    {
      inside = local_inside(p.f, p.q);
      if (inside) v = sample_local(p.f, p.cache, p.q.ix, p.q.iy, p.q.iz, p.q.ux, p.q.uy, p.q.uz);
    }
    if (!inside)
    {
      p.out[p.it] = term; ++p.written; ++p.kept; finish = true;
      if (a.route_exits)
      {
        const int face = exit_face(p.f, p.last, a.blocks[p.block].neighbor);
        if (face >= 0)
        {
          const unsigned int slot = atomicAdd(a.exit_count, 1u);
          pars_particle e;
          e.position[0] = p.last.x; e.position[1] = p.last.y; e.position[2] = p.last.z; e.position[3] = p.last.w;
          e.remaining_iterations = p.N - p.it;
          e.vector_field_index = -1;
          e.original_rank = 0;
          e.original_voxel[0] = e.original_voxel[1] = e.original_voxel[2] = 0;
          e.padding[0] = e.padding[1] = 0;
          const int destination = a.blocks[p.block].neighbor[face];
          a.exit_particles[slot] = e;
          a.exit_keys[slot] = ((unsigned long long)destination << 40) | (unsigned long long)p.i;
        }
      }
    }
    else if (MODE == trace_frozen ? is_zero(v) : is_zero_local(p.f, v)) { p.out[p.it] = term; ++p.written; ++p.kept; finish = true; }
    else
    {
      float4 next;
      if constexpr (MODE == trace_frozen) next = frozen_step(*p.frozen_rule, p.last, v, p.hist);
      else
      {
        if constexpr (MODE == trace_general) general_step_local(p.f, p.cache, p.rule, p.q, v, p.hist);
        else local_step(p.f, p.cache, p.rule.rk4, p.rule.h, p.q, v);
        next = to_absolute(p.f, p.q, p.last.w);
      }
      p.out[p.it] = next;
      ++p.written;
      p.kept += is_invalid_vertex(next) ? 0 : 1;
      p.last = next;
      ++steps;
      ++p.it;
    }
  }
  if (finish)
  {
    a.written[p.i] = p.written;
    a.kept[p.i] = p.kept;
  }
  return finish;
}

__device__ __forceinline__ void add_steps(const trace_launch& a, unsigned int steps)
{
  const unsigned int warp_steps = __reduce_add_sync(full_mask, steps);
  if ((threadIdx.x & 31) == 0 && warp_steps) atomicAdd(a.steps, (unsigned long long)warp_steps);
}

// One particle per thread: for launches with no more particles than resident
// lanes, where refilling cannot help and warp votes would only add latency.
template <int MODE>
__global__ void __launch_bounds__(128) trace_kernel(const __grid_constant__ trace_launch a)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int steps = 0;
  if (i < a.count)
  {
    lane_particle p;
    particle_start<MODE>(a, p, i);
    while (!particle_iteration<MODE>(a, p, steps)) {}
  }
  add_steps(a, steps);
}

// Persistent: warps take pools of particles from a device counter, and a lane
// whose particle has ended takes the next particle of the pool at once (warp
// ballot + prefix), so lanes do not idle while the rest of the warp finishes
// longer curves.  Every particle writes only its own slot range, its counts
// and its exit-queue entry, so the result does not depend on which lane traced
// it.
template <int MODE>
__global__ void __launch_bounds__(128) trace_persistent_kernel(const __grid_constant__ trace_launch a, int pool_size)
{
  const int lane = threadIdx.x & 31;
  const unsigned lanes_below = (1u << lane) - 1u;
  long long pool_next = 0, pool_end = 0;   // warp-uniform
  bool exhausted = false;
  unsigned int steps = 0;
  bool alive = false;
  lane_particle p;
  for (;;)
  {
    unsigned need = __ballot_sync(full_mask, !alive);
    if (need && !exhausted)
    {
      while (need)
      {
        if (pool_next < pool_end)
        {
          const long long s = pool_next + __popc(need & lanes_below);
          if (!alive && s < pool_end) { particle_start<MODE>(a, p, s); alive = true; }
          pool_next = min(pool_end, pool_next + (long long)__popc(need));
          need = __ballot_sync(full_mask, !alive);
          continue;
        }
        long long q = 0;
        if (lane == 0) q = (long long)atomicAdd(a.next, (unsigned long long)pool_size);
        q = __shfl_sync(full_mask, q, 0);
        if (q >= a.count) { exhausted = true; break; }
        pool_next = q;
        pool_end = min(q + pool_size, a.count);
      }
    }
    if (need == full_mask) break;   // every lane idle, and the pools are exhausted
    if (alive && particle_iteration<MODE>(a, p, steps)) alive = false;
  }
  add_steps(a, steps);
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
  const int mode = a.rule.frozen ? trace_frozen : (a.rule.scheme == scheme_classic ? trace_classic : trace_general);
  const void* persistent = mode == trace_frozen ? (const void*)trace_persistent_kernel<trace_frozen>
                         : mode == trace_classic ? (const void*)trace_persistent_kernel<trace_classic>
                                                 : (const void*)trace_persistent_kernel<trace_general>;
  int& per_sm = ctx.trace_ctas_per_sm[mode];
  if (ctx.sm_count <= 0) PARS_CUDA(cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, ctx.device));
  if (per_sm < 0) PARS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent, 128, 0));
  const int sms = ctx.sm_count;
  const long long resident_warps = (long long)std::max(per_sm, 1) * sms * 4;
  launch_scope scope(ctx, "trace_streamlines");
  if (a.count <= resident_warps * 32)
  {
    // every lane gets at most one particle: one per thread, narrow CTAs for
    // small counts so that the work spreads over all SMs
    const int threads = a.count <= 128LL * sms ? 32 : 128;
    const unsigned grid = (unsigned)((a.count + threads - 1) / threads);
    if (mode == trace_frozen)       trace_kernel<trace_frozen><<<grid, threads, 0, ctx.stream>>>(a);
    else if (mode == trace_classic) trace_kernel<trace_classic><<<grid, threads, 0, ctx.stream>>>(a);
    else                            trace_kernel<trace_general><<<grid, threads, 0, ctx.stream>>>(a);
    return;
  }
  // pools of 256 particles when every resident warp gets several, else 32
  const int pool = a.count >= resident_warps * 256 * 2 ? 256 : 32;
  const unsigned grid = (unsigned)std::min<long long>((long long)per_sm * sms, (a.count / pool + 4) / 4 + 1);
  int pool_size = pool;
  void* args[] = {(void*)&a, (void*)&pool_size};
  PARS_CUDA(cudaLaunchKernel(persistent, grid, 128, args, 0, ctx.stream));
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
