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
enum iteration_outcome { particle_stepped = 0, particle_ended = 1, particle_left = 2 };

// The per-particle part of one iteration: the termination tests and the step,
// the vertex written at slot p.it.  particle_left: the step-start point is
// outside the block (the caller routes the particle).
template <int MODE>
__device__ __forceinline__ int particle_advance(lane_particle& p, unsigned int& steps)
{
  const float4 term = termination_vertex();
  if (p.it >= p.N) return particle_ended;                              // remaining_iterations <= 1
  if (p.it == p.N - 1) { p.out[p.it] = term; ++p.written; ++p.kept; return particle_ended; }
  float3 v;
  bool inside;
  if constexpr (MODE == trace_frozen) inside = sample_inside_cached(p.f, p.cache, p.last, v);
  else
  {
    inside = local_inside(p.f, p.q);
    if (inside) v = sample_local(p.f, p.cache, p.q.ix, p.q.iy, p.q.iz, p.q.ux, p.q.uy, p.q.uz);
  }
  if (!inside) { p.out[p.it] = term; ++p.written; ++p.kept; return particle_left; }
  if (MODE == trace_frozen ? is_zero(v) : is_zero_local(p.f, v)) { p.out[p.it] = term; ++p.written; ++p.kept; return particle_ended; }
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
  return particle_stepped;
}

// The particle a block hands to its face neighbour: its last vertex and the
// iterations left (particle_tracer.cpp:280-309).
__device__ __forceinline__ pars_particle handed_over(const lane_particle& p)
{
  pars_particle e;
  e.position[0] = p.last.x; e.position[1] = p.last.y; e.position[2] = p.last.z; e.position[3] = p.last.w;
  e.remaining_iterations = p.N - p.it;
  e.vector_field_index = -1;
  e.original_rank = 0;
  e.original_voxel[0] = e.original_voxel[1] = e.original_voxel[2] = 0;
  e.padding[0] = e.padding[1] = 0;
  return e;
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
  const int outcome = particle_advance<MODE>(p, steps);
  if (outcome == particle_stepped) return false;
  if (outcome == particle_left && a.route_exits)
  {
    const int face = exit_face(p.f, p.last, a.blocks[p.block].neighbor);
    if (face >= 0)
    {
      const unsigned int slot = atomicAdd(a.exit_count, 1u);
      const int destination = a.blocks[p.block].neighbor[face];
      a.exit_particles[slot] = handed_over(p);
      a.exit_keys[slot] = ((unsigned long long)destination << 40) | (unsigned long long)p.i;
    }
  }
  a.written[p.i] = p.written;
  a.kept[p.i] = p.kept;
  return true;
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

// ---- Asynchronous rounds ---------------------------------------------------------
// Every round of a partitioned domain in one persistent launch (no round
// barrier): warps take segment ids in order, async_claims at a time, and hand
// them to idle lanes; a lane starts its segment once the record is published,
// and appends the continuation of a particle that leaves its block.  Vertex
// chunks come from warp-private slabs of async_slab chunks, so the global
// counters see one atomic per 32 claims or 64 chunks.  The launch ends when
// every allocated segment is done (done read before allocated: a segment is
// marked done only after its continuation was allocated and published).
constexpr unsigned int async_wait_limit = 1u << 23;   // warp-wide idle polls (about 2 s with the sleeps)

// Device-scope memory-model accesses (PTX ld.acquire / ld.relaxed /
// st.release): a segment's record is written before its ready flag is
// released, and read after the flag is acquired.
__device__ __forceinline__ unsigned long long load_acquire(const unsigned long long* p)
{
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long load_relaxed(const unsigned long long* p)
{
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int load_acquire(const int* p)
{
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void store_release(int* p, int v)
{
  asm volatile("st.release.gpu.global.b32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

template <int MODE>
__device__ __forceinline__ void async_start(const async_launch& a, lane_particle& p, long long s)
{
  p.i = s;
  p.block = a.seg_block[s];
  p.f = a.blocks[p.block].field;
  p.rule = a.rule;
  p.frozen_rule = &a.rule;
  p.hist = frozen_history();
  const float4* record = reinterpret_cast<const float4*>(a.seg_particle + s);
  p.last = record[0];
  p.N = __float_as_int(record[1].x);   // remaining_iterations
  p.written = 0;
  p.kept = 0;
  if constexpr (MODE != trace_frozen) p.q = to_local(p.f, p.last);
  p.cache = corner_cache();
  p.it = 0;   // the seed vertex is written by the first iteration
}

template <int MODE>
__global__ void __launch_bounds__(128) async_trace_kernel(const __grid_constant__ async_launch a)
{
  const int lane = threadIdx.x & 31;
  const unsigned lanes_below = (1u << lane) - 1u;
  unsigned int steps = 0, waits = 0;
  bool alive = false, finished = false;
  long long claim = -1;
  unsigned long long known_allocated = 0;      // allocated segments, as last read
  long long pool_next = 0, pool_end = 0;       // warp-uniform: claimed ids not yet handed out
  long long slab_next = 0, slab_end = 0;       // warp-uniform: chunks not yet handed out
  int chunk = -1;
  lane_particle p;
  for (;;)
  {
    // segment ids for idle lanes, from the warp's pool (refilled in order)
    const unsigned want = __ballot_sync(full_mask, !alive && claim < 0 && !finished);
    if (want)
    {
      const long long k = __popc(want), left = pool_end - pool_next;
      long long fresh = 0;
      if (k > left)
      {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(a.counters + async_head, (unsigned long long)async_claims);
        fresh = (long long)__shfl_sync(full_mask, base, 0);
      }
      if (!alive && claim < 0 && !finished)
      {
        const long long mine = __popc(want & lanes_below);
        claim = mine < left ? pool_next + mine : fresh + (mine - left);
      }
      if (k > left) { pool_next = fresh + (k - left); pool_end = fresh + async_claims; }
      else pool_next += k;
    }
    // start a claimed segment once published; finish when every segment is
    // done (done read before allocated: equal counts mean nothing is in flight)
    if (claim >= 0)
    {
      if (claim >= a.capacity) { finished = true; claim = -1; }
      else
      {
        if ((unsigned long long)claim >= known_allocated) known_allocated = load_relaxed(a.counters + async_alloc);
        if ((unsigned long long)claim < known_allocated)
        {
          if (load_acquire(a.seg_ready + claim))
          {
            async_start<MODE>(a, p, claim);
            chunk = -1;
            alive = true;
            claim = -1;
          }
        }
        else
        {
          const unsigned long long done = load_acquire(a.counters + async_done);
          const unsigned long long allocated = load_relaxed(a.counters + async_alloc);
          known_allocated = allocated;
          if ((unsigned long long)claim >= allocated && done == allocated) { finished = true; claim = -1; }
        }
      }
    }
    if (__all_sync(full_mask, finished)) break;
    if (!__any_sync(full_mask, alive))
    {
      // nothing to trace: stop on another lane's failure or after the wait limit
      if (load_acquire(a.error) != async_ok) break;
      if (++waits > async_wait_limit) { if (lane == 0) atomicCAS(a.error, async_ok, async_wait_limit); break; }
      __nanosleep(256);
      continue;
    }
    waits = 0;
    // a chunk for every lane whose next vertex starts one, from the warp's slab
    const bool need = alive && (p.it < p.N || p.it == 0) && (p.written % async_chunk) == 0;
    const unsigned needing = __ballot_sync(full_mask, need);
    if (needing)
    {
      const long long k = __popc(needing), left = slab_end - slab_next;
      long long fresh = 0;
      if (k > left)
      {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(a.counters + async_chunks, (unsigned long long)async_slab);
        fresh = (long long)__shfl_sync(full_mask, base, 0);
      }
      if (need)
      {
        const long long mine = __popc(needing & lanes_below);
        const long long c = mine < left ? slab_next + mine : fresh + (mine - left);
        if (c >= a.chunk_capacity) { atomicCAS(a.error, async_ok, async_chunks_full); alive = false; finished = true; }
        else
        {
          if (chunk >= 0) a.chunk_next[chunk] = int(c);
          else a.seg_first_chunk[p.i] = int(c);
          chunk = int(c);
          p.out = a.chunks + c * async_chunk - p.written;   // p.out[p.written] is the chunk's first vertex
        }
      }
      if (k > left) { slab_next = fresh + (k - left); slab_end = fresh + async_slab; }
      else slab_next += k;
    }
    if (!alive) continue;
    if (p.it == 0)
    {
      // the seed vertex (slot 0 of the reference's layout)
      p.out[0] = p.last;
      p.written = 1;
      p.kept = is_invalid_vertex(p.last) ? 0 : 1;
      p.it = 1;
      continue;
    }
    const int outcome = particle_advance<MODE>(p, steps);
    if (outcome == particle_stepped) continue;
    if (outcome == particle_left)
    {
      const int face = exit_face(p.f, p.last, a.blocks[p.block].neighbor);
      if (face >= 0)
      {
        const unsigned long long id = atomicAdd(a.counters + async_alloc, 1ULL);
        if ((long long)id >= a.capacity) atomicCAS(a.error, async_ok, async_segments_full);
        else
        {
          a.seg_particle[id] = handed_over(p);
          a.seg_block[id] = a.blocks[p.block].neighbor[face];
          a.seg_round[id] = a.seg_round[p.i] + 1;
          a.seg_parent[id] = p.i;
          store_release(a.seg_ready + id, 1);
        }
      }
    }
    a.seg_written[p.i] = p.written;
    a.seg_kept[p.i] = p.kept;
    __threadfence();
    atomicAdd(a.counters + async_done, 1ULL);
    alive = false;
  }
  const unsigned int warp_steps = __reduce_add_sync(full_mask, steps);
  if (lane == 0 && warp_steps) atomicAdd(a.counters + async_steps, (unsigned long long)warp_steps);
}

__global__ void async_seed_kernel(const async_launch a, const pars_particle* __restrict__ particles, const int* __restrict__ block_of,
                                  long long count)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  a.seg_particle[i] = particles[i];
  a.seg_block[i] = block_of ? block_of[i] : 0;
  a.seg_round[i] = 0;
  a.seg_parent[i] = -1;
  a.seg_ready[i] = 1;
  a.seg_first_chunk[i] = -1;
}

// The round kernels below meet long runs of equal keys (a round's segments
// are mostly allocated together), so each warp first combines its lanes'
// equal keys (__match_any_sync) and one lane per key does the atomic.
__global__ void round_histogram_kernel(const int* __restrict__ seg_round, long long count, int rounds_cap, int* __restrict__ histogram,
                                       int* __restrict__ max_round)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool valid = i < count;
  const int r = valid ? seg_round[i] : -1;
  const unsigned same = __match_any_sync(full_mask, r);
  const int top = __reduce_max_sync(full_mask, r);
  if (lane == 0 && top >= 0) atomicMax(max_round, top);
  if (valid && lane == __ffs(same) - 1 && r < rounds_cap) atomicAdd(histogram + r, __popc(same));
}

__global__ void round_scatter_kernel(const int* __restrict__ seg_round, long long count, const long long* __restrict__ first,
                                     int* __restrict__ cursor, unsigned int* __restrict__ ids)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool valid = i < count;
  const int r = valid ? seg_round[i] : -1;
  const unsigned same = __match_any_sync(full_mask, r);
  const int leader = __ffs(same) - 1;
  int base = 0;
  if (valid && lane == leader) base = atomicAdd(cursor + r, __popc(same));
  base = __shfl_sync(full_mask, base, leader);
  if (valid) ids[first[r] + base + __popc(same & ((1u << lane) - 1u))] = (unsigned int)i;
}

__global__ void round_keys_kernel(const unsigned int* __restrict__ ids, long long n, const int* __restrict__ seg_block,
                                  const long long* __restrict__ seg_parent, const long long* __restrict__ position,
                                  unsigned long long* __restrict__ keys)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const unsigned int s = ids[k];
  const long long parent = seg_parent[s];
  keys[k] = ((unsigned long long)seg_block[s] << 40) | (unsigned long long)(parent < 0 ? (long long)s : position[parent]);
}

__global__ void round_positions_kernel(const unsigned int* __restrict__ ids, long long n, long long first, long long* __restrict__ position)
{
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) position[ids[k]] = first + k;
}

__global__ void round_stats_kernel(const unsigned int* __restrict__ order, long long n, const int* __restrict__ seg_round,
                                   const int* __restrict__ seg_block, const pars_particle* __restrict__ seg_particle,
                                   const int* __restrict__ seg_kept, int blocks, int* __restrict__ stats, int* __restrict__ kept_ordered)
{
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool valid = g < n;
  long long cell = -1;
  int remaining = 0;
  if (valid)
  {
    const unsigned int s = order[g];
    cell = (long long)seg_round[s] * blocks + seg_block[s];
    remaining = seg_particle[s].remaining_iterations;
    kept_ordered[g] = seg_kept[s];
  }
  const unsigned same = __match_any_sync(full_mask, cell);
  const int top = __reduce_max_sync(same, remaining);
  if (valid && lane == __ffs(same) - 1)
  {
    atomicAdd(stats + 2 * cell, __popc(same));
    atomicMax(stats + 2 * cell + 1, top);
  }
}

// One warp per segment: its written vertices, chunk by chunk, minus invalid ones.
__global__ void __launch_bounds__(256) async_assemble_kernel(const async_launch a, const unsigned int* __restrict__ order,
                                                             const long long* __restrict__ offsets, long long n,
                                                             float4* __restrict__ out)
{
  const long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= n) return;
  const unsigned int s = order[g];
  const int written = a.seg_written[s];
  long long dst = offsets[g];
  int chunk = a.seg_first_chunk[s];
  for (int j0 = 0; j0 < written; j0 += async_chunk)
  {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    bool keep = false;
    if (j0 + lane < written) { v = a.chunks[(long long)chunk * async_chunk + lane]; keep = !is_invalid_vertex(v); }
    const unsigned mask = __ballot_sync(full_mask, keep);
    if (keep) out[dst + __popc(mask & ((1u << lane) - 1u))] = v;
    dst += __popc(mask);
    if (j0 + async_chunk < written) chunk = a.chunk_next[chunk];
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

long long launch_async_trace(pars_gpu_context& ctx, const async_launch& a, bool count_only)
{
  const int mode = a.rule.frozen ? trace_frozen : (a.rule.scheme == scheme_classic ? trace_classic : trace_general);
  const void* kernel = mode == trace_frozen ? (const void*)async_trace_kernel<trace_frozen>
                     : mode == trace_classic ? (const void*)async_trace_kernel<trace_classic>
                                             : (const void*)async_trace_kernel<trace_general>;
  if (ctx.sm_count <= 0) PARS_CUDA(cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, ctx.device));
  int& per_sm = ctx.async_ctas_per_sm[mode];
  if (per_sm < 0) PARS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0));
  // as many CTAs as are resident at once: lanes wait for segments that others publish
  const unsigned grid = (unsigned)(std::max(per_sm, 1) * ctx.sm_count);
  if (count_only) return (long long)grid * 4;
  launch_scope scope(ctx, "trace_async");
  void* args[] = {(void*)&a};
  PARS_CUDA(cudaLaunchKernel(kernel, grid, 128, args, 0, ctx.stream));
  return (long long)grid * 4;
}

void launch_async_seed(pars_gpu_context& ctx, const async_launch& a, const pars_particle* particles, const int* block_of, long long count)
{
  if (count <= 0) return;
  launch_scope scope(ctx, "async_seed");
  async_seed_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(a, particles, block_of, count);
}

void launch_round_histogram(pars_gpu_context& ctx, const int* seg_round, long long count, int rounds_cap, int* histogram, int* max_round)
{
  if (count <= 0) return;
  launch_scope scope(ctx, "round_histogram");
  round_histogram_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(seg_round, count, rounds_cap, histogram, max_round);
}

void launch_round_scatter(pars_gpu_context& ctx, const int* seg_round, long long count, const long long* first, int* cursor,
                          unsigned int* ids)
{
  if (count <= 0) return;
  launch_scope scope(ctx, "round_scatter");
  round_scatter_kernel<<<grid_for(count, 256), 256, 0, ctx.stream>>>(seg_round, count, first, cursor, ids);
}

void launch_round_keys(pars_gpu_context& ctx, const unsigned int* ids, long long n, const int* seg_block, const long long* seg_parent,
                       const long long* position, unsigned long long* keys)
{
  if (n <= 0) return;
  launch_scope scope(ctx, "round_keys");
  round_keys_kernel<<<grid_for(n, 256), 256, 0, ctx.stream>>>(ids, n, seg_block, seg_parent, position, keys);
}

void launch_round_positions(pars_gpu_context& ctx, const unsigned int* ids, long long n, long long first, long long* position)
{
  if (n <= 0) return;
  launch_scope scope(ctx, "round_positions");
  round_positions_kernel<<<grid_for(n, 256), 256, 0, ctx.stream>>>(ids, n, first, position);
}

void launch_round_stats(pars_gpu_context& ctx, const unsigned int* order, long long n, const int* seg_round, const int* seg_block,
                        const pars_particle* seg_particle, const int* seg_kept, int blocks, int* stats, int* kept_ordered)
{
  if (n <= 0) return;
  launch_scope scope(ctx, "round_stats");
  round_stats_kernel<<<grid_for(n, 256), 256, 0, ctx.stream>>>(order, n, seg_round, seg_block, seg_particle, seg_kept, blocks, stats,
                                                               kept_ordered);
}

void launch_async_assemble(pars_gpu_context& ctx, const async_launch& a, const unsigned int* order, const long long* offsets,
                           long long n, float4* out)
{
  if (n <= 0) return;
  launch_scope scope(ctx, "async_assemble");
  async_assemble_kernel<<<grid_for(n * 32, 256), 256, 0, ctx.stream>>>(a, order, offsets, n, out);
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
