// Host-side state of a pars_gpu context: device buffers, resident fields and
// domains, the curves of the last trace, scratch, and launch instrumentation.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pars_gpu.h"
#include "device_math.cuh"

namespace pars
{
// Error carrying a pars_gpu status; thrown inside the library and turned into
// a status code at the C boundary (no exception crosses it).
struct error : std::runtime_error
{
  int32_t status;
  error(int32_t s, const std::string& message) : std::runtime_error(message), status(s) {}
};

#define PARS_CUDA(call)                                                                            \
  do {                                                                                             \
    cudaError_t pars_e_ = (call);                                                                  \
    if (pars_e_ != cudaSuccess)                                                                    \
      throw ::pars::error(pars_e_ == cudaErrorMemoryAllocation ? PARS_ERR_OUT_OF_MEMORY : PARS_ERR_CUDA, \
                          std::string(#call) + ": " + cudaGetErrorString(pars_e_));                \
  } while (0)

#define PARS_REQUIRE(condition, message)                                                            \
  do { if (!(condition)) throw ::pars::error(PARS_ERR_INVALID_ARGUMENT, message); } while (0)

// Grow-only device allocation owned by the context.
class device_buffer
{
public:
  device_buffer() = default;
  device_buffer(const device_buffer&) = delete;
  device_buffer& operator=(const device_buffer&) = delete;
  device_buffer(device_buffer&& o) noexcept : ptr_(o.ptr_), bytes_(o.bytes_) { o.ptr_ = nullptr; o.bytes_ = 0; }
  device_buffer& operator=(device_buffer&& o) noexcept { release(); ptr_ = o.ptr_; bytes_ = o.bytes_; o.ptr_ = nullptr; o.bytes_ = 0; return *this; }
  ~device_buffer() { release(); }

  void reserve(std::size_t bytes)
  {
    if (bytes <= bytes_) return;
    release();
    if (bytes == 0) return;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess)
    {
      (void)cudaGetLastError();
      throw error(PARS_ERR_OUT_OF_MEMORY, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
    }
    ptr_ = p;
    bytes_ = bytes;
  }
  void release()
  {
    if (ptr_) cudaFree(ptr_);
    ptr_ = nullptr;
    bytes_ = 0;
  }
  template <typename T> T* as() const { return static_cast<T*>(ptr_); }
  void*       get()   const { return ptr_; }
  std::size_t bytes() const { return bytes_; }

private:
  void*       ptr_   = nullptr;
  std::size_t bytes_ = 0;
};

struct field_entry
{
  device_buffer data;          // float4 [slices][X][Y][Z]
  int           shape[3];
  float         offset[3], size[3], spacing[3];
  int           slices = 1;    // time slices (1 = steady)
  double        t0 = 0.0, slice_dt = 1.0;
  time_axis time() const
  {
    time_axis t;
    t.nt = slices;
    t.slice_stride = (long long)shape[0] * shape[1] * shape[2];
    t.t0 = t0;
    t.inv_slice_dt = 1.0 / slice_dt;
    return t;
  }
  field_view view() const
  {
    field_view v;
    v.data = data.as<const float4>();
    v.nx = shape[0]; v.ny = shape[1]; v.nz = shape[2];
    v.ox = offset[0]; v.oy = offset[1]; v.oz = offset[2];
    v.hx = spacing[0]; v.hy = spacing[1]; v.hz = spacing[2];
    v.maxx = offset[0] + size[0]; v.maxy = offset[1] + size[1]; v.maxz = offset[2] + size[2];
    v.inv_hx = 1.0f / spacing[0]; v.inv_hy = 1.0f / spacing[1]; v.inv_hz = 1.0f / spacing[2];
    return v;
  }
};

// One block of a traced domain as the tracing kernel sees it.
struct trace_block
{
  field_view field;
  int        neighbor[6];   // block index per face, -1 where absent
};

struct domain_entry
{
  int                      ranks = 0;
  bool                     owns_fields = true;   // false: blocks are the caller's fields (pars_gpu_domain_assemble)
  pars_partition_info      first {};
  std::vector<int>         fields;      // field handle per block
  std::vector<trace_block> blocks;
  device_buffer            device_blocks;
};

// A batch of integral curves resident on the device.
struct curves_batch
{
  long long vertex_offset = 0;   // into curves.vertices / colors
  long long vertex_count  = 0;
  long long index_offset  = 0;   // into curves.indices (valid after indexing)
  long long index_count   = 0;
  int       rank = 0, round = 0;
};

struct curves_store
{
  device_buffer             vertices;   // float4
  device_buffer             colors;     // float4
  device_buffer             indices;    // int32, the batches' indices packed one after the other
  long long                 vertex_total = 0;
  long long                 index_total = 0;
  bool                      indexed = false;
  bool                      colored = false;
  std::vector<curves_batch> batches;
  long long                 generation = 0;   // bumped whenever the curves or their indices / colours change
};

// The ray tracer's state (render_kernels.cu): the scene's capsules and their
// BVH, the volume, the camera, and the accumulated frames.
struct render_state
{
  render_state();
  // scene: one capsule per line index; prim_vertex[k] = its segment's start vertex
  long long     prims = 0;
  long long     leaves = 0;                     // BVH leaves (runs of 1 or 2 consecutive segments)
  const float4* vertices = nullptr;
  const float4* colors = nullptr;               // nullptr: white
  float         radius = 1.0f;
  long long     curves_generation = -1;         // >= 0: the context's curves at that generation
  device_buffer own_vertices, own_colors, prim_vertex, batch_bounds;
  // BVH (linear, Karras 2012)
  bool          tree_valid = false;
  bool          status_pending = false;         // the build's status word is not read yet
  device_buffer bounds, leaf_lo_unsorted, leaf_hi_unsorted, keys, values, leaf_lo, leaf_hi, leaf_vertex, nodes,
                node_parent, leaf_parent, arrivals, leaf_flags, leaf_index, leaf_first, leaf_run;
  // volume: float [x][y][z] (volume_data: the tracer's own copy in `volume`,
  // or a buffer the caller keeps alive, such as a service dataset)
  bool          has_volume = false;
  const float*  volume_data = nullptr;
  device_buffer volume;
  int           volume_shape[3] = {0, 0, 0};
  float         volume_offset[3] = {0, 0, 0}, volume_spacing[3] = {1, 1, 1};
  // camera and image
  bool          camera_set = false;
  float         position[3] = {0, 0, 0}, corner[3] = {0, 0, 0}, du[3] = {0, 0, 0}, dv[3] = {0, 0, 0};
  float         forward[3] = {0, 0, 1}, up[3] = {0, 1, 0};
  int           width = 0, height = 0;
  // accumulated frames
  bool          accum_valid = false;
  long long     frames = 0;
  device_buffer accum, jitter, status, image, thresholds;
  float         srgb_thresholds[255];
};

struct profile_entry
{
  double    milliseconds = 0.0;
  long long launches     = 0;
};

struct timed_launch
{
  std::string name;
  cudaEvent_t start, stop;
};

struct batch_engine;   // continuous batched advection (pars_gpu.cu)
}

struct pars_gpu_context
{
  int                                     device = 0;
  cudaStream_t                            own_stream = nullptr;
  cudaStream_t                            stream = nullptr;
  std::mutex                              mutex;
  std::string                             last_error;
  int                                     next_handle = 1;
  std::map<int, std::unique_ptr<pars::field_entry>>  fields;
  std::map<int, std::unique_ptr<pars::domain_entry>> domains;
  pars::curves_store                      curves;
  std::unique_ptr<pars::render_state>     render;     // created by the first ray-tracer call
  // scratch
  pars::device_buffer                     particles_in, particles_next, slots, kept, written, offsets, block_of,
                                          block_of_next, exits, exit_keys, exit_keys_sorted, exit_order,
                                          exit_order_sorted, counters, block_max, cub_temp, scan_input, tile_counts,
                                          tile_offsets, staging, boundary_positions, boundary_offsets, single_block,
                                          slot_layouts, curve_bounds, color_specs;
  pars::device_buffer                     ftle;
  long long                               ftle_count = 0;
  // asynchronous rounds: segment table, vertex chunks, round order
  pars::device_buffer                     async_segments, async_chunks, async_counters, async_order, async_positions,
                                          async_cursor;
  // round-by-round tracing (pars_gpu_round_trace): the next round's
  // particles stay in particles_in / block_of; their per-block counts and
  // largest remaining_iterations, the round they belong to, and the tracing
  // call that left them (trace_serial counts every tracing call)
  long long                               trace_serial = 0, round_serial = -1;
  int                                     round_domain = -1, round_next = 0;
  long long                               round_count = 0;
  std::vector<long long>                  round_block_count;
  std::vector<int>                        round_block_max;
  // Released field buffers kept for reuse (bytes -> buffer), so that a caller
  // that uploads, traces and releases every request does not pay cudaMalloc /
  // cudaFree (and their device-wide synchronisation) each time.
  std::multimap<std::size_t, pars::device_buffer> buffer_cache;
  std::size_t                             buffer_cache_bytes = 0;
  // batched advection: job table, counters, and the autotuned launch variant
  // per job class (0 = steady, 1 = unsteady); -1 = not tuned yet
  pars::device_buffer                     batch_jobs, batch_counters;
  int                                     batch_variant[3] = {-1, -1, -1};
  // tracing kernel: resident CTAs of 128 threads per SM (frozen, re-sampled
  // RK4 / Euler, re-sampled general schemes)
  // and the device's SM count, queried once
  int                                     trace_ctas_per_sm[3] = {-1, -1, -1};
  int                                     async_ctas_per_sm[3] = {-1, -1, -1};
  int                                     sm_count = 0;
  // batched engine: resident CTAs per SM per job class and launch shape
  int                                     batch_ctas_per_sm[3][4] = {{-1, -1, -1, -1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}};
  int                                     horizon_ctas_per_sm[3][4] = {{-1, -1, -1, -1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}};
  // continuous batched advection: job tables that grow between horizon launches
  std::shared_ptr<pars::batch_engine>     engine;
  static constexpr std::size_t            buffer_cache_limit = std::size_t(8) << 30;
  // instrumentation
  bool                                    profile = false;
  std::map<std::string, pars::profile_entry> profile_totals;
  std::vector<pars::timed_launch>         pending;
  std::vector<cudaEvent_t>                event_pool;
  cudaEvent_t                             legacy_event = nullptr;   // orders the own stream after the legacy default stream
  long long                               launches = 0;
  long long                               held_bytes() const;
};

namespace pars
{
// Brackets one kernel launch for the instrumentation: call begin() just before
// and end() just after the launch (same stream).
class launch_scope
{
public:
  launch_scope(pars_gpu_context& ctx, const char* name);
  ~launch_scope() noexcept(false);
private:
  pars_gpu_context& ctx_;
  const char*       name_;
  cudaEvent_t       start_ = nullptr;
};

// A device buffer of at least `bytes` (at most twice that) from the context's
// cache, or a new allocation.
device_buffer acquire_buffer(pars_gpu_context& ctx, std::size_t bytes);
// Returns a buffer to the cache (freed instead when the cache is full).
void recycle_buffer(pars_gpu_context& ctx, device_buffer&& buffer);
// Frees every scratch buffer and the buffer cache after the stream drains
// (fields and domains stay); the last trace's curves are dropped.
void release_scratch(pars_gpu_context& ctx);
// Resolves the context's timed launches and moves its per-kernel totals into
// `into` (adding), leaving the context's totals empty.
void take_profile(pars_gpu_context& ctx, std::map<std::string, profile_entry>& into);

// Integrator parameters for (integrator, stage mode, step size); throws
// pars::error for integrators the kernels do not implement.
step_rule make_step_rule(int integrator, int stage_mode, float h);

// Kernel launchers (defined in the *_kernels.cu translation units).
void launch_pack_field(pars_gpu_context& ctx, const float* xyz, float4* out, long long count);
void launch_unpack_field(pars_gpu_context& ctx, const float4* data, float* xyz, long long count);
void launch_field_sample(pars_gpu_context& ctx, const field_view& f, const float4* positions, long long n, uint8_t* inside, float* velocity);
void launch_seed_generate(pars_gpu_context& ctx, const float offset[3], const float stride[3], const int per_dimension[3],
                          int iterations, int rank, pars_particle* out);

// Where a block's particles keep their vertex slots: particle i (of this
// block) owns slots [origin + i * stride, origin + (i + 1) * stride), stride =
// the block's largest remaining_iterations (the reference's per-curve layout,
// particle_tracer.cpp:235-252, with each block padded to its own maximum).
struct slot_layout
{
  long long origin, stride;
};

struct trace_launch
{
  const trace_block*   blocks;
  const pars_particle* particles;
  const int*           block_of;      // nullptr: every particle is in block 0
  long long            count;
  const slot_layout*   block_slots;   // per block (device)
  float4*              slots;
  int*                 written;
  int*                 kept;
  step_rule            rule;
  const step_rule*     block_rules;   // per-block rules (same stage mode as `rule`), or nullptr
  int                  route_exits;   // 0: particles leaving the block are dropped
  pars_particle*       exit_particles;
  unsigned long long*  exit_keys;     // (destination block << 40) | particle index
  unsigned int*        exit_count;
  unsigned long long*  steps;
  unsigned long long*  next;          // pool counter (zero before the launch)
};
void launch_trace(pars_gpu_context& ctx, const trace_launch& a);

// Asynchronous rounds: every round of a partitioned domain traced in one
// persistent launch.  A segment is one particle's trace through one block in
// one round; the launch starts with the seeds as round-0 segments, and a
// particle that leaves its block through a face with a neighbour appends its
// continuation (round + 1, the neighbour's block) to the segment table, where
// any lane picks it up at once.  Vertices go to chunks of async_chunk
// vertices taken from a pool and linked per segment; the rounds' order and
// batches are rebuilt afterwards.
constexpr int async_chunk = 32;
constexpr int async_slab = 64;      // chunks a warp takes from the pool at once
constexpr int async_claims = 32;    // segment ids a warp takes at once
enum async_counter { async_head = 0, async_alloc = 1, async_done = 2, async_chunks = 3, async_steps = 4, async_counters = 5 };
enum async_error { async_ok = 0, async_segments_full = 1, async_chunks_full = 2, async_wait_limit = 3 };
struct async_launch
{
  const trace_block*  blocks;
  step_rule           rule;
  pars_particle*      seg_particle;     // segment start state
  int*                seg_block;
  int*                seg_round;
  long long*          seg_parent;       // the segment it continues (-1: a seed)
  int*                seg_ready;        // 1 once the record is written
  int*                seg_written;      // vertices written (slots of the reference's layout)
  int*                seg_kept;         // of them not invalid
  int*                seg_first_chunk;
  long long           capacity;         // segments
  float4*             chunks;           // async_chunk vertices each
  int*                chunk_next;
  long long           chunk_capacity;
  unsigned long long* counters;         // async_counter
  int*                error;            // async_error
};
// Launches the persistent kernel; returns its warps (each may leave part of a
// chunk slab unused).
long long launch_async_trace(pars_gpu_context& ctx, const async_launch& a, bool count_only = false);
// Round-0 segments from ctx.particles_in / block_of (count particles).
void launch_async_seed(pars_gpu_context& ctx, const async_launch& a, const pars_particle* particles, const int* block_of,
                       long long count);
// Histogram of segment rounds (rounds_cap bins) and the largest round.
void launch_round_histogram(pars_gpu_context& ctx, const int* seg_round, long long count, int rounds_cap, int* histogram,
                            int* max_round);
// Segment ids grouped by round: ids[first[r] + k] for the k-th segment of round r met (any order).
void launch_round_scatter(pars_gpu_context& ctx, const int* seg_round, long long count, const long long* first, int* cursor,
                          unsigned int* ids);
// key[k] = (seg_block[ids[k]] << 40) | position[seg_parent[ids[k]]] for a round's segments (the
// segment's own id for seeds).
void launch_round_keys(pars_gpu_context& ctx, const unsigned int* ids, long long n, const int* seg_block, const long long* seg_parent,
                       const long long* position, unsigned long long* keys);
// position[ids[k]] = first + k.
void launch_round_positions(pars_gpu_context& ctx, const unsigned int* ids, long long n, long long first, long long* position);
// Per (round, block): segments and largest remaining_iterations, stats[2 * (round * blocks + block) + {0, 1}];
// kept_ordered[g] = seg_kept[order[g]].
void launch_round_stats(pars_gpu_context& ctx, const unsigned int* order, long long n, const int* seg_round, const int* seg_block,
                        const pars_particle* seg_particle, const int* seg_kept, int blocks, int* stats, int* kept_ordered);
// Copies each segment's kept vertices (chunk by chunk) to out + offsets[g], in the order `order`.
void launch_async_assemble(pars_gpu_context& ctx, const async_launch& a, const unsigned int* order, const long long* offsets,
                           long long n, float4* out);
void launch_compact_vertices(pars_gpu_context& ctx, const float4* slots, const slot_layout* block_slots, const int* block_of,
                             const int* written,
                             const long long* offsets, long long count, float4* out);
// Exclusive sum of `count` int32 into int64 offsets; offsets[count] = total.
void exclusive_sum(pars_gpu_context& ctx, const int* in, long long* out, long long count);
// Stable sort of (key, value) pairs by the low `bits` bits of the key.
void sort_pairs(pars_gpu_context& ctx, const unsigned long long* keys_in, unsigned long long* keys_out,
                const unsigned int* values_in, unsigned int* values_out, long long count, int bits);
// Gathers the sorted exit queue into the next round's particle list and
// accumulates per-block maximum remaining_iterations and particle counts.
void launch_gather_exits(pars_gpu_context& ctx, const pars_particle* exits, const unsigned int* order,
                         const unsigned long long* keys, long long count, pars_particle* out, int* block_of,
                         int* block_max, int* block_count);
void launch_iota(pars_gpu_context& ctx, unsigned int* out, long long count);
// out[k] = offsets[positions[k]] for k < n.
void launch_gather_offsets(pars_gpu_context& ctx, const long long* offsets, const long long* positions, long long n, long long* out);
// block_max[0] = max remaining_iterations over particles (block_of == nullptr).
void launch_particle_stats(pars_gpu_context& ctx, const pars_particle* particles, const int* block_of, long long count, int* block_max);
// Copies the ghosted block at voxel `offset` of a device [X][Y][Z][3] domain into float4 [shape].
void launch_extract_block(pars_gpu_context& ctx, const float* domain_xyz, const int32_t domain[3], const int32_t offset[3],
                          const int shape[3], float4* out);

long long launch_index_generate(pars_gpu_context& ctx, const float4* vertices, long long n, int* indices);
void launch_color_generate(pars_gpu_context& ctx, const float4* vertices, const int* indices, long long index_count,
                           int mode, float parameter, float4* colors);

// Colour mode and parameter of one curve batch.
struct color_spec
{
  int   mode;
  float parameter;
};
// index_generator::generate on every batch of a curves store in one pass
// (three launches and one host read for all batches): sets each batch's
// index_offset / index_count into the packed index buffer.
void index_batches(pars_gpu_context& ctx, curves_store& c);
// color_generator::generate on every batch (after index_batches) in one
// launch, with each batch's own mode and parameter.
void color_batches(pars_gpu_context& ctx, curves_store& c, const std::vector<color_spec>& specs);

// One job of a batched advection launch, as the persistent kernel reads it.
struct batch_job_device
{
  field_view          field;
  time_axis           time;
  step_rule           rule;
  int                 max_steps;
  double              time_begin;
  slice_clock         clock;          // set by execute_batch from time, time_begin and rule.h
  long long           seed_count;
  const float4*       seeds;          // explicit seeds, or nullptr for the lattice
  float               ox, oy, oz, sx, sy, sz;
  int                 px, py, pz;
  int                 ux, uy, uz;     // lattice seeds: output voxel shape (0 = output per seed)
  float4*             end_positions;  // may be nullptr
  int*                end_steps;      // may be nullptr
  long long           first_pool;     // pools of all earlier jobs
  unsigned long long* steps;          // per-job step counter
};
// Job classes of the batched engine: each class runs in its own launch.
enum batch_class { batch_steady = 0, batch_unsteady = 1, batch_frozen = 2, batch_classes = 3 };
int  batch_variant_count();
// Resident warps per SM of a job class's launch shape.
int  batch_resident_warps(pars_gpu_context& ctx, int job_class, int variant);
int  batch_variant_threads(int variant);
int  batch_pool_seeds();
// job_class: batch_steady, batch_unsteady or batch_frozen.
void launch_batch_advect(pars_gpu_context& ctx, int job_class, int variant, const batch_job_device* jobs, int njobs,
                         long long total_chunks, unsigned long long* counter);

// Horizon launches of the batched engine.  A warp that has taken `iterations`
// steps, or that sees another warp's stop flag, parks as one group: its job (an index into the launch's job table),
// the unconsumed seeds [pool_next, pool_end) of its pool, a pool it has taken
// but not begun (pending, or -1), and its live particles, `count` lane
// records at lanes[32 g ..].  The next launch resumes each group in a warp of
// its own before the warps take new pools.
struct batch_parked_group
{
  int       job;
  int       count;
  long long pool_next, pool_end;
  long long pending;
};
struct batch_parked_lane
{
  long long seed;
  int       steps;
  int       started;             // frozen multistep schemes: history present
  float4    pos;                 // frozen: absolute position
  float3    hist_v;              // frozen multistep schemes: previous velocity
  int       ix, iy, iz;          // re-sampled: cell
  float     ux, uy, uz, lx, ly, lz;   // re-sampled: offset and compensation
};
struct batch_horizon_args
{
  int                       iterations = 0;   // steps per warp before it parks
  int                       in_count = 0;     // parked groups to resume
  const batch_parked_group* in_groups = nullptr;
  const batch_parked_lane*  in_lanes = nullptr;
  unsigned int*             in_counter = nullptr;   // groups resumed (zero before the launch)
  batch_parked_group*       out_groups = nullptr;
  batch_parked_lane*        out_lanes = nullptr;
  unsigned int*             out_count = nullptr;    // groups parked (zero before the launch)
  unsigned int*             stop = nullptr;         // raised by the first warp at the horizon (zero before the launch)
};
// Warps of a horizon launch of (class, variant) when every CTA is resident:
// the most groups one launch can park.
long long batch_horizon_warps(pars_gpu_context& ctx, int job_class, int variant);
// warps: the warps the launch's work can use (at least the parked groups).
void launch_batch_advect_horizon(pars_gpu_context& ctx, int job_class, int variant, const batch_job_device* jobs, int njobs,
                                 long long total_pools, unsigned long long* counter, const batch_horizon_args& hz, long long warps);

// Continuous batched advection.  engine_submit appends a job (re-sampled RK4
// / Euler on steady or unsteady fields, or the frozen scheme on steady ones)
// to its class's job table and returns its ticket; engine_advance runs one
// horizon launch of `iterations` steps per warp for every class with work and
// returns the jobs that completed (ticket, particle-steps); engine_open
// counts the jobs submitted and not yet returned.
long long engine_submit(pars_gpu_context& ctx, const batch_job_device& job);
std::vector<std::pair<long long, unsigned long long>> engine_advance(pars_gpu_context& ctx, int iterations);
long long engine_open(const pars_gpu_context& ctx);

// The tracing round loop over particles already in ctx.particles_in (grouped
// by block, ctx.block_of when there are several blocks); fills ctx.curves.
// device_block_rules (optional, one per block) override `rule`'s step size and
// integrator per block; the stage mode of `rule` applies to every block.
void trace_rounds(pars_gpu_context& ctx, const std::vector<trace_block>& blocks, const trace_block* device_blocks, long long count,
                  std::vector<long long> block_count, std::vector<int> block_max, const step_rule& rule, bool route_exits,
                  pars_gpu_trace_summary* summary, const step_rule* device_block_rules = nullptr);
// Batched advection of `jobs` (one persistent launch per job class: steady,
// unsteady); returns each job's steps.
std::vector<unsigned long long> run_batch(pars_gpu_context& ctx, std::vector<batch_job_device>& jobs, int variant);
pars_partition_info partition(int ranks, int rank, const int32_t domain[3]);

void launch_flow_map(pars_gpu_context& ctx, const field_view& f, const step_rule& rule, int iterations,
                     const float offset[3], const float fm_spacing[3], const int seeds_per_dimension[3],
                     const int fm_shape[3], float4* flow, unsigned long long* steps);
void launch_ftle(pars_gpu_context& ctx, const field_view& flow, double time, int mode, float* out);

// Ray tracer (render_kernels.cu).
void render_jitter(long long frame, float& jx, float& jy);
void render_camera(const float position[3], const float forward[3], const float up[3], int width, int height,
                   float corner[3], float du[3], float dv[3]);
void render_clear(render_state& r);
void render_use_context_curves(pars_gpu_context& ctx, render_state& r);
// Prims of curve spans inside caller-owned buffers: each span is (start vertex
// of its batch in `vertices`, first index in `indices`, index count).
void render_use_spans(pars_gpu_context& ctx, render_state& r, const float4* vertices, const float4* colors, const int* indices,
                      const std::vector<std::array<long long, 3>>& spans);
// Camera and image size (ray_tracer.cpp:213-229); clears the accumulation.
void render_set_view(render_state& r, const float position[3], const float forward[3], const float up[3], int width, int height);
void render_build(pars_gpu_context& ctx, render_state& r);
void render_frames(pars_gpu_context& ctx, render_state& r, int iterations);
void render_encode(pars_gpu_context& ctx, render_state& r, uint8_t* host_rgba);

// Runs body under the context's lock and turns exceptions into a status (the
// wrapper of every C entry point on a context).
int32_t run_guarded(pars_gpu_context* ctx, const std::function<void()>& body);
}
