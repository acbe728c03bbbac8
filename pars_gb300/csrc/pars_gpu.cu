// C ABI of libpars_gpu (include/pars_gpu.h): context, fields, domains, the
// tracing round loop, curve stages, flow map / FTLE, instrumentation.
//
// The round loop follows pars::pipeline::execute (pars/source/pipeline.cpp:
// 160-208) with load balancing off: per round and per block, round info
// (particle_tracer.cpp:210-234), trace (:253-337), prune (:402-409), and the
// out-of-bounds exchange (:376-393) — here a device exit queue sorted by
// destination block, so the next round's particles never leave the GPU.
#include <algorithm>
#include <map>
#include <mutex>
#include <utility>
#include <cstring>
#include <limits>
#include <new>

#include "context.hpp"

using pars::device_buffer;

namespace
{
// Every grow-only scratch buffer of a context (not its fields or domains).
template <typename context_type, typename visit_type>
void for_each_scratch(context_type& c, visit_type&& visit)
{
  for (auto* b : {&c.particles_in, &c.particles_next, &c.slots, &c.kept, &c.written, &c.offsets, &c.block_of,
                  &c.block_of_next, &c.exits, &c.exit_keys, &c.exit_keys_sorted, &c.exit_order,
                  &c.exit_order_sorted, &c.counters, &c.block_max, &c.cub_temp, &c.scan_input, &c.tile_counts,
                  &c.tile_offsets, &c.staging, &c.ftle, &c.curves.vertices, &c.curves.colors,
                  &c.curves.indices, &c.boundary_positions, &c.boundary_offsets, &c.batch_jobs,
                  &c.batch_counters, &c.single_block, &c.slot_layouts, &c.curve_bounds, &c.color_specs})
    visit(*b);
}
}

long long pars_gpu_context::held_bytes() const
{
  long long total = 0;
  for (auto& f : fields) total += (long long)f.second->data.bytes();
  for (auto& d : domains) total += (long long)d.second->device_blocks.bytes();
  for_each_scratch(*this, [&](const pars::device_buffer& b) { total += (long long)b.bytes(); });
  return total + (long long)buffer_cache_bytes;
}

namespace pars
{
device_buffer acquire_buffer(pars_gpu_context& ctx, std::size_t bytes)
{
  auto it = ctx.buffer_cache.lower_bound(bytes);
  if (it != ctx.buffer_cache.end() && it->first <= 2 * bytes)
  {
    device_buffer b = std::move(it->second);
    ctx.buffer_cache_bytes -= it->first;
    ctx.buffer_cache.erase(it);
    return b;
  }
  device_buffer b;
  try { b.reserve(bytes); }
  catch (const error&)
  {
    // Out of memory: give the cache back to the device and try once more.
    PARS_CUDA(cudaStreamSynchronize(ctx.stream));
    ctx.buffer_cache.clear();
    ctx.buffer_cache_bytes = 0;
    b.reserve(bytes);
  }
  return b;
}

void recycle_buffer(pars_gpu_context& ctx, device_buffer&& buffer)
{
  const std::size_t bytes = buffer.bytes();
  if (bytes == 0) return;
  if (ctx.buffer_cache_bytes + bytes > pars_gpu_context::buffer_cache_limit)
  {
    // Work still queued may read the buffer: free it only after the stream drains.
    PARS_CUDA(cudaStreamSynchronize(ctx.stream));
    buffer.release();
    return;
  }
  ctx.buffer_cache_bytes += bytes;
  ctx.buffer_cache.emplace(bytes, std::move(buffer));
}

void release_scratch(pars_gpu_context& ctx)
{
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  for_each_scratch(ctx, [](device_buffer& b) { b.release(); });
  ctx.buffer_cache.clear();
  ctx.buffer_cache_bytes = 0;
  ctx.curves.vertex_total = 0;
  ctx.curves.index_total = 0;
  ctx.curves.indexed = ctx.curves.colored = false;
  ctx.curves.batches.clear();
  ++ctx.curves.generation;
  ctx.ftle_count = 0;
}

launch_scope::launch_scope(pars_gpu_context& ctx, const char* name) : ctx_(ctx), name_(name)
{
  ++ctx_.launches;
  if (!ctx_.profile) return;
  if (ctx_.event_pool.empty())
  {
    cudaEvent_t e;
    PARS_CUDA(cudaEventCreate(&e));
    ctx_.event_pool.push_back(e);
  }
  start_ = ctx_.event_pool.back();
  ctx_.event_pool.pop_back();
  PARS_CUDA(cudaEventRecord(start_, ctx_.stream));
}

launch_scope::~launch_scope() noexcept(false)
{
  const cudaError_t launch_error = cudaGetLastError();
  if (start_)
  {
    cudaEvent_t stop;
    if (ctx_.event_pool.empty()) cudaEventCreate(&stop);
    else { stop = ctx_.event_pool.back(); ctx_.event_pool.pop_back(); }
    cudaEventRecord(stop, ctx_.stream);
    ctx_.pending.push_back(timed_launch{name_, start_, stop});
  }
  if (launch_error != cudaSuccess && std::uncaught_exceptions() == 0)
    throw error(PARS_ERR_CUDA, std::string("launch of ") + name_ + ": " + cudaGetErrorString(launch_error));
}

namespace
{
void flush_profile(pars_gpu_context& ctx)
{
  if (ctx.pending.empty()) return;
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  for (auto& p : ctx.pending)
  {
    float ms = 0.0f;
    PARS_CUDA(cudaEventElapsedTime(&ms, p.start, p.stop));
    auto& entry = ctx.profile_totals[p.name];
    entry.milliseconds += ms;
    entry.launches += 1;
    ctx.event_pool.push_back(p.start);
    ctx.event_pool.push_back(p.stop);
  }
  ctx.pending.clear();
}
}

void take_profile(pars_gpu_context& ctx, std::map<std::string, profile_entry>& into)
{
  flush_profile(ctx);
  for (auto& t : ctx.profile_totals)
  {
    into[t.first].milliseconds += t.second.milliseconds;
    into[t.first].launches += t.second.launches;
  }
  ctx.profile_totals.clear();
}

namespace
{
template <typename body_type>
int32_t guarded(pars_gpu_context* ctx, body_type&& body)
{
  if (!ctx) return PARS_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(ctx->mutex);
  try
  {
    PARS_CUDA(cudaSetDevice(ctx->device));
    if (ctx->stream == ctx->own_stream)
    {
      // The context's own stream does not synchronise with the legacy default
      // stream, where a caller's device inputs are usually produced: the
      // call's work starts after the work already submitted there.
      if (!ctx->legacy_event) PARS_CUDA(cudaEventCreateWithFlags(&ctx->legacy_event, cudaEventDisableTiming));
      PARS_CUDA(cudaEventRecord(ctx->legacy_event, cudaStreamLegacy));
      PARS_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->legacy_event, 0));
    }
    body();
    if (ctx->pending.size() > 4096) flush_profile(*ctx);
    ctx->last_error.clear();
    return PARS_OK;
  }
  catch (const error& e) { ctx->last_error = e.what(); return e.status; }
  catch (const std::bad_alloc&) { ctx->last_error = "host allocation failed"; return PARS_ERR_OUT_OF_MEMORY; }
  catch (const std::exception& e) { ctx->last_error = e.what(); return PARS_ERR_STATE; }
}

}

int32_t run_guarded(pars_gpu_context* ctx, const std::function<void()>& body)
{
  return guarded(ctx, body);
}

namespace
{
field_entry& find_field(pars_gpu_context& ctx, int32_t handle)
{
  auto it = ctx.fields.find(handle);
  if (it == ctx.fields.end()) throw error(PARS_ERR_NOT_FOUND, "no field with handle " + std::to_string(handle));
  return *it->second;
}

void check_field_args(const int32_t shape[3], const float spacing[3])
{
  PARS_REQUIRE(shape && spacing, "shape and spacing are required");
  for (int i = 0; i < 3; ++i)
  {
    PARS_REQUIRE(shape[i] >= 2, "every field extent must be >= 2");
    PARS_REQUIRE(spacing[i] > 0.0f, "spacing must be positive");
  }
  PARS_REQUIRE((long long)shape[0] * shape[1] * shape[2] < (1LL << 40), "field too large");
}

int32_t add_field(pars_gpu_context& ctx, std::unique_ptr<field_entry> entry)
{
  const int32_t handle = ctx.next_handle++;
  ctx.fields[handle] = std::move(entry);
  return handle;
}

std::unique_ptr<field_entry> make_field(const int32_t shape[3], const float offset[3], const float size[3], const float spacing[3])
{
  auto entry = std::make_unique<field_entry>();
  for (int i = 0; i < 3; ++i)
  {
    entry->shape[i] = shape[i];
    entry->offset[i] = offset ? offset[i] : 0.0f;
    entry->spacing[i] = spacing[i];
    entry->size[i] = size ? size[i] : float(shape[i]) * spacing[i];
  }
  return entry;
}

// FP32 quotient p / q and product with h, each rounded once (kept out of
// constant folding at another precision).
float weight_times(int p, int q, float h)
{
  const volatile float num = float(p), den = float(q);
  const volatile float b = num / den;
  const volatile float c = b * h;
  return c;
}

step_rule make_rule(int integrator, int stage_mode, float h)
{
  PARS_REQUIRE(stage_mode == PARS_STAGES_FROZEN || stage_mode == PARS_STAGES_RESAMPLED, "unknown stage mode");
  PARS_REQUIRE(integrator >= PARS_EULER && integrator <= PARS_ADAMS_BASHFORTH_MOULTON_2, "unknown integrator");
  step_rule r {};
  r.frozen = stage_mode == PARS_STAGES_FROZEN ? 1 : 0;
  r.rk4 = integrator == PARS_RUNGE_KUTTA_4 ? 1 : 0;
  r.h = h;
  r.method = frozen_weighted_sum;
  // re-sampled stages ("true form") of each integrator
  r.scheme = scheme_classic;
  switch (integrator)
  {
  case PARS_MODIFIED_MIDPOINT:            r.scheme = scheme_tableau; r.tableau = tableau_midpoint; break;
  case PARS_RUNGE_KUTTA_CASH_KARP_54:     r.scheme = scheme_tableau; r.tableau = tableau_cash_karp; break;
  case PARS_RUNGE_KUTTA_DORMAND_PRINCE_5: r.scheme = scheme_tableau; r.tableau = tableau_dormand_prince; break;
  case PARS_RUNGE_KUTTA_FEHLBERG_78:      r.scheme = scheme_tableau; r.tableau = tableau_fehlberg; break;
  case PARS_ADAMS_BASHFORTH_2:            r.scheme = scheme_adams_bashforth; break;
  case PARS_ADAMS_BASHFORTH_MOULTON_2:    r.scheme = scheme_adams_moulton; break;
  default: break;
  }
  // Frozen coefficients (the odeint 1.69 schemes of integrators.hpp:16-23 with
  // every stage seeing the step-start velocity): b_i * h, b_i = float(p) /
  // float(q) in FP32, as the generic RK scale-sum forms them.
  auto weights = [&](std::initializer_list<std::pair<int, int>> b) {
    r.count = 0;
    for (const auto& q : b) r.c[r.count++] = q.first == 0 ? 0.0f * h : weight_times(q.first, q.second, h);
  };
  switch (integrator)
  {
  case PARS_EULER: r.count = 1; r.c[0] = h; break;
  case PARS_MODIFIED_MIDPOINT:
  {
    const volatile float H = h / 2.0f;
    r.method = frozen_midpoint;
    r.c[0] = H;
    r.c[1] = 2.0f * H;
    r.c[2] = 0.5f * H;
    break;
  }
  case PARS_RUNGE_KUTTA_CASH_KARP_54: weights({{37, 378}, {0, 1}, {250, 621}, {125, 594}, {0, 1}, {512, 1771}}); break;
  case PARS_RUNGE_KUTTA_DORMAND_PRINCE_5: weights({{35, 384}, {0, 1}, {500, 1113}, {125, 192}, {-2187, 6784}, {11, 84}}); break;
  case PARS_RUNGE_KUTTA_FEHLBERG_78:
    weights({{41, 840}, {0, 1}, {0, 1}, {0, 1}, {0, 1}, {34, 105}, {9, 35}, {9, 35}, {9, 280}, {9, 280}, {41, 840}, {0, 1}, {0, 1}});
    break;
  case PARS_ADAMS_BASHFORTH_2:
    weights({{1, 6}, {1, 3}, {1, 3}, {1, 6}});          // the first step is RK4
    r.method = frozen_multistep;
    r.c[4] = weight_times(3, 2, h);
    r.c[5] = weight_times(-1, 2, h);
    break;
  case PARS_ADAMS_BASHFORTH_MOULTON_2: weights({{1, 2}, {1, 2}}); break;
  default: weights({{1, 6}, {1, 3}, {1, 3}, {1, 6}}); break;    // RK4
  }
  return r;
}

// ---- partitioner restated (partitioner.cpp:8-53, prime_factorize.hpp:11-32) ----
pars_partition_info partition_of(int ranks, int rank, const int32_t domain[3])
{
  std::vector<int> factors;
  int value = ranks, d = 2;
  while (d * d <= value)
  {
    if (value % d == 0) { factors.push_back(d); value /= d; }
    else ++d;
  }
  if (value > 1) factors.push_back(value);
  pars_partition_info info {};
  int current[3] = {domain[0], domain[1], domain[2]};
  for (int i = 0; i < 3; ++i) info.grid_size[i] = 1;
  while (!factors.empty())
  {
    int dim = 0;
    for (int i = 0; i < 3; ++i) if (current[i] > current[dim]) dim = i;
    current[dim] /= factors.back();
    info.grid_size[dim] *= factors.back();
    factors.pop_back();
  }
  long long r = rank;
  for (int i = 2; i >= 0; --i) { info.multi_rank[i] = int(r % info.grid_size[i]); r /= info.grid_size[i]; }
  for (int i = 0; i < 3; ++i)
  {
    info.block_size[i] = domain[i] / info.grid_size[i];
    info.offset[i] = info.block_size[i] * info.multi_rank[i];
    info.ghosted_block_size[i] = info.block_size[i] + (info.multi_rank[i] + 1 < info.grid_size[i] ? 1 : 0);
  }
  for (int face = 0; face < 6; ++face)
  {
    int n[3] = {info.multi_rank[0], info.multi_rank[1], info.multi_rank[2]};
    n[face / 2] += (face % 2 == 0) ? -1 : 1;
    const bool exists = n[face / 2] >= 0 && n[face / 2] < info.grid_size[face / 2];
    info.neighbor_rank[face] = exists ? int(((long long)n[0] * info.grid_size[1] + n[1]) * info.grid_size[2] + n[2]) : -1;
  }
  return info;
}

void grow_curves(pars_gpu_context& ctx, long long needed_vertices)
{
  auto& c = ctx.curves;
  const std::size_t bytes = sizeof(float4) * (std::size_t)needed_vertices;
  if (bytes <= c.vertices.bytes()) return;
  device_buffer bigger;
  bigger.reserve(std::max<std::size_t>(bytes, c.vertices.bytes() + c.vertices.bytes() / 2));
  if (c.vertex_total > 0)
    PARS_CUDA(cudaMemcpyAsync(bigger.get(), c.vertices.get(), sizeof(float4) * c.vertex_total, cudaMemcpyDeviceToDevice, ctx.stream));
  c.vertices = std::move(bigger);
}

// The round loop over device-resident particles grouped by block.
// particles/block_of live in ctx.particles_in / ctx.block_of; block_count and
// block_max give each block's particle count and maximum remaining_iterations.
// What one tracing round needs from the previous one: the particles of the
// round (in ctx.particles_in, grouped by block in block order, with
// ctx.block_of when there are several blocks), each block's particle count
// and largest remaining_iterations.
struct round_plan
{
  long long              count = 0;
  std::vector<long long> block_count;
  std::vector<int>       block_max;
};

// The tracing counters: steps (accumulated over rounds), the exit-queue size
// (32-bit) and the tracing kernel's pool counter.
struct round_counters
{
  unsigned long long* steps;
  unsigned int*       exits;
  unsigned long long* pool;
};

round_counters tracing_counters(pars_gpu_context& ctx)
{
  ctx.counters.reserve(sizeof(unsigned long long) * 3);
  auto* base = ctx.counters.as<unsigned long long>();
  return {base, reinterpret_cast<unsigned int*>(base + 1), base + 2};
}

void clear_curves(pars_gpu_context& ctx)
{
  auto& curves = ctx.curves;
  curves.batches.clear();
  curves.vertex_total = 0;
  curves.index_total = 0;
  curves.indexed = curves.colored = false;
  ++curves.generation;
}

// One round of the reference's loop (particle_tracer.cpp:210-393) for every
// block at once: compute_round_info's batch split per block, the slots
// (allocate / initialize), one tracing launch, prune into batches tagged
// `round` appended to ctx.curves, and the exchange: the exit queue, stably
// ordered by (destination block, source order), becomes the next round's
// particles in ctx.particles_in, and `plan` describes them.
void trace_one_round(pars_gpu_context& ctx, const std::vector<trace_block>& blocks, const trace_block* device_blocks,
                     round_plan& plan, const step_rule& rule, bool route_exits, int round, const round_counters& counters,
                     const step_rule* device_block_rules)
{
  auto& curves = ctx.curves;
  const int nblocks = int(blocks.size());
  int key_bits = 40;
  while ((1 << (key_bits - 40)) < nblocks) ++key_bits;
  const long long count = plan.count;
  auto& block_count = plan.block_count;
  auto& block_max = plan.block_max;

  // The round's particles are grouped by block in block order (seeds per
  // rank; exits sorted by destination block), so each block's slots follow
  // the previous block's.
  std::vector<slot_layout> layout(nblocks);
  long long total_slots = 0, first_particle = 0;
  for (int b = 0; b < nblocks; ++b)
  {
    const long long stride = std::max(1, block_max[b]);
    layout[b].origin = total_slots - first_particle * stride;
    layout[b].stride = stride;
    total_slots += block_count[b] * stride;
    first_particle += block_count[b];
  }
  PARS_REQUIRE(first_particle == count, "block particle counts do not add up to the particle count");
  ctx.slots.reserve(sizeof(float4) * (std::size_t)total_slots);
  ctx.slot_layouts.reserve(sizeof(slot_layout) * nblocks);
  PARS_CUDA(cudaMemcpyAsync(ctx.slot_layouts.get(), layout.data(), sizeof(slot_layout) * nblocks, cudaMemcpyHostToDevice, ctx.stream));
  ctx.written.reserve(sizeof(int) * count);
  ctx.kept.reserve(sizeof(int) * count);
  ctx.offsets.reserve(sizeof(long long) * (count + 1));
  if (route_exits)
  {
    ctx.exits.reserve(sizeof(pars_particle) * count);
    ctx.exit_keys.reserve(sizeof(unsigned long long) * count);
  }
  PARS_CUDA(cudaMemsetAsync(counters.exits, 0, sizeof(unsigned int), ctx.stream));
  PARS_CUDA(cudaMemsetAsync(counters.pool, 0, sizeof(unsigned long long), ctx.stream));

  trace_launch a {};
  a.blocks = device_blocks;
  a.particles = ctx.particles_in.as<const pars_particle>();
  a.block_of = nblocks > 1 ? ctx.block_of.as<const int>() : nullptr;
  a.count = count;
  a.block_slots = ctx.slot_layouts.as<const slot_layout>();
  a.slots = ctx.slots.as<float4>();
  a.written = ctx.written.as<int>();
  a.kept = ctx.kept.as<int>();
  a.rule = rule;
  a.block_rules = device_block_rules;
  a.route_exits = route_exits ? 1 : 0;
  a.exit_particles = route_exits ? ctx.exits.as<pars_particle>() : nullptr;
  a.exit_keys = route_exits ? ctx.exit_keys.as<unsigned long long>() : nullptr;
  a.exit_count = counters.exits;
  a.steps = counters.steps;
  a.next = counters.pool;
  launch_trace(ctx, a);

  // prune: packed offsets of every particle's kept vertices.
  exclusive_sum(ctx, ctx.kept.as<int>(), ctx.offsets.as<long long>(), count);

  // Batch boundaries per block (compute_round_info), as particle indices.
  struct pending_batch { long long first, last; int rank; };
  std::vector<pending_batch> pending;
  long long first = 0;
  for (int b = 0; b < nblocks; ++b)
  {
    const long long n = block_count[b];
    if (n == 0) continue;
    const long long max_vertices = std::numeric_limits<int32_t>::max() / 16;
    const long long ppc = max_vertices / std::max(1, block_max[b]);
    PARS_REQUIRE(ppc > 0, "remaining_iterations exceeds the batch vertex limit");
    const long long curve_count = 1 + n / ppc;
    for (long long k = 0; k < curve_count; ++k)
      pending.push_back({first + std::min(n, k * ppc), first + std::min(n, (k + 1) * ppc), b});
    first += n;
  }
  std::vector<long long> positions;
  positions.reserve(pending.size() * 2 + 1);
  for (auto& p : pending) { positions.push_back(p.first); positions.push_back(p.last); }
  positions.push_back(count);
  std::vector<long long> boundary(positions.size());
  ctx.boundary_positions.reserve(sizeof(long long) * positions.size());
  ctx.boundary_offsets.reserve(sizeof(long long) * positions.size());
  PARS_CUDA(cudaMemcpyAsync(ctx.boundary_positions.get(), positions.data(), sizeof(long long) * positions.size(), cudaMemcpyHostToDevice, ctx.stream));
  launch_gather_offsets(ctx, ctx.offsets.as<const long long>(), ctx.boundary_positions.as<const long long>(), (long long)positions.size(),
                        ctx.boundary_offsets.as<long long>());
  unsigned int exit_total = 0;
  PARS_CUDA(cudaMemcpyAsync(boundary.data(), ctx.boundary_offsets.get(), sizeof(long long) * boundary.size(), cudaMemcpyDeviceToHost, ctx.stream));
  PARS_CUDA(cudaMemcpyAsync(&exit_total, counters.exits, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  const long long round_vertices = boundary.back();

  grow_curves(ctx, curves.vertex_total + round_vertices);
  launch_compact_vertices(ctx, ctx.slots.as<const float4>(), ctx.slot_layouts.as<const slot_layout>(), a.block_of,
                          ctx.written.as<const int>(), ctx.offsets.as<const long long>(), count,
                          curves.vertices.as<float4>() + curves.vertex_total);
  for (std::size_t k = 0; k < pending.size(); ++k)
  {
    curves_batch batch;
    batch.vertex_offset = curves.vertex_total + boundary[2 * k];
    batch.vertex_count = boundary[2 * k + 1] - boundary[2 * k];
    batch.rank = pending[k].rank;
    batch.round = round;
    curves.batches.push_back(batch);
  }
  curves.vertex_total += round_vertices;

  // Exchange: the exit queue, stably ordered by (destination block, source
  // order), becomes the next round's particle list.
  const long long next = route_exits ? (long long)exit_total : 0;
  std::fill(block_count.begin(), block_count.end(), 0);
  std::fill(block_max.begin(), block_max.end(), 0);
  if (next > 0)
  {
    ctx.exit_keys_sorted.reserve(sizeof(unsigned long long) * next);
    ctx.exit_order.reserve(sizeof(unsigned int) * next);
    ctx.exit_order_sorted.reserve(sizeof(unsigned int) * next);
    ctx.particles_next.reserve(sizeof(pars_particle) * next);
    ctx.block_of_next.reserve(sizeof(int) * next);
    ctx.block_max.reserve(sizeof(int) * 2 * nblocks);
    PARS_CUDA(cudaMemsetAsync(ctx.block_max.get(), 0, sizeof(int) * 2 * nblocks, ctx.stream));
    launch_iota(ctx, ctx.exit_order.as<unsigned int>(), next);
    sort_pairs(ctx, ctx.exit_keys.as<const unsigned long long>(), ctx.exit_keys_sorted.as<unsigned long long>(),
               ctx.exit_order.as<const unsigned int>(), ctx.exit_order_sorted.as<unsigned int>(), next, key_bits);
    launch_gather_exits(ctx, ctx.exits.as<const pars_particle>(), ctx.exit_order_sorted.as<const unsigned int>(),
                        ctx.exit_keys_sorted.as<const unsigned long long>(), next, ctx.particles_next.as<pars_particle>(),
                        ctx.block_of_next.as<int>(), ctx.block_max.as<int>(), ctx.block_max.as<int>() + nblocks);
    std::vector<int> stats(2 * nblocks);
    PARS_CUDA(cudaMemcpyAsync(stats.data(), ctx.block_max.get(), sizeof(int) * 2 * nblocks, cudaMemcpyDeviceToHost, ctx.stream));
    PARS_CUDA(cudaStreamSynchronize(ctx.stream));
    for (int b = 0; b < nblocks; ++b) { block_max[b] = stats[b]; block_count[b] = stats[nblocks + b]; }
    std::swap(ctx.particles_in, ctx.particles_next);
    std::swap(ctx.block_of, ctx.block_of_next);
  }
  plan.count = next;
}

// The whole round loop (particle_tracer::trace, particle_tracer.cpp:39-56)
// over device-resident particles grouped by block: rounds until no particle
// is left, the curves of every round in ctx.curves.
void run_rounds(pars_gpu_context& ctx, const std::vector<trace_block>& blocks, const trace_block* device_blocks,
                long long count, std::vector<long long> block_count, std::vector<int> block_max,
                const step_rule& rule, bool route_exits, pars_gpu_trace_summary* summary,
                const step_rule* device_block_rules = nullptr)
{
  clear_curves(ctx);
  ++ctx.trace_serial;
  const round_counters counters = tracing_counters(ctx);
  PARS_CUDA(cudaMemsetAsync(counters.steps, 0, sizeof(unsigned long long), ctx.stream));
  round_plan plan;
  plan.count = count;
  plan.block_count = std::move(block_count);
  plan.block_max = std::move(block_max);
  int round = 0;
  while (plan.count > 0)
  {
    trace_one_round(ctx, blocks, device_blocks, plan, rule, route_exits, round, counters, device_block_rules);
    ++round;
  }

  unsigned long long steps = 0;
  PARS_CUDA(cudaMemcpyAsync(&steps, counters.steps, sizeof(steps), cudaMemcpyDeviceToHost, ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  if (summary)
  {
    summary->batches = (long long)ctx.curves.batches.size();
    summary->vertices = ctx.curves.vertex_total;
    summary->steps = (long long)steps;
    summary->rounds = round;
    summary->padding = 0;
  }
}

// ---- Asynchronous rounds -------------------------------------------------------------
// Every round of a partitioned domain in one persistent launch (async_launch,
// trace_kernels.cu): no round waits for the slowest particle of the previous
// one.  The rounds' order is rebuilt afterwards exactly as the round loop
// forms it (a block's particles of round r + 1 ordered by the sender's
// position in round r), then compute_round_info's batches per (round, block),
// prune, and the packed vertices.  Returns false, with nothing kept, when the
// segment table, the vertex chunks or the round histogram overflowed, a wait
// ran out, or the buffers would take more than a quarter of the free device
// memory: the caller then traces round by round.
bool run_rounds_async(pars_gpu_context& ctx, const std::vector<trace_block>& blocks, const trace_block* device_blocks,
                      long long count, const std::vector<long long>& block_count, const std::vector<int>& block_max,
                      const step_rule& rule, pars_gpu_trace_summary* summary)
{
  const int nblocks = int(blocks.size());
  if (count <= 0) return false;
  async_launch a {};
  a.blocks = device_blocks;
  a.rule = rule;
  long long vertex_bound = 0;   // sum of remaining_iterations over the seeds, at most
  for (int b = 0; b < nblocks; ++b) vertex_bound += block_count[b] * std::max(1, block_max[b]);
  const long long warps = launch_async_trace(ctx, a, true);
  const long long capacity = std::min<long long>(std::max<long long>(16 * count, 1 << 16), (1LL << 31) - 1);
  // every segment's vertices in whole chunks, plus the slabs warps leave unused
  const long long chunk_capacity = (vertex_bound + capacity) / async_chunk + capacity + async_slab * (warps + 1);
  if (chunk_capacity > (1LL << 31) - 1) return false;
  auto align = [](std::size_t b) { return (b + 255) & ~std::size_t(255); };
  const std::size_t seg_bytes = align(sizeof(pars_particle) * capacity) + 6 * align(sizeof(int) * capacity) +
                                align(sizeof(long long) * capacity);
  const std::size_t chunk_bytes = align(sizeof(float4) * async_chunk * chunk_capacity) + align(sizeof(int) * chunk_capacity);
  if (seg_bytes > ctx.async_segments.bytes() || chunk_bytes > ctx.async_chunks.bytes())
  {
    std::size_t free_bytes = 0, total_bytes = 0;
    PARS_CUDA(cudaMemGetInfo(&free_bytes, &total_bytes));
    const std::size_t have = ctx.async_segments.bytes() + ctx.async_chunks.bytes();
    if (seg_bytes + chunk_bytes > have + free_bytes / 4) return false;
  }

  ctx.async_segments.reserve(seg_bytes);
  ctx.async_chunks.reserve(chunk_bytes);
  ctx.async_counters.reserve(sizeof(unsigned long long) * async_counters + 256);
  char* sp = ctx.async_segments.as<char>();
  auto carve = [&](std::size_t bytes) { char* p = sp; sp += align(bytes); return p; };
  a.seg_particle = reinterpret_cast<pars_particle*>(carve(sizeof(pars_particle) * capacity));
  a.seg_block = reinterpret_cast<int*>(carve(sizeof(int) * capacity));
  a.seg_round = reinterpret_cast<int*>(carve(sizeof(int) * capacity));
  a.seg_ready = reinterpret_cast<int*>(carve(sizeof(int) * capacity));
  a.seg_written = reinterpret_cast<int*>(carve(sizeof(int) * capacity));
  a.seg_kept = reinterpret_cast<int*>(carve(sizeof(int) * capacity));
  a.seg_first_chunk = reinterpret_cast<int*>(carve(sizeof(int) * capacity));
  a.seg_parent = reinterpret_cast<long long*>(carve(sizeof(long long) * capacity));
  a.capacity = capacity;
  a.chunks = ctx.async_chunks.as<float4>();
  a.chunk_next = reinterpret_cast<int*>(ctx.async_chunks.as<char>() + align(sizeof(float4) * async_chunk * chunk_capacity));
  a.chunk_capacity = chunk_capacity;
  a.counters = ctx.async_counters.as<unsigned long long>();
  a.error = reinterpret_cast<int*>(a.counters + async_counters);

  // the seeds as round-0 segments; nothing else published
  PARS_CUDA(cudaMemsetAsync(a.seg_ready, 0, sizeof(int) * capacity, ctx.stream));
  PARS_CUDA(cudaMemsetAsync(ctx.async_counters.get(), 0, sizeof(unsigned long long) * async_counters + sizeof(int), ctx.stream));
  const unsigned long long allocated0 = (unsigned long long)count;
  PARS_CUDA(cudaMemcpyAsync(a.counters + async_alloc, &allocated0, sizeof(allocated0), cudaMemcpyHostToDevice, ctx.stream));
  launch_async_seed(ctx, a, ctx.particles_in.as<const pars_particle>(), nblocks > 1 ? ctx.block_of.as<const int>() : nullptr, count);
  launch_async_trace(ctx, a);
  unsigned long long counters[async_counters + 1] = {};
  PARS_CUDA(cudaMemcpyAsync(counters, a.counters, sizeof(unsigned long long) * async_counters + sizeof(int), cudaMemcpyDeviceToHost,
                            ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  int error = 0;
  std::memcpy(&error, counters + async_counters, sizeof(int));
  if (error != async_ok) return false;
  const long long n = (long long)counters[async_alloc];

  // rounds: histogram, then each round's segments sorted by (block, the
  // sender's position in the previous round), positions concatenated
  constexpr int rounds_cap = 65536;
  ctx.async_cursor.reserve(sizeof(int) * (2 * rounds_cap + 1));
  int* histogram = ctx.async_cursor.as<int>();
  int* max_round = histogram + rounds_cap;
  int* cursor = max_round + 1;
  PARS_CUDA(cudaMemsetAsync(histogram, 0, sizeof(int) * (2 * rounds_cap + 1), ctx.stream));
  launch_round_histogram(ctx, a.seg_round, n, rounds_cap, histogram, max_round);
  int rounds = 0;
  PARS_CUDA(cudaMemcpyAsync(&rounds, max_round, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  ++rounds;
  if (rounds > rounds_cap) return false;
  std::vector<int> per_round(rounds);
  PARS_CUDA(cudaMemcpyAsync(per_round.data(), histogram, sizeof(int) * rounds, cudaMemcpyDeviceToHost, ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  std::vector<long long> first(rounds + 1, 0);
  long long widest = 0;
  for (int r = 0; r < rounds; ++r) { first[r + 1] = first[r] + per_round[r]; widest = std::max<long long>(widest, per_round[r]); }

  ctx.async_order.reserve(sizeof(unsigned int) * 2 * n + sizeof(long long) * (rounds + 1) + 256);
  unsigned int* grouped = ctx.async_order.as<unsigned int>();
  unsigned int* order = grouped + n;
  long long* device_first = reinterpret_cast<long long*>(ctx.async_order.as<char>() + align(sizeof(unsigned int) * 2 * n));
  ctx.async_positions.reserve(sizeof(long long) * (n + 1));
  long long* position = ctx.async_positions.as<long long>();
  PARS_CUDA(cudaMemcpyAsync(device_first, first.data(), sizeof(long long) * (rounds + 1), cudaMemcpyHostToDevice, ctx.stream));
  launch_round_scatter(ctx, a.seg_round, n, device_first, cursor, grouped);
  ctx.exit_keys.reserve(sizeof(unsigned long long) * widest);
  ctx.exit_keys_sorted.reserve(sizeof(unsigned long long) * widest);
  int key_bits = 40;
  while ((1 << (key_bits - 40)) < nblocks) ++key_bits;
  for (int r = 0; r < rounds; ++r)
  {
    const long long m = per_round[r];
    if (m == 0) continue;
    launch_round_keys(ctx, grouped + first[r], m, a.seg_block, a.seg_parent, position, ctx.exit_keys.as<unsigned long long>());
    sort_pairs(ctx, ctx.exit_keys.as<const unsigned long long>(), ctx.exit_keys_sorted.as<unsigned long long>(), grouped + first[r],
               order + first[r], m, key_bits);
    launch_round_positions(ctx, order + first[r], m, first[r], position);
  }

  // per (round, block): segments and largest remaining_iterations; kept
  // vertices in that order, and their offsets in the packed buffer
  ctx.block_max.reserve(sizeof(int) * 2 * (std::size_t)rounds * nblocks);
  int* stats = ctx.block_max.as<int>();
  PARS_CUDA(cudaMemsetAsync(stats, 0, sizeof(int) * 2 * (std::size_t)rounds * nblocks, ctx.stream));
  ctx.kept.reserve(sizeof(int) * n);
  ctx.offsets.reserve(sizeof(long long) * (n + 1));
  launch_round_stats(ctx, order, n, a.seg_round, a.seg_block, a.seg_particle, a.seg_kept, nblocks, stats, ctx.kept.as<int>());
  exclusive_sum(ctx, ctx.kept.as<int>(), ctx.offsets.as<long long>(), n);
  std::vector<int> host_stats(2 * (std::size_t)rounds * nblocks);
  PARS_CUDA(cudaMemcpyAsync(host_stats.data(), stats, sizeof(int) * host_stats.size(), cudaMemcpyDeviceToHost, ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));

  // compute_round_info's batches of every (round, block), as positions
  struct pending_batch { long long first, last; int rank, round; };
  std::vector<pending_batch> pending;
  long long g = 0;
  for (int r = 0; r < rounds; ++r)
    for (int b = 0; b < nblocks; ++b)
    {
      const long long m = host_stats[2 * ((std::size_t)r * nblocks + b)];
      const int maximum = host_stats[2 * ((std::size_t)r * nblocks + b) + 1];
      if (m == 0) continue;
      const long long max_vertices = std::numeric_limits<int32_t>::max() / 16;
      const long long ppc = max_vertices / std::max(1, maximum);
      PARS_REQUIRE(ppc > 0, "remaining_iterations exceeds the batch vertex limit");
      const long long curve_count = 1 + m / ppc;
      for (long long k = 0; k < curve_count; ++k)
        pending.push_back({g + std::min(m, k * ppc), g + std::min(m, (k + 1) * ppc), b, r});
      g += m;
    }
  PARS_REQUIRE(g == n, "round statistics do not cover the segments");
  std::vector<long long> positions;
  positions.reserve(pending.size() * 2 + 1);
  for (auto& p : pending) { positions.push_back(p.first); positions.push_back(p.last); }
  positions.push_back(n);
  std::vector<long long> boundary(positions.size());
  ctx.boundary_positions.reserve(sizeof(long long) * positions.size());
  ctx.boundary_offsets.reserve(sizeof(long long) * positions.size());
  PARS_CUDA(cudaMemcpyAsync(ctx.boundary_positions.get(), positions.data(), sizeof(long long) * positions.size(), cudaMemcpyHostToDevice,
                            ctx.stream));
  launch_gather_offsets(ctx, ctx.offsets.as<const long long>(), ctx.boundary_positions.as<const long long>(), (long long)positions.size(),
                        ctx.boundary_offsets.as<long long>());
  PARS_CUDA(cudaMemcpyAsync(boundary.data(), ctx.boundary_offsets.get(), sizeof(long long) * boundary.size(), cudaMemcpyDeviceToHost,
                            ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  const long long total_vertices = boundary.back();

  clear_curves(ctx);
  ++ctx.trace_serial;
  auto& curves = ctx.curves;
  grow_curves(ctx, total_vertices);
  launch_async_assemble(ctx, a, order, ctx.offsets.as<const long long>(), n, curves.vertices.as<float4>());
  for (std::size_t k = 0; k < pending.size(); ++k)
  {
    curves_batch batch;
    batch.vertex_offset = boundary[2 * k];
    batch.vertex_count = boundary[2 * k + 1] - boundary[2 * k];
    batch.rank = pending[k].rank;
    batch.round = pending[k].round;
    curves.batches.push_back(batch);
  }
  curves.vertex_total = total_vertices;
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  if (summary)
  {
    summary->batches = (long long)curves.batches.size();
    summary->vertices = total_vertices;
    summary->steps = (long long)counters[async_steps];
    summary->rounds = rounds;
    summary->padding = 0;
  }
  return true;
}

// Single block: one trace_block with no neighbours, kept in a small device array.
const trace_block* single_block(pars_gpu_context& ctx, const field_entry& f, std::vector<trace_block>& blocks)
{
  trace_block b;
  b.field = f.view();
  for (int i = 0; i < 6; ++i) b.neighbor[i] = -1;
  blocks.assign(1, b);
  ctx.single_block.reserve(sizeof(trace_block));
  PARS_CUDA(cudaMemcpyAsync(ctx.single_block.get(), &b, sizeof(trace_block), cudaMemcpyHostToDevice, ctx.stream));
  return ctx.single_block.as<const trace_block>();
}

void trace_single(pars_gpu_context& ctx, int32_t field, long long count, int32_t integrator, int32_t stage_mode,
                  float step_size, pars_gpu_trace_summary* summary)
{
  auto& f = find_field(ctx, field);
  const step_rule rule = make_rule(integrator, stage_mode, step_size);
  std::vector<trace_block> blocks;
  const trace_block* device_blocks = single_block(ctx, f, blocks);
  std::vector<long long> block_count(1, count);
  std::vector<int> block_max(1, 0);
  if (count > 0)
  {
    ctx.block_max.reserve(sizeof(int) * 2);
    PARS_CUDA(cudaMemsetAsync(ctx.block_max.get(), 0, sizeof(int) * 2, ctx.stream));
    launch_particle_stats(ctx, ctx.particles_in.as<const pars_particle>(), nullptr, count, ctx.block_max.as<int>());
    PARS_CUDA(cudaMemcpyAsync(block_max.data(), ctx.block_max.get(), sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
    PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  }
  run_rounds(ctx, blocks, device_blocks, count, block_count, block_max, rule, false, summary);
}

int class_of_job(const batch_job_device& j)
{
  return j.rule.frozen ? batch_frozen : (j.time.nt > 1 ? batch_unsteady : batch_steady);
}

long long pools_of(long long seeds)
{
  const int pool = batch_pool_seeds();
  return (seeds + pool - 1) / pool;
}

// Chooses the launch shape of job class c from `jobs` (all of class c, clocks
// set): every shape runs a probe of the jobs twice (seed counts capped at four
// times the seeds the GPU holds resident), timed with CUDA events.
// Tuned launch shapes of the process's contexts, per device and job class: a
// context whose class is untuned takes the shape another context of the same
// device chose (the service's lanes are contexts of one device).
std::mutex tuned_mutex;
std::map<std::pair<int, int>, int> tuned_shapes;

void tune_class(pars_gpu_context& ctx, int c, std::vector<batch_job_device> jobs)
{
  const int count = int(jobs.size());
  if (count == 0) return;
  {
    std::lock_guard<std::mutex> lock(tuned_mutex);
    const auto it = tuned_shapes.find({ctx.device, c});
    if (it != tuned_shapes.end()) { ctx.batch_variant[c] = it->second; return; }
  }
  ctx.batch_jobs.reserve(sizeof(batch_job_device) * count);
  ctx.batch_counters.reserve(sizeof(unsigned long long) * (count + 1));
  auto* counters = ctx.batch_counters.as<unsigned long long>();
  auto* device_jobs = ctx.batch_jobs.as<batch_job_device>();
  if (ctx.sm_count <= 0) PARS_CUDA(cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, ctx.device));
  const long long probe = std::max(16384LL, 4LL * 2048LL * ctx.sm_count);
  long long pools = 0;
  for (int k = 0; k < count; ++k)
  {
    jobs[k].seed_count = std::min(jobs[k].seed_count, probe);
    jobs[k].first_pool = pools;
    jobs[k].steps = counters + 1 + k;
    pools += pools_of(jobs[k].seed_count);
  }
  cudaEvent_t a, b;
  PARS_CUDA(cudaEventCreate(&a));
  PARS_CUDA(cudaEventCreate(&b));
  std::vector<float> fastest(batch_variant_count(), 0.0f);
  for (int v = 0; v < batch_variant_count(); ++v)
  {
    for (int rep = 0; rep < 2; ++rep)
    {
      PARS_CUDA(cudaMemcpyAsync(device_jobs, jobs.data(), sizeof(batch_job_device) * count, cudaMemcpyHostToDevice, ctx.stream));
      PARS_CUDA(cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * (count + 1), ctx.stream));
      PARS_CUDA(cudaEventRecord(a, ctx.stream));
      launch_batch_advect(ctx, c, v, device_jobs, count, pools, counters);
      PARS_CUDA(cudaEventRecord(b, ctx.stream));
      PARS_CUDA(cudaEventSynchronize(b));
      float ms = 0.0f;
      PARS_CUDA(cudaEventElapsedTime(&ms, a, b));
      fastest[v] = rep == 0 ? ms : std::min(fastest[v], ms);
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  // The probe's particles take a few hundred steps each, so its last
  // particles' tail blurs differences of a few per cent between shapes:
  // among the shapes within 3 % of the fastest, keep the one with the most
  // resident warps per SM (on the 256^3 flow map the 96-register shape, five
  // CTAs of 128, beats the 104-register ones by 7 %, which the probes alone
  // do not resolve reliably).
  const float best_time = *std::min_element(fastest.begin(), fastest.end());
  int best_v = -1, best_warps = -1;
  for (int v = 0; v < batch_variant_count(); ++v)
  {
    if (fastest[v] > 1.03f * best_time) continue;
    const int warps = batch_resident_warps(ctx, c, v);
    if (warps > best_warps || (warps == best_warps && fastest[v] < fastest[best_v])) { best_v = v; best_warps = warps; }
  }
  ctx.batch_variant[c] = best_v;
  std::lock_guard<std::mutex> lock(tuned_mutex);
  tuned_shapes.emplace(std::make_pair(ctx.device, c), best_v);
}

// Runs batched jobs and returns each job's steps.  Re-sampled jobs on steady
// fields (one slice), re-sampled jobs on unsteady fields and frozen-scheme
// jobs run in up to three persistent launches, one per job class, so that a
// job's arithmetic, and so its result, does not depend on the other jobs of
// the batch.  variant < 0 uses the context's tuned launch shape for each
// class, tuning it first if needed (tune_class): every job of the class
// capped at four times the seeds the GPU holds resident (2048 lanes per SM),
// so that each shape runs at its own occupancy in steady state, each shape
// timed twice with CUDA events, the fastest kept.  (A cap of 16384 seeds fills
// a sixth of a GB300's lanes and picked a 104-register shape that was 7 %
// slower on the 256^3 flow map than the 96-register one.)
std::vector<unsigned long long> execute_batch(pars_gpu_context& ctx, std::vector<batch_job_device>& jobs, int variant)
{
  const int count = int(jobs.size());
  // jobs grouped by class; order[k] = caller's index of job k
  std::vector<int> order;
  order.reserve(count);
  int first[batch_classes], size[batch_classes];
  for (int c = 0; c < batch_classes; ++c)
  {
    first[c] = int(order.size());
    for (int j = 0; j < count; ++j) if (class_of_job(jobs[j]) == c) order.push_back(j);
    size[c] = int(order.size()) - first[c];
  }
  std::vector<batch_job_device> queue(count);
  for (int k = 0; k < count; ++k)
  {
    queue[k] = jobs[order[k]];
    queue[k].clock = make_slice_clock(queue[k].time, queue[k].time_begin, queue[k].rule.h);
  }
  constexpr int C = batch_classes;
  for (int c = 0; c < C; ++c)
    if (variant < 0 && size[c] > 0 && ctx.batch_variant[c] < 0)
      tune_class(ctx, c, std::vector<batch_job_device>(queue.begin() + first[c], queue.begin() + first[c] + size[c]));

  // The device queues: each job's seeds in pools of batch_pool_seeds(), numbered
  // per class; counters 0 .. C-1 hand out the pools of the classes, counters
  // C.. count each job's steps.
  ctx.batch_jobs.reserve(sizeof(batch_job_device) * count);
  ctx.batch_counters.reserve(sizeof(unsigned long long) * (count + C));
  auto* counters = ctx.batch_counters.as<unsigned long long>();
  auto* device_jobs = ctx.batch_jobs.as<batch_job_device>();
  long long pools[C] = {};
  for (int c = 0; c < C; ++c)
    for (int k = first[c]; k < first[c] + size[c]; ++k)
    {
      queue[k].first_pool = pools[c];
      queue[k].steps = counters + C + k;
      pools[c] += pools_of(queue[k].seed_count);
    }
  PARS_CUDA(cudaMemcpyAsync(device_jobs, queue.data(), sizeof(batch_job_device) * count, cudaMemcpyHostToDevice, ctx.stream));
  PARS_CUDA(cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * (count + C), ctx.stream));
  for (int c = 0; c < C; ++c)
    if (size[c] > 0)
      launch_batch_advect(ctx, c, variant >= 0 ? variant : ctx.batch_variant[c], device_jobs + first[c], size[c], pools[c], counters + c);
  std::vector<unsigned long long> steps(count + C);
  PARS_CUDA(cudaMemcpyAsync(steps.data(), counters, sizeof(unsigned long long) * (count + C), cudaMemcpyDeviceToHost, ctx.stream));
  PARS_CUDA(cudaStreamSynchronize(ctx.stream));
  std::vector<unsigned long long> result(count);
  for (int k = 0; k < count; ++k) result[order[k]] = steps[C + k];
  return result;
}

std::size_t checked_bytes(long long count, std::size_t element)
{
  PARS_REQUIRE(count >= 0, "negative count");
  return (std::size_t)count * element;
}
}

step_rule make_step_rule(int integrator, int stage_mode, float h) { return make_rule(integrator, stage_mode, h); }

void trace_rounds(pars_gpu_context& ctx, const std::vector<trace_block>& blocks, const trace_block* device_blocks, long long count,
                  std::vector<long long> block_count, std::vector<int> block_max, const step_rule& rule, bool route_exits,
                  pars_gpu_trace_summary* summary, const step_rule* device_block_rules)
{
  run_rounds(ctx, blocks, device_blocks, count, std::move(block_count), std::move(block_max), rule, route_exits, summary,
             device_block_rules);
}

std::vector<unsigned long long> run_batch(pars_gpu_context& ctx, std::vector<batch_job_device>& jobs, int variant)
{
  return execute_batch(ctx, jobs, variant);
}

pars_partition_info partition(int ranks, int rank, const int32_t domain[3]) { return partition_of(ranks, rank, domain); }

// ---- continuous batched advection ------------------------------------------------
// One job table per job class.  Jobs are appended between horizon launches;
// their pools continue the class's pool numbering, so the table's pool
// counter hands them out after the earlier jobs' pools.  A launch's warps
// that find the counter past the table's last pool increment it once more
// each; the host puts it back to the number of pools before the next launch.
// Completed jobs stay in the table until every job of the class is complete,
// then the table starts again from zero.
struct batch_engine_class
{
  std::vector<batch_job_device> jobs;       // host copy of the device table
  std::vector<long long>        tickets;
  std::vector<char>             complete;
  std::vector<char>             counted;         // the job's device counters are zeroed
  int                           uploaded = 0;    // jobs copied to the device table
  int                           capacity = 0;    // jobs the device buffers hold
  device_buffer                 table;
  // [0] pools handed out, [1] groups resumed (u32), [2] groups parked (u32),
  // [3] stop flag (u32), [4, 4 + capacity) steps per job
  device_buffer                 counters;
  device_buffer                 groups[2], lanes[2];
  long long                     group_capacity = 0;
  int                           parity = 0;      // parked groups are in groups[parity]
  unsigned int                  parked = 0;
  long long                     total_pools = 0;
  unsigned long long            handed = 0;      // pools handed out (at most total_pools)
  int                           variant = -1;
  long long                     open = 0;
  // steps per launch chosen for a launch time (iterations = 0): the last
  // launch's kernel time per step of its horizon, measured with CUDA events
  double                        ms_per_iteration = 0.0;
  int                           last_iterations = 0;
};

struct batch_engine
{
  batch_engine_class classes[batch_classes];
  long long          next_ticket = 1;
  cudaEvent_t        launch_start = nullptr, launch_stop = nullptr;
  ~batch_engine()
  {
    if (launch_start) cudaEventDestroy(launch_start);
    if (launch_stop) cudaEventDestroy(launch_stop);
  }
  std::vector<std::pair<long long, unsigned long long>> ready;   // completions not yet returned (C ABI)
};

namespace
{
// Launch time the engine aims at when it chooses the steps per launch itself:
// about the longest a job submitted meanwhile waits before it starts.
constexpr double engine_launch_ms = 2.0;

void engine_reserve(pars_gpu_context& ctx, batch_engine_class& E, int jobs)
{
  if (jobs <= E.capacity) return;
  const int capacity = std::max(jobs, std::max(64, 2 * E.capacity));
  device_buffer table, counters;
  table.reserve(sizeof(batch_job_device) * capacity);
  counters.reserve(sizeof(unsigned long long) * (4 + std::size_t(capacity)));
  PARS_CUDA(cudaMemsetAsync(counters.get(), 0, counters.bytes(), ctx.stream));
  auto* fresh = counters.as<unsigned long long>();
  if (E.capacity > 0)
  {
    // keep the pool counter and the jobs' step counts
    PARS_CUDA(cudaMemcpyAsync(fresh, E.counters.get(), sizeof(unsigned long long) * (4 + E.capacity), cudaMemcpyDeviceToDevice,
                              ctx.stream));
  }
  E.table = std::move(table);
  E.counters = std::move(counters);
  E.capacity = capacity;
  for (std::size_t k = 0; k < E.jobs.size(); ++k) E.jobs[k].steps = fresh + 4 + k;
  E.uploaded = 0;   // the steps pointers changed: upload the whole table again
}

void engine_reset(batch_engine_class& E)
{
  E.jobs.clear();
  E.tickets.clear();
  E.complete.clear();
  E.counted.clear();
  E.uploaded = 0;
  E.parity = 0;
  E.parked = 0;
  E.total_pools = 0;
  E.handed = 0;
  E.open = 0;
}
}

long long engine_submit(pars_gpu_context& ctx, const batch_job_device& job)
{
  if (!ctx.engine) ctx.engine = std::make_shared<batch_engine>();
  batch_engine& engine = *ctx.engine;
  const int c = class_of_job(job);
  batch_engine_class& E = engine.classes[c];
  batch_job_device j = job;
  j.clock = make_slice_clock(j.time, j.time_begin, j.rule.h);
  if (ctx.batch_variant[c] < 0) tune_class(ctx, c, {j});
  if (E.open == 0) E.variant = ctx.batch_variant[c];   // fixed while the class has work
  engine_reserve(ctx, E, int(E.jobs.size()) + 1);
  j.first_pool = E.total_pools;
  j.steps = E.counters.as<unsigned long long>() + 4 + E.jobs.size();
  E.total_pools += pools_of(j.seed_count);
  E.jobs.push_back(j);
  const long long ticket = engine.next_ticket++;
  E.tickets.push_back(ticket);
  E.complete.push_back(0);
  E.counted.push_back(0);
  ++E.open;
  return ticket;
}

long long engine_open(const pars_gpu_context& ctx)
{
  if (!ctx.engine) return 0;
  long long open = 0;
  for (const auto& E : ctx.engine->classes) open += E.open;
  return open;
}

std::vector<std::pair<long long, unsigned long long>> engine_advance(pars_gpu_context& ctx, int iterations)
{
  PARS_REQUIRE(iterations >= 0, "iterations must be >= 0");
  std::vector<std::pair<long long, unsigned long long>> done;
  if (!ctx.engine) return done;
  batch_engine& engine = *ctx.engine;
  if (!engine.launch_start)
  {
    PARS_CUDA(cudaEventCreate(&engine.launch_start));
    PARS_CUDA(cudaEventCreate(&engine.launch_stop));
  }
  for (int c = 0; c < batch_classes; ++c)
  {
    batch_engine_class& E = ctx.engine->classes[c];
    if (E.open == 0) continue;
    const int n = int(E.jobs.size());
    auto* counters = E.counters.as<unsigned long long>();
    if (E.uploaded < n)
    {
      PARS_CUDA(cudaMemcpyAsync(E.table.as<batch_job_device>() + E.uploaded, E.jobs.data() + E.uploaded,
                                sizeof(batch_job_device) * (n - E.uploaded), cudaMemcpyHostToDevice, ctx.stream));
      // new jobs start from zero steps (the slots may hold the counts of
      // the jobs of an earlier table)
      for (int k = E.uploaded; k < n; ++k)
        if (E.counted[k] == 0)
        {
          PARS_CUDA(cudaMemsetAsync(counters + 4 + k, 0, sizeof(unsigned long long), ctx.stream));
          E.counted[k] = 1;
        }
      E.uploaded = n;
    }
    const long long resident = batch_horizon_warps(ctx, c, E.variant);
    if (E.group_capacity < resident)
    {
      PARS_REQUIRE(E.parked == 0, "the engine's launch shape changed while groups are parked");
      for (int b = 0; b < 2; ++b)
      {
        E.groups[b].reserve(sizeof(batch_parked_group) * resident);
        E.lanes[b].reserve(sizeof(batch_parked_lane) * 32 * resident);
      }
      E.group_capacity = resident;
    }
    const long long remaining = E.total_pools - (long long)E.handed;
    if (remaining > 0 || E.parked > 0)
    {
      const unsigned long long start[4] = {E.handed, 0, 0, 0};
      PARS_CUDA(cudaMemcpyAsync(counters, start, sizeof(start), cudaMemcpyHostToDevice, ctx.stream));
      batch_horizon_args hz;
      // iterations 0: steps per launch for a launch of engine_launch_ms, from
      // the last launch's time per step (a first launch takes 256 steps)
      int steps = iterations;
      if (steps == 0)
      {
        steps = E.ms_per_iteration > 0.0 ? int(std::min(1.0e6, std::max(16.0, engine_launch_ms / E.ms_per_iteration))) : 256;
      }
      hz.iterations = steps;
      hz.in_count = int(E.parked);
      hz.in_groups = E.groups[E.parity].as<const batch_parked_group>();
      hz.in_lanes = E.lanes[E.parity].as<const batch_parked_lane>();
      hz.in_counter = reinterpret_cast<unsigned int*>(counters + 1);
      hz.out_groups = E.groups[1 - E.parity].as<batch_parked_group>();
      hz.out_lanes = E.lanes[1 - E.parity].as<batch_parked_lane>();
      hz.out_count = reinterpret_cast<unsigned int*>(counters + 2);
      hz.stop = reinterpret_cast<unsigned int*>(counters + 3);
      PARS_CUDA(cudaEventRecord(engine.launch_start, ctx.stream));
      launch_batch_advect_horizon(ctx, c, E.variant, E.table.as<const batch_job_device>(), n, E.total_pools, counters, hz,
                                  remaining + E.parked);
      PARS_CUDA(cudaEventRecord(engine.launch_stop, ctx.stream));
      E.parity = 1 - E.parity;
      E.last_iterations = steps;
    }
    std::vector<unsigned long long> host(4 + std::size_t(E.capacity));
    PARS_CUDA(cudaMemcpyAsync(host.data(), counters, sizeof(unsigned long long) * host.size(), cudaMemcpyDeviceToHost, ctx.stream));
    PARS_CUDA(cudaStreamSynchronize(ctx.stream));
    E.handed = std::min<unsigned long long>(host[0], (unsigned long long)E.total_pools);
    E.parked = (unsigned int)(host[2] & 0xffffffffu);
    if (E.last_iterations > 0 && E.parked > 0)
    {
      // a launch that parked ran its full horizon: its time per step sets the next one's
      float ms = 0.0f;
      PARS_CUDA(cudaEventElapsedTime(&ms, engine.launch_start, engine.launch_stop));
      E.ms_per_iteration = double(ms) / double(E.last_iterations);
    }
    E.last_iterations = 0;
    PARS_REQUIRE(E.parked <= (unsigned long long)E.group_capacity, "parked group count out of range");
    // No warp runs between launches: a job's particles are all retired once
    // all its pools are handed out and no parked group holds its particles,
    // the rest of one of its pools, or one of its pools not yet begun.
    std::vector<char> held(n, 0);
    if (E.parked > 0)
    {
      std::vector<batch_parked_group> groups(E.parked);
      PARS_CUDA(cudaMemcpyAsync(groups.data(), E.groups[E.parity].get(), sizeof(batch_parked_group) * groups.size(),
                                cudaMemcpyDeviceToHost, ctx.stream));
      PARS_CUDA(cudaStreamSynchronize(ctx.stream));
      auto job_of_pool = [&](long long pool) {
        int lo = 0, hi = n - 1;
        while (lo < hi)
        {
          const int mid = (lo + hi + 1) / 2;
          if (E.jobs[mid].first_pool <= pool) lo = mid;
          else hi = mid - 1;
        }
        return lo;
      };
      for (const auto& g : groups)
      {
        PARS_REQUIRE(g.job >= 0 && g.job < n && g.count >= 0 && g.count <= 32, "parked group out of range");
        held[g.job] = 1;
        if (g.pending >= 0) held[job_of_pool(g.pending)] = 1;
      }
    }
    for (int k = 0; k < n; ++k)
    {
      const long long last_pool = E.jobs[k].first_pool + pools_of(E.jobs[k].seed_count);
      if (E.complete[k] || held[k] || (long long)E.handed < last_pool) continue;
      E.complete[k] = 1;
      --E.open;
      done.emplace_back(E.tickets[k], host[4 + k]);
    }
    if (E.open == 0)
    {
      PARS_REQUIRE(E.parked == 0, "groups parked after every job completed");
      engine_reset(E);
    }
  }
  return done;
}

// A public batch job as the engine reads it (field, rule and seeds checked).
batch_job_device device_job(pars_gpu_context& ctx, const pars_gpu_batch_job& in)
{
  auto& f = find_field(ctx, in.field);
  batch_job_device d {};
  d.field = f.view();
  d.time = f.time();
  d.rule = make_rule(in.integrator, in.stage_mode, in.step_size);
  if (d.rule.frozen && d.time.nt > 1)
    throw error(PARS_ERR_UNSUPPORTED, "batched frozen-scheme jobs run on steady fields");
  if (!d.rule.frozen && d.rule.scheme != scheme_classic)
    throw error(PARS_ERR_UNSUPPORTED, "batched re-sampled advection integrates with RK4 or Euler");
  d.ux = d.uy = d.uz = 0;
  PARS_REQUIRE(in.max_steps >= 0, "max_steps must be >= 0");
  d.max_steps = in.max_steps;
  d.time_begin = in.time_begin;
  d.seeds = reinterpret_cast<const float4*>(in.seeds);
  if (in.seeds) { PARS_REQUIRE(in.seed_count >= 0, "seed_count must be >= 0"); d.seed_count = in.seed_count; }
  else
  {
    for (int i = 0; i < 3; ++i) PARS_REQUIRE(in.lattice_count[i] >= 0, "lattice counts must be >= 0");
    d.seed_count = (long long)in.lattice_count[0] * in.lattice_count[1] * in.lattice_count[2];
  }
  d.ox = in.lattice_offset[0]; d.oy = in.lattice_offset[1]; d.oz = in.lattice_offset[2];
  d.sx = in.lattice_stride[0]; d.sy = in.lattice_stride[1]; d.sz = in.lattice_stride[2];
  d.px = in.lattice_count[0]; d.py = in.lattice_count[1]; d.pz = in.lattice_count[2];
  d.end_positions = reinterpret_cast<float4*>(in.end_positions);
  d.end_steps = in.end_steps;
  return d;
}
}

using namespace pars;

// The library is built with hidden visibility; only the C ABI is exported.
#pragma GCC visibility push(default)
extern "C" {

int32_t pars_gpu_abi_version(void) { return PARS_GPU_ABI_VERSION; }

int32_t pars_gpu_create(pars_gpu_context** context, int32_t device)
{
  if (!context) return PARS_ERR_INVALID_ARGUMENT;
  *context = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) { (void)cudaGetLastError(); return PARS_ERR_CUDA; }
  if (device < 0 || device >= count) return PARS_ERR_INVALID_ARGUMENT;
  auto* ctx = new (std::nothrow) pars_gpu_context();
  if (!ctx) return PARS_ERR_OUT_OF_MEMORY;
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess)
  {
    (void)cudaGetLastError();
    delete ctx;
    return PARS_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  *context = ctx;
  return PARS_OK;
}

int32_t pars_gpu_destroy(pars_gpu_context* ctx)
{
  if (!ctx) return PARS_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lock(ctx->mutex);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& p : ctx->pending) { cudaEventDestroy(p.start); cudaEventDestroy(p.stop); }
    for (auto e : ctx->event_pool) cudaEventDestroy(e);
    if (ctx->legacy_event) cudaEventDestroy(ctx->legacy_event);
    ctx->pending.clear();
    ctx->event_pool.clear();
    ctx->fields.clear();
    ctx->domains.clear();
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  }
  delete ctx;
  return PARS_OK;
}

const char* pars_gpu_last_error(const pars_gpu_context* ctx)
{
  return ctx ? ctx->last_error.c_str() : "null context";
}

int32_t pars_gpu_set_stream(pars_gpu_context* ctx, void* stream)
{
  return guarded(ctx, [&] {
    flush_profile(*ctx);
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  });
}

int32_t pars_gpu_synchronize(pars_gpu_context* ctx)
{
  return guarded(ctx, [&] { PARS_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

int32_t pars_gpu_memory_in_use(pars_gpu_context* ctx, int64_t* bytes)
{
  return guarded(ctx, [&] { PARS_REQUIRE(bytes, "bytes is required"); *bytes = ctx->held_bytes(); });
}

// ---- fields -------------------------------------------------------------------
int32_t pars_gpu_field_upload(pars_gpu_context* ctx, const float* xyz, const int32_t shape[3], const float offset[3],
                              const float size[3], const float spacing[3], int32_t* field)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(xyz && field, "xyz and field are required");
    check_field_args(shape, spacing);
    auto entry = make_field(shape, offset, size, spacing);
    const long long count = (long long)shape[0] * shape[1] * shape[2];
    ctx->staging.reserve(sizeof(float) * 3 * count);
    entry->data = acquire_buffer(*ctx, sizeof(float4) * count);
    PARS_CUDA(cudaMemcpyAsync(ctx->staging.get(), xyz, sizeof(float) * 3 * count, cudaMemcpyHostToDevice, ctx->stream));
    launch_pack_field(*ctx, ctx->staging.as<const float>(), entry->data.as<float4>(), count);
    // the caller may reuse or free its buffer once the call returns
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    *field = add_field(*ctx, std::move(entry));
  });
}

int32_t pars_gpu_field_upload_device(pars_gpu_context* ctx, const float* device_xyz, const int32_t shape[3], const float offset[3],
                                     const float size[3], const float spacing[3], int32_t* field)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(device_xyz && field, "device_xyz and field are required");
    check_field_args(shape, spacing);
    auto entry = make_field(shape, offset, size, spacing);
    const long long count = (long long)shape[0] * shape[1] * shape[2];
    entry->data = acquire_buffer(*ctx, sizeof(float4) * count);
    launch_pack_field(*ctx, device_xyz, entry->data.as<float4>(), count);
    // the caller may reuse or free its buffer once the call returns
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    *field = add_field(*ctx, std::move(entry));
  });
}

int32_t pars_gpu_unsteady_field_upload(pars_gpu_context* ctx, const float* xyz, const int32_t shape[3], int32_t slices,
                                       const float offset[3], const float size[3], const float spacing[3], double t0,
                                       double slice_dt, int32_t* field)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(xyz && field, "xyz and field are required");
    PARS_REQUIRE(slices >= 1 && slice_dt > 0.0, "slices must be >= 1 and slice_dt positive");
    check_field_args(shape, spacing);
    auto entry = make_field(shape, offset, size, spacing);
    entry->slices = slices; entry->t0 = t0; entry->slice_dt = slice_dt;
    const long long count = (long long)shape[0] * shape[1] * shape[2] * slices;
    ctx->staging.reserve(sizeof(float) * 3 * count);
    entry->data = acquire_buffer(*ctx, sizeof(float4) * count);
    PARS_CUDA(cudaMemcpyAsync(ctx->staging.get(), xyz, sizeof(float) * 3 * count, cudaMemcpyHostToDevice, ctx->stream));
    launch_pack_field(*ctx, ctx->staging.as<const float>(), entry->data.as<float4>(), count);
    // the caller may reuse or free its buffer once the call returns
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    *field = add_field(*ctx, std::move(entry));
  });
}

int32_t pars_gpu_unsteady_field_upload_device(pars_gpu_context* ctx, const float* device_xyz, const int32_t shape[3], int32_t slices,
                                              const float offset[3], const float size[3], const float spacing[3], double t0,
                                              double slice_dt, int32_t* field)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(device_xyz && field, "device_xyz and field are required");
    PARS_REQUIRE(slices >= 1 && slice_dt > 0.0, "slices must be >= 1 and slice_dt positive");
    check_field_args(shape, spacing);
    auto entry = make_field(shape, offset, size, spacing);
    entry->slices = slices; entry->t0 = t0; entry->slice_dt = slice_dt;
    const long long count = (long long)shape[0] * shape[1] * shape[2] * slices;
    entry->data = acquire_buffer(*ctx, sizeof(float4) * count);
    launch_pack_field(*ctx, device_xyz, entry->data.as<float4>(), count);
    // the caller may reuse or free its buffer once the call returns
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    *field = add_field(*ctx, std::move(entry));
  });
}

int32_t pars_gpu_field_release(pars_gpu_context* ctx, int32_t field)
{
  return guarded(ctx, [&] {
    auto it = ctx->fields.find(field);
    if (it == ctx->fields.end()) throw error(PARS_ERR_NOT_FOUND, "no field with handle " + std::to_string(field));
    for (auto& d : ctx->domains)
      for (int f : d.second->fields)
        if (f == field) throw error(PARS_ERR_STATE, "field belongs to a domain; release the domain instead");
    // Work queued on the context's stream may still read the buffer; anything
    // that reuses it is queued behind that work on the same stream.
    recycle_buffer(*ctx, std::move(it->second->data));
    ctx->fields.erase(it);
  });
}

int32_t pars_gpu_field_info(pars_gpu_context* ctx, int32_t field, int32_t shape[3], float offset[3], float size[3], float spacing[3])
{
  return guarded(ctx, [&] {
    auto& f = find_field(*ctx, field);
    for (int i = 0; i < 3; ++i)
    {
      if (shape) shape[i] = f.shape[i];
      if (offset) offset[i] = f.offset[i];
      if (size) size[i] = f.size[i];
      if (spacing) spacing[i] = f.spacing[i];
    }
  });
}

int32_t pars_gpu_field_download(pars_gpu_context* ctx, int32_t field, float* xyz)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(xyz, "xyz is required");
    auto& f = find_field(*ctx, field);
    const long long count = (long long)f.shape[0] * f.shape[1] * f.shape[2];
    ctx->staging.reserve(sizeof(float) * 3 * count);
    launch_unpack_field(*ctx, f.data.as<const float4>(), ctx->staging.as<float>(), count);
    PARS_CUDA(cudaMemcpyAsync(xyz, ctx->staging.get(), sizeof(float) * 3 * count, cudaMemcpyDeviceToHost, ctx->stream));
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int32_t pars_gpu_field_sample(pars_gpu_context* ctx, int32_t field, const float* positions, int64_t n, uint8_t* inside, float* velocity)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(n >= 0, "negative count");
    if (n == 0) return;
    PARS_REQUIRE(positions && inside && velocity, "positions, inside and velocity are required");
    auto& f = find_field(*ctx, field);
    device_buffer p, in, v;
    p.reserve(checked_bytes(n, sizeof(float4)));
    in.reserve(checked_bytes(n, 1));
    v.reserve(checked_bytes(n, 3 * sizeof(float)));
    PARS_CUDA(cudaMemcpyAsync(p.get(), positions, sizeof(float4) * n, cudaMemcpyHostToDevice, ctx->stream));
    launch_field_sample(*ctx, f.view(), p.as<const float4>(), n, in.as<uint8_t>(), v.as<float>());
    PARS_CUDA(cudaMemcpyAsync(inside, in.get(), n, cudaMemcpyDeviceToHost, ctx->stream));
    PARS_CUDA(cudaMemcpyAsync(velocity, v.get(), sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

// ---- seeds / partition -----------------------------------------------------------
int32_t pars_gpu_seed_generate(pars_gpu_context* ctx, const float offset[3], const float size[3], const float stride[3],
                               int32_t iterations, int32_t rank, pars_particle* particles, int64_t capacity, int64_t* count)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(offset && size && stride && count, "offset, size, stride and count are required");
    int per_dimension[3];
    long long total = 1;
    for (int i = 0; i < 3; ++i)
    {
      // (size / stride).cast<integer>() (seed_generator.cpp:11): FP32 quotient, truncated.
      const float q = size[i] / stride[i];
      per_dimension[i] = (q > 0.0f && q < 2147483647.0f) ? int(q) : 0;
      total *= per_dimension[i];
    }
    *count = total;
    if (!particles || total == 0) return;
    PARS_REQUIRE(capacity >= total, "capacity is smaller than the seed count");
    device_buffer out;
    out.reserve(checked_bytes(total, sizeof(pars_particle)));
    launch_seed_generate(*ctx, offset, stride, per_dimension, iterations, rank, out.as<pars_particle>());
    PARS_CUDA(cudaMemcpyAsync(particles, out.get(), sizeof(pars_particle) * total, cudaMemcpyDeviceToHost, ctx->stream));
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int32_t pars_gpu_partition(int32_t ranks, int32_t rank, const int32_t domain_size[3], pars_partition_info* info)
{
  if (!domain_size || !info || ranks < 1 || rank < 0 || rank >= ranks) return PARS_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < 3; ++i) if (domain_size[i] < 1) return PARS_ERR_INVALID_ARGUMENT;
  *info = partition_of(ranks, rank, domain_size);
  return PARS_OK;
}

// ---- tracing --------------------------------------------------------------------
int32_t pars_gpu_trace(pars_gpu_context* ctx, int32_t field, const pars_particle* particles, int64_t count,
                       int32_t integrator, int32_t stage_mode, float step_size, pars_gpu_trace_summary* summary)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(count >= 0 && (count == 0 || particles), "particles are required");
    ctx->particles_in.reserve(checked_bytes(std::max<long long>(count, 1), sizeof(pars_particle)));
    if (count > 0)
      PARS_CUDA(cudaMemcpyAsync(ctx->particles_in.get(), particles, sizeof(pars_particle) * count, cudaMemcpyHostToDevice, ctx->stream));
    trace_single(*ctx, field, count, integrator, stage_mode, step_size, summary);
  });
}

int32_t pars_gpu_trace_device(pars_gpu_context* ctx, int32_t field, const pars_particle* device_particles, int64_t count,
                              int32_t integrator, int32_t stage_mode, float step_size, pars_gpu_trace_summary* summary)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(count >= 0 && (count == 0 || device_particles), "particles are required");
    ctx->particles_in.reserve(checked_bytes(std::max<long long>(count, 1), sizeof(pars_particle)));
    if (count > 0)
      PARS_CUDA(cudaMemcpyAsync(ctx->particles_in.get(), device_particles, sizeof(pars_particle) * count, cudaMemcpyDeviceToDevice, ctx->stream));
    trace_single(*ctx, field, count, integrator, stage_mode, step_size, summary);
  });
}

namespace
{
// Splits a DEVICE [X][Y][Z][3] domain field into the partitioner's ghosted
// blocks (data_io.cpp:91-115 without the file) and registers the domain.
int32_t build_domain(pars_gpu_context* ctx, const float* device_xyz, const int32_t domain_size[3], const float spacing[3], int32_t ranks)
{
  auto entry = std::make_unique<domain_entry>();
  entry->ranks = ranks;
  entry->first = partition_of(ranks, 0, domain_size);
  for (int i = 0; i < 3; ++i) PARS_REQUIRE(entry->first.block_size[i] >= 1, "more blocks than voxels along an axis");
  for (int r = 0; r < ranks; ++r)
  {
    const pars_partition_info info = partition_of(ranks, r, domain_size);
    auto f = std::make_unique<field_entry>();
    for (int i = 0; i < 3; ++i)
    {
      f->shape[i] = info.ghosted_block_size[i];
      f->spacing[i] = spacing[i];
      f->offset[i] = float(info.offset[i]) * spacing[i];          // data_io.cpp:113
      f->size[i] = float(info.block_size[i]) * spacing[i];        // data_io.cpp:114
    }
    for (int i = 0; i < 3; ++i) PARS_REQUIRE(f->shape[i] >= 2, "blocks must be at least 2 voxels wide");
    f->data = acquire_buffer(*ctx, sizeof(float4) * (std::size_t)f->shape[0] * f->shape[1] * f->shape[2]);
    launch_extract_block(*ctx, device_xyz, domain_size, info.offset, f->shape, f->data.as<float4>());
    trace_block b;
    b.field = f->view();
    for (int face = 0; face < 6; ++face) b.neighbor[face] = info.neighbor_rank[face];
    entry->blocks.push_back(b);
    entry->fields.push_back(add_field(*ctx, std::move(f)));
  }
  entry->device_blocks.reserve(sizeof(trace_block) * ranks);
  PARS_CUDA(cudaMemcpyAsync(entry->device_blocks.get(), entry->blocks.data(), sizeof(trace_block) * ranks, cudaMemcpyHostToDevice, ctx->stream));
  PARS_CUDA(cudaStreamSynchronize(ctx->stream));
  const int32_t handle = ctx->next_handle++;
  ctx->domains[handle] = std::move(entry);
  return handle;
}
}

int32_t pars_gpu_domain_create_device(pars_gpu_context* ctx, const float* device_xyz, const int32_t domain_size[3], const float spacing[3],
                                      int32_t ranks, int32_t* domain)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(device_xyz && domain_size && spacing && domain, "device_xyz, domain_size, spacing and domain are required");
    PARS_REQUIRE(ranks >= 1, "ranks must be >= 1");
    check_field_args(domain_size, spacing);
    *domain = build_domain(ctx, device_xyz, domain_size, spacing, ranks);
  });
}

int32_t pars_gpu_domain_create(pars_gpu_context* ctx, const float* xyz, const int32_t domain_size[3], const float spacing[3],
                               int32_t ranks, int32_t* domain)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(xyz && domain_size && spacing && domain, "xyz, domain_size, spacing and domain are required");
    PARS_REQUIRE(ranks >= 1, "ranks must be >= 1");
    check_field_args(domain_size, spacing);
    const long long total = (long long)domain_size[0] * domain_size[1] * domain_size[2];
    ctx->staging.reserve(sizeof(float) * 3 * total);
    PARS_CUDA(cudaMemcpyAsync(ctx->staging.get(), xyz, sizeof(float) * 3 * total, cudaMemcpyHostToDevice, ctx->stream));
    *domain = build_domain(ctx, ctx->staging.as<const float>(), domain_size, spacing, ranks);
  });
}

int32_t pars_gpu_domain_release(pars_gpu_context* ctx, int32_t domain)
{
  return guarded(ctx, [&] {
    auto it = ctx->domains.find(domain);
    if (it == ctx->domains.end()) throw error(PARS_ERR_NOT_FOUND, "no domain with handle " + std::to_string(domain));
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    if (it->second->owns_fields)
    for (int f : it->second->fields)
    {
      auto fit = ctx->fields.find(f);
      if (fit == ctx->fields.end()) continue;
      recycle_buffer(*ctx, std::move(fit->second->data));
      ctx->fields.erase(fit);
    }
    ctx->domains.erase(it);
  });
}

int32_t pars_gpu_trace_domain(pars_gpu_context* ctx, int32_t domain, const pars_particle* particles, const int64_t* seed_offsets,
                              int32_t integrator, int32_t stage_mode, float step_size, pars_gpu_trace_summary* summary)
{
  return guarded(ctx, [&] {
    auto it = ctx->domains.find(domain);
    if (it == ctx->domains.end()) throw error(PARS_ERR_NOT_FOUND, "no domain with handle " + std::to_string(domain));
    auto& d = *it->second;
    PARS_REQUIRE(seed_offsets, "seed_offsets is required");
    const step_rule rule = make_rule(integrator, stage_mode, step_size);
    const int nblocks = d.ranks;
    const long long count = seed_offsets[nblocks] - seed_offsets[0];
    PARS_REQUIRE(count >= 0 && (count == 0 || particles), "particles are required");
    std::vector<long long> block_count(nblocks);
    std::vector<int> block_max(nblocks, 0);
    std::vector<int> block_of(std::max<long long>(count, 1));
    for (int b = 0; b < nblocks; ++b)
    {
      const long long begin = seed_offsets[b] - seed_offsets[0], end = seed_offsets[b + 1] - seed_offsets[0];
      PARS_REQUIRE(end >= begin, "seed_offsets must be non-decreasing");
      block_count[b] = end - begin;
      for (long long i = begin; i < end; ++i)
      {
        block_of[i] = b;
        block_max[b] = std::max(block_max[b], particles[seed_offsets[0] + i].remaining_iterations);
      }
    }
    ctx->particles_in.reserve(checked_bytes(std::max<long long>(count, 1), sizeof(pars_particle)));
    ctx->block_of.reserve(checked_bytes(std::max<long long>(count, 1), sizeof(int)));
    if (count > 0)
    {
      PARS_CUDA(cudaMemcpyAsync(ctx->particles_in.get(), particles + seed_offsets[0], sizeof(pars_particle) * count, cudaMemcpyHostToDevice, ctx->stream));
      PARS_CUDA(cudaMemcpyAsync(ctx->block_of.get(), block_of.data(), sizeof(int) * count, cudaMemcpyHostToDevice, ctx->stream));
    }
    // one persistent launch over all rounds; round by round when its
    // buffers do not fit or overflow
    if (!run_rounds_async(*ctx, d.blocks, d.device_blocks.as<const trace_block>(), count, block_count, block_max, rule, summary))
      run_rounds(*ctx, d.blocks, d.device_blocks.as<const trace_block>(), count, block_count, block_max, rule, true, summary);
  });
}

// ---- round-by-round tracing ----------------------------------------------------------
int32_t pars_gpu_domain_assemble(pars_gpu_context* ctx, int32_t ranks, const int32_t domain_size[3], const int32_t* fields,
                                 int32_t* domain)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(domain_size && fields && domain, "domain_size, fields and domain are required");
    PARS_REQUIRE(ranks >= 1, "ranks must be >= 1");
    for (int i = 0; i < 3; ++i) PARS_REQUIRE(domain_size[i] >= 2, "every domain extent must be >= 2");
    auto entry = std::make_unique<domain_entry>();
    entry->ranks = ranks;
    entry->owns_fields = false;
    entry->first = partition_of(ranks, 0, domain_size);
    for (int r = 0; r < ranks; ++r)
    {
      const pars_partition_info info = partition_of(ranks, r, domain_size);
      auto& f = find_field(*ctx, fields[r]);
      PARS_REQUIRE(f.slices == 1, "domain blocks must be steady fields");
      for (int i = 0; i < 3; ++i)
        PARS_REQUIRE(f.shape[i] == info.ghosted_block_size[i],
                     "field of rank " + std::to_string(r) + " is not its ghosted block of the partition");
      trace_block b;
      b.field = f.view();
      for (int face = 0; face < 6; ++face) b.neighbor[face] = info.neighbor_rank[face];
      entry->blocks.push_back(b);
      entry->fields.push_back(fields[r]);
    }
    entry->device_blocks.reserve(sizeof(trace_block) * ranks);
    PARS_CUDA(cudaMemcpyAsync(entry->device_blocks.get(), entry->blocks.data(), sizeof(trace_block) * ranks, cudaMemcpyHostToDevice,
                              ctx->stream));
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    const int32_t handle = ctx->next_handle++;
    ctx->domains[handle] = std::move(entry);
    *domain = handle;
  });
}

int32_t pars_gpu_round_trace(pars_gpu_context* ctx, int32_t domain, int32_t round, const pars_particle* particles,
                             const int64_t* offsets, int32_t integrator, int32_t stage_mode, float step_size, int64_t* next_offsets,
                             pars_gpu_trace_summary* summary)
{
  return guarded(ctx, [&] {
    auto it = ctx->domains.find(domain);
    if (it == ctx->domains.end()) throw error(PARS_ERR_NOT_FOUND, "no domain with handle " + std::to_string(domain));
    auto& d = *it->second;
    PARS_REQUIRE(round >= 0, "round must be >= 0");
    const step_rule rule = make_rule(integrator, stage_mode, step_size);
    const int nblocks = d.ranks;
    round_plan plan;
    if (particles)
    {
      PARS_REQUIRE(offsets, "offsets are required with host particles");
      const long long count = offsets[nblocks] - offsets[0];
      PARS_REQUIRE(count >= 0, "offsets must be non-decreasing");
      plan.count = count;
      plan.block_count.assign(nblocks, 0);
      plan.block_max.assign(nblocks, 0);
      std::vector<int> block_of(std::max<long long>(count, 1));
      for (int b = 0; b < nblocks; ++b)
      {
        const long long begin = offsets[b] - offsets[0], end = offsets[b + 1] - offsets[0];
        PARS_REQUIRE(end >= begin, "offsets must be non-decreasing");
        plan.block_count[b] = end - begin;
        for (long long i = begin; i < end; ++i)
        {
          block_of[i] = b;
          plan.block_max[b] = std::max(plan.block_max[b], particles[offsets[0] + i].remaining_iterations);
        }
      }
      ctx->particles_in.reserve(checked_bytes(std::max<long long>(count, 1), sizeof(pars_particle)));
      ctx->block_of.reserve(checked_bytes(std::max<long long>(count, 1), sizeof(int)));
      if (count > 0)
      {
        PARS_CUDA(cudaMemcpyAsync(ctx->particles_in.get(), particles + offsets[0], sizeof(pars_particle) * count,
                                  cudaMemcpyHostToDevice, ctx->stream));
        PARS_CUDA(cudaMemcpyAsync(ctx->block_of.get(), block_of.data(), sizeof(int) * count, cudaMemcpyHostToDevice, ctx->stream));
      }
    }
    else
    {
      if (ctx->round_serial != ctx->trace_serial || ctx->round_domain != domain || ctx->round_next != round)
        throw error(PARS_ERR_STATE, "no device-resident particles of round " + std::to_string(round) + " on this domain");
      plan.count = ctx->round_count;
      plan.block_count = ctx->round_block_count;
      plan.block_max = ctx->round_block_max;
    }
    if (round == 0) clear_curves(*ctx);
    ++ctx->trace_serial;
    const long long batches_before = (long long)ctx->curves.batches.size();
    const long long vertices_before = ctx->curves.vertex_total;
    const round_counters counters = tracing_counters(*ctx);
    PARS_CUDA(cudaMemsetAsync(counters.steps, 0, sizeof(unsigned long long), ctx->stream));
    if (plan.count > 0)
      trace_one_round(*ctx, d.blocks, d.device_blocks.as<const trace_block>(), plan, rule, true, round, counters, nullptr);
    else
      std::fill(plan.block_count.begin(), plan.block_count.end(), 0);
    unsigned long long steps = 0;
    PARS_CUDA(cudaMemcpyAsync(&steps, counters.steps, sizeof(steps), cudaMemcpyDeviceToHost, ctx->stream));
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->round_serial = ctx->trace_serial;
    ctx->round_domain = domain;
    ctx->round_next = round + 1;
    ctx->round_count = plan.count;
    ctx->round_block_count = plan.block_count;
    ctx->round_block_max = plan.block_max;
    if (next_offsets)
    {
      next_offsets[0] = 0;
      for (int b = 0; b < nblocks; ++b) next_offsets[b + 1] = next_offsets[b] + plan.block_count[b];
    }
    if (summary)
    {
      summary->batches = (long long)ctx->curves.batches.size() - batches_before;
      summary->vertices = ctx->curves.vertex_total - vertices_before;
      summary->steps = (long long)steps;
      summary->rounds = round + 1;
      summary->padding = 0;
    }
  });
}

int32_t pars_gpu_round_particles(pars_gpu_context* ctx, pars_particle* particles)
{
  return guarded(ctx, [&] {
    if (ctx->round_serial != ctx->trace_serial) throw error(PARS_ERR_STATE, "no round-by-round tracing to read particles from");
    PARS_REQUIRE(particles || ctx->round_count == 0, "particles is required");
    if (ctx->round_count > 0)
    {
      PARS_CUDA(cudaMemcpyAsync(particles, ctx->particles_in.get(), sizeof(pars_particle) * ctx->round_count, cudaMemcpyDeviceToHost,
                                ctx->stream));
      PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    }
  });
}

// ---- curve stages -----------------------------------------------------------------
int32_t pars_gpu_curves_index(pars_gpu_context* ctx)
{
  return guarded(ctx, [&] {
    auto& c = ctx->curves;
    index_batches(*ctx, c);
    c.indexed = true;
    c.colored = false;
    ++c.generation;
  });
}

int32_t pars_gpu_curves_color(pars_gpu_context* ctx, int32_t mode, float parameter)
{
  return guarded(ctx, [&] {
    auto& c = ctx->curves;
    if (!c.indexed) throw error(PARS_ERR_STATE, "curves must be indexed before they are coloured");
    PARS_REQUIRE(mode >= PARS_COLOR_HSL_CONSTANT_S && mode <= PARS_COLOR_RGB, "unknown colour mode");
    color_batches(*ctx, c, std::vector<color_spec>(c.batches.size(), color_spec{mode, parameter}));
    c.colored = true;
    ++c.generation;
  });
}

int32_t pars_gpu_curves_batch_info(pars_gpu_context* ctx, int64_t batch, int64_t* vertices, int64_t* indices, int32_t* rank, int32_t* round)
{
  return guarded(ctx, [&] {
    auto& c = ctx->curves;
    PARS_REQUIRE(batch >= 0 && batch < (int64_t)c.batches.size(), "batch out of range");
    const auto& b = c.batches[batch];
    if (vertices) *vertices = b.vertex_count;
    if (indices) *indices = c.indexed ? b.index_count : 0;
    if (rank) *rank = b.rank;
    if (round) *round = b.round;
  });
}

int32_t pars_gpu_curves_download(pars_gpu_context* ctx, int64_t batch, float* vertices, float* colors, int32_t* indices)
{
  return guarded(ctx, [&] {
    auto& c = ctx->curves;
    PARS_REQUIRE(batch >= 0 && batch < (int64_t)c.batches.size(), "batch out of range");
    const auto& b = c.batches[batch];
    if (vertices && b.vertex_count)
      PARS_CUDA(cudaMemcpyAsync(vertices, c.vertices.as<float4>() + b.vertex_offset, sizeof(float4) * b.vertex_count, cudaMemcpyDeviceToHost, ctx->stream));
    if (colors && b.vertex_count)
    {
      if (!c.colored) throw error(PARS_ERR_STATE, "curves are not coloured");
      PARS_CUDA(cudaMemcpyAsync(colors, c.colors.as<float4>() + b.vertex_offset, sizeof(float4) * b.vertex_count, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (indices && c.indexed && b.index_count)
      PARS_CUDA(cudaMemcpyAsync(indices, c.indices.as<int>() + b.index_offset, sizeof(int) * b.index_count, cudaMemcpyDeviceToHost, ctx->stream));
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int32_t pars_gpu_index_generate(pars_gpu_context* ctx, const float* vertices, int64_t n, int32_t* indices, int64_t* index_count)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(index_count && n >= 0 && (n == 0 || (vertices && indices)), "vertices, indices and index_count are required");
    *index_count = 0;
    if (n < 2) return;
    device_buffer v, i;
    v.reserve(checked_bytes(n, sizeof(float4)));
    i.reserve(checked_bytes(n, sizeof(int)));
    PARS_CUDA(cudaMemcpyAsync(v.get(), vertices, sizeof(float4) * n, cudaMemcpyHostToDevice, ctx->stream));
    const long long m = launch_index_generate(*ctx, v.as<const float4>(), n, i.as<int>());
    if (m) PARS_CUDA(cudaMemcpyAsync(indices, i.get(), sizeof(int) * m, cudaMemcpyDeviceToHost, ctx->stream));
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    *index_count = m;
  });
}

int32_t pars_gpu_color_generate(pars_gpu_context* ctx, const float* vertices, int64_t n, const int32_t* indices, int64_t index_count,
                                int32_t mode, float parameter, float* colors)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(n >= 0 && index_count >= 0 && (n == 0 || (vertices && colors)) && (index_count == 0 || indices), "buffers are required");
    PARS_REQUIRE(mode >= PARS_COLOR_HSL_CONSTANT_S && mode <= PARS_COLOR_RGB, "unknown colour mode");
    if (n == 0 || index_count == 0) return;
    for (int64_t k = 0; k < index_count; ++k)
      PARS_REQUIRE(indices[k] >= 0 && indices[k] + 1 < n, "index out of range");
    device_buffer v, i, c;
    v.reserve(checked_bytes(n, sizeof(float4)));
    i.reserve(checked_bytes(index_count, sizeof(int)));
    c.reserve(checked_bytes(n, sizeof(float4)));
    PARS_CUDA(cudaMemcpyAsync(v.get(), vertices, sizeof(float4) * n, cudaMemcpyHostToDevice, ctx->stream));
    PARS_CUDA(cudaMemcpyAsync(i.get(), indices, sizeof(int) * index_count, cudaMemcpyHostToDevice, ctx->stream));
    PARS_CUDA(cudaMemcpyAsync(c.get(), colors, sizeof(float4) * n, cudaMemcpyHostToDevice, ctx->stream));
    launch_color_generate(*ctx, v.as<const float4>(), i.as<const int>(), index_count, mode, parameter, c.as<float4>());
    PARS_CUDA(cudaMemcpyAsync(colors, c.get(), sizeof(float4) * n, cudaMemcpyDeviceToHost, ctx->stream));
    PARS_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

// ---- flow map / FTLE -------------------------------------------------------------
int32_t pars_gpu_flow_map_generate(pars_gpu_context* ctx, int32_t field, int32_t iterations, float resolution_scale,
                                   int32_t integrator, int32_t stage_mode, float step_size, int32_t* flow_map, int64_t* steps)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(flow_map, "flow_map is required");
    PARS_REQUIRE(resolution_scale > 0.0f, "resolution_scale must be positive");
    auto& f = find_field(*ctx, field);
    const step_rule rule = make_rule(integrator, stage_mode, step_size);
    auto entry = std::make_unique<field_entry>();
    int seeds[3];
    for (int i = 0; i < 3; ++i)
    {
      entry->shape[i] = int(float(f.shape[i]) * resolution_scale);      // flow_map_generator.cpp:27-30
      entry->spacing[i] = f.spacing[i] / resolution_scale;              // :34-37
      entry->offset[i] = f.offset[i];
      entry->size[i] = f.size[i];
      const float q = f.size[i] / entry->spacing[i];                     // seed_generator.cpp:11
      seeds[i] = (q > 0.0f && q < 2147483647.0f) ? int(q) : 0;
      PARS_REQUIRE(entry->shape[i] >= 1, "flow map would be empty");
      // The seed lattice covers the flow map's voxels (one seed per vertex,
      // plus at most one that rounding of size / spacing can add); a larger
      // lattice would write nothing more and would overflow the seed count.
      PARS_REQUIRE(seeds[i] <= entry->shape[i] + 1, "size / spacing gives more seeds than the flow map has voxels");
    }
    const long long voxels = (long long)entry->shape[0] * entry->shape[1] * entry->shape[2];
    entry->data = acquire_buffer(*ctx, sizeof(float4) * voxels);
    // Voxels no seed reaches stay NaN (the reference leaves them unassigned);
    // when the seed lattice covers the flow map every voxel is written.
    if (seeds[0] < entry->shape[0] || seeds[1] < entry->shape[1] || seeds[2] < entry->shape[2])
      PARS_CUDA(cudaMemsetAsync(entry->data.get(), 0xff, sizeof(float4) * voxels, ctx->stream));
    if (rule.scheme != scheme_classic && f.slices > 1)
      throw error(PARS_ERR_UNSUPPORTED, "unsteady flow maps integrate with RK4 or Euler");
    if (rule.frozen || iterations <= 1 || rule.scheme != scheme_classic)
    {
      // One seed per thread: the reference's scheme bit for bit (one field
      // sample per step: at 64 registers this kernel keeps more warps
      // resident than the batched engine's frozen class, 57 against 53 G
      // steps/s on the 256^3 flow map), the iterations <= 1 case, where every
      // voxel keeps its seed position, and the re-sampled stages of the
      // general schemes.
      ctx->counters.reserve(sizeof(unsigned long long) * 2);
      auto* counter = ctx->counters.as<unsigned long long>();
      PARS_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream));
      launch_flow_map(*ctx, f.view(), rule, iterations, f.offset, entry->spacing, seeds, entry->shape, entry->data.as<float4>(), counter);
      if (steps)
      {
        unsigned long long s = 0;
        PARS_CUDA(cudaMemcpyAsync(&s, counter, sizeof(s), cudaMemcpyDeviceToHost, ctx->stream));
        PARS_CUDA(cudaStreamSynchronize(ctx->stream));
        *steps = (int64_t)s;
      }
    }
    else
    {
      // Re-sampled RK4 / Euler: one job of the persistent batched engine.
      std::vector<batch_job_device> job(1);
      batch_job_device& d = job[0];
      d.field = f.view();
      d.time = f.time();
      d.rule = rule;
      d.max_steps = iterations - 1;
      d.time_begin = f.t0;
      d.seeds = nullptr;
      d.seed_count = (long long)seeds[0] * seeds[1] * seeds[2];
      d.ox = f.offset[0]; d.oy = f.offset[1]; d.oz = f.offset[2];
      d.sx = entry->spacing[0]; d.sy = entry->spacing[1]; d.sz = entry->spacing[2];
      d.px = seeds[0]; d.py = seeds[1]; d.pz = seeds[2];
      d.ux = entry->shape[0]; d.uy = entry->shape[1]; d.uz = entry->shape[2];
      d.end_positions = entry->data.as<float4>();
      d.end_steps = nullptr;
      const auto s = execute_batch(*ctx, job, -1);
      if (steps) *steps = (int64_t)s[0];
    }
    *flow_map = add_field(*ctx, std::move(entry));
  });
}

int32_t pars_gpu_ftle_generate(pars_gpu_context* ctx, int32_t flow_map, float time, int32_t mode, float* ftle)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(mode == PARS_FTLE_REGULAR || mode == PARS_FTLE_FRACTIONAL_ANISOTROPY, "unknown FTLE mode");
    PARS_REQUIRE(time != 0.0f, "time must be non-zero");
    auto& f = find_field(*ctx, flow_map);
    const long long voxels = (long long)f.shape[0] * f.shape[1] * f.shape[2];
    ctx->ftle.reserve(sizeof(float) * voxels);
    ctx->ftle_count = voxels;
    launch_ftle(*ctx, f.view(), double(time), mode, ctx->ftle.as<float>());
    if (ftle)
    {
      PARS_CUDA(cudaMemcpyAsync(ftle, ctx->ftle.get(), sizeof(float) * voxels, cudaMemcpyDeviceToHost, ctx->stream));
      PARS_CUDA(cudaStreamSynchronize(ctx->stream));
    }
  });
}

int32_t pars_gpu_batch_variants(pars_gpu_context* ctx, int32_t* count)
{
  return guarded(ctx, [&] { PARS_REQUIRE(count, "count is required"); *count = batch_variant_count(); });
}

int32_t pars_gpu_batch_tuned(pars_gpu_context* ctx, int32_t job_class, int32_t* variant, int32_t* threads)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(job_class >= 0 && job_class < batch_classes, "job_class is 0 (steady), 1 (unsteady) or 2 (frozen)");
    const int v = ctx->batch_variant[job_class];
    if (variant) *variant = v;
    if (threads) *threads = v >= 0 ? batch_variant_threads(v) : 0;
  });
}

int32_t pars_gpu_batch_advect(pars_gpu_context* ctx, pars_gpu_batch_job* jobs, int32_t count, int32_t variant)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(count >= 0 && (count == 0 || jobs), "jobs are required");
    PARS_REQUIRE(variant >= -1 && variant < batch_variant_count(), "unknown launch variant");
    if (count == 0) return;
    std::vector<batch_job_device> device_jobs(count);
    for (int j = 0; j < count; ++j) device_jobs[j] = device_job(*ctx, jobs[j]);
    const std::vector<unsigned long long> steps = execute_batch(*ctx, device_jobs, variant);
    for (int j = 0; j < count; ++j) jobs[j].steps = (int64_t)steps[j];
  });
}

int32_t pars_gpu_engine_submit(pars_gpu_context* ctx, const pars_gpu_batch_job* job, int64_t* ticket)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(job && ticket, "job and ticket are required");
    *ticket = engine_submit(*ctx, device_job(*ctx, *job));
  });
}

int32_t pars_gpu_engine_advance(pars_gpu_context* ctx, int32_t iterations, pars_gpu_engine_done* done, int32_t capacity,
                                int32_t* done_count, int64_t* open)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(capacity >= 0 && (capacity == 0 || done), "done is required when capacity > 0");
    PARS_REQUIRE(done_count, "done_count is required");
    const auto finished = engine_advance(*ctx, iterations);
    if (!ctx->engine) ctx->engine = std::make_shared<batch_engine>();
    auto& ready = ctx->engine->ready;
    ready.insert(ready.end(), finished.begin(), finished.end());
    const int32_t n = int32_t(std::min<std::size_t>(ready.size(), std::size_t(capacity)));
    for (int32_t i = 0; i < n; ++i) { done[i].ticket = ready[i].first; done[i].steps = (int64_t)ready[i].second; }
    ready.erase(ready.begin(), ready.begin() + n);
    *done_count = n;
    if (open) *open = engine_open(*ctx) + (int64_t)ready.size();
  });
}

int32_t pars_gpu_ftle_device_pointer(pars_gpu_context* ctx, const float** device_ftle, int64_t* count)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(device_ftle && count, "device_ftle and count are required");
    *device_ftle = ctx->ftle.as<const float>();
    *count = ctx->ftle_count;
  });
}

// ---- instrumentation ------------------------------------------------------------
int32_t pars_gpu_profile_enable(pars_gpu_context* ctx, int32_t enable)
{
  return guarded(ctx, [&] { flush_profile(*ctx); ctx->profile = enable != 0; });
}

int32_t pars_gpu_profile_reset(pars_gpu_context* ctx)
{
  return guarded(ctx, [&] { flush_profile(*ctx); ctx->profile_totals.clear(); });
}

int32_t pars_gpu_profile_get(pars_gpu_context* ctx, const char* name, double* milliseconds, int64_t* launches)
{
  return guarded(ctx, [&] {
    PARS_REQUIRE(name, "name is required");
    flush_profile(*ctx);
    auto it = ctx->profile_totals.find(name);
    if (milliseconds) *milliseconds = it == ctx->profile_totals.end() ? 0.0 : it->second.milliseconds;
    if (launches) *launches = it == ctx->profile_totals.end() ? 0 : it->second.launches;
  });
}

int32_t pars_gpu_launch_count(pars_gpu_context* ctx, int64_t* launches)
{
  return guarded(ctx, [&] { PARS_REQUIRE(launches, "launches is required"); *launches = ctx->launches; });
}

}
#pragma GCC visibility pop
