// pars_service-compatible request service with continuous batching.
//
// The reference's service (pars/source/service.cpp:20-69) receives one binary
// `settings` message at a time, runs pipeline::execute on it and replies.
// Here requests are queued as they arrive and several lanes (each a context
// with its own CUDA stream and worker thread) take batches from the queue:
//  * admission: a request enters a batch only while the device memory that
//    the running batches are estimated to need, plus the results held on the
//    device, stays within the budget;
//  * results: each request's buffers stay on the device until the client
//    copies them into its own host buffers and releases the request — an FTLE
//    field in one allocation from the service's stream-ordered pool, curves
//    as ranges of their batch's curve buffers, which the batch's requests share
//    (no device copy) and which return to the lanes once all have let go; when
//    no queued request fits and no batch runs, held results move to host
//    memory so that the queue moves on;
//  * batching: a lane takes every queued request of the same kind that fits
//    (up to max_batch) and runs them as one launch — FTLE requests as jobs of
//    the persistent batched advection engine, streamline requests as blocks of
//    one tracing round loop;
//  * overlap: while one lane's batch runs, another lane admits the requests
//    that arrived meanwhile and launches them on its own stream.
// Datasets (the requests' dataset_filepath) are fields registered with the
// service and kept resident across requests; scalar volumes (volume_type)
// likewise.  A streamline request that carries an image size is also ray
// traced (pipeline.cpp:264-337): its image is rendered on the lane right after
// its batch and kept in host memory with the request.
#include <algorithm>
#include <atomic>
#include <array>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "context.hpp"
#include "settings.hpp"

namespace pars
{
namespace
{
using clock_type = std::chrono::steady_clock;

enum request_state { queued = 0, running = 1, done = 2 };
enum request_kind { streamlines = 0, ftle = 1 };

struct dataset
{
  std::string name;
  int32_t     field;   // handle in the service's owner context
  field_view  view;
  int         shape[3];
  float       offset[3], size[3], spacing[3];
};

// A scalar volume for the ray tracer (the reference's load_local_scalar_field
// of `volume_type`, data_io.cpp:41-49,76-81): float [X][Y][Z] on the device.
struct volume_dataset
{
  device_buffer data;
  int           shape[3];
  float         offset[3], spacing[3];
};

// One integral_curves batch of a streamline request: its place in the
// request's own layout (vertex_offset, index_offset; used once its buffers
// have moved to host memory) and in the batch's shared curve store.
struct curve_span
{
  int64_t vertex_offset, vertex_count, index_offset, index_count;
  int64_t store_vertex_offset, store_index_offset;
};

// The curve buffers of one streamline batch (vertices, colours, packed
// indices), shared by the batch's requests until the last of them is
// released or moved to host memory; the buffers then return to the service's
// free list, from which the lanes take their next curve buffers.
struct curve_store
{
  pars_gpu_service* svc = nullptr;
  device_buffer     vertices, colors, indices;
  std::size_t       counted = 0;   // bytes booked against the budget
  std::size_t bytes() const { return vertices.bytes() + colors.bytes() + indices.bytes(); }
  ~curve_store();
};

struct request
{
  int64_t            ticket = 0;
  settings           s;
  int                kind = streamlines;
  int                dataset = -1;
  int                integrator = PARS_RUNGE_KUTTA_4;
  int                stage_mode = PARS_STAGES_RESAMPLED;
  int                color_mode = PARS_COLOR_RGB;
  int                ftle_mode = PARS_FTLE_REGULAR;
  std::size_t        estimate = 0;
  int32_t            state = queued;
  int32_t            status = PARS_OK;
  std::string        error;
  clock_type::time_point submitted, started, finished;
  long long          steps = 0;
  int                ftle_shape[3] = {0, 0, 0};
  // Results.  FTLE: one device allocation from the service's pool (float
  // [voxels]).  Streamlines: sub-ranges of the batch's curve store.  Once
  // moved to host memory, `spilled` holds them in the request's own layout:
  // vertices (float4 [vertex_total]), colours (float4 [vertex_total]), indices
  // (int32 [index_total]) — or the FTLE values.
  std::mutex              result_mutex;
  char*                   result = nullptr;
  std::size_t             result_bytes = 0;
  std::shared_ptr<curve_store> store;
  std::vector<char>       spilled;
  bool                    released = false;
  std::vector<curve_span> spans;   // streamlines: one per integral_curves batch
  int64_t                 vertex_total = 0, index_total = 0;
  // ray tracing (streamline requests with an image size)
  bool                    trace_curves = true;   // false for a "volume"-only request
  bool                    wants_image = false;
  int                     volume = -1;           // volume dataset, -1 without
  std::vector<uint8_t>    image;                 // sRGB RGBA8, rows from the top
  int32_t                 image_size[2] = {0, 0};
};

int integrator_of(const std::string& name)
{
  static const char* names[] = {"euler", "modified_midpoint", "runge_kutta_4", "runge_kutta_cash_karp_54",
                                "runge_kutta_dormand_prince_5", "runge_kutta_fehlberg_78", "adams_bashforth_2",
                                "adams_bashforth_moulton_2"};
  for (int i = 0; i < 8; ++i) if (name == names[i]) return i;
  return -1;
}

int color_of(const std::string& name)
{
  static const char* names[] = {"hsl_constant_s", "hsl_constant_l", "hsv_constant_s", "hsv_constant_v", "rgb"};
  for (int i = 0; i < 5; ++i) if (name == names[i]) return i;
  return PARS_COLOR_RGB;
}
}
}

struct pars_gpu_service
{
  int                                  device = 0;
  std::size_t                          budget = 0;
  std::size_t                          in_use = 0;      // running batches' estimates + held results
  std::size_t                          held = 0;        // result bytes held on the device
  std::size_t                          lane_keep = 0;   // scratch a lane keeps between batches
  int                                  max_batch = 64;
  cudaMemPool_t                        pool = nullptr;  // result allocations
  cudaStream_t                         copy_stream = nullptr;   // client copies and frees
  std::vector<std::unique_ptr<pars::curve_store>> spare_stores;   // curve buffers for the next batches
  std::size_t                          spare_bytes = 0;
  pars_gpu_context*                    owner = nullptr;
  std::vector<pars_gpu_context*>       lanes;
  std::vector<std::thread>             workers;
  std::mutex                           mutex;
  std::condition_variable              work, finished;
  std::deque<std::shared_ptr<pars::request>> queue;
  std::map<int64_t, std::shared_ptr<pars::request>> requests;
  std::vector<pars::dataset>           datasets;
  std::map<std::string, int>           dataset_index;
  std::vector<std::unique_ptr<pars::volume_dataset>> volumes;
  std::map<std::string, int>           volume_index;
  bool                                 stopping = false;
  bool                                 spilling = false;
  // instrumentation: per-kernel CUDA-event totals of all lanes and wall time
  // of each batch phase, collected while profile is set
  bool                                 profile = false;
  std::map<std::string, pars::profile_entry> profile_totals;
  int64_t                              next_ticket = 1;
  int                                  running_batches = 0;
  // FTLE requests: steps per warp of each continuous-engine launch (0: each
  // batch runs to completion in one launch; -1: the engine chooses them for
  // launches of about 2 ms)
  std::atomic<int>                     horizon {-1};
};

namespace pars
{
namespace
{
// Keeps spare curve buffers up to a quarter of the budget; frees the rest.
void return_buffers(pars_gpu_service& svc, std::unique_ptr<curve_store> spare)
{
  std::lock_guard<std::mutex> lock(svc.mutex);
  const std::size_t bytes = spare->bytes();
  if (svc.spare_bytes + bytes <= svc.budget / 4)
  {
    svc.spare_bytes += bytes;
    svc.spare_stores.push_back(std::move(spare));
  }
}

// The last request of the batch let go: unbook the bytes and keep the buffers
// for the lanes (no work on them is pending: the batch's stream was drained
// and every client copy is synchronised before its call returns).
curve_store::~curve_store()
{
  if (!svc) return;
  auto spare = std::make_unique<curve_store>();
  spare->vertices = std::move(vertices);
  spare->colors = std::move(colors);
  spare->indices = std::move(indices);
  if (counted)
  {
    {
      std::lock_guard<std::mutex> lock(svc->mutex);
      svc->held -= std::min(svc->held, counted);
      svc->in_use -= std::min(svc->in_use, counted);
    }
    svc->work.notify_all();
  }
  return_buffers(*svc, std::move(spare));
}

// Device bytes a request needs while it runs (a conservative estimate).
std::size_t estimate_bytes(const request& r, const dataset* dp)
{
  std::size_t image = 0;
  if (r.wants_image)
    image = std::size_t(r.s.raytracing_image_size[0]) * std::size_t(r.s.raytracing_image_size[1]) * (sizeof(float4) + 4);
  if (!dp) return image + (1 << 20);
  const dataset& d = *dp;
  if (r.kind == ftle)
  {
    const float scale = 1.0f / float(std::max(1, r.s.seed_generation_stride.empty() ? 1 : r.s.seed_generation_stride[0]));
    std::size_t voxels = 1;
    for (int i = 0; i < 3; ++i) voxels *= std::size_t(std::max(1, int(float(d.shape[i]) * scale)));
    return voxels * (sizeof(float4) + sizeof(float)) + (1 << 20);
  }
  std::size_t seeds = 1;
  for (int i = 0; i < 3; ++i)
  {
    const int stride = r.s.seed_generation_stride.size() > std::size_t(i) ? std::max(1, r.s.seed_generation_stride[i]) : 1;
    seeds *= std::size_t(std::max(0, int(d.size[i] / (d.spacing[i] * float(stride)))));
  }
  const std::size_t slots = seeds * std::size_t(std::max(1, r.s.seed_generation_iterations));
  // padded slots + packed vertices + colours + indices + particle records,
  // and the result (vertices, colours, indices); with an image, the tracer's
  // BVH (about 200 B per segment) and frame buffers
  std::size_t bytes = slots * (sizeof(float4) * 5 + sizeof(int32_t) * 2) + seeds * (sizeof(pars_particle) * 2 + 32) + (1 << 20);
  if (r.wants_image) bytes += slots * 200 + image;
  return bytes;
}

void fail(request& r, int32_t status, const std::string& message)
{
  r.status = status;
  r.error = message;
}

void allocate_result(pars_gpu_service& svc, pars_gpu_context& c, request& r, std::size_t bytes)
{
  void* p = nullptr;
  PARS_CUDA(cudaMallocFromPoolAsync(&p, std::max<std::size_t>(bytes, 256), svc.pool, c.stream));
  r.result = static_cast<char*>(p);
  r.result_bytes = bytes;
}

// Wall time of the phases of one batch, recorded when the service profiles:
// mark() drains the lane's stream and books the time since the previous mark.
struct phase_clock
{
  pars_gpu_service&      svc;
  pars_gpu_context&      c;
  bool                   on;
  clock_type::time_point t = clock_type::now();
  void mark(const char* name)
  {
    if (!on) return;
    cudaStreamSynchronize(c.stream);
    const auto now = clock_type::now();
    std::lock_guard<std::mutex> lock(svc.mutex);
    auto& e = svc.profile_totals[name];
    e.milliseconds += std::chrono::duration<double, std::milli>(now - t).count();
    e.launches += 1;
    t = now;
  }
};

// Returns a request's device result to the pool (stream-ordered on `stream`).
void free_result(request& r, cudaStream_t stream)
{
  if (r.result) cudaFreeAsync(r.result, stream);
  r.result = nullptr;
}

// Copies `bytes` at `offset` of a finished request's result into host `out`,
// from the device (on the service's copy stream) or from its spilled copy.
// The caller holds r.result_mutex and synchronises the copy stream.
void copy_result(pars_gpu_service& svc, const request& r, std::size_t offset, void* out, std::size_t bytes)
{
  if (!out || bytes == 0) return;
  if (r.result)
    PARS_CUDA(cudaMemcpyAsync(out, r.result + offset, bytes, cudaMemcpyDeviceToHost, svc.copy_stream));
  else if (offset + bytes <= r.spilled.size())
    std::memcpy(out, r.spilled.data() + offset, bytes);
  else
    throw error(PARS_ERR_STATE, "the request has no result");
}

// One FTLE request's flow-map job and flow-map buffer (the flow_map_generator
// stage of pipeline::execute_ftle, pars/source/pipeline.cpp:345-409): seeds on
// the dataset's lattice at 1 / stride resolution, flow map of that shape.
struct ftle_work
{
  std::shared_ptr<request> r;
  batch_job_device         job {};
  device_buffer            flow;
};

ftle_work prepare_ftle(pars_gpu_service& svc, pars_gpu_context& c, const std::shared_ptr<request>& rp)
{
  request& r = *rp;
  const dataset& d = svc.datasets[r.dataset];
  const float scale = 1.0f / float(std::max(1, r.s.seed_generation_stride.empty() ? 1 : r.s.seed_generation_stride[0]));
  ftle_work w;
  w.r = rp;
  batch_job_device& j = w.job;
  j.field = d.view;
  j.time.nt = 1; j.time.slice_stride = 0; j.time.t0 = 0.0; j.time.inv_slice_dt = 1.0;
  j.rule = make_step_rule(r.integrator, r.stage_mode, r.s.particle_tracing_step_size);
  j.max_steps = std::max(0, r.s.seed_generation_iterations - 1);
  j.time_begin = 0.0;
  j.seeds = nullptr;
  int fm[3], seeds[3];
  float fm_spacing[3];
  for (int i = 0; i < 3; ++i)
  {
    fm[i] = std::max(1, int(float(d.shape[i]) * scale));
    fm_spacing[i] = d.spacing[i] / scale;
    const float q = d.size[i] / fm_spacing[i];
    seeds[i] = (q > 0.0f && q < 2147483647.0f) ? int(q) : 0;
    r.ftle_shape[i] = fm[i];
  }
  j.seed_count = (long long)seeds[0] * seeds[1] * seeds[2];
  j.ox = d.offset[0]; j.oy = d.offset[1]; j.oz = d.offset[2];
  j.sx = fm_spacing[0]; j.sy = fm_spacing[1]; j.sz = fm_spacing[2];
  j.px = seeds[0]; j.py = seeds[1]; j.pz = seeds[2];
  j.ux = fm[0]; j.uy = fm[1]; j.uz = fm[2];
  w.flow = acquire_buffer(c, sizeof(float4) * (std::size_t)fm[0] * fm[1] * fm[2]);
  if (seeds[0] < fm[0] || seeds[1] < fm[1] || seeds[2] < fm[2])
    PARS_CUDA(cudaMemsetAsync(w.flow.get(), 0xff, w.flow.bytes(), c.stream));
  j.end_positions = w.flow.as<float4>();
  j.end_steps = nullptr;
  return w;
}

// RK4 / Euler requests and the reference's frozen scheme run on the batched
// engine; the other integrators' re-sampled schemes on the per-seed flow-map
// kernel.
bool engine_job(const batch_job_device& j) { return j.rule.frozen || j.rule.scheme == scheme_classic; }

// The per-seed flow-map kernel for one request; returns its steps.
long long per_seed_flow_map(pars_gpu_context& c, const ftle_work& w)
{
  device_buffer counter;
  counter.reserve(sizeof(unsigned long long));
  PARS_CUDA(cudaMemsetAsync(counter.get(), 0, sizeof(unsigned long long), c.stream));
  const batch_job_device& j = w.job;
  const float offset[3] = {j.ox, j.oy, j.oz}, spacing[3] = {j.sx, j.sy, j.sz};
  const int seeds[3] = {j.px, j.py, j.pz}, shape[3] = {j.ux, j.uy, j.uz};
  launch_flow_map(c, j.field, j.rule, w.r->s.seed_generation_iterations, offset, spacing, seeds, shape,
                  w.flow.as<float4>(), counter.as<unsigned long long>());
  unsigned long long steps = 0;
  PARS_CUDA(cudaMemcpyAsync(&steps, counter.get(), sizeof(steps), cudaMemcpyDeviceToHost, c.stream));
  PARS_CUDA(cudaStreamSynchronize(c.stream));
  return (long long)steps;
}

// The ftle_map_generator stage of a request whose flow map is complete: the
// result allocation and the FTLE kernel (queued on the lane's stream).
void finish_ftle(pars_gpu_service& svc, pars_gpu_context& c, ftle_work& w, long long steps)
{
  request& r = *w.r;
  r.steps = steps;
  field_view fv {};
  fv.data = w.flow.as<const float4>();
  fv.nx = r.ftle_shape[0]; fv.ny = r.ftle_shape[1]; fv.nz = r.ftle_shape[2];
  fv.hx = w.job.sx; fv.hy = w.job.sy; fv.hz = w.job.sz;
  const long long voxels = (long long)fv.nx * fv.ny * fv.nz;
  allocate_result(svc, c, r, sizeof(float) * voxels);
  // time = step * iterations in FP32, as pipeline.cpp:403 sets it
  const float time = r.s.particle_tracing_step_size * float(r.s.seed_generation_iterations);
  launch_ftle(c, fv, time == 0.0f ? 1.0 : double(time), r.ftle_mode, reinterpret_cast<float*>(r.result));
}

// FTLE requests run to completion as one batch: flow maps as jobs of one
// batched launch, then the FTLE kernel per request.
void run_ftle_batch(pars_gpu_service& svc, pars_gpu_context& c, std::vector<std::shared_ptr<request>>& batch)
{
  phase_clock clock {svc, c, c.profile};
  std::vector<ftle_work> work;
  for (auto& rp : batch) work.push_back(prepare_ftle(svc, c, rp));
  clock.mark("ftle.setup");
  std::vector<batch_job_device> classic;
  std::vector<std::size_t> classic_of;
  std::vector<long long> steps(work.size(), 0);
  for (std::size_t k = 0; k < work.size(); ++k)
    if (engine_job(work[k].job)) { classic.push_back(work[k].job); classic_of.push_back(k); }
  if (!classic.empty())
  {
    const auto s = run_batch(c, classic, -1);
    for (std::size_t i = 0; i < classic_of.size(); ++i) steps[classic_of[i]] = (long long)s[i];
  }
  for (std::size_t k = 0; k < work.size(); ++k)
    if (!engine_job(work[k].job)) steps[k] = per_seed_flow_map(c, work[k]);
  clock.mark("ftle.advect");
  for (std::size_t k = 0; k < work.size(); ++k) finish_ftle(svc, c, work[k], steps[k]);
  PARS_CUDA(cudaStreamSynchronize(c.stream));
  clock.mark("ftle.field");
  for (auto& w : work) recycle_buffer(c, std::move(w.flow));
}

// FTLE requests through the context's continuous engine: each request's flow
// map is a job of the engine's table, advanced one horizon launch (svc.horizon
// steps per warp, or as many as fill about 2 ms) at a time.  Between launches the requests whose flow maps
// completed get their FTLE field and are handed to the client at once, and
// FTLE requests that arrived meanwhile are admitted (within the budget and
// max_batch in flight) and join the running table.  Admission pauses while
// requests of the other kind wait and no other lane is free, so streamline
// requests are not starved.  Requests leave `batch` as they finish; their
// estimates leave `reserved`.  Returns the number of requests served.
std::size_t run_ftle_continuous(pars_gpu_service& svc, pars_gpu_context& c, std::vector<std::shared_ptr<request>>& batch,
                                std::size_t& reserved)
{
  std::map<long long, ftle_work> in_engine;   // by engine ticket
  std::size_t served = batch.size();
  auto complete = [&](ftle_work& w, long long steps) {
    {
      phase_clock clock {svc, c, c.profile};
      finish_ftle(svc, c, w, steps);
      PARS_CUDA(cudaStreamSynchronize(c.stream));
      clock.mark("ftle.field");
    }
    recycle_buffer(c, std::move(w.flow));
    {
      std::lock_guard<std::mutex> lock(svc.mutex);
      request& r = *w.r;
      svc.in_use -= std::min(svc.in_use, r.estimate);
      reserved -= std::min(reserved, r.estimate);
      if (r.result) { svc.in_use += r.result_bytes; svc.held += r.result_bytes; }
      r.state = done;
      r.finished = clock_type::now();
      const auto it = std::find(batch.begin(), batch.end(), w.r);
      if (it != batch.end()) batch.erase(it);
    }
    svc.finished.notify_all();
    svc.work.notify_all();
  };
  auto start = [&](const std::shared_ptr<request>& rp) {
    ftle_work w = prepare_ftle(svc, c, rp);
    if (engine_job(w.job))
    {
      const long long ticket = engine_submit(c, w.job);
      in_engine.emplace(ticket, std::move(w));
    }
    else complete(w, per_seed_flow_map(c, w));
  };
  try
  {
    const std::vector<std::shared_ptr<request>> first(batch);
    for (const auto& rp : first) start(rp);
    while (engine_open(c) > 0)
    {
      {
        phase_clock clock {svc, c, c.profile};
        const auto finished = engine_advance(c, std::max(0, svc.horizon.load()));
        clock.mark("ftle.advect");
        for (const auto& d : finished)
        {
          auto it = in_engine.find(d.first);
          if (it == in_engine.end()) throw error(PARS_ERR_STATE, "the engine reported an unknown job");
          complete(it->second, (long long)d.second);
          in_engine.erase(it);
        }
      }
      std::vector<std::shared_ptr<request>> joined;
      {
        std::lock_guard<std::mutex> lock(svc.mutex);
        bool other_waiting = false;
        for (const auto& q : svc.queue) other_waiting = other_waiting || q->kind != ftle;
        if (!(other_waiting && svc.running_batches >= int(svc.lanes.size())))
        {
          for (auto it = svc.queue.begin(); it != svc.queue.end() && (int)batch.size() < svc.max_batch;)
          {
            request& r = **it;
            if (r.kind == ftle && svc.in_use + r.estimate <= svc.budget)
            {
              svc.in_use += r.estimate;
              reserved += r.estimate;
              r.state = running;
              r.started = clock_type::now();
              batch.push_back(*it);
              joined.push_back(*it);
              it = svc.queue.erase(it);
            }
            else ++it;
          }
        }
      }
      served += joined.size();
      for (const auto& rp : joined) start(rp);
    }
  }
  catch (...)
  {
    // the table's jobs write into flow maps that are about to be freed
    cudaStreamSynchronize(c.stream);
    c.engine.reset();
    for (auto& entry : in_engine) recycle_buffer(c, std::move(entry.second.flow));
    throw;
  }
  return served;
}

// Streamline requests: one block per request in one tracing round loop, then
// index and colour per batch (pipeline::execute, pipeline.cpp:107-260).
// Returns the bytes of the batch's curve store (shared by its requests).
// Renders one request's curves (its spans of the batch's store) and, when it
// names one, its volume: set_integral_curves, set_volume, set_camera,
// set_image_size, trace and serialize of ray_tracer.cpp on the lane's tracer.
void render_request(pars_gpu_service& svc, pars_gpu_context& c, request& r, const curve_store& store)
{
  if (!c.render) c.render = std::make_unique<render_state>();
  render_state& rs = *c.render;
  std::vector<std::array<long long, 3>> spans;
  for (const auto& s : r.spans) spans.push_back({s.store_vertex_offset, s.store_index_offset, s.index_count});
  render_use_spans(c, rs, store.vertices.as<const float4>(), store.colors.as<const float4>(), store.indices.as<const int>(), spans);
  const float radius = r.s.raytracing_streamline_radius;
  rs.radius = radius != 0.0f ? radius : 1.0f;                       // pipeline.cpp:306
  rs.has_volume = false;
  rs.volume_data = nullptr;
  if (r.volume >= 0)
  {
    const volume_dataset& v = *svc.volumes[r.volume];
    rs.has_volume = true;
    rs.volume_data = v.data.as<const float>();
    for (int i = 0; i < 3; ++i)
    {
      rs.volume_shape[i] = v.shape[i];
      rs.volume_offset[i] = v.offset[i];
      rs.volume_spacing[i] = v.spacing[i];
    }
  }
  render_set_view(rs, r.s.raytracing_camera_position.data(), r.s.raytracing_camera_forward.data(), r.s.raytracing_camera_up.data(),
                  r.s.raytracing_image_size[0], r.s.raytracing_image_size[1]);
  render_frames(c, rs, std::max(0, r.s.raytracing_iterations));
  r.image.resize(std::size_t(rs.width) * rs.height * 4);
  render_encode(c, rs, r.image.data());
  r.image_size[0] = rs.width;
  r.image_size[1] = rs.height;
  rs.vertices = rs.colors = nullptr;       // the store may go once the request lets go
  rs.prims = 0;
  rs.tree_valid = false;
}

std::size_t run_streamline_batch(pars_gpu_service& svc, pars_gpu_context& c, std::vector<std::shared_ptr<request>>& batch, int stage_mode)
{
  phase_clock clock {svc, c, c.profile};
  std::size_t store_bytes = 0;
  // curve buffers left by an earlier batch whose requests have all let go
  {
    std::unique_ptr<curve_store> spare;
    {
      std::lock_guard<std::mutex> lock(svc.mutex);
      if (!svc.spare_stores.empty() && !c.curves.vertices.get())
      {
        spare = std::move(svc.spare_stores.back());
        svc.spare_stores.pop_back();
        svc.spare_bytes -= std::min(svc.spare_bytes, spare->bytes());
      }
    }
    if (spare)
    {
      c.curves.vertices = std::move(spare->vertices);
      c.curves.colors = std::move(spare->colors);
      c.curves.indices = std::move(spare->indices);
    }
  }
  std::vector<trace_block> blocks;
  std::vector<step_rule> rules;
  std::vector<long long> block_count;
  std::vector<int> block_max;
  long long total = 0;
  std::vector<std::array<int, 3>> per_dim;
  for (auto& rp : batch)
  {
    request& r = *rp;
    std::array<int, 3> pd {0, 0, 0};
    long long n = 0;
    trace_block b {};
    for (int f = 0; f < 6; ++f) b.neighbor[f] = -1;
    if (r.trace_curves)
    {
      const dataset& d = svc.datasets[r.dataset];
      n = 1;
      for (int i = 0; i < 3; ++i)
      {
        const int stride = r.s.seed_generation_stride.size() > std::size_t(i) ? std::max(1, r.s.seed_generation_stride[i]) : 1;
        const float st = d.spacing[i] * float(stride);               // pipeline.cpp:117
        const float q = d.size[i] / st;                              // seed_generator.cpp:11
        pd[i] = (q > 0.0f && q < 2147483647.0f) ? int(q) : 0;
        n *= pd[i];
      }
      b.field = d.view;
    }
    else
      b.field = svc.datasets.empty() ? field_view {} : svc.datasets[0].view;   // no particles sample it
    per_dim.push_back(pd);
    blocks.push_back(b);
    rules.push_back(r.trace_curves ? make_step_rule(r.integrator, stage_mode, r.s.particle_tracing_step_size)
                                   : make_step_rule(PARS_RUNGE_KUTTA_4, stage_mode, 1.0f));
    block_count.push_back(n);
    block_max.push_back(n > 0 ? r.s.seed_generation_iterations : 0);
    total += n;
  }
  c.particles_in.reserve(sizeof(pars_particle) * std::max<long long>(total, 1));
  c.block_of.reserve(sizeof(int) * std::max<long long>(total, 1));
  std::vector<int> block_of(std::max<long long>(total, 1));
  long long first = 0;
  for (std::size_t k = 0; k < batch.size(); ++k)
  {
    request& r = *batch[k];
    if (block_count[k] == 0) continue;
    const dataset& d = svc.datasets[r.dataset];
    float stride[3];
    for (int i = 0; i < 3; ++i)
    {
      const int s = r.s.seed_generation_stride.size() > std::size_t(i) ? std::max(1, r.s.seed_generation_stride[i]) : 1;
      stride[i] = d.spacing[i] * float(s);
    }
    launch_seed_generate(c, d.offset, stride, per_dim[k].data(), r.s.seed_generation_iterations, 0,
                         c.particles_in.as<pars_particle>() + first);
    std::fill(block_of.begin() + first, block_of.begin() + first + block_count[k], int(k));
    first += block_count[k];
  }
  if (total > 0)
    PARS_CUDA(cudaMemcpyAsync(c.block_of.get(), block_of.data(), sizeof(int) * total, cudaMemcpyHostToDevice, c.stream));
  device_buffer device_blocks, device_rules;
  device_blocks.reserve(sizeof(trace_block) * blocks.size());
  device_rules.reserve(sizeof(step_rule) * rules.size());
  PARS_CUDA(cudaMemcpyAsync(device_blocks.get(), blocks.data(), sizeof(trace_block) * blocks.size(), cudaMemcpyHostToDevice, c.stream));
  PARS_CUDA(cudaMemcpyAsync(device_rules.get(), rules.data(), sizeof(step_rule) * rules.size(), cudaMemcpyHostToDevice, c.stream));
  clock.mark("streamlines.seed");
  pars_gpu_trace_summary summary {};
  // the launch's kernel follows the most general scheme among the requests'
  // rules; each block then integrates with its own rule
  step_rule launch_rule = rules[0];
  for (const auto& r : rules) if (r.scheme != scheme_classic) launch_rule = r;
  trace_rounds(c, blocks, device_blocks.as<const trace_block>(), total, block_count, block_max, launch_rule, false, &summary,
               device_rules.as<const step_rule>());

  clock.mark("streamlines.trace");
  auto& curves = c.curves;
  // index and colour every request's batches together, each with its mode
  index_batches(c, curves);
  std::vector<color_spec> specs;
  specs.reserve(curves.batches.size());
  for (auto& b : curves.batches)
    specs.push_back(color_spec{batch[b.rank]->color_mode, batch[b.rank]->s.color_generation_free_parameter});
  color_batches(c, curves, specs);
  curves.indexed = curves.colored = true;
  clock.mark("streamlines.index_color");
  // The curve buffers become the batch's store, shared by its requests: each
  // request keeps its batches' ranges in it (no copy); the lane takes fresh
  // buffers for its next batch.
  auto store = std::make_shared<curve_store>();
  store->svc = &svc;
  store->vertices = std::move(curves.vertices);
  store->colors = std::move(curves.colors);
  store->indices = std::move(curves.indices);
  for (const auto& b : curves.batches)
  {
    request& r = *batch[b.rank];
    r.spans.push_back({r.vertex_total, b.vertex_count, r.index_total, b.index_count, b.vertex_offset, b.index_offset});
    r.vertex_total += b.vertex_count;
    r.index_total += b.index_count;
    r.store = store;
  }
  store_bytes = store->bytes();
  curves.batches.clear();
  curves.vertex_total = curves.index_total = 0;
  curves.indexed = curves.colored = false;
  ++curves.generation;
  PARS_CUDA(cudaStreamSynchronize(c.stream));
  clock.mark("streamlines.results");
  // ray tracing (pipeline.cpp:264-337): one image per request that asks for one
  bool rendered = false;
  for (auto& rp : batch)
  {
    if (!rp->wants_image) continue;
    render_request(svc, c, *rp, *store);
    rendered = true;
  }
  if (rendered) clock.mark("streamlines.render");
  // Steps per request: each curve holds its seed, one vertex per step and the
  // termination vertex (remaining_iterations >= 2; one block, one round).
  for (std::size_t k = 0; k < batch.size(); ++k)
    batch[k]->steps = batch[k]->s.seed_generation_iterations >= 2 ? std::max(0LL, (long long)batch[k]->vertex_total - 2 * block_count[k]) : 0;
  (void)summary;
  return store_bytes;
}

// Moves every finished request's device result to host memory (the queue is
// blocked on held results and no batch runs); returns the FTLE bytes freed
// (curve stores unbook themselves when their last request lets go).
std::size_t spill_results(pars_gpu_service& svc, pars_gpu_context& c, const std::vector<std::shared_ptr<request>>& finished)
{
  std::size_t freed = 0;
  for (auto& rp : finished)
  {
    request& r = *rp;
    std::lock_guard<std::mutex> lock(r.result_mutex);
    if (r.released) continue;
    if (r.store)
    {
      // the request's own layout: vertices, colours, indices
      const std::size_t colors = sizeof(float4) * r.vertex_total, indices = 2 * colors;
      r.spilled.resize(indices + sizeof(int32_t) * r.index_total);
      for (const auto& sp : r.spans)
      {
        if (sp.vertex_count)
        {
          PARS_CUDA(cudaMemcpyAsync(r.spilled.data() + sizeof(float4) * sp.vertex_offset,
                                    r.store->vertices.as<float4>() + sp.store_vertex_offset, sizeof(float4) * sp.vertex_count,
                                    cudaMemcpyDeviceToHost, c.stream));
          PARS_CUDA(cudaMemcpyAsync(r.spilled.data() + colors + sizeof(float4) * sp.vertex_offset,
                                    r.store->colors.as<float4>() + sp.store_vertex_offset, sizeof(float4) * sp.vertex_count,
                                    cudaMemcpyDeviceToHost, c.stream));
        }
        if (sp.index_count)
          PARS_CUDA(cudaMemcpyAsync(r.spilled.data() + indices + sizeof(int32_t) * sp.index_offset,
                                    r.store->indices.as<int32_t>() + sp.store_index_offset, sizeof(int32_t) * sp.index_count,
                                    cudaMemcpyDeviceToHost, c.stream));
      }
      PARS_CUDA(cudaStreamSynchronize(c.stream));
      r.store.reset();
      continue;
    }
    if (!r.result) continue;
    r.spilled.resize(r.result_bytes);
    if (r.result_bytes)
      PARS_CUDA(cudaMemcpyAsync(r.spilled.data(), r.result, r.result_bytes, cudaMemcpyDeviceToHost, c.stream));
    PARS_CUDA(cudaStreamSynchronize(c.stream));
    free_result(r, c.stream);
    freed += r.result_bytes;
  }
  PARS_CUDA(cudaStreamSynchronize(c.stream));
  return freed;
}

// Returns scratch beyond what a lane keeps between batches.
void trim_lane(pars_gpu_service& svc, pars_gpu_context& c)
{
  if ((std::size_t)c.held_bytes() > svc.lane_keep) release_scratch(c);
}

void worker(pars_gpu_service* svc, int lane)
{
  pars_gpu_context& c = *svc->lanes[lane];
  cudaSetDevice(svc->device);
  for (;;)
  {
    std::vector<std::shared_ptr<request>> batch;
    int kind = -1, stage_mode = -1;
    std::size_t reserved = 0;
    {
      std::unique_lock<std::mutex> lock(svc->mutex);
      for (;;)
      {
        if (svc->stopping && svc->queue.empty()) return;
        // Admit, in arrival order, requests of the first admissible request's
        // kind (and stage mode) that fit into the remaining budget.
        for (auto it = svc->queue.begin(); it != svc->queue.end() && (int)batch.size() < svc->max_batch;)
        {
          request& r = **it;
          const bool same = kind < 0 || (r.kind == kind && r.stage_mode == stage_mode);
          if (same && svc->in_use + reserved + r.estimate <= svc->budget)
          {
            kind = r.kind;
            stage_mode = r.stage_mode;
            reserved += r.estimate;
            r.state = running;
            r.started = clock_type::now();
            batch.push_back(*it);
            it = svc->queue.erase(it);
          }
          else ++it;
        }
        if (!batch.empty()) break;
        if (!svc->queue.empty() && svc->running_batches == 0 && svc->held > 0 && !svc->spilling)
        {
          // Nothing fits because finished results hold the budget: move them
          // to host memory (the client still collects them the same way).
          std::vector<std::shared_ptr<request>> finished;
          for (auto& t : svc->requests) if (t.second->state == done) finished.push_back(t.second);
          svc->spilling = true;
          lock.unlock();
          std::size_t freed = 0;
          try { freed = spill_results(*svc, c, finished); } catch (const std::exception&) {}
          lock.lock();
          svc->spilling = false;
          svc->held -= std::min(svc->held, freed);
          svc->in_use -= std::min(svc->in_use, freed);
          continue;
        }
        svc->work.wait(lock);
      }
      svc->in_use += reserved;
      ++svc->running_batches;
      c.profile = svc->profile;
    }
    bool ok = true;
    std::size_t store_bytes = 0;
    std::size_t served = batch.size();
    try
    {
      if (kind == ftle && svc->horizon.load() != 0) served = run_ftle_continuous(*svc, c, batch, reserved);
      else if (kind == ftle) run_ftle_batch(*svc, c, batch);
      else store_bytes = run_streamline_batch(*svc, c, batch, stage_mode);
    }
    catch (const error& e) { ok = false; for (auto& r : batch) fail(*r, e.status, e.what()); }
    catch (const std::exception& e) { ok = false; for (auto& r : batch) fail(*r, PARS_ERR_STATE, e.what()); }
    if (!ok)
    {
      for (auto& r : batch) { free_result(*r, c.stream); r->result_bytes = 0; r->spans.clear(); r->store.reset(); }
      cudaStreamSynchronize(c.stream);
    }
    {
      phase_clock clock {*svc, c, c.profile};
      try { trim_lane(*svc, c); } catch (const std::exception&) {}
      clock.mark("lane.trim");
    }
    if (c.profile)
    {
      std::map<std::string, profile_entry> kernels;
      try { take_profile(c, kernels); } catch (const std::exception&) {}
      std::lock_guard<std::mutex> lock(svc->mutex);
      for (auto& k : kernels)
      {
        svc->profile_totals[k.first].milliseconds += k.second.milliseconds;
        svc->profile_totals[k.first].launches += k.second.launches;
      }
      auto& b = svc->profile_totals[kind == ftle ? "batches.ftle" : "batches.streamlines"];
      b.launches += 1;
      b.milliseconds += double(served);   // requests in these batches
    }
    {
      std::lock_guard<std::mutex> lock(svc->mutex);
      svc->in_use -= reserved;
      for (auto& r : batch)
        if (r->result) { svc->in_use += r->result_bytes; svc->held += r->result_bytes; }
      if (ok && store_bytes && !batch.empty() && batch[0]->store)
      {
        batch[0]->store->counted = store_bytes;
        svc->in_use += store_bytes;
        svc->held += store_bytes;
      }
      --svc->running_batches;
      for (auto& r : batch) { r->state = done; r->finished = clock_type::now(); }
    }
    svc->finished.notify_all();
    svc->work.notify_all();
  }
}

std::shared_ptr<request> find_request(pars_gpu_service* svc, int64_t ticket)
{
  auto it = svc->requests.find(ticket);
  if (it == svc->requests.end()) throw error(PARS_ERR_NOT_FOUND, "no request with ticket " + std::to_string(ticket));
  return it->second;
}

// A field uploaded into the owner context becomes a dataset.
void register_dataset(pars_gpu_service* svc, const char* name, int32_t handle)
{
  PARS_CUDA(cudaSetDevice(svc->device));
  dataset d;
  d.name = name;
  d.field = handle;
  {
    std::lock_guard<std::mutex> owner_lock(svc->owner->mutex);
    auto& f = *svc->owner->fields.at(handle);
    d.view = f.view();
    for (int i = 0; i < 3; ++i) { d.shape[i] = f.shape[i]; d.offset[i] = f.offset[i]; d.size[i] = f.size[i]; d.spacing[i] = f.spacing[i]; }
    PARS_CUDA(cudaStreamSynchronize(svc->owner->stream));
  }
  std::lock_guard<std::mutex> lock(svc->mutex);
  svc->dataset_index[d.name] = int(svc->datasets.size());
  svc->datasets.push_back(d);
}

template <typename body_type>
int32_t service_guard(pars_gpu_service* svc, body_type&& body)
{
  if (!svc) return PARS_ERR_INVALID_ARGUMENT;
  try { body(); return PARS_OK; }
  catch (const error& e) { return e.status; }
  catch (const std::bad_alloc&) { return PARS_ERR_OUT_OF_MEMORY; }
  catch (const std::exception&) { return PARS_ERR_STATE; }
}
}
}

using namespace pars;

#pragma GCC visibility push(default)
extern "C" {

int32_t pars_gpu_settings_from_json(const char* json, int64_t length, uint8_t* message, int64_t capacity, int64_t* message_length)
{
  if ((!json && length > 0) || length < 0 || !message_length) return PARS_ERR_INVALID_ARGUMENT;
  try
  {
    settings s;
    std::string problem;
    if (!settings_from_json(json, std::size_t(length), s, problem)) return PARS_ERR_INVALID_ARGUMENT;
    const std::vector<uint8_t> bytes = encode_settings(s);
    *message_length = int64_t(bytes.size());
    if (!message) return PARS_OK;
    if (capacity < int64_t(bytes.size())) return PARS_ERR_INVALID_ARGUMENT;
    if (!bytes.empty()) std::memcpy(message, bytes.data(), bytes.size());
    return PARS_OK;
  }
  catch (const std::bad_alloc&) { return PARS_ERR_OUT_OF_MEMORY; }
  catch (...) { return PARS_ERR_STATE; }
}

int32_t pars_gpu_settings_decode(const uint8_t* bytes, int64_t length, pars_gpu_settings_summary* out)
{
  if ((!bytes && length > 0) || length < 0 || !out) return PARS_ERR_INVALID_ARGUMENT;
  settings s;
  std::string message;
  if (!decode_settings(bytes, std::size_t(length), s, message)) return PARS_ERR_INVALID_ARGUMENT;
  std::memset(out, 0, sizeof(*out));
  std::snprintf(out->mode, sizeof(out->mode), "%s", s.mode.c_str());
  std::snprintf(out->dataset_filepath, sizeof(out->dataset_filepath), "%s", s.dataset_filepath.c_str());
  std::snprintf(out->particle_tracing_integrator, sizeof(out->particle_tracing_integrator), "%s", s.particle_tracing_integrator.c_str());
  std::snprintf(out->color_generation_mode, sizeof(out->color_generation_mode), "%s", s.color_generation_mode.c_str());
  for (int i = 0; i < 3 && i < (int)s.seed_generation_stride.size(); ++i) out->seed_generation_stride[i] = s.seed_generation_stride[i];
  out->seed_generation_iterations = s.seed_generation_iterations;
  out->particle_tracing_step_size = s.particle_tracing_step_size;
  out->particle_tracing_load_balance = s.particle_tracing_load_balance ? 1 : 0;
  out->color_generation_free_parameter = s.color_generation_free_parameter;
  for (int i = 0; i < 3 && i < (int)s.raytracing_camera_position.size(); ++i) out->raytracing_camera_position[i] = s.raytracing_camera_position[i];
  for (int i = 0; i < 2 && i < (int)s.raytracing_image_size.size(); ++i) out->raytracing_image_size[i] = s.raytracing_image_size[i];
  out->raytracing_streamline_radius = s.raytracing_streamline_radius;
  out->raytracing_iterations = s.raytracing_iterations;
  return PARS_OK;
}

int32_t pars_gpu_service_create(pars_gpu_service** service, int32_t device, int64_t budget_bytes, int32_t lanes, int32_t max_batch)
{
  if (!service || budget_bytes <= 0 || lanes < 1 || lanes > 16 || max_batch < 1) return PARS_ERR_INVALID_ARGUMENT;
  *service = nullptr;
  auto* svc = new (std::nothrow) pars_gpu_service();
  if (!svc) return PARS_ERR_OUT_OF_MEMORY;
  svc->device = device;
  svc->budget = std::size_t(budget_bytes);
  svc->lane_keep = svc->budget / (4 * std::size_t(lanes));
  svc->max_batch = max_batch;
  int32_t status = pars_gpu_create(&svc->owner, device);
  if (status == PARS_OK)
  {
    // A pool that keeps up to a quarter of the budget of freed results mapped.
    cudaMemPoolProps props {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    uint64_t keep = svc->budget / 4;
    if (cudaSetDevice(device) != cudaSuccess || cudaMemPoolCreate(&svc->pool, &props) != cudaSuccess ||
        cudaMemPoolSetAttribute(svc->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess ||
        cudaStreamCreateWithFlags(&svc->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    {
      (void)cudaGetLastError();
      status = PARS_ERR_CUDA;
    }
  }
  for (int i = 0; status == PARS_OK && i < lanes; ++i)
  {
    pars_gpu_context* c = nullptr;
    status = pars_gpu_create(&c, device);
    if (status == PARS_OK) svc->lanes.push_back(c);
  }
  if (status != PARS_OK)
  {
    for (auto* c : svc->lanes) pars_gpu_destroy(c);
    if (svc->owner) pars_gpu_destroy(svc->owner);
    if (svc->copy_stream) cudaStreamDestroy(svc->copy_stream);
    if (svc->pool) cudaMemPoolDestroy(svc->pool);
    delete svc;
    return status;
  }
  for (int i = 0; i < lanes; ++i) svc->workers.emplace_back(worker, svc, i);
  *service = svc;
  return PARS_OK;
}

int32_t pars_gpu_service_set_horizon(pars_gpu_service* svc, int32_t iterations)
{
  return service_guard(svc, [&] {
    PARS_REQUIRE(iterations >= -1, "iterations must be >= -1");
    svc->horizon.store(iterations);
  });
}

int32_t pars_gpu_service_destroy(pars_gpu_service* svc)
{
  if (!svc) return PARS_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lock(svc->mutex);
    svc->stopping = true;
  }
  svc->work.notify_all();
  for (auto& t : svc->workers) t.join();
  cudaSetDevice(svc->device);
  std::vector<std::shared_ptr<request>> left;
  for (auto& t : svc->requests) left.push_back(t.second);
  svc->requests.clear();
  for (auto& r : left)
  {
    std::lock_guard<std::mutex> lock(r->result_mutex);
    free_result(*r, svc->copy_stream);
    r->store.reset();
  }
  left.clear();
  cudaStreamSynchronize(svc->copy_stream);
  svc->spare_stores.clear();
  for (auto* c : svc->lanes) pars_gpu_destroy(c);
  pars_gpu_destroy(svc->owner);
  cudaStreamDestroy(svc->copy_stream);
  cudaMemPoolDestroy(svc->pool);
  delete svc;
  return PARS_OK;
}

int32_t pars_gpu_service_add_dataset(pars_gpu_service* svc, const char* name, const float* xyz, const int32_t shape[3],
                                     const float offset[3], const float size[3], const float spacing[3])
{
  return service_guard(svc, [&] {
    PARS_REQUIRE(name && xyz, "name and xyz are required");
    int32_t handle = -1;
    const int32_t status = pars_gpu_field_upload(svc->owner, xyz, shape, offset, size, spacing, &handle);
    if (status != PARS_OK) throw error(status, pars_gpu_last_error(svc->owner));
    register_dataset(svc, name, handle);
  });
}

int32_t pars_gpu_service_add_dataset_device(pars_gpu_service* svc, const char* name, const float* device_xyz, const int32_t shape[3],
                                            const float offset[3], const float size[3], const float spacing[3])
{
  return service_guard(svc, [&] {
    PARS_REQUIRE(name && device_xyz, "name and device_xyz are required");
    int32_t handle = -1;
    const int32_t status = pars_gpu_field_upload_device(svc->owner, device_xyz, shape, offset, size, spacing, &handle);
    if (status != PARS_OK) throw error(status, pars_gpu_last_error(svc->owner));
    register_dataset(svc, name, handle);
  });
}

namespace
{
void add_volume(pars_gpu_service* svc, const char* name, const float* values, bool device, const int32_t shape[3],
                const float offset[3], const float spacing[3])
{
  PARS_REQUIRE(name && values && shape && offset && spacing, "name, values, shape, offset and spacing are required");
  auto v = std::make_unique<volume_dataset>();
  std::size_t count = 1;
  for (int i = 0; i < 3; ++i)
  {
    PARS_REQUIRE(shape[i] >= 2 && spacing[i] > 0.0f, "volume extents must be >= 2 and spacings positive");
    v->shape[i] = shape[i];
    v->offset[i] = offset[i];
    v->spacing[i] = spacing[i];
    count *= std::size_t(shape[i]);
  }
  PARS_CUDA(cudaSetDevice(svc->device));
  v->data.reserve(sizeof(float) * count);
  PARS_CUDA(cudaMemcpy(v->data.get(), values, sizeof(float) * count, device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
  std::lock_guard<std::mutex> lock(svc->mutex);
  PARS_REQUIRE(svc->volume_index.count(name) == 0, "a volume with this name exists");
  svc->volume_index[name] = int(svc->volumes.size());
  svc->volumes.push_back(std::move(v));
}
}

int32_t pars_gpu_service_add_volume(pars_gpu_service* svc, const char* name, const float* values, const int32_t shape[3],
                                    const float offset[3], const float spacing[3])
{
  return service_guard(svc, [&] { add_volume(svc, name, values, false, shape, offset, spacing); });
}

int32_t pars_gpu_service_add_volume_device(pars_gpu_service* svc, const char* name, const float* device_values,
                                           const int32_t shape[3], const float offset[3], const float spacing[3])
{
  return service_guard(svc, [&] { add_volume(svc, name, device_values, true, shape, offset, spacing); });
}

int32_t pars_gpu_service_submit(pars_gpu_service* svc, const uint8_t* message, int64_t length, int64_t* ticket)
{
  return service_guard(svc, [&] {
    PARS_REQUIRE(ticket && (message || length == 0) && length >= 0, "message and ticket are required");
    auto r = std::make_shared<request>();
    std::string problem;
    if (!decode_settings(message, std::size_t(length), r->s, problem)) throw error(PARS_ERR_INVALID_ARGUMENT, problem);
    // mode substrings as pipeline.cpp:21-23 and service.cpp:79 read them
    const std::string& mode = r->s.mode;
    r->kind = mode.find("ftle") != std::string::npos ? ftle : streamlines;
    if (mode.find("fractional_anisotropy") != std::string::npos) r->ftle_mode = PARS_FTLE_FRACTIONAL_ANISOTROPY;
    r->stage_mode = mode.find("reference") != std::string::npos ? PARS_STAGES_FROZEN : PARS_STAGES_RESAMPLED;
    const bool with_volume = mode.find("volume") != std::string::npos;
    if (r->kind == streamlines)
    {
      // "volume" without "streamlines" renders the volume alone (pipeline.cpp:21-22, 76-92)
      r->trace_curves = mode.find("streamlines") != std::string::npos || !with_volume;
      const auto& size = r->s.raytracing_image_size;
      r->wants_image = mode.find("export") == std::string::npos && size.size() >= 2 && size[0] > 0 && size[1] > 0;
      if (r->wants_image)
      {
        PARS_REQUIRE((long long)size[0] * size[1] <= (1LL << 28), "raytracing_image_size too large");
        PARS_REQUIRE(r->s.raytracing_camera_position.size() >= 3 && r->s.raytracing_camera_forward.size() >= 3 &&
                     r->s.raytracing_camera_up.size() >= 3, "ray tracing needs camera position, forward and up");
      }
      PARS_REQUIRE(r->trace_curves || r->wants_image, "a volume request needs an image size");
    }
    if (r->trace_curves || r->kind == ftle)
    {
      r->integrator = integrator_of(r->s.particle_tracing_integrator);
      if (r->integrator < 0) throw error(PARS_ERR_UNSUPPORTED, "unknown integrator '" + r->s.particle_tracing_integrator + "'");
      PARS_REQUIRE(r->s.particle_tracing_step_size != 0.0f, "particle_tracing_step_size must be non-zero");
    }
    r->color_mode = color_of(r->s.color_generation_mode);
    std::unique_lock<std::mutex> lock(svc->mutex);
    if (r->trace_curves || r->kind == ftle)
    {
      auto d = svc->dataset_index.find(r->s.dataset_filepath);
      if (d == svc->dataset_index.end()) throw error(PARS_ERR_NOT_FOUND, "unknown dataset '" + r->s.dataset_filepath + "'");
      r->dataset = d->second;
    }
    if (r->wants_image && with_volume)
    {
      auto v = svc->volume_index.find(r->s.volume_type);
      if (v == svc->volume_index.end()) throw error(PARS_ERR_NOT_FOUND, "unknown volume '" + r->s.volume_type + "'");
      r->volume = v->second;
    }
    r->estimate = estimate_bytes(*r, r->dataset >= 0 ? &svc->datasets[r->dataset] : nullptr);
    if (r->estimate > svc->budget) throw error(PARS_ERR_BUDGET, "request needs more device memory than the service budget");
    r->ticket = svc->next_ticket++;
    r->submitted = clock_type::now();
    svc->requests[r->ticket] = r;
    svc->queue.push_back(r);
    *ticket = r->ticket;
    lock.unlock();
    svc->work.notify_all();
  });
}

int32_t pars_gpu_service_wait(pars_gpu_service* svc, int64_t ticket, int32_t timeout_ms, int32_t* state)
{
  return service_guard(svc, [&] {
    std::unique_lock<std::mutex> lock(svc->mutex);
    auto r = find_request(svc, ticket);
    if (timeout_ms != 0)
      svc->finished.wait_for(lock, std::chrono::milliseconds(timeout_ms < 0 ? 24 * 3600 * 1000 : timeout_ms),
                             [&] { return r->state == done; });
    if (state) *state = r->state;
    if (r->state == done && r->status != PARS_OK) throw error(r->status, r->error);
  });
}

int32_t pars_gpu_service_result_info(pars_gpu_service* svc, int64_t ticket, pars_gpu_request_info* info)
{
  return service_guard(svc, [&] {
    PARS_REQUIRE(info, "info is required");
    std::lock_guard<std::mutex> lock(svc->mutex);
    auto r = find_request(svc, ticket);
    std::memset(info, 0, sizeof(*info));
    info->state = r->state;
    info->status = r->status;
    info->kind = r->kind;
    info->batches = r->state == done ? (int64_t)r->spans.size() : 0;
    for (int i = 0; i < 3; ++i) info->ftle_shape[i] = r->ftle_shape[i];
    info->steps = r->steps;
    if (r->state == done) { info->image_size[0] = r->image_size[0]; info->image_size[1] = r->image_size[1]; }
    using ms = std::chrono::duration<double, std::milli>;
    if (r->state >= running) info->queue_ms = ms(r->started - r->submitted).count();
    if (r->state == done) { info->run_ms = ms(r->finished - r->started).count(); info->latency_ms = ms(r->finished - r->submitted).count(); }
  });
}

int32_t pars_gpu_service_result_batch(pars_gpu_service* svc, int64_t ticket, int64_t batch, int64_t* vertices, int64_t* indices,
                                      float* vertex_data, float* color_data, int32_t* index_data)
{
  return service_guard(svc, [&] {
    std::shared_ptr<request> r;
    {
      std::lock_guard<std::mutex> lock(svc->mutex);
      r = find_request(svc, ticket);
      if (r->state != done) throw error(PARS_ERR_STATE, "request has not finished");
    }
    std::lock_guard<std::mutex> lock(r->result_mutex);
    if (r->released) throw error(PARS_ERR_NOT_FOUND, "request was released");
    PARS_REQUIRE(r->kind == streamlines, "not a streamline request");
    PARS_REQUIRE(batch >= 0 && batch < (int64_t)r->spans.size(), "batch out of range");
    const curve_span& s = r->spans[batch];
    if (vertices) *vertices = s.vertex_count;
    if (indices) *indices = s.index_count;
    PARS_CUDA(cudaSetDevice(svc->device));
    if (r->store)
    {
      // straight from the batch's curve store
      auto d2h = [&](void* out, const void* in, std::size_t bytes) {
        if (out && bytes) PARS_CUDA(cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToHost, svc->copy_stream));
      };
      d2h(vertex_data, r->store->vertices.as<float4>() + s.store_vertex_offset, sizeof(float4) * s.vertex_count);
      d2h(color_data, r->store->colors.as<float4>() + s.store_vertex_offset, sizeof(float4) * s.vertex_count);
      d2h(index_data, r->store->indices.as<int32_t>() + s.store_index_offset, sizeof(int32_t) * s.index_count);
    }
    else
    {
      const std::size_t colors = sizeof(float4) * r->vertex_total, index_base = 2 * colors;
      copy_result(*svc, *r, sizeof(float4) * s.vertex_offset, vertex_data, sizeof(float4) * s.vertex_count);
      copy_result(*svc, *r, colors + sizeof(float4) * s.vertex_offset, color_data, sizeof(float4) * s.vertex_count);
      copy_result(*svc, *r, index_base + sizeof(int32_t) * s.index_offset, index_data, sizeof(int32_t) * s.index_count);
    }
    PARS_CUDA(cudaStreamSynchronize(svc->copy_stream));
  });
}

int32_t pars_gpu_service_result_ftle(pars_gpu_service* svc, int64_t ticket, float* values)
{
  return service_guard(svc, [&] {
    PARS_REQUIRE(values, "values is required");
    std::shared_ptr<request> r;
    {
      std::lock_guard<std::mutex> lock(svc->mutex);
      r = find_request(svc, ticket);
      if (r->state != done) throw error(PARS_ERR_STATE, "request has not finished");
    }
    std::lock_guard<std::mutex> lock(r->result_mutex);
    if (r->released) throw error(PARS_ERR_NOT_FOUND, "request was released");
    PARS_REQUIRE(r->kind == ftle, "not an FTLE request");
    PARS_CUDA(cudaSetDevice(svc->device));
    copy_result(*svc, *r, 0, values, r->result_bytes);
    PARS_CUDA(cudaStreamSynchronize(svc->copy_stream));
  });
}

int32_t pars_gpu_service_result_image(pars_gpu_service* svc, int64_t ticket, uint8_t* rgba, int32_t size[2])
{
  return service_guard(svc, [&] {
    std::shared_ptr<request> r;
    {
      std::lock_guard<std::mutex> lock(svc->mutex);
      r = find_request(svc, ticket);
      if (r->state != done) throw error(PARS_ERR_STATE, "request has not finished");
    }
    std::lock_guard<std::mutex> lock(r->result_mutex);
    if (r->released) throw error(PARS_ERR_NOT_FOUND, "request was released");
    if (size) { size[0] = r->image_size[0]; size[1] = r->image_size[1]; }
    if (rgba && !r->image.empty()) std::memcpy(rgba, r->image.data(), r->image.size());
  });
}

int32_t pars_gpu_service_release(pars_gpu_service* svc, int64_t ticket)
{
  return service_guard(svc, [&] {
    std::shared_ptr<request> r;
    {
      std::lock_guard<std::mutex> lock(svc->mutex);
      r = find_request(svc, ticket);
      if (r->state == running) throw error(PARS_ERR_STATE, "request is running");
      if (r->state == queued)
      {
        svc->queue.erase(std::remove(svc->queue.begin(), svc->queue.end(), r), svc->queue.end());
        r->status = PARS_ERR_CANCELLED;
      }
      svc->requests.erase(ticket);
    }
    std::size_t freed = 0;
    {
      std::lock_guard<std::mutex> lock(r->result_mutex);
      r->released = true;
      if (r->result)
      {
        PARS_CUDA(cudaSetDevice(svc->device));
        free_result(*r, svc->copy_stream);
        freed = r->result_bytes;
      }
      r->store.reset();   // the last request of its batch hands the curve buffers back
      std::vector<char>().swap(r->spilled);
    }
    if (freed)
    {
      {
        std::lock_guard<std::mutex> lock(svc->mutex);
        svc->held -= std::min(svc->held, freed);
        svc->in_use -= std::min(svc->in_use, freed);
      }
      svc->work.notify_all();
    }
  });
}

int32_t pars_gpu_service_profile_enable(pars_gpu_service* svc, int32_t enable)
{
  return service_guard(svc, [&] {
    std::lock_guard<std::mutex> lock(svc->mutex);
    svc->profile = enable != 0;
    if (svc->profile) svc->profile_totals.clear();
  });
}

int32_t pars_gpu_service_profile_get(pars_gpu_service* svc, const char* name, double* milliseconds, int64_t* count)
{
  return service_guard(svc, [&] {
    PARS_REQUIRE(name, "name is required");
    std::lock_guard<std::mutex> lock(svc->mutex);
    auto it = svc->profile_totals.find(name);
    if (milliseconds) *milliseconds = it == svc->profile_totals.end() ? 0.0 : it->second.milliseconds;
    if (count) *count = it == svc->profile_totals.end() ? 0 : it->second.launches;
  });
}

}
#pragma GCC visibility pop
