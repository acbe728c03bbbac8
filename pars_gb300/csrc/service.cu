// pars_service-compatible request service with continuous batching.
//
// The reference's service (pars/source/service.cpp:20-69) receives one binary
// `settings` message at a time, runs pipeline::execute on it and replies.
// Here requests are queued as they arrive and several lanes (each a context
// with its own CUDA stream and worker thread) take batches from the queue:
//  * admission: a request enters a batch only while the device memory the
//    running batches are estimated to need stays within the budget; memory is
//    returned when a batch completes (its results are then on the host);
//  * batching: a lane takes every queued request of the same kind that fits
//    (up to max_batch) and runs them as one launch — FTLE requests as jobs of
//    the persistent batched advection engine, streamline requests as blocks of
//    one tracing round loop;
//  * overlap: while one lane's batch runs, another lane admits the requests
//    that arrived meanwhile and launches them on its own stream.
// Datasets (the requests' dataset_filepath) are fields registered with the
// service and kept resident across requests.
#include <algorithm>
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
  // results on the host
  std::vector<std::vector<float4>>  vertices, colors;
  std::vector<std::vector<int32_t>> indices;
  std::vector<float> ftle_values;
  int                ftle_shape[3] = {0, 0, 0};
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
  std::size_t                          in_use = 0;
  int                                  max_batch = 64;
  pars_gpu_context*                    owner = nullptr;
  std::vector<pars_gpu_context*>       lanes;
  std::vector<std::thread>             workers;
  std::mutex                           mutex;
  std::condition_variable              work, finished;
  std::deque<std::shared_ptr<pars::request>> queue;
  std::map<int64_t, std::shared_ptr<pars::request>> requests;
  std::vector<pars::dataset>           datasets;
  std::map<std::string, int>           dataset_index;
  bool                                 stopping = false;
  int64_t                              next_ticket = 1;
  int                                  running_batches = 0;
};

namespace pars
{
namespace
{
// Device bytes a request needs while it runs (a conservative estimate).
std::size_t estimate_bytes(const request& r, const dataset& d)
{
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
  // padded slots + packed vertices + colours + indices + particle records
  return slots * (sizeof(float4) * 3 + sizeof(int32_t)) + seeds * (sizeof(pars_particle) * 2 + 32) + (1 << 20);
}

void fail(request& r, int32_t status, const std::string& message)
{
  r.status = status;
  r.error = message;
}

// FTLE requests: flow maps as jobs of one batched launch, then the FTLE kernel
// per request (pipeline::execute_ftle, pars/source/pipeline.cpp:345-409).
void run_ftle_batch(pars_gpu_service& svc, pars_gpu_context& c, std::vector<std::shared_ptr<request>>& batch)
{
  std::vector<batch_job_device> jobs;
  std::vector<device_buffer> flows;
  std::vector<int> shapes;
  for (auto& rp : batch)
  {
    request& r = *rp;
    const dataset& d = svc.datasets[r.dataset];
    const float scale = 1.0f / float(std::max(1, r.s.seed_generation_stride.empty() ? 1 : r.s.seed_generation_stride[0]));
    batch_job_device j {};
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
    flows.push_back(acquire_buffer(c, sizeof(float4) * (std::size_t)fm[0] * fm[1] * fm[2]));
    if (seeds[0] < fm[0] || seeds[1] < fm[1] || seeds[2] < fm[2])
      PARS_CUDA(cudaMemsetAsync(flows.back().get(), 0xff, flows.back().bytes(), c.stream));
    j.end_positions = flows.back().as<float4>();
    j.end_steps = nullptr;
    jobs.push_back(j);
  }
  const auto steps = run_batch(c, jobs, 0, -1);
  device_buffer values;
  for (std::size_t k = 0; k < batch.size(); ++k)
  {
    request& r = *batch[k];
    r.steps = (long long)steps[k];
    field_view fv {};
    fv.data = flows[k].as<const float4>();
    fv.nx = r.ftle_shape[0]; fv.ny = r.ftle_shape[1]; fv.nz = r.ftle_shape[2];
    fv.hx = jobs[k].sx; fv.hy = jobs[k].sy; fv.hz = jobs[k].sz;
    const long long voxels = (long long)fv.nx * fv.ny * fv.nz;
    values.reserve(sizeof(float) * voxels);
    // time = step * iterations in FP32, as pipeline.cpp:403 sets it
    const float time = r.s.particle_tracing_step_size * float(r.s.seed_generation_iterations);
    launch_ftle(c, fv, time == 0.0f ? 1.0 : double(time), r.ftle_mode, values.as<float>());
    r.ftle_values.resize(voxels);
    PARS_CUDA(cudaMemcpyAsync(r.ftle_values.data(), values.get(), sizeof(float) * voxels, cudaMemcpyDeviceToHost, c.stream));
  }
  PARS_CUDA(cudaStreamSynchronize(c.stream));
  for (auto& f : flows) recycle_buffer(c, std::move(f));
}

// Streamline requests: one block per request in one tracing round loop, then
// index and colour per batch (pipeline::execute, pipeline.cpp:107-260).
void run_streamline_batch(pars_gpu_service& svc, pars_gpu_context& c, std::vector<std::shared_ptr<request>>& batch, int stage_mode)
{
  std::vector<trace_block> blocks;
  std::vector<step_rule> rules;
  std::vector<long long> block_count;
  std::vector<int> block_max;
  long long total = 0;
  std::vector<std::array<int, 3>> per_dim;
  for (auto& rp : batch)
  {
    request& r = *rp;
    const dataset& d = svc.datasets[r.dataset];
    std::array<int, 3> pd;
    long long n = 1;
    for (int i = 0; i < 3; ++i)
    {
      const int stride = r.s.seed_generation_stride.size() > std::size_t(i) ? std::max(1, r.s.seed_generation_stride[i]) : 1;
      const float st = d.spacing[i] * float(stride);               // pipeline.cpp:117
      const float q = d.size[i] / st;                              // seed_generator.cpp:11
      pd[i] = (q > 0.0f && q < 2147483647.0f) ? int(q) : 0;
      n *= pd[i];
    }
    per_dim.push_back(pd);
    trace_block b;
    b.field = d.view;
    for (int f = 0; f < 6; ++f) b.neighbor[f] = -1;
    blocks.push_back(b);
    rules.push_back(make_step_rule(r.integrator, stage_mode, r.s.particle_tracing_step_size));
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
  pars_gpu_trace_summary summary {};
  trace_rounds(c, blocks, device_blocks.as<const trace_block>(), total, block_count, block_max, rules[0], false, &summary,
               device_rules.as<const step_rule>());

  auto& curves = c.curves;
  curves.indices.reserve(sizeof(int) * (std::size_t)std::max<long long>(curves.vertex_total, 1));
  curves.colors.reserve(sizeof(float4) * (std::size_t)std::max<long long>(curves.vertex_total, 1));
  if (curves.vertex_total > 0)
    PARS_CUDA(cudaMemsetAsync(curves.colors.get(), 0, sizeof(float4) * curves.vertex_total, c.stream));
  for (auto& b : curves.batches)
  {
    request& r = *batch[b.rank];
    b.index_offset = b.vertex_offset;
    b.index_count = launch_index_generate(c, curves.vertices.as<const float4>() + b.vertex_offset, b.vertex_count,
                                          curves.indices.as<int>() + b.index_offset);
    launch_color_generate(c, curves.vertices.as<const float4>() + b.vertex_offset, curves.indices.as<const int>() + b.index_offset,
                          b.index_count, r.color_mode, r.s.color_generation_free_parameter, curves.colors.as<float4>() + b.vertex_offset);
  }
  curves.indexed = curves.colored = true;
  for (auto& b : curves.batches)
  {
    request& r = *batch[b.rank];
    r.vertices.emplace_back(b.vertex_count);
    r.colors.emplace_back(b.vertex_count);
    r.indices.emplace_back(b.index_count);
    if (b.vertex_count)
    {
      PARS_CUDA(cudaMemcpyAsync(r.vertices.back().data(), curves.vertices.as<float4>() + b.vertex_offset, sizeof(float4) * b.vertex_count,
                                cudaMemcpyDeviceToHost, c.stream));
      PARS_CUDA(cudaMemcpyAsync(r.colors.back().data(), curves.colors.as<float4>() + b.vertex_offset, sizeof(float4) * b.vertex_count,
                                cudaMemcpyDeviceToHost, c.stream));
    }
    if (b.index_count)
      PARS_CUDA(cudaMemcpyAsync(r.indices.back().data(), curves.indices.as<int>() + b.index_offset, sizeof(int) * b.index_count,
                                cudaMemcpyDeviceToHost, c.stream));
  }
  PARS_CUDA(cudaStreamSynchronize(c.stream));
  // Steps per request: each curve holds its seed, one vertex per step and the
  // termination vertex (remaining_iterations >= 2; one block, one round).
  for (std::size_t k = 0; k < batch.size(); ++k)
  {
    long long vertices = 0;
    for (auto& v : batch[k]->vertices) vertices += (long long)v.size();
    batch[k]->steps = batch[k]->s.seed_generation_iterations >= 2 ? std::max(0LL, vertices - 2 * block_count[k]) : 0;
  }
  (void)summary;
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
        svc->work.wait(lock);
      }
      svc->in_use += reserved;
      ++svc->running_batches;
    }
    try
    {
      if (kind == ftle) run_ftle_batch(*svc, c, batch);
      else run_streamline_batch(*svc, c, batch, stage_mode);
    }
    catch (const error& e) { for (auto& r : batch) fail(*r, e.status, e.what()); }
    catch (const std::exception& e) { for (auto& r : batch) fail(*r, PARS_ERR_STATE, e.what()); }
    {
      std::lock_guard<std::mutex> lock(svc->mutex);
      svc->in_use -= reserved;
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
  svc->max_batch = max_batch;
  int32_t status = pars_gpu_create(&svc->owner, device);
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
    delete svc;
    return status;
  }
  for (int i = 0; i < lanes; ++i) svc->workers.emplace_back(worker, svc, i);
  *service = svc;
  return PARS_OK;
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
  for (auto* c : svc->lanes) pars_gpu_destroy(c);
  pars_gpu_destroy(svc->owner);
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
    PARS_CUDA(cudaSetDevice(svc->device));
    pars_gpu_synchronize(svc->owner);
    dataset d;
    d.name = name;
    d.field = handle;
    auto& f = *svc->owner->fields.at(handle);
    d.view = f.view();
    for (int i = 0; i < 3; ++i) { d.shape[i] = f.shape[i]; d.offset[i] = f.offset[i]; d.size[i] = f.size[i]; d.spacing[i] = f.spacing[i]; }
    std::lock_guard<std::mutex> lock(svc->mutex);
    svc->dataset_index[d.name] = int(svc->datasets.size());
    svc->datasets.push_back(d);
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
    pars_gpu_synchronize(svc->owner);
    dataset d;
    d.name = name;
    d.field = handle;
    auto& f = *svc->owner->fields.at(handle);
    d.view = f.view();
    for (int i = 0; i < 3; ++i) { d.shape[i] = f.shape[i]; d.offset[i] = f.offset[i]; d.size[i] = f.size[i]; d.spacing[i] = f.spacing[i]; }
    std::lock_guard<std::mutex> lock(svc->mutex);
    svc->dataset_index[d.name] = int(svc->datasets.size());
    svc->datasets.push_back(d);
  });
}

int32_t pars_gpu_service_submit(pars_gpu_service* svc, const uint8_t* message, int64_t length, int64_t* ticket)
{
  return service_guard(svc, [&] {
    PARS_REQUIRE(ticket && (message || length == 0) && length >= 0, "message and ticket are required");
    auto r = std::make_shared<request>();
    std::string problem;
    if (!decode_settings(message, std::size_t(length), r->s, problem)) throw error(PARS_ERR_INVALID_ARGUMENT, problem);
    // mode substrings as pipeline.cpp:21-23 and service.cpp:79 read them
    r->kind = r->s.mode.find("ftle") != std::string::npos ? ftle : streamlines;
    if (r->s.mode.find("fractional_anisotropy") != std::string::npos) r->ftle_mode = PARS_FTLE_FRACTIONAL_ANISOTROPY;
    r->stage_mode = r->s.mode.find("reference") != std::string::npos ? PARS_STAGES_FROZEN : PARS_STAGES_RESAMPLED;
    if (r->kind == ftle && r->stage_mode == PARS_STAGES_FROZEN)
      throw error(PARS_ERR_UNSUPPORTED, "served FTLE integrates with re-sampled stages");
    r->integrator = integrator_of(r->s.particle_tracing_integrator);
    if (r->integrator != PARS_EULER && r->integrator != PARS_RUNGE_KUTTA_4)
      throw error(PARS_ERR_UNSUPPORTED, "integrator '" + r->s.particle_tracing_integrator + "' is not supported");
    r->color_mode = color_of(r->s.color_generation_mode);
    PARS_REQUIRE(r->s.particle_tracing_step_size != 0.0f, "particle_tracing_step_size must be non-zero");
    std::unique_lock<std::mutex> lock(svc->mutex);
    auto d = svc->dataset_index.find(r->s.dataset_filepath);
    if (d == svc->dataset_index.end()) throw error(PARS_ERR_NOT_FOUND, "unknown dataset '" + r->s.dataset_filepath + "'");
    r->dataset = d->second;
    r->estimate = estimate_bytes(*r, svc->datasets[r->dataset]);
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
    info->batches = (int64_t)r->vertices.size();
    for (int i = 0; i < 3; ++i) info->ftle_shape[i] = r->ftle_shape[i];
    info->steps = r->steps;
    using ms = std::chrono::duration<double, std::milli>;
    if (r->state >= running) info->queue_ms = ms(r->started - r->submitted).count();
    if (r->state == done) { info->run_ms = ms(r->finished - r->started).count(); info->latency_ms = ms(r->finished - r->submitted).count(); }
  });
}

int32_t pars_gpu_service_result_batch(pars_gpu_service* svc, int64_t ticket, int64_t batch, int64_t* vertices, int64_t* indices,
                                      float* vertex_data, float* color_data, int32_t* index_data)
{
  return service_guard(svc, [&] {
    std::lock_guard<std::mutex> lock(svc->mutex);
    auto r = find_request(svc, ticket);
    if (r->state != done) throw error(PARS_ERR_STATE, "request has not finished");
    PARS_REQUIRE(batch >= 0 && batch < (int64_t)r->vertices.size(), "batch out of range");
    if (vertices) *vertices = (int64_t)r->vertices[batch].size();
    if (indices) *indices = (int64_t)r->indices[batch].size();
    if (vertex_data && !r->vertices[batch].empty()) std::memcpy(vertex_data, r->vertices[batch].data(), 16 * r->vertices[batch].size());
    if (color_data && !r->colors[batch].empty()) std::memcpy(color_data, r->colors[batch].data(), 16 * r->colors[batch].size());
    if (index_data && !r->indices[batch].empty()) std::memcpy(index_data, r->indices[batch].data(), 4 * r->indices[batch].size());
  });
}

int32_t pars_gpu_service_result_ftle(pars_gpu_service* svc, int64_t ticket, float* values)
{
  return service_guard(svc, [&] {
    std::lock_guard<std::mutex> lock(svc->mutex);
    auto r = find_request(svc, ticket);
    if (r->state != done) throw error(PARS_ERR_STATE, "request has not finished");
    PARS_REQUIRE(values, "values is required");
    if (!r->ftle_values.empty()) std::memcpy(values, r->ftle_values.data(), sizeof(float) * r->ftle_values.size());
  });
}

int32_t pars_gpu_service_release(pars_gpu_service* svc, int64_t ticket)
{
  return service_guard(svc, [&] {
    std::lock_guard<std::mutex> lock(svc->mutex);
    auto r = find_request(svc, ticket);
    if (r->state == running) throw error(PARS_ERR_STATE, "request is running");
    if (r->state == queued)
    {
      svc->queue.erase(std::remove(svc->queue.begin(), svc->queue.end(), r), svc->queue.end());
      r->status = PARS_ERR_CANCELLED;
    }
    svc->requests.erase(ticket);
  });
}

}
#pragma GCC visibility pop
