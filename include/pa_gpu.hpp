// pa_gpu.hpp — C++17 drop-in for the pa:: stage classes of the particle-tracing
// hot path, over the C ABI in pars_gpu.h (header-only; link libpars_gpu.so).
//
// Mirrors the reference interfaces (same class and method names, argument
// meaning and call order as pars::pipeline::execute uses them):
//   pa::particle_tracer     pa/include/pa/stages/particle_tracer.hpp:21-71
//   pa::index_generator     pa/include/pa/stages/index_generator.hpp:9-13
//   pa::color_generator     pa/include/pa/stages/color_generator.hpp:11-32
//   pa::seed_generator      pa/include/pa/stages/seed_generator.hpp:10-14
//   pa::partitioner         pa/include/pa/stages/partitioner.hpp:12-53
//   pa::flow_map_generator  pa/include/pa/stages/flow_map_generator.hpp:10-28
//   pa::ftle_map_generator  pa/include/pa/stages/ftle_map_generator.hpp:11-40
//   pa::data_io             pa/include/pa/stages/data_io.hpp (on "pars raw" files)
//   pars::ray_tracer        pars/include/pars/stages/ray_tracer.hpp:24-44
// The value types are layout-compatible with the reference's (pa::particle is
// 48 bytes with the same field offsets; vector4 is 16 bytes), so a caller
// holding the reference's std::vector<pa::particle> can pass its data()
// through pars_gpu.h directly.  Errors are reported as std::runtime_error, as
// the reference does (data_io.cpp:198, ray_tracer.cpp:10-12).
#ifndef PA_GPU_HPP
#define PA_GPU_HPP

#include <array>
#include <cstdint>
#include <cstring>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <vector>

#include "pars_gpu.h"

namespace pa_gpu
{
using scalar   = float;
using integer  = std::int32_t;
struct alignas(16) vector4 { float data[4]; float& operator[](int i) { return data[i]; } float operator[](int i) const { return data[i]; } };
struct vector3 { float data[3]; float& operator[](int i) { return data[i]; } float operator[](int i) const { return data[i]; } };
struct ivector3 { integer data[3]; integer& operator[](int i) { return data[i]; } integer operator[](int i) const { return data[i]; } };

// pa::particle (particle.hpp:30-35); 48 bytes like the reference's.
struct alignas(16) particle
{
  vector4  position {};
  integer  remaining_iterations = 0;
  integer  vector_field_index   = 0;
  integer  original_rank        = 0;
  ivector3 original_voxel       {};
};
static_assert(sizeof(particle) == sizeof(pars_particle), "particle matches pars_particle");

// pa::integral_curves (integral_curves.hpp:11-20).
struct integral_curves
{
  std::vector<vector4> vertices {};
  std::vector<vector4> colors   {};
  std::vector<integer> indices  {};
};
inline const vector4 termination_vertex {{-2.0f, -2.0f, -2.0f, 0.0f}};
inline const vector4 invalid_vertex     {{-1.0f, -1.0f, -1.0f, 0.0f}};
inline const integer invalid_index      = -1;

// pa::vector_field (vector_field.hpp:14-24): shape plus xyz data in C order.
struct vector_field
{
  std::array<integer, 3> shape {};
  std::vector<float>     data  {};   // shape[0]*shape[1]*shape[2]*3
  vector3                offset {};
  vector3                size   {};
  vector3                spacing {};
};

// pa::scalar_field (scalar_field.hpp:11-17).
struct scalar_field
{
  std::array<integer, 3> shape {};
  std::vector<float>     data  {};
  vector3                offset {}, size {}, spacing {};
};

// The integrator choice of pa::variant_integrator, by index.
enum class integrator { euler = PARS_EULER, modified_midpoint = PARS_MODIFIED_MIDPOINT, runge_kutta_4 = PARS_RUNGE_KUTTA_4,
                        runge_kutta_cash_karp_54 = PARS_RUNGE_KUTTA_CASH_KARP_54,
                        runge_kutta_dormand_prince_5 = PARS_RUNGE_KUTTA_DORMAND_PRINCE_5,
                        runge_kutta_fehlberg_78 = PARS_RUNGE_KUTTA_FEHLBERG_78, adams_bashforth_2 = PARS_ADAMS_BASHFORTH_2,
                        adams_bashforth_moulton_2 = PARS_ADAMS_BASHFORTH_MOULTON_2 };

inline void check(pars_gpu_context* ctx, int32_t status, const char* what)
{
  if (status != PARS_OK)
    throw std::runtime_error(std::string(what) + " failed (" + std::to_string(status) + "): " + pars_gpu_last_error(ctx));
}

// One GPU context shared by the stages of a pipeline.
class device
{
public:
  explicit device(int32_t index = 0)
  {
    pars_gpu_context* c = nullptr;
    if (pars_gpu_create(&c, index) != PARS_OK) throw std::runtime_error("pars_gpu_create failed");
    context_.reset(c);
  }
  pars_gpu_context* get() const { return context_.get(); }

  // Uploads a field and returns its handle (kept until the device is destroyed
  // or release() is called).
  int32_t upload(const vector_field& f)
  {
    int32_t handle = -1;
    check(get(), pars_gpu_field_upload(get(), f.data.data(), f.shape.data(), f.offset.data, f.size.data, f.spacing.data, &handle),
          "pars_gpu_field_upload");
    return handle;
  }
  void release(int32_t handle) { check(get(), pars_gpu_field_release(get(), handle), "pars_gpu_field_release"); }

private:
  struct deleter { void operator()(pars_gpu_context* c) const { pars_gpu_destroy(c); } };
  std::unique_ptr<pars_gpu_context, deleter> context_;
};

// pa::partitioner: the same block grid and neighbour table, computed on the host.
class partitioner
{
public:
  struct rank_info
  {
    integer  rank = 0;
    ivector3 multi_rank {}, offset {}, ghosted_block_size {};
  };
  partitioner(integer ranks, integer rank) : ranks_(ranks), rank_(rank) {}
  void set_domain_size(const ivector3& domain_size)
  {
    domain_size_ = domain_size;
    pars_partition_info info {};
    if (pars_gpu_partition(ranks_, rank_, domain_size.data, &info) != PARS_OK) throw std::runtime_error("pars_gpu_partition failed");
    for (int i = 0; i < 3; ++i)
    {
      grid_size_[i] = info.grid_size[i];
      block_size_[i] = info.block_size[i];
    }
    local_ = make_info(rank_);
    for (int f = 0; f < 6; ++f)
      neighbors_[f] = info.neighbor_rank[f] >= 0 ? std::optional<rank_info>(make_info(info.neighbor_rank[f])) : std::nullopt;
  }
  const ivector3& domain_size() const { return domain_size_; }
  const ivector3& grid_size  () const { return grid_size_; }
  const ivector3& block_size () const { return block_size_; }
  const std::optional<rank_info>& local_rank_info() const { return local_; }
  const std::array<std::optional<rank_info>, 6>& neighbor_rank_info() const { return neighbors_; }
  integer size() const { return ranks_; }

private:
  rank_info make_info(integer r) const
  {
    pars_partition_info info {};
    if (pars_gpu_partition(ranks_, r, domain_size_.data, &info) != PARS_OK) throw std::runtime_error("pars_gpu_partition failed");
    rank_info out;
    out.rank = r;
    for (int i = 0; i < 3; ++i)
    {
      out.multi_rank[i] = info.multi_rank[i];
      out.offset[i] = info.offset[i];
      out.ghosted_block_size[i] = info.ghosted_block_size[i];
    }
    return out;
  }
  integer ranks_, rank_;
  ivector3 domain_size_ {}, grid_size_ {}, block_size_ {};
  std::optional<rank_info> local_;
  std::array<std::optional<rank_info>, 6> neighbors_ {};
};

// pa::seed_generator::generate (seed_generator.hpp:13).
struct seed_generator
{
  static std::vector<particle> generate(device& dev, const vector3& offset, const vector3& size, const vector3& stride,
                                        integer remaining_iterations, integer rank)
  {
    int64_t count = 0;
    check(dev.get(), pars_gpu_seed_generate(dev.get(), offset.data, size.data, stride.data, remaining_iterations, rank, nullptr, 0, &count),
          "pars_gpu_seed_generate");
    std::vector<particle> out(count);
    if (count)
      check(dev.get(), pars_gpu_seed_generate(dev.get(), offset.data, size.data, stride.data, remaining_iterations, rank,
                                              reinterpret_cast<pars_particle*>(out.data()), count, &count), "pars_gpu_seed_generate");
    return out;
  }
};

// pa::particle_tracer for one block.  trace(particles) runs the rounds, prune,
// and leaves the curves on the device; the curves are returned as host
// integral_curves batches (vertices only, as the reference's trace returns).
// index_generator / color_generator below work on the same device-resident
// curves when given the tracer, or on host buffers.
class particle_tracer
{
public:
  explicit particle_tracer(device& dev) : dev_(dev) {}
  void set_local_vector_field(int32_t field_handle) { field_ = field_handle; }
  void set_integrator(integrator i) { integrator_ = i; }
  void set_step_size(scalar h) { step_size_ = h; }
  // PARS_STAGES_FROZEN (the reference's scheme, default) or PARS_STAGES_RESAMPLED.
  void set_stage_mode(int32_t mode) { stage_mode_ = mode; }

  std::vector<integral_curves> trace(const std::vector<particle>& particles)
  {
    pars_gpu_trace_summary s {};
    check(dev_.get(), pars_gpu_trace(dev_.get(), field_, reinterpret_cast<const pars_particle*>(particles.data()),
                                     (int64_t)particles.size(), (int32_t)integrator_, stage_mode_, step_size_, &s), "pars_gpu_trace");
    batches_ = s.batches;
    std::vector<integral_curves> out(s.batches);
    for (int64_t b = 0; b < s.batches; ++b)
    {
      int64_t nv = 0;
      check(dev_.get(), pars_gpu_curves_batch_info(dev_.get(), b, &nv, nullptr, nullptr, nullptr), "pars_gpu_curves_batch_info");
      out[b].vertices.resize(nv);
      check(dev_.get(), pars_gpu_curves_download(dev_.get(), b, out[b].vertices.empty() ? nullptr : out[b].vertices[0].data,
                                                 nullptr, nullptr), "pars_gpu_curves_download");
    }
    return out;
  }
  // Index and colour the device-resident curves of the last trace and
  // download everything (the pipeline's stages 4.0 and 5.0 in one pass).
  std::vector<integral_curves> finish(int32_t color_mode, scalar parameter)
  {
    check(dev_.get(), pars_gpu_curves_index(dev_.get()), "pars_gpu_curves_index");
    if (color_mode >= 0) check(dev_.get(), pars_gpu_curves_color(dev_.get(), color_mode, parameter), "pars_gpu_curves_color");
    std::vector<integral_curves> out(batches_);
    for (int64_t b = 0; b < batches_; ++b)
    {
      int64_t nv = 0, ni = 0;
      check(dev_.get(), pars_gpu_curves_batch_info(dev_.get(), b, &nv, &ni, nullptr, nullptr), "pars_gpu_curves_batch_info");
      out[b].vertices.resize(nv);
      out[b].indices.resize(ni);
      if (color_mode >= 0) out[b].colors.resize(nv);
      check(dev_.get(), pars_gpu_curves_download(dev_.get(), b, nv ? out[b].vertices[0].data : nullptr,
                                                 (color_mode >= 0 && nv) ? out[b].colors[0].data : nullptr,
                                                 ni ? out[b].indices.data() : nullptr), "pars_gpu_curves_download");
    }
    return out;
  }

private:
  device&    dev_;
  int32_t    field_ = -1;
  integrator integrator_ = integrator::euler;   // the reference's default (particle_tracer.hpp:67)
  scalar     step_size_ = 1.0f;                  // particle_tracer.hpp:68
  int32_t    stage_mode_ = PARS_STAGES_FROZEN;
  int64_t    batches_ = 0;
};

// pa::index_generator::generate on a host batch.
struct index_generator
{
  static void generate(device& dev, integral_curves* curves)
  {
    curves->indices.resize(curves->vertices.size());
    int64_t n = 0;
    if (curves->vertices.size() >= 2)
      check(dev.get(), pars_gpu_index_generate(dev.get(), curves->vertices[0].data, (int64_t)curves->vertices.size(),
                                               curves->indices.data(), &n), "pars_gpu_index_generate");
    curves->indices.resize(n);
  }
};

// pa::color_generator::generate on a host batch.
struct color_generator
{
  enum class mode { hsl_constant_s = 0, hsl_constant_l = 1, hsv_constant_s = 2, hsv_constant_v = 3, rgb = 4 };
  static void generate(device& dev, integral_curves* curves, mode m = mode::rgb, scalar constant_parameter = 0.5f)
  {
    curves->colors.resize(curves->vertices.size());
    if (curves->vertices.empty() || curves->indices.empty()) return;
    check(dev.get(), pars_gpu_color_generate(dev.get(), curves->vertices[0].data, (int64_t)curves->vertices.size(),
                                             curves->indices.data(), (int64_t)curves->indices.size(), (int32_t)m,
                                             constant_parameter, curves->colors[0].data), "pars_gpu_color_generate");
  }
};

// pa::flow_map_generator: the flow map stays on the device as a field handle.
class flow_map_generator
{
public:
  explicit flow_map_generator(device& dev) : dev_(dev) {}
  void set_vector_field(int32_t field_handle) { field_ = field_handle; }
  void set_integrator(integrator i) { integrator_ = i; }
  void set_step_size(scalar h) { step_size_ = h; }
  void set_stage_mode(int32_t mode) { stage_mode_ = mode; }
  int32_t generate(std::size_t iterations, scalar resolution_scale = 1)
  {
    int32_t handle = -1;
    int64_t steps = 0;
    check(dev_.get(), pars_gpu_flow_map_generate(dev_.get(), field_, (int32_t)iterations, resolution_scale, (int32_t)integrator_,
                                                 stage_mode_, step_size_, &handle, &steps), "pars_gpu_flow_map_generate");
    last_steps_ = steps;
    return handle;
  }
  int64_t last_steps() const { return last_steps_; }

private:
  device&    dev_;
  int32_t    field_ = -1;
  integrator integrator_ = integrator::euler;
  scalar     step_size_ = 1.0f;
  int32_t    stage_mode_ = PARS_STAGES_FROZEN;
  int64_t    last_steps_ = 0;
};

// pa::ftle_map_generator.
class ftle_map_generator
{
public:
  enum class mode { regular = PARS_FTLE_REGULAR, fractional_anisotropy = PARS_FTLE_FRACTIONAL_ANISOTROPY };
  ftle_map_generator(device& dev, mode m = mode::regular) : dev_(dev), mode_(m) {}
  void set_flow_map(int32_t flow_map_handle) { flow_map_ = flow_map_handle; }
  void set_time(scalar time) { time_ = time; }
  std::unique_ptr<scalar_field> generate()
  {
    auto out = std::make_unique<scalar_field>();
    check(dev_.get(), pars_gpu_field_info(dev_.get(), flow_map_, out->shape.data(), out->offset.data, out->size.data, out->spacing.data),
          "pars_gpu_field_info");
    out->data.resize((std::size_t)out->shape[0] * out->shape[1] * out->shape[2]);
    check(dev_.get(), pars_gpu_ftle_generate(dev_.get(), flow_map_, time_, (int32_t)mode_, out->data.data()), "pars_gpu_ftle_generate");
    return out;
  }

private:
  device& dev_;
  mode    mode_;
  int32_t flow_map_ = -1;
  scalar  time_ = 1;
};

// pa::data_io on "pars raw" files (pars_gpu.h): the rank's ghosted block of a
// file's vector field (uploaded) or scalar field, and FTLE write-back.
class data_io
{
public:
  data_io(device& dev, integer ranks = 1, integer rank = 0) : dev_(dev), ranks_(ranks), rank_(rank) {}
  void set_file(const std::string& path) { path_ = path; }
  ivector3 load_dimensions() const
  {
    int32_t components = 0;
    int64_t shape[3];
    float spacing[3];
    check(dev_.get(), pars_gpu_raw_info(path_.c_str(), &components, shape, spacing), "pars_gpu_raw_info");
    return ivector3 {{integer(shape[0]), integer(shape[1]), integer(shape[2])}};
  }
  // The block as a resident field handle (data_io.cpp:50-58, 90-114).
  int32_t load_local_vector_field()
  {
    int32_t handle = -1;
    check(dev_.get(), pars_gpu_field_load(dev_.get(), path_.c_str(), ranks_, rank_, &handle, nullptr), "pars_gpu_field_load");
    return handle;
  }
  // A scalar dataset's block (data_io.cpp:41-49, 76-89); `file` names its own file.
  scalar_field load_local_scalar_field(const std::string& file) const
  {
    scalar_field out;
    check(dev_.get(), pars_gpu_scalar_load(file.c_str(), ranks_, rank_, nullptr, out.shape.data(), out.offset.data,
                                           out.spacing.data, out.size.data), "pars_gpu_scalar_load");
    out.data.resize((std::size_t)out.shape[0] * out.shape[1] * out.shape[2]);
    check(dev_.get(), pars_gpu_scalar_load(file.c_str(), ranks_, rank_, out.data.data(), out.shape.data(), out.offset.data,
                                           out.spacing.data, out.size.data), "pars_gpu_scalar_load");
    return out;
  }
  // save_ftle_field (data_io.cpp:117-140): this rank's block at its voxel offset.
  void save_ftle_field(const std::string& file, const scalar_field& ftle, const std::array<integer, 3>& domain,
                       const std::array<integer, 3>& voxel_offset) const
  {
    check(dev_.get(), pars_gpu_ftle_save(file.c_str(), domain.data(), voxel_offset.data(), ftle.shape.data(), ftle.data.data(),
                                         ftle.spacing.data), "pars_gpu_ftle_save");
  }
  // save_integral_curves (data_io.cpp:142-196) of the device's current curves.
  void save_integral_curves(const std::string& file) const
  {
    check(dev_.get(), pars_gpu_curves_export_vtk(dev_.get(), file.c_str()), "pars_gpu_curves_export_vtk");
  }

private:
  device&     dev_;
  integer     ranks_, rank_;
  std::string path_;
};

// pars::ray_tracer (ray_tracer.hpp:24-44) on the device; serialize() returns
// the `image` reply (image.proto) as bytes.
class ray_tracer
{
public:
  explicit ray_tracer(device& dev) : dev_(dev) {}
  void set_volume(const scalar_field& volume)
  {
    check(dev_.get(), pars_gpu_ray_tracer_set_volume(dev_.get(), volume.data.data(), volume.shape.data(), volume.offset.data,
                                                     volume.spacing.data), "pars_gpu_ray_tracer_set_volume");
  }
  // The device's current curves (traced, indexed, coloured).
  void set_integral_curves(float radius)
  {
    check(dev_.get(), pars_gpu_ray_tracer_set_integral_curves(dev_.get(), radius), "pars_gpu_ray_tracer_set_integral_curves");
  }
  void set_integral_curves(const std::vector<integral_curves>& curves, float radius)
  {
    std::vector<int64_t> vertex_counts, index_counts;
    std::vector<const float*> vertices, colors;
    std::vector<const int32_t*> indices;
    for (const auto& c : curves)
    {
      vertex_counts.push_back((int64_t)c.vertices.size());
      index_counts.push_back((int64_t)c.indices.size());
      vertices.push_back(c.vertices.empty() ? nullptr : c.vertices[0].data);
      colors.push_back(c.colors.size() == c.vertices.size() && !c.colors.empty() ? c.colors[0].data : nullptr);
      indices.push_back(c.indices.empty() ? nullptr : c.indices.data());
    }
    check(dev_.get(), pars_gpu_ray_tracer_set_integral_curves_host(dev_.get(), (int64_t)curves.size(), vertex_counts.data(),
                                                                   vertices.data(), colors.data(), index_counts.data(),
                                                                   indices.data(), radius),
          "pars_gpu_ray_tracer_set_integral_curves_host");
  }
  void set_camera(const vector3& position, const vector3& forward, const vector3& up)
  {
    check(dev_.get(), pars_gpu_ray_tracer_set_camera(dev_.get(), position.data, forward.data, up.data), "pars_gpu_ray_tracer_set_camera");
  }
  void set_image_size(integer width, integer height)
  {
    check(dev_.get(), pars_gpu_ray_tracer_set_image_size(dev_.get(), width, height), "pars_gpu_ray_tracer_set_image_size");
  }
  void trace(std::size_t iterations = 1)
  {
    check(dev_.get(), pars_gpu_ray_tracer_trace(dev_.get(), (int32_t)iterations), "pars_gpu_ray_tracer_trace");
  }
  std::string serialize()
  {
    int32_t size[2] = {0, 0};
    check(dev_.get(), pars_gpu_ray_tracer_serialize(dev_.get(), nullptr, size), "pars_gpu_ray_tracer_serialize");
    std::vector<uint8_t> rgba((std::size_t)size[0] * size[1] * 4);
    check(dev_.get(), pars_gpu_ray_tracer_serialize(dev_.get(), rgba.data(), size), "pars_gpu_ray_tracer_serialize");
    int64_t length = 0;
    if (pars_gpu_image_encode(size, rgba.data(), (int64_t)rgba.size(), nullptr, 0, &length) != PARS_OK)
      throw std::runtime_error("pars_gpu_image_encode failed");
    std::string message((std::size_t)length, '\0');
    if (pars_gpu_image_encode(size, rgba.data(), (int64_t)rgba.size(), reinterpret_cast<uint8_t*>(&message[0]), length, &length) != PARS_OK)
      throw std::runtime_error("pars_gpu_image_encode failed");
    return message;
  }

private:
  device& dev_;
};
}

#endif
