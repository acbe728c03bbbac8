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

#include <algorithm>
#include <array>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
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

// ---- the ranks of one GPU ---------------------------------------------------------
// pars runs one MPI process per rank (boost::mpi::communicator,
// pipeline.cpp:14-17).  On one GPU every rank's block is resident in one device
// context, and the drop-in's ranks are threads of one process that share a
// `world`: its collectives (the round exchange and check_completion) wait for
// every rank as MPI's would, and a round of all ranks is one tracing launch on
// the device.  A rank that never joins makes the others' collectives fail
// after `timeout_seconds` with std::runtime_error.
class world
{
public:
  world(device& dev, integer size, double timeout_seconds = 120.0)
    : dev_(dev), size_(size), timeout_(timeout_seconds), fields_(size, -1), submitted_(size), next_(size), batches_(size)
  {
    if (size < 1) throw std::runtime_error("a world needs at least one rank");
  }
  world(const world&) = delete;
  world& operator=(const world&) = delete;
  ~world() { if (domain_ >= 0) pars_gpu_domain_release(dev_.get(), domain_); }

  device& get_device() const { return dev_; }
  integer size() const { return size_; }

  // A rank's local block (its ghosted field handle) and the domain size.
  void set_block(integer rank, int32_t field, const ivector3& domain_size)
  {
    std::lock_guard<std::mutex> lock(mutex_);
    fields_.at(rank) = field;
    domain_size_ = domain_size;
    drop_domain();
  }

  // particle_tracer::trace(particles, curves, round_info) of `rank` in `round`.
  void submit(integer rank, int round, const std::vector<particle>& particles, int32_t integrator, int32_t stage_mode, scalar step)
  {
    std::lock_guard<std::mutex> lock(mutex_);
    if (round != submit_round_)
    {
      submit_round_ = round;
      submitted_count_ = 0;
      for (auto& s : submitted_) s.clear();
    }
    submitted_.at(rank) = particles;
    ++submitted_count_;
    integrator_ = integrator;
    stage_mode_ = stage_mode;
    step_ = step;
    cv_.notify_all();
  }

  // out_of_bounds_distribute: once every rank has submitted `round`, the round
  // runs on the device (once); returns `rank`'s particles of the next round.
  std::vector<particle> exchange(integer rank, int round)
  {
    std::unique_lock<std::mutex> lock(mutex_);
    wait(lock, [&] { return done_round_ >= round || (submit_round_ == round && submitted_count_ == size_); });
    if (done_round_ < round) run_round(round);
    return next_.at(rank);
  }

  // check_completion: true when no rank holds particles (a collective).
  bool all_empty(std::size_t count)
  {
    std::unique_lock<std::mutex> lock(mutex_);
    const long long generation = barrier_generation_;
    any_left_ = any_left_ || count > 0;
    if (++barrier_arrived_ == size_)
    {
      barrier_result_ = !any_left_;
      if (barrier_result_) { submit_round_ = -1; done_round_ = -1; }   // the next round is the first of a new trace
      any_left_ = false;
      barrier_arrived_ = 0;
      ++barrier_generation_;
      cv_.notify_all();
      return barrier_result_;
    }
    wait(lock, [&] { return barrier_generation_ != generation; });
    return barrier_result_;
  }

  // The device batch indices of `rank`'s curves, in round order.
  std::vector<int64_t> batches(integer rank)
  {
    std::lock_guard<std::mutex> lock(mutex_);
    return batches_.at(rank);
  }

private:
  template <typename predicate> void wait(std::unique_lock<std::mutex>& lock, predicate ready)
  {
    if (!cv_.wait_for(lock, std::chrono::duration<double>(timeout_), ready))
      throw std::runtime_error("a rank did not join the collective within the timeout");
  }
  void drop_domain()
  {
    if (domain_ >= 0) pars_gpu_domain_release(dev_.get(), domain_);
    domain_ = -1;
  }
  void run_round(int round)
  {
    pars_gpu_context* ctx = dev_.get();
    if (domain_ < 0)
    {
      for (integer r = 0; r < size_; ++r)
        if (fields_[r] < 0) throw std::runtime_error("rank " + std::to_string(r) + " has no local vector field");
      check(ctx, pars_gpu_domain_assemble(ctx, size_, domain_size_.data, fields_.data(), &domain_), "pars_gpu_domain_assemble");
    }
    std::vector<pars_particle> all;
    std::vector<int64_t> offsets(size_ + 1, 0);
    for (integer r = 0; r < size_; ++r)
    {
      offsets[r + 1] = offsets[r] + (int64_t)submitted_[r].size();
      const auto* p = reinterpret_cast<const pars_particle*>(submitted_[r].data());
      all.insert(all.end(), p, p + submitted_[r].size());
    }
    if (round == 0) for (auto& b : batches_) b.clear();
    int64_t before = 0;
    if (round > 0)
      for (const auto& b : batches_) before += (int64_t)b.size();
    std::vector<int64_t> next_offsets(size_ + 1, 0);
    pars_gpu_trace_summary summary {};
    static const pars_particle none {};
    check(ctx, pars_gpu_round_trace(ctx, domain_, round, all.empty() ? &none : all.data(), offsets.data(), integrator_,
                                    stage_mode_, step_, next_offsets.data(), &summary), "pars_gpu_round_trace");
    for (int64_t b = before; b < before + summary.batches; ++b)
    {
      int32_t rank = 0;
      check(ctx, pars_gpu_curves_batch_info(ctx, b, nullptr, nullptr, &rank, nullptr), "pars_gpu_curves_batch_info");
      batches_.at(rank).push_back(b);
    }
    std::vector<particle> moved((std::size_t)next_offsets[size_]);
    if (!moved.empty())
      check(ctx, pars_gpu_round_particles(ctx, reinterpret_cast<pars_particle*>(moved.data())), "pars_gpu_round_particles");
    for (integer r = 0; r < size_; ++r)
      next_[r].assign(moved.begin() + next_offsets[r], moved.begin() + next_offsets[r + 1]);
    done_round_ = round;
    cv_.notify_all();
  }

  device&                            dev_;
  integer                            size_;
  double                             timeout_;
  std::mutex                         mutex_;
  std::condition_variable            cv_;
  std::vector<int32_t>               fields_;
  ivector3                           domain_size_ {};
  int32_t                            domain_ = -1;
  int32_t                            integrator_ = PARS_EULER, stage_mode_ = PARS_STAGES_FROZEN;
  scalar                             step_ = 1.0f;
  int                                submit_round_ = -1, submitted_count_ = 0, done_round_ = -1;
  std::vector<std::vector<particle>> submitted_, next_;
  std::vector<std::vector<int64_t>>  batches_;
  long long                          barrier_generation_ = 0;
  integer                            barrier_arrived_ = 0;
  bool                               any_left_ = false, barrier_result_ = false;
};

// boost::mpi::communicator as the stages see it: one rank of a world.
class communicator
{
public:
  communicator(world& w, integer rank) : world_(&w), rank_(rank)
  {
    if (rank < 0 || rank >= w.size()) throw std::runtime_error("rank outside the world");
  }
  integer rank() const { return rank_; }
  integer size() const { return world_->size(); }
  world&  get_world() const { return *world_; }

private:
  world*  world_;
  integer rank_;
};

// pa::partitioner (partitioner.hpp:14-53): the same block grid and neighbour
// table, computed on the host.
class partitioner
{
public:
  struct rank_info
  {
    integer  rank = 0;
    ivector3 multi_rank {}, offset {}, ghosted_block_size {};
  };
  explicit partitioner(pa_gpu::communicator* communicator) : communicator_(communicator) {}
  void set_domain_size(const ivector3& domain_size)
  {
    domain_size_ = domain_size;
    pars_partition_info info {};
    if (pars_gpu_partition(communicator_->size(), communicator_->rank(), domain_size.data, &info) != PARS_OK)
      throw std::runtime_error("pars_gpu_partition failed");
    for (int i = 0; i < 3; ++i)
    {
      grid_size_[i] = info.grid_size[i];
      block_size_[i] = info.block_size[i];
    }
    local_ = make_info(communicator_->rank());
    for (int f = 0; f < 6; ++f)
      neighbors_[f] = info.neighbor_rank[f] >= 0 ? std::optional<rank_info>(make_info(info.neighbor_rank[f])) : std::nullopt;
  }
  pa_gpu::communicator* communicator() { return communicator_; }
  const ivector3& domain_size() const { return domain_size_; }
  const ivector3& grid_size  () const { return grid_size_; }
  const ivector3& block_size () const { return block_size_; }
  const std::optional<rank_info>& local_rank_info() const { return local_; }
  const std::array<std::optional<rank_info>, 6>& neighbor_rank_info() const { return neighbors_; }

private:
  rank_info make_info(integer r) const
  {
    pars_partition_info info {};
    if (pars_gpu_partition(communicator_->size(), r, domain_size_.data, &info) != PARS_OK)
      throw std::runtime_error("pars_gpu_partition failed");
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
  pa_gpu::communicator* communicator_;
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

// pa::particle_tracer (particle_tracer.hpp:21-71) with the reference's
// construction, setters, whole trace() and the sub-methods pipeline::execute
// calls one by one per round (pipeline.cpp:130-131, 155-205).  On one GPU:
//  * set_local_vector_field uploads the rank's block; set_neighbor_vector_fields
//    is kept for the interface: the neighbours are the other ranks' resident
//    blocks;
//  * compute_round_info is the reference's arithmetic (particle_tracer.cpp:
//    210-234; an empty particle list gives no batch instead of the reference's
//    undefined max_element);
//  * allocate appends the round's batches; their vertices live on the device
//    until prune() copies the pruned vertices in (initialize's seed vertices
//    are written there too);
//  * trace submits the rank's particles; out_of_bounds_distribute runs the
//    round of all ranks once every rank has submitted (one launch) and hands
//    this rank the particles its face neighbours passed on, in the reference's
//    order (by sending rank, then the sender's order); round_info's particle
//    maps stay empty (the exchange happens on the device);
//  * load_balance_distribute / load_balance_collect do nothing: they move
//    particles between MPI ranks, and here every rank shares one GPU;
//  * check_completion is the collective "no rank holds particles".
class particle_tracer
{
public:
  struct round_info
  {
    using particle_map = std::map<integer, std::vector<particle>>;
    std::size_t  maximum_remaining_iterations     = 0;
    std::size_t  vertices_per_integral_curve      = 0;
    std::size_t  vertices_per_integral_curve_last = 0;
    std::size_t  integral_curve_offset            = 0;
    std::size_t  integral_curve_count             = 0;
    particle_map out_of_bounds_particles          {};
    particle_map neighbor_out_of_bounds_particles {};
  };

  explicit particle_tracer(pa_gpu::partitioner* partitioner) : partitioner_(partitioner) {}
  particle_tracer(const particle_tracer&) = delete;
  particle_tracer& operator=(const particle_tracer&) = delete;
  ~particle_tracer()
  {
    if (field_ >= 0) pars_gpu_field_release(dev().get(), field_);
  }

  void set_local_vector_field(std::optional<vector_field>* local_vector_field)
  {
    local_vector_field_ = local_vector_field;
    if (field_ >= 0) { pars_gpu_field_release(dev().get(), field_); field_ = -1; }
    if (local_vector_field_ && local_vector_field_->has_value())
    {
      field_ = dev().upload(local_vector_field_->value());
      partitioner_->communicator()->get_world().set_block(rank(), field_, partitioner_->domain_size());
    }
  }
  void set_neighbor_vector_fields(std::array<std::optional<vector_field>, 6>* neighbor_vector_fields)
  {
    neighbor_vector_fields_ = neighbor_vector_fields;
  }
  void set_integrator(integrator i) { integrator_ = i; }
  void set_step_size(scalar h) { step_size_ = h; }
  // Extension: PARS_STAGES_FROZEN (the reference's scheme, default) or PARS_STAGES_RESAMPLED.
  void set_stage_mode(int32_t mode) { stage_mode_ = mode; }

  // particle_tracer::trace(particles) (particle_tracer.cpp:39-56).
  std::vector<integral_curves> trace(std::vector<particle> particles)
  {
    std::vector<integral_curves> curves;
    while (!check_completion(particles))
    {
      load_balance_distribute(particles);
      auto info = compute_round_info(particles, curves);
      allocate(curves, info);
      initialize(particles, curves, info);
      trace(particles, curves, info);
      load_balance_collect(info);
      out_of_bounds_distribute(particles, info);
    }
    prune(curves);
    return curves;
  }

  void load_balance_distribute(std::vector<particle>&) {}
  round_info compute_round_info(const std::vector<particle>& particles, const std::vector<integral_curves>& curves)
  {
    round_info info;
    info.integral_curve_offset = curves.size();
    if (particles.empty()) return info;
    integer maximum = 0;
    for (const auto& p : particles) maximum = std::max(maximum, p.remaining_iterations);
    info.maximum_remaining_iterations = (std::size_t)std::max(maximum, 1);
    const std::size_t per_curve = (std::size_t)std::numeric_limits<integer>::max() / sizeof(vector4) / info.maximum_remaining_iterations;
    info.vertices_per_integral_curve = per_curve * info.maximum_remaining_iterations;
    info.vertices_per_integral_curve_last = particles.size() % per_curve * info.maximum_remaining_iterations;
    info.integral_curve_count = 1 + particles.size() / per_curve;
    return info;
  }
  void allocate(std::vector<integral_curves>& curves, const round_info& info)
  {
    curves.resize(info.integral_curve_offset + info.integral_curve_count);
  }
  void initialize(const std::vector<particle>&, std::vector<integral_curves>&, const round_info&) {}
  void trace(const std::vector<particle>& particles, std::vector<integral_curves>&, round_info&)
  {
    partitioner_->communicator()->get_world().submit(rank(), round_, particles, (int32_t)integrator_, stage_mode_, step_size_);
  }
  void load_balance_collect(round_info&) {}
  void out_of_bounds_distribute(std::vector<particle>& particles, const round_info&)
  {
    particles = partitioner_->communicator()->get_world().exchange(rank(), round_);
    ++round_;
  }
  bool check_completion(const std::vector<particle>& particles)
  {
    const bool complete = partitioner_->communicator()->get_world().all_empty(particles.size());
    if (complete) round_ = 0;
    return complete;
  }
  // prune (particle_tracer.cpp:402-409): this rank's batches, pruned on the
  // device, copied into its integral_curves (vertices).
  void prune(std::vector<integral_curves>& curves)
  {
    const auto batches = partitioner_->communicator()->get_world().batches(rank());
    if (batches.size() != curves.size())
      throw std::runtime_error("prune: " + std::to_string(curves.size()) + " batches allocated, " +
                               std::to_string(batches.size()) + " traced");
    for (std::size_t k = 0; k < batches.size(); ++k)
    {
      int64_t nv = 0;
      check(dev().get(), pars_gpu_curves_batch_info(dev().get(), batches[k], &nv, nullptr, nullptr, nullptr),
            "pars_gpu_curves_batch_info");
      curves[k].vertices.resize((std::size_t)nv);
      check(dev().get(), pars_gpu_curves_download(dev().get(), batches[k], nv ? curves[k].vertices[0].data : nullptr, nullptr,
                                                  nullptr), "pars_gpu_curves_download");
    }
  }
  // Extension: index and colour every traced batch on the device and copy
  // this rank's batches out with vertices, colours and indices (the
  // pipeline's stages 4.0 and 5.0 in one pass; one rank's call serves the
  // device-resident curves of all ranks, so call it from one rank).
  std::vector<integral_curves> finish(int32_t color_mode, scalar parameter)
  {
    check(dev().get(), pars_gpu_curves_index(dev().get()), "pars_gpu_curves_index");
    if (color_mode >= 0) check(dev().get(), pars_gpu_curves_color(dev().get(), color_mode, parameter), "pars_gpu_curves_color");
    const auto batches = partitioner_->communicator()->get_world().batches(rank());
    std::vector<integral_curves> out(batches.size());
    for (std::size_t k = 0; k < batches.size(); ++k)
    {
      int64_t nv = 0, ni = 0;
      check(dev().get(), pars_gpu_curves_batch_info(dev().get(), batches[k], &nv, &ni, nullptr, nullptr), "pars_gpu_curves_batch_info");
      out[k].vertices.resize(nv);
      out[k].indices.resize(ni);
      if (color_mode >= 0) out[k].colors.resize(nv);
      check(dev().get(), pars_gpu_curves_download(dev().get(), batches[k], nv ? out[k].vertices[0].data : nullptr,
                                                  (color_mode >= 0 && nv) ? out[k].colors[0].data : nullptr,
                                                  ni ? out[k].indices.data() : nullptr), "pars_gpu_curves_download");
    }
    return out;
  }

private:
  device& dev() const { return partitioner_->communicator()->get_world().get_device(); }
  integer rank() const { return partitioner_->communicator()->rank(); }

  pa_gpu::partitioner*                        partitioner_ = nullptr;
  std::optional<vector_field>*                local_vector_field_ = nullptr;
  std::array<std::optional<vector_field>, 6>* neighbor_vector_fields_ = nullptr;
  integrator                                  integrator_ = integrator::euler;   // particle_tracer.hpp:67
  scalar                                      step_size_ = 1.0f;                  // particle_tracer.hpp:68
  int32_t                                     stage_mode_ = PARS_STAGES_FROZEN;
  int32_t                                     field_ = -1;
  int                                         round_ = 0;
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
