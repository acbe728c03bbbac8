// C-ABI driver around the reference's own hot-path classes, compiled from the
// unmodified reference sources against the stand-ins in oracle/ref_shim.
// It runs the stage sequence of pars::pipeline::execute (pars/source/pipeline.cpp:
// 153-260, load balancing off) and pipeline::execute_ftle (pipeline.cpp:339-409)
// and hands the results back as flat arrays.  Test infrastructure only: it is
// used in the development container to pin the CPU restatement (oracle/
// pars_oracle.cpp) and to write the golden fixtures under tests/golden/.
#include <pa/math/integral_curves.hpp>
#include <pa/math/integrators.hpp>
#include <pa/math/particle.hpp>
#include <pa/math/vector_field.hpp>
#include <pa/stages/color_generator.hpp>
#include <pa/stages/flow_map_generator.hpp>
#include <pa/stages/ftle_map_generator.hpp>
#include <pa/stages/index_generator.hpp>
#include <pa/stages/particle_tracer.hpp>
#include <pa/stages/partitioner.hpp>
#include <pa/stages/seed_generator.hpp>

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

static_assert(sizeof(pa::particle) == 48, "pa::particle is 48 bytes");
static_assert(offsetof(pa::particle, remaining_iterations) == 16, "layout");
static_assert(offsetof(pa::particle, vector_field_index) == 20, "layout");
static_assert(offsetof(pa::particle, original_rank) == 24, "layout");
static_assert(offsetof(pa::particle, original_voxel) == 28, "layout");

namespace
{
pa::variant_integrator make_integrator(int kind)
{
  switch (kind)
  {
  case 0: return pa::euler_integrator();
  case 1: return pa::modified_midpoint_integrator();
  case 2: return pa::runge_kutta_4_integrator();
  case 3: return pa::runge_kutta_cash_karp_54_integrator();
  case 4: return pa::runge_kutta_dormand_prince_5_integrator();
  case 5: return pa::runge_kutta_fehlberg_78_integrator();
  case 6: return pa::adams_bashforth_2_integrator();
  default: return pa::adams_bashforth_moulton_2_integrator();
  }
}

void fill_field(pa::vector_field& field, const float* xyz, const int dims[3], const float offset[3], const float size[3], const float spacing[3])
{
  field.data.resize(std::array<int, 3>{dims[0], dims[1], dims[2]});
  const std::size_t count = std::size_t(dims[0]) * dims[1] * dims[2];
  for (std::size_t i = 0; i < count; ++i)
    field.data.data()[i] = pa::vector3(xyz[3 * i + 0], xyz[3 * i + 1], xyz[3 * i + 2]);
  field.offset  = pa::vector3(offset[0], offset[1], offset[2]);
  field.size    = pa::vector3(size[0], size[1], size[2]);
  field.spacing = pa::vector3(spacing[0], spacing[1], spacing[2]);
}

pa::color_generator::mode color_mode(int mode)
{
  switch (mode)
  {
  case 0: return pa::color_generator::mode::hsl_constant_s;
  case 1: return pa::color_generator::mode::hsl_constant_l;
  case 2: return pa::color_generator::mode::hsv_constant_s;
  case 3: return pa::color_generator::mode::hsv_constant_v;
  default: return pa::color_generator::mode::rgb;
  }
}

// Colours the reference never writes keep this marker (color_generator.cpp:46
// resizes without initialising), so tests can tell them apart.
const float unwritten_color = std::numeric_limits<float>::quiet_NaN();

void index_and_color(pa::integral_curves& curves, int mode, float parameter)
{
  // index_generator::generate on an empty batch iterates up to size()-1 = SIZE_MAX
  // (index_generator.cpp:17), which is undefined; such batches are skipped.
  if (curves.vertices.empty()) return;
  pa::index_generator::generate(&curves);
  curves.colors.assign(curves.vertices.size(), pa::vector4::Constant(unwritten_color));
  if (mode >= 0) pa::color_generator::generate(&curves, color_mode(mode), parameter);
}
}

struct ref_curves
{
  std::vector<pa::integral_curves> batches;
  std::vector<int>                 batch_rank;
  std::vector<int>                 batch_round;
};

extern "C" {

long long ref_curves_batches(const ref_curves* c) { return (long long)c->batches.size(); }
long long ref_curves_vertex_count(const ref_curves* c, long long b) { return (long long)c->batches[b].vertices.size(); }
long long ref_curves_index_count(const ref_curves* c, long long b) { return (long long)c->batches[b].indices.size(); }
long long ref_curves_color_count(const ref_curves* c, long long b) { return (long long)c->batches[b].colors.size(); }
const float* ref_curves_vertices(const ref_curves* c, long long b) { return c->batches[b].vertices.empty() ? nullptr : c->batches[b].vertices[0].data(); }
const float* ref_curves_colors(const ref_curves* c, long long b) { return c->batches[b].colors.empty() ? nullptr : c->batches[b].colors[0].data(); }
const int* ref_curves_indices(const ref_curves* c, long long b) { return c->batches[b].indices.empty() ? nullptr : c->batches[b].indices.data(); }
int ref_curves_batch_rank(const ref_curves* c, long long b) { return c->batch_rank[b]; }
int ref_curves_batch_round(const ref_curves* c, long long b) { return c->batch_round[b]; }
void ref_curves_free(ref_curves* c) { delete c; }

// vector_field::contains and ::interpolate at n positions (vector_field.cpp:12-48).
void ref_field_sample(const float* xyz, const int dims[3], const float offset[3], const float size[3], const float spacing[3],
                      const float* positions, long long n, unsigned char* inside, float* velocity)
{
  pa::vector_field field;
  fill_field(field, xyz, dims, offset, size, spacing);
  for (long long i = 0; i < n; ++i)
  {
    const pa::vector4 p(positions[4 * i], positions[4 * i + 1], positions[4 * i + 2], positions[4 * i + 3]);
    inside[i] = field.contains(p) ? 1 : 0;
    if (inside[i])
    {
      const pa::vector3 v = field.interpolate(p);
      velocity[3 * i] = v[0]; velocity[3 * i + 1] = v[1]; velocity[3 * i + 2] = v[2];
    }
    else velocity[3 * i] = velocity[3 * i + 1] = velocity[3 * i + 2] = 0.0f;
  }
}

// seed_generator::generate (seed_generator.cpp:9-21).  Returns the count; writes
// the particles when out is not null.
long long ref_seed_generate(const float offset[3], const float size[3], const float stride[3], int iterations, int rank, void* out)
{
  auto particles = pa::seed_generator::generate(pa::vector3(offset[0], offset[1], offset[2]), pa::vector3(size[0], size[1], size[2]),
                                                pa::vector3(stride[0], stride[1], stride[2]), iterations, rank);
  if (out) std::memcpy(out, particles.data(), particles.size() * sizeof(pa::particle));
  return (long long)particles.size();
}

// partitioner::set_domain_size for `ranks` ranks as seen from `rank`
// (partitioner.cpp:8-53).  info = grid[3], block[3], multi_rank[3], offset[3],
// ghosted_block_size[3], neighbor ranks[6] (-1 where absent).
void ref_partition(int ranks, int rank, const int domain[3], int* info)
{
  auto world = std::make_shared<pars_shim::world>(ranks);
  boost::mpi::communicator comm(world, rank);
  pa::partitioner partitioner(&comm);
  partitioner.set_domain_size(pa::ivector3(domain[0], domain[1], domain[2]));
  for (int i = 0; i < 3; ++i)
  {
    info[i]      = partitioner.grid_size()[i];
    info[3 + i]  = partitioner.block_size()[i];
    info[6 + i]  = partitioner.local_rank_info()->multi_rank[i];
    info[9 + i]  = partitioner.local_rank_info()->offset[i];
    info[12 + i] = partitioner.local_rank_info()->ghosted_block_size[i];
  }
  for (int f = 0; f < 6; ++f)
    info[15 + f] = partitioner.neighbor_rank_info()[f] ? partitioner.neighbor_rank_info()[f]->rank : -1;
}

// One rank, one block: the round loop of pipeline.cpp:160-208 (load balancing
// off), prune (:219), index (:230-233) and colour (:256-259) per batch.
// color_mode < 0 skips colouring.
ref_curves* ref_trace_single(const float* xyz, const int dims[3], const float offset[3], const float size[3], const float spacing[3],
                             const void* particles_in, long long n, int integrator, float step, int color, float parameter)
{
  boost::mpi::communicator comm;
  pa::partitioner partitioner(&comm);
  partitioner.set_domain_size(pa::ivector3(dims[0], dims[1], dims[2]));

  std::optional<pa::vector_field> local;
  local.emplace();
  fill_field(*local, xyz, dims, offset, size, spacing);
  std::array<std::optional<pa::vector_field>, 6> neighbors;

  pa::particle_tracer tracer(&partitioner);
  tracer.set_local_vector_field(&local);
  tracer.set_neighbor_vector_fields(&neighbors);
  tracer.set_step_size(step);
  tracer.set_integrator(make_integrator(integrator));

  std::vector<pa::particle> seeds(n);
  if (n) std::memcpy(seeds.data(), particles_in, n * sizeof(pa::particle));

  auto* result = new ref_curves();
  int round = 0;
  bool complete = seeds.empty();
  while (!complete)
  {
    auto info = tracer.compute_round_info(seeds, result->batches);
    tracer.allocate(result->batches, info);
    tracer.initialize(seeds, result->batches, info);
    tracer.trace(seeds, result->batches, info);
    tracer.out_of_bounds_distribute(seeds, info);
    complete = tracer.check_completion(seeds);
    while (result->batch_rank.size() < result->batches.size()) { result->batch_rank.push_back(0); result->batch_round.push_back(round); }
    ++round;
  }
  tracer.prune(result->batches);
  for (auto& batch : result->batches) index_and_color(batch, color, parameter);
  return result;
}

// Several blocks, one thread per rank (in-process MPI stand-in), load balancing
// off: each rank holds its ghosted block of the domain field (data_io.cpp:91-115
// without the file), traces the seeds it owns, and hands particles that leave
// its block to the face neighbour every round (particle_tracer.cpp:280-309,
// 376-393).  seed_offsets[r]..seed_offsets[r+1] are rank r's seeds.
ref_curves* ref_trace_multi(const float* xyz, const int domain[3], const float spacing[3], int ranks,
                            const long long* seed_offsets, const void* seeds_in, int integrator, float step, int color, float parameter)
{
  auto world = std::make_shared<pars_shim::world>(ranks);
  std::vector<ref_curves> per_rank(ranks);
  std::vector<std::thread> threads;
  for (int rank = 0; rank < ranks; ++rank)
  {
    threads.emplace_back([&, rank]
    {
      pars_shim::set_serial(true);
      boost::mpi::communicator comm(world, rank);
      pa::partitioner partitioner(&comm);
      partitioner.set_domain_size(pa::ivector3(domain[0], domain[1], domain[2]));
      const auto& info = *partitioner.local_rank_info();

      std::optional<pa::vector_field> local;
      local.emplace();
      local->data.resize(std::array<int, 3>{info.ghosted_block_size[0], info.ghosted_block_size[1], info.ghosted_block_size[2]});
      for (int x = 0; x < info.ghosted_block_size[0]; ++x)
        for (int y = 0; y < info.ghosted_block_size[1]; ++y)
          for (int z = 0; z < info.ghosted_block_size[2]; ++z)
          {
            const std::size_t g = (std::size_t(info.offset[0] + x) * domain[1] + (info.offset[1] + y)) * domain[2] + (info.offset[2] + z);
            local->data[x][y][z] = pa::vector3(xyz[3 * g], xyz[3 * g + 1], xyz[3 * g + 2]);
          }
      const pa::vector3 h(spacing[0], spacing[1], spacing[2]);
      local->spacing = h;
      local->offset  = info.offset.cast<float>().array() * h.array();
      local->size    = partitioner.block_size().cast<float>().array() * h.array();
      std::array<std::optional<pa::vector_field>, 6> neighbors;

      pa::particle_tracer tracer(&partitioner);
      tracer.set_local_vector_field(&local);
      tracer.set_neighbor_vector_fields(&neighbors);
      tracer.set_step_size(step);
      tracer.set_integrator(make_integrator(integrator));

      const long long begin = seed_offsets[rank], end = seed_offsets[rank + 1];
      std::vector<pa::particle> seeds(end - begin);
      if (end > begin) std::memcpy(seeds.data(), static_cast<const pa::particle*>(seeds_in) + begin, (end - begin) * sizeof(pa::particle));

      auto& result = per_rank[rank];
      int round = 0;
      bool complete = tracer.check_completion(seeds);
      while (!complete)
      {
        // compute_round_info dereferences max_element of an empty list
        // (particle_tracer.cpp:214), so a rank without particles this round
        // only builds the neighbour map the exchange needs.
        pa::particle_tracer::round_info round_info;
        if (!seeds.empty())
        {
          round_info = tracer.compute_round_info(seeds, result.batches);
          tracer.allocate(result.batches, round_info);
          tracer.initialize(seeds, result.batches, round_info);
          tracer.trace(seeds, result.batches, round_info);
        }
        else
        {
          round_info.maximum_remaining_iterations = round_info.vertices_per_integral_curve = 0;
          round_info.vertices_per_integral_curve_last = 0;
          round_info.integral_curve_offset = result.batches.size();
          round_info.integral_curve_count = 0;
          for (auto& neighbor : partitioner.neighbor_rank_info())
            if (neighbor)
            {
              round_info.out_of_bounds_particles.emplace(neighbor->rank, std::vector<pa::particle>());
              round_info.neighbor_out_of_bounds_particles.emplace(neighbor->rank, std::vector<pa::particle>());
            }
        }
        tracer.out_of_bounds_distribute(seeds, round_info);
        complete = tracer.check_completion(seeds);
        while (result.batch_round.size() < result.batches.size()) { result.batch_rank.push_back(rank); result.batch_round.push_back(round); }
        ++round;
      }
      tracer.prune(result.batches);
      for (auto& batch : result.batches) index_and_color(batch, color, parameter);
    });
  }
  for (auto& t : threads) t.join();

  auto* result = new ref_curves();
  for (auto& r : per_rank)
    for (std::size_t b = 0; b < r.batches.size(); ++b)
    {
      result->batches.push_back(std::move(r.batches[b]));
      result->batch_rank.push_back(r.batch_rank[b]);
      result->batch_round.push_back(r.batch_round[b]);
    }
  return result;
}

// index_generator::generate on one vertex buffer (index_generator.cpp:10-24).
long long ref_index_generate(const float* vertices, long long n, int* indices)
{
  pa::integral_curves curves;
  curves.vertices.resize(n);
  if (n) std::memcpy(curves.vertices[0].data(), vertices, n * 16);
  if (n == 0) return 0;
  pa::index_generator::generate(&curves);
  if (indices) std::memcpy(indices, curves.indices.data(), curves.indices.size() * sizeof(int));
  return (long long)curves.indices.size();
}

// color_generator::generate on one vertex/index buffer (color_generator.cpp:16-39).
void ref_color_generate(const float* vertices, long long n, const int* indices, long long n_indices, int mode, float parameter, float* colors)
{
  pa::integral_curves curves;
  curves.vertices.resize(n);
  if (n) std::memcpy(curves.vertices[0].data(), vertices, n * 16);
  curves.indices.assign(indices, indices + n_indices);
  curves.colors.assign(n, pa::vector4::Constant(unwritten_color));
  pa::color_generator::generate(&curves, color_mode(mode), parameter);
  if (n) std::memcpy(colors, curves.colors[0].data(), n * 16);
}

// flow_map_generator::generate (flow_map_generator.cpp:12-52) on one block.
// flow is [X'][Y'][Z'][3] with X' = int(dims * resolution_scale); returns the
// number of flow-map voxels.  out_dims receives X', Y', Z'.
long long ref_flow_map(const float* xyz, const int dims[3], const float offset[3], const float size[3], const float spacing[3],
                       int iterations, float resolution_scale, int integrator, float step, float* flow, int* out_dims)
{
  boost::mpi::communicator comm;
  pa::partitioner partitioner(&comm);
  partitioner.set_domain_size(pa::ivector3(dims[0], dims[1], dims[2]));
  pa::vector_field field;
  fill_field(field, xyz, dims, offset, size, spacing);
  pa::flow_map_generator generator(&partitioner);
  generator.set_vector_field(&field);
  generator.set_integrator(make_integrator(integrator));
  generator.set_step_size(step);
  std::cout.setstate(std::ios::failbit);
  auto flow_map = generator.generate(std::size_t(iterations), resolution_scale);
  std::cout.clear();
  for (int i = 0; i < 3; ++i) out_dims[i] = int(flow_map->data.shape()[i]);
  const std::size_t count = flow_map->data.num_elements();
  if (flow)
    for (std::size_t i = 0; i < count; ++i)
      for (int c = 0; c < 3; ++c) flow[3 * i + c] = flow_map->data.data()[i][c];
  return (long long)count;
}

// ftle_map_generator::generate (ftle_map_generator.cpp:22-60), as written: it
// inherits the reference gradient's defects (vector_field.cpp:49-93).
void ref_ftle(const float* flow, const int dims[3], const float offset[3], const float size[3], const float spacing[3], float time, int mode, float* out)
{
  boost::mpi::communicator comm;
  pa::partitioner partitioner(&comm);
  partitioner.set_domain_size(pa::ivector3(dims[0], dims[1], dims[2]));
  pa::vector_field flow_map;
  fill_field(flow_map, flow, dims, offset, size, spacing);
  pa::ftle_map_generator generator(&partitioner, mode == 0 ? pa::ftle_map_generator::mode::regular : pa::ftle_map_generator::mode::fractional_anisotropy);
  generator.set_flow_map(&flow_map);
  generator.set_time(time);
  auto ftle = generator.generate();
  std::memcpy(out, ftle->data.data(), ftle->data.num_elements() * sizeof(float));
}

}
