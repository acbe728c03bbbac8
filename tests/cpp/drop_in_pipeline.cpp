// The stage sequence of pars::pipeline::execute (pars/source/pipeline.cpp:
// 107-337) and execute_ftle (:345-409), written against the C++ drop-in
// (include/pa_gpu.hpp).  Writes the curves, the `image` reply of the ray
// tracer and the FTLE field as raw files for tests/test_gpu_drop_in.py to
// compare with the oracle.
//
// usage:
//   drop_in_pipeline single field.bin nx ny nz spacing stride iterations step out_dir
//     one rank: seeds, the round loop, prune, index, colour, ray tracer, FTLE
//   drop_in_pipeline multi domain.bin nx ny nz spacing ranks seeds.bin offsets.bin step out_dir
//     `ranks` threads, one per rank as pars runs one MPI process per rank, each
//     running pipeline.cpp's round loop (:153-209) stage by stage on its own
//     ghosted block, then prune, index and rgb colours; seeds.bin holds the
//     pa::particle records of all ranks, offsets.bin (int64, ranks + 1) where
//     each rank's begin.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <thread>

#include "pa_gpu.hpp"

namespace
{
template <typename T> std::vector<T> read_file(const std::string& path, std::size_t count)
{
  std::vector<T> out(count);
  std::ifstream in(path, std::ios::binary);
  in.read(reinterpret_cast<char*>(out.data()), (std::streamsize)(count * sizeof(T)));
  if (!in) throw std::runtime_error("cannot read " + path);
  return out;
}

template <typename T> void write_file(const std::string& path, const std::vector<T>& data)
{
  std::ofstream out(path, std::ios::binary);
  out.write(reinterpret_cast<const char*>(data.data()), (std::streamsize)(data.size() * sizeof(T)));
}

// data_io::load_local_vector_field (data_io.cpp:90-114) on an in-memory
// domain: the rank's ghosted block, offset = voxel offset * spacing, size =
// block size * spacing.
pa_gpu::vector_field local_block(const std::vector<float>& domain, const pa_gpu::ivector3& domain_size, float spacing,
                                 const pa_gpu::partitioner& partitioner)
{
  const auto& info = partitioner.local_rank_info().value();
  pa_gpu::vector_field f;
  for (int i = 0; i < 3; ++i)
  {
    f.shape[i] = info.ghosted_block_size[i];
    f.spacing[i] = spacing;
    f.offset[i] = float(info.offset[i]) * spacing;
    f.size[i] = float(partitioner.block_size()[i]) * spacing;
  }
  f.data.resize((std::size_t)f.shape[0] * f.shape[1] * f.shape[2] * 3);
  for (int x = 0; x < f.shape[0]; ++x)
    for (int y = 0; y < f.shape[1]; ++y)
      for (int z = 0; z < f.shape[2]; ++z)
      {
        const std::size_t src = (((std::size_t)(info.offset[0] + x) * domain_size[1] + (info.offset[1] + y)) * domain_size[2] +
                                 (info.offset[2] + z)) * 3;
        const std::size_t dst = (((std::size_t)x * f.shape[1] + y) * f.shape[2] + z) * 3;
        for (int c = 0; c < 3; ++c) f.data[dst + c] = domain[src + c];
      }
  return f;
}

// One rank of the multi-rank run: pipeline.cpp's stages 3.0-5.0.
void run_rank(pa_gpu::world& world, int rank, const std::vector<float>& domain, const pa_gpu::ivector3& domain_size,
              float spacing, std::vector<pa_gpu::particle> seeds, float step, const std::string& out, std::string& error)
{
  try
  {
    pa_gpu::communicator communicator(world, rank);
    pa_gpu::partitioner partitioner(&communicator);
    partitioner.set_domain_size(domain_size);
    std::optional<pa_gpu::vector_field> local_vector_field = local_block(domain, domain_size, spacing, partitioner);
    std::array<std::optional<pa_gpu::vector_field>, 6> neighbor_vector_fields {};

    // 3.0 particle_tracer::initialize (pipeline.cpp:127-131)
    pa_gpu::particle_tracer particle_tracer(&partitioner);
    particle_tracer.set_local_vector_field(&local_vector_field);
    particle_tracer.set_neighbor_vector_fields(&neighbor_vector_fields);
    particle_tracer.set_step_size(step);
    particle_tracer.set_integrator(pa_gpu::integrator::runge_kutta_4);

    // 3.1 particle_tracer::trace, round by round (pipeline.cpp:153-209)
    std::vector<pa_gpu::integral_curves> integral_curves;
    std::vector<int> batch_round;
    int  round_counter = 0;
    bool complete      = false;
    while (!complete)
    {
      pa_gpu::particle_tracer::round_info round_info;
      round_info = particle_tracer.compute_round_info(seeds, integral_curves);
      particle_tracer.allocate(integral_curves, round_info);
      particle_tracer.initialize(seeds, integral_curves, round_info);
      particle_tracer.trace(seeds, integral_curves, round_info);
      particle_tracer.out_of_bounds_distribute(seeds, round_info);
      complete = particle_tracer.check_completion(seeds);
      batch_round.insert(batch_round.end(), round_info.integral_curve_count, round_counter);
      round_counter++;
    }
    // 3.2 prune, 4.0 index_generator, 5.0 color_generator (pipeline.cpp:213-260)
    particle_tracer.prune(integral_curves);
    pa_gpu::device& device = world.get_device();
    std::ofstream meta(out + "/rank_" + std::to_string(rank) + ".txt");
    for (std::size_t b = 0; b < integral_curves.size(); ++b)
    {
      pa_gpu::index_generator::generate(device, &integral_curves[b]);
      pa_gpu::color_generator::generate(device, &integral_curves[b], pa_gpu::color_generator::mode::rgb);
      const std::string name = out + "/rank_" + std::to_string(rank) + "_batch_" + std::to_string(b);
      write_file(name + "_vertices.bin", integral_curves[b].vertices);
      write_file(name + "_colors.bin", integral_curves[b].colors);
      write_file(name + "_indices.bin", integral_curves[b].indices);
      meta << batch_round[b] << " " << integral_curves[b].vertices.size() << " " << integral_curves[b].indices.size() << "\n";
    }
  }
  catch (const std::exception& e)
  {
    error = e.what();
  }
}

int run_multi(char** argv)
{
  pa_gpu::ivector3 domain_size;
  for (int i = 0; i < 3; ++i) domain_size[i] = std::atoi(argv[3 + i]);
  const float spacing = std::strtof(argv[6], nullptr);
  const int ranks = std::atoi(argv[7]);
  const float step = std::strtof(argv[10], nullptr);
  const std::string out = argv[11];
  const auto domain = read_file<float>(argv[2], (std::size_t)domain_size[0] * domain_size[1] * domain_size[2] * 3);
  const auto offsets = read_file<int64_t>(argv[9], (std::size_t)ranks + 1);
  const auto seeds = read_file<pa_gpu::particle>(argv[8], (std::size_t)offsets[ranks]);

  pa_gpu::device device(0);
  pa_gpu::world world(device, ranks);
  std::vector<std::thread> threads;
  std::vector<std::string> errors(ranks);
  for (int r = 0; r < ranks; ++r)
    threads.emplace_back(run_rank, std::ref(world), r, std::cref(domain), domain_size, spacing,
                         std::vector<pa_gpu::particle>(seeds.begin() + offsets[r], seeds.begin() + offsets[r + 1]), step, out,
                         std::ref(errors[r]));
  for (auto& t : threads) t.join();
  for (int r = 0; r < ranks; ++r)
    if (!errors[r].empty()) { std::fprintf(stderr, "rank %d: %s\n", r, errors[r].c_str()); return 1; }
  std::printf("ok %d ranks\n", ranks);
  return 0;
}

int run_single(char** argv)
{
  pa_gpu::vector_field field;
  for (int i = 0; i < 3; ++i) field.shape[i] = std::atoi(argv[3 + i]);
  const float spacing = std::strtof(argv[6], nullptr);
  const int stride = std::atoi(argv[7]);
  const int iterations = std::atoi(argv[8]);
  const float step = std::strtof(argv[9], nullptr);
  const std::string out = argv[10];
  field.data = read_file<float>(argv[2], (std::size_t)field.shape[0] * field.shape[1] * field.shape[2] * 3);
  for (int i = 0; i < 3; ++i)
  {
    field.spacing[i] = spacing;
    field.offset[i] = 0.0f;
    field.size[i] = float(field.shape[i]) * spacing;   // data_io.cpp:114
  }

  pa_gpu::device device(0);
  pa_gpu::world world(device, 1);
  pa_gpu::communicator communicator(world, 0);
  pa_gpu::partitioner partitioner(&communicator);
  partitioner.set_domain_size({{field.shape[0], field.shape[1], field.shape[2]}});
  std::optional<pa_gpu::vector_field> local = field;

  // 2.0 seed_generator::generate (pipeline.cpp:113-119)
  pa_gpu::vector3 seed_stride;
  for (int i = 0; i < 3; ++i) seed_stride[i] = field.spacing[i] * float(stride);
  auto seeds = pa_gpu::seed_generator::generate(device, field.offset, field.size, seed_stride, iterations, 0);

  // 3.0 / 3.1 particle_tracer (pipeline.cpp:130-209: the whole trace of
  // particle_tracer.cpp:39-56), 3.2 prune, then 4.0 index and 5.0 colour of
  // the device-resident curves
  pa_gpu::particle_tracer tracer(&partitioner);
  tracer.set_local_vector_field(&local);
  tracer.set_step_size(step);
  tracer.set_integrator(pa_gpu::integrator::runge_kutta_4);
  auto traced = tracer.trace(seeds);
  auto curves = tracer.finish(PARS_COLOR_HSV_CONSTANT_S, 0.75f);
  std::ofstream meta(out + "/curves.txt");
  meta << curves.size() << "\n";
  for (std::size_t b = 0; b < curves.size(); ++b)
  {
    if (traced[b].vertices.size() != curves[b].vertices.size()) { std::fprintf(stderr, "trace/finish mismatch\n"); return 1; }
    meta << curves[b].vertices.size() << " " << curves[b].indices.size() << "\n";
    write_file(out + "/vertices_" + std::to_string(b) + ".bin", curves[b].vertices);
    write_file(out + "/colors_" + std::to_string(b) + ".bin", curves[b].colors);
    write_file(out + "/indices_" + std::to_string(b) + ".bin", curves[b].indices);
    // The host-buffer stage drop-ins agree with the device-resident pass.
    pa_gpu::integral_curves again;
    again.vertices = curves[b].vertices;
    pa_gpu::index_generator::generate(device, &again);
    if (again.indices != curves[b].indices) { std::fprintf(stderr, "index_generator mismatch\n"); return 1; }
  }

  // 6.0-6.6 ray_tracer: camera, image size, the curves, trace, serialize
  pa_gpu::ray_tracer tracer6(device);
  tracer6.set_camera(pa_gpu::vector3 {{3.0f, 3.2f, 13.0f}}, pa_gpu::vector3 {{0.0f, 0.0f, -1.0f}}, pa_gpu::vector3 {{0.0f, 1.0f, 0.0f}});
  tracer6.set_image_size(64, 48);
  tracer6.set_integral_curves(curves, 0.05f);
  tracer6.trace(2);
  const std::string image = tracer6.serialize();
  std::ofstream im(out + "/image.bin", std::ios::binary);
  im.write(image.data(), (std::streamsize)image.size());

  // execute_ftle: 2.1 flow_map_generator, 3.0-3.1 ftle_map_generator
  const int32_t handle = device.upload(field);
  pa_gpu::flow_map_generator flow(device);
  flow.set_vector_field(handle);
  flow.set_step_size(step);
  flow.set_integrator(pa_gpu::integrator::runge_kutta_4);
  const int32_t flow_map = flow.generate(iterations, 1.0f);
  pa_gpu::ftle_map_generator ftle(device);
  ftle.set_flow_map(flow_map);
  ftle.set_time(step * float(iterations - 1));
  auto result = ftle.generate();
  write_file(out + "/ftle.bin", result->data);
  std::printf("ok %zu batches, %lld flow-map steps\n", curves.size(), (long long)flow.last_steps());
  return 0;
}
}

int main(int argc, char** argv)
{
  try
  {
    if (argc == 11 && std::string(argv[1]) == "single") return run_single(argv);
    if (argc == 12 && std::string(argv[1]) == "multi") return run_multi(argv);
  }
  catch (const std::exception& e)
  {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  std::fprintf(stderr, "usage: %s single field.bin nx ny nz spacing stride iterations step out_dir\n"
                       "       %s multi domain.bin nx ny nz spacing ranks seeds.bin offsets.bin step out_dir\n", argv[0], argv[0]);
  return 2;
}
