// The stage sequence of pars::pipeline::execute (pars/source/pipeline.cpp:
// 107-337) and execute_ftle (:345-409), written against the C++ drop-in
// (include/pa_gpu.hpp).  Reads a raw field, writes the curves, the `image`
// reply of the ray tracer and the FTLE field as raw files for
// tests/test_gpu_drop_in.py to compare with the oracle.
//
// usage: drop_in_pipeline field.bin nx ny nz spacing stride iterations step out_dir
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>

#include "pa_gpu.hpp"

int main(int argc, char** argv)
{
  if (argc != 10) { std::fprintf(stderr, "usage: %s field.bin nx ny nz spacing stride iterations step out_dir\n", argv[0]); return 2; }
  pa_gpu::vector_field field;
  for (int i = 0; i < 3; ++i) field.shape[i] = std::atoi(argv[2 + i]);
  const float spacing = std::strtof(argv[5], nullptr);
  const int stride = std::atoi(argv[6]);
  const int iterations = std::atoi(argv[7]);
  const float step = std::strtof(argv[8], nullptr);
  const std::string out = argv[9];
  field.data.resize((std::size_t)field.shape[0] * field.shape[1] * field.shape[2] * 3);
  std::ifstream in(argv[1], std::ios::binary);
  in.read(reinterpret_cast<char*>(field.data.data()), field.data.size() * sizeof(float));
  if (!in) { std::fprintf(stderr, "cannot read %s\n", argv[1]); return 2; }
  for (int i = 0; i < 3; ++i)
  {
    field.spacing[i] = spacing;
    field.offset[i] = 0.0f;
    field.size[i] = float(field.shape[i]) * spacing;   // data_io.cpp:114
  }

  try
  {
    pa_gpu::device device(0);
    pa_gpu::partitioner partitioner(1, 0);
    partitioner.set_domain_size({{field.shape[0], field.shape[1], field.shape[2]}});
    const int32_t local = device.upload(field);

    // 2.0 seed_generator::generate (pipeline.cpp:113-119)
    pa_gpu::vector3 seed_stride;
    for (int i = 0; i < 3; ++i) seed_stride[i] = field.spacing[i] * float(stride);
    auto seeds = pa_gpu::seed_generator::generate(device, field.offset, field.size, seed_stride, iterations, 0);

    // 3.0 / 3.1 particle_tracer (pipeline.cpp:130-209), 3.2 prune, 4.0 index, 5.0 colour
    pa_gpu::particle_tracer tracer(device);
    tracer.set_local_vector_field(local);
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
      std::ofstream v(out + "/vertices_" + std::to_string(b) + ".bin", std::ios::binary);
      v.write(reinterpret_cast<const char*>(curves[b].vertices.data()), curves[b].vertices.size() * 16);
      std::ofstream c(out + "/colors_" + std::to_string(b) + ".bin", std::ios::binary);
      c.write(reinterpret_cast<const char*>(curves[b].colors.data()), curves[b].colors.size() * 16);
      std::ofstream i(out + "/indices_" + std::to_string(b) + ".bin", std::ios::binary);
      i.write(reinterpret_cast<const char*>(curves[b].indices.data()), curves[b].indices.size() * 4);
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
    pa_gpu::flow_map_generator flow(device);
    flow.set_vector_field(local);
    flow.set_step_size(step);
    flow.set_integrator(pa_gpu::integrator::runge_kutta_4);
    const int32_t flow_map = flow.generate(iterations, 1.0f);
    pa_gpu::ftle_map_generator ftle(device);
    ftle.set_flow_map(flow_map);
    ftle.set_time(step * float(iterations - 1));
    auto result = ftle.generate();
    std::ofstream f(out + "/ftle.bin", std::ios::binary);
    f.write(reinterpret_cast<const char*>(result->data.data()), result->data.size() * sizeof(float));
    std::printf("ok %zu batches, %lld flow-map steps\n", curves.size(), (long long)flow.last_steps());
  }
  catch (const std::exception& e)
  {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
