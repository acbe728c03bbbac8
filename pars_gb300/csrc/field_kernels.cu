// Field packing (xyz FP32 -> float4, the repack of data_io.cpp:99-106), field
// sampling (vector_field::contains + ::interpolate at given positions) and
// lattice seeding (seed_generator::generate, seed_generator.cpp:9-21).
#include "context.hpp"

namespace pars
{
namespace
{
__global__ void pack_field_kernel(const float* __restrict__ xyz, float4* __restrict__ out, long long count)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  out[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f);
}

__global__ void unpack_field_kernel(const float4* __restrict__ data, float* __restrict__ xyz, long long count)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float4 v = data[i];
  xyz[3 * i] = v.x; xyz[3 * i + 1] = v.y; xyz[3 * i + 2] = v.z;
}

__global__ void sample_kernel(const field_view f, const float4* __restrict__ positions, long long n,
                              uint8_t* __restrict__ inside, float* __restrict__ velocity)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float3 v = make_float3(0.f, 0.f, 0.f);
  const bool in = sample_inside(f, positions[i], v);
  inside[i] = in ? 1 : 0;
  velocity[3 * i] = in ? v.x : 0.0f;
  velocity[3 * i + 1] = in ? v.y : 0.0f;
  velocity[3 * i + 2] = in ? v.z : 0.0f;
}

struct seed_args
{
  float ox, oy, oz, sx, sy, sz;
  int   px, py, pz;
  int   iterations, rank;
  pars_particle* out;
};

// position = offset + stride * index (FP32, no contraction); C-order index.
__global__ void seed_kernel(const seed_args a)
{
  const long long total = (long long)a.px * a.py * a.pz;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int iz = int(i % a.pz);
  const int iy = int((i / a.pz) % a.py);
  const int ix = int(i / ((long long)a.pz * a.py));
  pars_particle p;
  p.position[0] = __fadd_rn(a.ox, __fmul_rn(a.sx, float(ix)));
  p.position[1] = __fadd_rn(a.oy, __fmul_rn(a.sy, float(iy)));
  p.position[2] = __fadd_rn(a.oz, __fmul_rn(a.sz, float(iz)));
  p.position[3] = 0.0f;
  p.remaining_iterations = a.iterations;
  p.vector_field_index = -1;
  p.original_rank = a.rank;
  p.original_voxel[0] = ix; p.original_voxel[1] = iy; p.original_voxel[2] = iz;
  p.padding[0] = p.padding[1] = 0;
  a.out[i] = p;
}
}

void launch_pack_field(pars_gpu_context& ctx, const float* xyz, float4* out, long long count)
{
  if (count <= 0) return;
  launch_scope scope(ctx, "field_pack");
  pack_field_kernel<<<(unsigned)((count + 255) / 256), 256, 0, ctx.stream>>>(xyz, out, count);
}

void launch_unpack_field(pars_gpu_context& ctx, const float4* data, float* xyz, long long count)
{
  if (count <= 0) return;
  launch_scope scope(ctx, "field_unpack");
  unpack_field_kernel<<<(unsigned)((count + 255) / 256), 256, 0, ctx.stream>>>(data, xyz, count);
}

void launch_field_sample(pars_gpu_context& ctx, const field_view& f, const float4* positions, long long n, uint8_t* inside, float* velocity)
{
  if (n <= 0) return;
  launch_scope scope(ctx, "field_sample");
  sample_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx.stream>>>(f, positions, n, inside, velocity);
}

void launch_seed_generate(pars_gpu_context& ctx, const float offset[3], const float stride[3], const int per_dimension[3],
                          int iterations, int rank, pars_particle* out)
{
  seed_args a;
  a.ox = offset[0]; a.oy = offset[1]; a.oz = offset[2];
  a.sx = stride[0]; a.sy = stride[1]; a.sz = stride[2];
  a.px = per_dimension[0]; a.py = per_dimension[1]; a.pz = per_dimension[2];
  a.iterations = iterations; a.rank = rank; a.out = out;
  const long long total = (long long)a.px * a.py * a.pz;
  if (total <= 0) return;
  launch_scope scope(ctx, "seed_generate");
  seed_kernel<<<(unsigned)((total + 255) / 256), 256, 0, ctx.stream>>>(a);
}
}
