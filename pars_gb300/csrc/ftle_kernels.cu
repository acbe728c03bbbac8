// Flow-map advection and the fused FTLE kernel.
//
// flow map: one thread per seed of flow_map_generator's lattice
//   (flow_map_generator.cpp:23-43 + seed_generator.cpp:9-21, seeds generated in
//   the kernel from the voxel index), advected with particle_advector's rules
//   (particle_advector.cpp:74-139, one block: a particle stops with its current
//   position when it leaves the grid, meets a zero velocity, or has taken
//   iterations - 1 steps) and written to its voxel (flow_map_generator.cpp:44-52).
// FTLE: per voxel, the flow map's central-difference gradient J (FP32, one-sided
//   at the borders), the Cauchy-Green tensor C = J^T J and its largest
//   eigenvalue in FP64 by the trigonometric closed form (O. K. Smith, CACM 4(4),
//   1961; its cosine refined by Newton steps, see largest_eigenvalue), then
//   log(sqrt(lambda)) / |T| = 0.5 log(lambda) / |T| in FP64, stored as FP32 — the intent of
//   vector_field::gradient + ftle_map_generator::generate
//   (vector_field.cpp:49-93, ftle_map_generator.cpp:22-60).
#include "context.hpp"

namespace pars
{
namespace
{
struct flow_map_args
{
  field_view f;
  step_rule  rule;
  int        iterations;
  float      ox, oy, oz;          // seed lattice offset
  float      sx, sy, sz;          // seed lattice spacing (field spacing / scale)
  int        px, py, pz;          // seeds per dimension
  int        fx, fy, fz;          // flow-map shape
  float4*    flow;
  unsigned long long* steps;
};

template <bool FROZEN>
__global__ void __launch_bounds__(256) flow_map_kernel(const __grid_constant__ flow_map_args a)
{
  const long long total = (long long)a.px * a.py * a.pz;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int steps = 0;
  if (i < total)
  {
    const int iz = int(i % a.pz);
    const int iy = int((i / a.pz) % a.py);
    const int ix = int(i / ((long long)a.pz * a.py));
    float4 pos = make_float4(__fadd_rn(a.ox, __fmul_rn(a.sx, float(ix))), __fadd_rn(a.oy, __fmul_rn(a.sy, float(iy))),
                             __fadd_rn(a.oz, __fmul_rn(a.sz, float(iz))), 0.0f);
    bool finished = false;
    float3 lo = make_float3(0.0f, 0.0f, 0.0f);
    corner_cache cache;
    frozen_history hist;
    for (int it = 1; it < a.iterations; ++it)
    {
      float3 v;
      bool inside;
      if (FROZEN) inside = sample_inside(a.f, pos, v);
      else        inside = sample_start(a.f, cache, pos, v);
      if (!inside) { finished = true; break; }
      if (is_zero(v)) { finished = true; break; }
      if (FROZEN) pos = frozen_step(a.rule, pos, v, hist);
      else resampled_step_cached(a.f, cache, a.rule, pos, lo, v);
      ++steps;
      if (it + 1 == a.iterations) { finished = true; break; }
    }
    // With iterations <= 1 the reference never assigns the voxel; it keeps the
    // seed position here.
    (void)finished;
    if (ix < a.fx && iy < a.fy && iz < a.fz)
      a.flow[((long long)ix * a.fy + iy) * a.fz + iz] = pos;
  }
  const unsigned int warp_steps = __reduce_add_sync(0xffffffffu, steps);
  if ((threadIdx.x & 31) == 0 && warp_steps) atomicAdd(a.steps, (unsigned long long)warp_steps);
}

// Eigenvalues of a symmetric 3x3 matrix in descending order (trigonometric form).
__device__ void symmetric_eigenvalues(double a00, double a01, double a02, double a11, double a12, double a22, double out[3])
{
  const double p1 = a01 * a01 + a02 * a02 + a12 * a12;
  if (p1 == 0.0)
  {
    double x = a00, y = a11, z = a22, t;
    if (x < y) { t = x; x = y; y = t; }
    if (y < z) { t = y; y = z; z = t; }
    if (x < y) { t = x; x = y; y = t; }
    out[0] = x; out[1] = y; out[2] = z;
    return;
  }
  const double q  = (a00 + a11 + a22) / 3.0;
  const double d0 = a00 - q, d1 = a11 - q, d2 = a22 - q;
  const double p  = sqrt((d0 * d0 + d1 * d1 + d2 * d2 + 2.0 * p1) / 6.0);
  const double inv = 1.0 / p;
  const double b00 = d0 * inv, b11 = d1 * inv, b22 = d2 * inv, b01 = a01 * inv, b02 = a02 * inv, b12 = a12 * inv;
  const double det = b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02);
  double r = 0.5 * det;
  r = r < -1.0 ? -1.0 : (r > 1.0 ? 1.0 : r);
  const double phi = acos(r) / 3.0;
  out[0] = q + 2.0 * p * cos(phi);
  out[2] = q + 2.0 * p * cos(phi + 2.0943951023931954923);   // 2 pi / 3
  out[1] = 3.0 * q - out[0] - out[2];
}

// Largest eigenvalue of a symmetric 3x3 matrix in FP64 (the trigonometric
// form above, lambda = q + 2 p cos(acos(r) / 3)), with c = cos(acos(r) / 3)
// found as the largest root of 4 c^3 - 3 c = r (cos 3t = 4 cos^3 t - 3 cos t)
// in [1/2, 1]: an FP32 start from acosf / cosf, then Newton steps on the
// cubic in FP64 whose derivative 12 c^2 - 3 is inverted in FP32 (each step
// multiplies the error by about the FP32 relative error of that reciprocal,
// plus the quadratic term), which is far cheaper than FP64 acos and cos.  Near
// the double root c = 1/2 (r -> -1: the two largest eigenvalues meet) the
// derivative vanishes, and the FP64 trigonometric evaluation is used instead.
__device__ __forceinline__ double largest_eigenvalue(double a00, double a01, double a02, double a11, double a12, double a22)
{
  const double p1 = a01 * a01 + a02 * a02 + a12 * a12;
  if (p1 == 0.0) return fmax(a00, fmax(a11, a22));
  const double q  = (a00 + a11 + a22) * (1.0 / 3.0);
  const double d0 = a00 - q, d1 = a11 - q, d2 = a22 - q;
  const double s  = (d0 * d0 + d1 * d1 + d2 * d2 + 2.0 * p1) * (1.0 / 6.0);
  const double inv = rsqrt(s);   // 1 / p
  const double p  = s * inv;
  const double b00 = d0 * inv, b11 = d1 * inv, b22 = d2 * inv, b01 = a01 * inv, b02 = a02 * inv, b12 = a12 * inv;
  const double det = b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02);
  double r = 0.5 * det;
  r = r < -1.0 ? -1.0 : (r > 1.0 ? 1.0 : r);
  const float cf = cosf(acosf(float(r)) * (1.0f / 3.0f));
  double c;
  if (cf > 0.52f)
  {
    c = cf;
    #pragma unroll
    for (int k = 0; k < 3; ++k)
    {
      const double f = fma(4.0 * c, c * c, fma(-3.0, c, -r));   // 4 c^3 - 3 c - r
      const float slope = fmaf(12.0f * float(c), float(c), -3.0f);
      c = fma(-f, double(__frcp_rn(slope)), c);
    }
  }
  else
    c = cos(acos(r) * (1.0 / 3.0));
  return fma(2.0 * p, c, q);
}

struct ftle_args
{
  const float4* flow;
  int           nx, ny, nz;
  float         hx, hy, hz;
  double        inverse_time;     // 1 / |T|
  int           mode;
  float*        out;
};

template <int MODE>
__global__ void __launch_bounds__(256) ftle_kernel(const ftle_args a)
{
  const long long total = (long long)a.nx * a.ny * a.nz;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int z = int(i % a.nz);
  const int y = int((i / a.nz) % a.ny);
  const int x = int(i / ((long long)a.nz * a.ny));
  const long long sy = a.nz, sx = (long long)a.ny * a.nz;

  // Column j of J: (phi(+e_j) - phi(-e_j)) / (2 h_j), one-sided at borders.
  float J[3][3];
  const int   idx[3] = {x, y, z};
  const int   ext[3] = {a.nx, a.ny, a.nz};
  const float h[3]   = {a.hx, a.hy, a.hz};
  const long long stride[3] = {sx, sy, 1};
  #pragma unroll
  for (int j = 0; j < 3; ++j)
  {
    if (ext[j] == 1) { J[0][j] = J[1][j] = J[2][j] = 0.0f; continue; }
    long long lo = i, hi = i;
    float denominator;
    if (idx[j] == 0)                 { hi = i + stride[j]; denominator = h[j]; }
    else if (idx[j] == ext[j] - 1)   { lo = i - stride[j]; denominator = h[j]; }
    else                             { lo = i - stride[j]; hi = i + stride[j]; denominator = 2.0f * h[j]; }
    const float4 A = __ldg(a.flow + lo), B = __ldg(a.flow + hi);
    J[0][j] = __fdiv_rn(__fsub_rn(B.x, A.x), denominator);
    J[1][j] = __fdiv_rn(__fsub_rn(B.y, A.y), denominator);
    J[2][j] = __fdiv_rn(__fsub_rn(B.z, A.z), denominator);
  }
  // Cauchy-Green tensor in FP64.
  double C[3][3];
  #pragma unroll
  for (int r = 0; r < 3; ++r)
    #pragma unroll
    for (int c = r; c < 3; ++c)
      C[r][c] = double(J[0][r]) * double(J[0][c]) + double(J[1][r]) * double(J[1][c]) + double(J[2][r]) * double(J[2][c]);
  double value;
  if constexpr (MODE == PARS_FTLE_REGULAR)
  {
    // log(sqrt(lambda_max)) / |T|
    const double lambda = largest_eigenvalue(C[0][0], C[0][1], C[0][2], C[1][1], C[1][2], C[2][2]);
    value = 0.5 * log(lambda) * a.inverse_time;
  }
  else
  {
    double lambda[3];
    symmetric_eigenvalues(C[0][0], C[0][1], C[0][2], C[1][1], C[1][2], C[2][2], lambda);
    const double d01 = lambda[0] - lambda[1], d12 = lambda[1] - lambda[2], d20 = lambda[2] - lambda[0];
    value = sqrt(0.5) * sqrt(d01 * d01 + d12 * d12 + d20 * d20) /
            sqrt(lambda[0] * lambda[0] + lambda[1] * lambda[1] + lambda[2] * lambda[2]);
  }
  a.out[i] = float(value);
}

void launch_ftle_kernel(const ftle_args& a, unsigned grid, cudaStream_t stream)
{
  if (a.mode == PARS_FTLE_REGULAR) ftle_kernel<PARS_FTLE_REGULAR><<<grid, 256, 0, stream>>>(a);
  else                             ftle_kernel<PARS_FTLE_FRACTIONAL_ANISOTROPY><<<grid, 256, 0, stream>>>(a);
}
}

void launch_flow_map(pars_gpu_context& ctx, const field_view& f, const step_rule& rule, int iterations,
                     const float offset[3], const float fm_spacing[3], const int seeds_per_dimension[3],
                     const int fm_shape[3], float4* flow, unsigned long long* steps)
{
  flow_map_args a;
  a.f = f; a.rule = rule; a.iterations = iterations;
  a.ox = offset[0]; a.oy = offset[1]; a.oz = offset[2];
  a.sx = fm_spacing[0]; a.sy = fm_spacing[1]; a.sz = fm_spacing[2];
  a.px = seeds_per_dimension[0]; a.py = seeds_per_dimension[1]; a.pz = seeds_per_dimension[2];
  a.fx = fm_shape[0]; a.fy = fm_shape[1]; a.fz = fm_shape[2];
  a.flow = flow; a.steps = steps;
  const long long total = (long long)a.px * a.py * a.pz;
  if (total <= 0) return;
  launch_scope scope(ctx, "advect_flow_map");
  if (rule.frozen) flow_map_kernel<true><<<(unsigned)((total + 127) / 128), 128, 0, ctx.stream>>>(a);
  else             flow_map_kernel<false><<<(unsigned)((total + 127) / 128), 128, 0, ctx.stream>>>(a);
}

void launch_ftle(pars_gpu_context& ctx, const field_view& flow, double time, int mode, float* out)
{
  ftle_args a;
  a.flow = flow.data; a.nx = flow.nx; a.ny = flow.ny; a.nz = flow.nz;
  a.hx = flow.hx; a.hy = flow.hy; a.hz = flow.hz;
  a.inverse_time = 1.0 / fabs(time);
  a.mode = mode;
  a.out = out;
  const long long total = (long long)a.nx * a.ny * a.nz;
  if (total <= 0) return;
  launch_scope scope(ctx, "ftle_fused");
  launch_ftle_kernel(a, (unsigned)((total + 255) / 256), ctx.stream);
}

// ---- Allocation-free FTLE ------------------------------------------------------
// pars_gpu_ftle_no_alloc (declared in pars_gpu.h) runs the same pack, flow-map
// and FTLE kernels as the context path, but keeps its scratch — the float4
// copy of the field, the flow map, and the step counter — in the one
// file-scope device array below instead of allocating it.  Every GPU that
// loads this library holds the array (no_alloc_max_voxels * 32 bytes + 256,
// 8 MiB) until the process exits.
namespace
{
constexpr long long no_alloc_max_voxels = 1LL << 18;   // 64^3
constexpr long long no_alloc_entries = 2 * no_alloc_max_voxels + 16;   // field | flow map | counter
static __device__ __align__(256) float4 no_alloc_scratch[no_alloc_entries];

__global__ void pack_into_scratch_kernel(const float* __restrict__ xyz, float4* __restrict__ out, long long count)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f);
}

__global__ void steps_to_int64_kernel(const unsigned long long* __restrict__ counter, int64_t* __restrict__ out)
{
  *out = (int64_t)*counter;
}

// Host code must not use the array's name as a device address: it is a host
// stand-in.  The device address is looked up once per device, with that device
// current, and cached; later calls on the device reuse it.
constexpr int no_alloc_max_devices = 64;
std::mutex no_alloc_mutex;
float4* no_alloc_address[no_alloc_max_devices] = {};

int32_t no_alloc_scratch_address(int device, float4** out)
{
  if (device < 0 || device >= no_alloc_max_devices) return PARS_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(no_alloc_mutex);
  if (!no_alloc_address[device])
  {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, no_alloc_scratch) != cudaSuccess) { (void)cudaGetLastError(); return PARS_ERR_CUDA; }
    no_alloc_address[device] = static_cast<float4*>(p);
  }
  *out = no_alloc_address[device];
  return PARS_OK;
}
}
}

#pragma GCC visibility push(default)
extern "C" int32_t pars_gpu_ftle_no_alloc(const float* device_xyz, const int32_t shape[3], const float offset[3], const float size[3],
                                          const float spacing[3], int32_t iterations, int32_t integrator, int32_t stage_mode,
                                          float step_size, float time, int32_t mode, float* device_ftle, int64_t* device_steps,
                                          void* stream)
{
  using namespace pars;
  if (!device_xyz || !shape || !offset || !size || !spacing || !device_ftle) return PARS_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < 3; ++i)
    if (shape[i] < 2 || !(spacing[i] > 0.0f)) return PARS_ERR_INVALID_ARGUMENT;
  if (mode != PARS_FTLE_REGULAR && mode != PARS_FTLE_FRACTIONAL_ANISOTROPY) return PARS_ERR_INVALID_ARGUMENT;
  if (time == 0.0f) return PARS_ERR_INVALID_ARGUMENT;
  const long long voxels = (long long)shape[0] * shape[1] * shape[2];
  if (voxels > no_alloc_max_voxels) return PARS_ERR_BUDGET;   // larger than the static scratch
  step_rule rule;
  try { rule = make_step_rule(integrator, stage_mode, step_size); }
  catch (const error& e) { return e.status; }
  // Flow map at the field's own resolution (resolution scale 1): one seed per
  // vertex (seed_generator.cpp:11), so every flow-map voxel is written and the
  // flow-map part of the scratch needs no clearing.
  int seeds[3];
  for (int i = 0; i < 3; ++i)
  {
    const float q = size[i] / spacing[i];
    seeds[i] = (q > 0.0f && q < 2147483647.0f) ? int(q) : 0;
    if (seeds[i] < shape[i]) return PARS_ERR_INVALID_ARGUMENT;
  }

  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) { (void)cudaGetLastError(); return PARS_ERR_CUDA; }
  float4* scratch = nullptr;
  const int32_t status = no_alloc_scratch_address(device, &scratch);
  if (status != PARS_OK) return status;
  float4* field_data = scratch;
  float4* flow = scratch + no_alloc_max_voxels;
  auto* counter = reinterpret_cast<unsigned long long*>(scratch + 2 * no_alloc_max_voxels);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  field_view f;
  f.data = field_data;
  f.nx = shape[0]; f.ny = shape[1]; f.nz = shape[2];
  f.ox = offset[0]; f.oy = offset[1]; f.oz = offset[2];
  f.hx = spacing[0]; f.hy = spacing[1]; f.hz = spacing[2];
  f.maxx = offset[0] + size[0]; f.maxy = offset[1] + size[1]; f.maxz = offset[2] + size[2];
  f.inv_hx = 1.0f / spacing[0]; f.inv_hy = 1.0f / spacing[1]; f.inv_hz = 1.0f / spacing[2];

  // The counter keeps the previous call's value: clear it first.
  if (cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s) != cudaSuccess) { (void)cudaGetLastError(); return PARS_ERR_CUDA; }
  pack_into_scratch_kernel<<<(unsigned)((voxels + 255) / 256), 256, 0, s>>>(device_xyz, field_data, voxels);

  flow_map_args a;
  a.f = f; a.rule = rule; a.iterations = iterations;
  a.ox = offset[0]; a.oy = offset[1]; a.oz = offset[2];
  a.sx = spacing[0]; a.sy = spacing[1]; a.sz = spacing[2];
  a.px = seeds[0]; a.py = seeds[1]; a.pz = seeds[2];
  a.fx = shape[0]; a.fy = shape[1]; a.fz = shape[2];
  a.flow = flow; a.steps = counter;
  const long long total = (long long)a.px * a.py * a.pz;
  if (rule.frozen) flow_map_kernel<true><<<(unsigned)((total + 127) / 128), 128, 0, s>>>(a);
  else             flow_map_kernel<false><<<(unsigned)((total + 127) / 128), 128, 0, s>>>(a);

  ftle_args t;
  t.flow = flow; t.nx = shape[0]; t.ny = shape[1]; t.nz = shape[2];
  t.hx = spacing[0]; t.hy = spacing[1]; t.hz = spacing[2];
  t.inverse_time = 1.0 / fabs(double(time));
  t.mode = mode;
  t.out = device_ftle;
  launch_ftle_kernel(t, (unsigned)((voxels + 255) / 256), s);
  if (device_steps) steps_to_int64_kernel<<<1, 1, 0, s>>>(counter, device_steps);
  if (cudaGetLastError() != cudaSuccess) return PARS_ERR_CUDA;
  return PARS_OK;
}
#pragma GCC visibility pop
