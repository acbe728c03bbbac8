// Flow-map advection and the fused FTLE kernel.
//
// flow map: one thread per seed of flow_map_generator's lattice
//   (flow_map_generator.cpp:23-43 + seed_generator.cpp:9-21, seeds generated in
//   the kernel from the voxel index), advected with particle_advector's rules
//   (particle_advector.cpp:74-139, one block: a particle stops with its current
//   position when it leaves the grid, meets a zero velocity, or has taken
//   iterations - 1 steps) and written to its voxel (flow_map_generator.cpp:44-52).
//   Frozen stages keep absolute positions and the reference's arithmetic;
//   re-sampled stages of the tableau and Adams schemes run in local cell
//   coordinates.
// FTLE: per voxel, the flow map's central-difference gradient J (FP32, one-sided
//   at the borders), the Cauchy-Green tensor C = J^T J (FP32) and its
//   eigenvalues by four sweeps of the cyclic Jacobi method (FP32 rotations;
//   Jacobi is backward stable, so every eigenvalue carries an error of a few
//   FP32 ulps of ||C||, also where two of them nearly coincide and closed
//   forms lose half their digits), then log(sqrt(lambda_max)) / |T| =
//   0.5 log(lambda_max) / |T| — the intent of vector_field::gradient +
//   ftle_map_generator::generate (vector_field.cpp:49-93,
//   ftle_map_generator.cpp:22-60).  All FP32: a GB300 SM issues FP64 at 1/64
//   of its FP32 rate, and FP64 evaluation made this kernel FP64-pipe bound.
//   The fractional-anisotropy mode (ftle_map_generator.cpp:51-54) needs no
//   eigen-solve: it is evaluated from the invariants of C.
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
    corner_cache cache;
    frozen_history hist;
    if constexpr (FROZEN)
    {
      for (int it = 1; it < a.iterations; ++it)
      {
        float3 v;
        if (!sample_inside_cached(a.f, cache, pos, v) || is_zero(v)) break;
        pos = frozen_step(a.rule, pos, v, hist);
        ++steps;
      }
    }
    else
    {
      // Re-sampled schemes in local cell coordinates (cell + offset +
      // compensation); the position leaves them once, at the end.
      local_position q = to_local(a.f, pos);
      for (int it = 1; it < a.iterations; ++it)
      {
        if (!local_inside(a.f, q)) break;
        const float3 v = sample_local(a.f, cache, q.ix, q.iy, q.iz, q.ux, q.uy, q.uz);
        if (is_zero_local(a.f, v)) break;
        general_step_local(a.f, cache, a.rule, q, v, hist);
        ++steps;
      }
      if (steps) pos = flow_position(a.f, q);
    }
    // With iterations <= 1 the reference never assigns the voxel; it keeps the
    // seed position here.
    if (ix < a.fx && iy < a.fy && iz < a.fz)
      a.flow[((long long)ix * a.fy + iy) * a.fz + iz] = pos;
  }
  const unsigned int warp_steps = __reduce_add_sync(0xffffffffu, steps);
  if ((threadIdx.x & 31) == 0 && warp_steps) atomicAdd(a.steps, (unsigned long long)warp_steps);
}

// Eigenvalues of the symmetric 3x3 matrix a (in place on its diagonal) by
// cyclic Jacobi rotations (Jacobi 1846; the rotation of Rutishauser's
// formulation, Numer. Math. 9, 1966): each rotation zeroes a_pq with
// t = sgn(theta) / (|theta| + sqrt(theta^2 + 1)), theta = (a_qq - a_pp) / (2 a_pq).
// Four sweeps of the three pivots: the off-diagonal mass shrinks
// quadratically, and the FP32 eigenvalues settle after three.
__device__ __forceinline__ void jacobi_eigenvalues(float& a00, float& a11, float& a22, float a01, float a02, float a12)
{
  #pragma unroll
  for (int sweep = 0; sweep < 4; ++sweep)
  {
    #pragma unroll
    for (int pivot = 0; pivot < 3; ++pivot)
    {
      // (p, q, r) = (0, 1, 2), (0, 2, 1), (1, 2, 0)
      float& app = pivot == 2 ? a11 : a00;
      float& aqq = pivot == 0 ? a11 : a22;
      float& apq = pivot == 0 ? a01 : (pivot == 1 ? a02 : a12);
      float& arp = pivot == 0 ? a02 : (pivot == 1 ? a01 : a01);
      float& arq = pivot == 0 ? a12 : (pivot == 1 ? a12 : a02);
      if (apq == 0.0f) continue;
      const float theta = __fdiv_rn(aqq - app, 2.0f * apq);
      float t;
      if (fabsf(theta) > 1e18f) t = __fdiv_rn(0.5f, theta);
      else t = copysignf(__frcp_rn(fabsf(theta) + __fsqrt_rn(fmaf(theta, theta, 1.0f))), theta);
      const float c = __frsqrt_rn(fmaf(t, t, 1.0f)), s = t * c;
      app = fmaf(-t, apq, app);
      aqq = fmaf(t, apq, aqq);
      apq = 0.0f;
      const float rp = arp, rq = arq;
      // pivot (1, 2): a01 is row 0's p-entry and a02 its q-entry
      arp = fmaf(c, rp, -s * rq);
      arq = fmaf(s, rp, c * rq);
    }
  }
}

struct ftle_args
{
  const float4* flow;
  int           nx, ny, nz;
  float         hx, hy, hz;
  float         inverse_time;     // 1 / |T|
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
    // positions with their sub-ulp residuals (w = 0: none); the FP32
    // difference of neighbouring coordinates is exact where they lie within a
    // factor of two of each other (Sterbenz), the residuals' difference is
    // added to it
    const float4 A = __ldg(a.flow + lo), B = __ldg(a.flow + hi);
    const unsigned wa = __float_as_uint(A.w), wb = __float_as_uint(B.w);
    J[0][j] = __fdiv_rn(__fsub_rn(B.x, A.x) + (residual_value(B.x, wb, 0) - residual_value(A.x, wa, 0)), denominator);
    J[1][j] = __fdiv_rn(__fsub_rn(B.y, A.y) + (residual_value(B.y, wb, 10) - residual_value(A.y, wa, 10)), denominator);
    J[2][j] = __fdiv_rn(__fsub_rn(B.z, A.z) + (residual_value(B.z, wb, 20) - residual_value(A.z, wa, 20)), denominator);
  }
  // Cauchy-Green tensor C = J^T J (FP32) and its eigenvalues.
  float C[3][3];
  #pragma unroll
  for (int r = 0; r < 3; ++r)
    #pragma unroll
    for (int c = r; c < 3; ++c)
      C[r][c] = fmaf(J[2][r], J[2][c], fmaf(J[1][r], J[1][c], J[0][r] * J[0][c]));
  float value;
  if constexpr (MODE == PARS_FTLE_REGULAR)
  {
    // log(sqrt(lambda_max)) / |T|
    float l0 = C[0][0], l1 = C[1][1], l2 = C[2][2];
    jacobi_eigenvalues(l0, l1, l2, C[0][1], C[0][2], C[1][2]);
    const float lambda = fmaxf(l0, fmaxf(l1, l2));
    value = 0.5f * logf(lambda) * a.inverse_time;
  }
  else
  {
    // Fractional anisotropy of the eigenvalues (ftle_map_generator.cpp:51-54),
    // sqrt(1/2) sqrt(sum_{i<j} (l_i - l_j)^2) / sqrt(sum_i l_i^2), from the
    // invariants: sum_{i<j} (l_i - l_j)^2 = 3 |C - (tr C / 3) I|_F^2 and
    // sum_i l_i^2 = |C|_F^2, so FA = sqrt(3/2) |dev C|_F / |C|_F — no
    // eigen-solve, and the deviator's diagonal is formed before squaring, so
    // nearly isotropic tensors keep their small anisotropy.
    const float m = (C[0][0] + C[1][1] + C[2][2]) * (1.0f / 3.0f);
    const float d0 = C[0][0] - m, d1 = C[1][1] - m, d2 = C[2][2] - m;
    const float off = fmaf(C[0][1], C[0][1], fmaf(C[0][2], C[0][2], C[1][2] * C[1][2]));
    const float dev = fmaf(2.0f, off, fmaf(d0, d0, fmaf(d1, d1, d2 * d2)));
    const float all = fmaf(2.0f, off, fmaf(C[0][0], C[0][0], fmaf(C[1][1], C[1][1], C[2][2] * C[2][2])));
    value = 1.22474487f * __fsqrt_rn(__fdiv_rn(dev, all));
  }
  a.out[i] = value;
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
  a.inverse_time = float(1.0 / fabs(time));
  a.mode = mode;
  a.out = out;
  const long long total = (long long)a.nx * a.ny * a.nz;
  if (total <= 0) return;
  launch_scope scope(ctx, "ftle_fused");
  launch_ftle_kernel(a, (unsigned)((total + 255) / 256), ctx.stream);
}

// ---- Allocation-free FTLE ------------------------------------------------------
// pars_gpu_ftle_no_alloc (declared in pars_gpu.h) runs the pack kernel, the
// per-seed flow-map kernel (flow_map_kernel, frozen or re-sampled stages) and
// the FTLE kernel, and keeps its scratch — the float4 copy of the field, the
// flow map, and the step counter — in the one file-scope device array below
// instead of allocating it.  The context path runs re-sampled RK4 / Euler
// flow maps through the batched engine instead, so for those the two paths
// agree to rounding (the engine's per-step arithmetic differs), not bit for
// bit; frozen stages and the other schemes use the same kernel in both.
// Every GPU that loads this library holds the array (no_alloc_max_voxels * 32
// bytes + 256, 8 MiB) until the process exits.
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

// Checks the geometry of an allocation-free call before anything is
// multiplied or launched: every shape entry within the static scratch on its
// own (so the voxel product cannot overflow), the product within it, and the
// seed lattice int(size / spacing) per axis between shape and shape + 1 (the
// lattice flow_map_generator builds over a block: one seed per vertex), so
// the seed count and the launch's grid stay small.  Host-only; no CUDA call.
static int32_t no_alloc_geometry(const int32_t shape[3], const float size[3], const float spacing[3], long long* voxels,
                          int seeds[3])
{
  for (int i = 0; i < 3; ++i)
  {
    if (shape[i] < 2 || !(spacing[i] > 0.0f)) return PARS_ERR_INVALID_ARGUMENT;
    if (shape[i] > no_alloc_max_voxels) return PARS_ERR_BUDGET;
  }
  const long long v = (long long)shape[0] * shape[1] * shape[2];   // each factor <= 2^18: no overflow
  if (v > no_alloc_max_voxels) return PARS_ERR_BUDGET;
  for (int i = 0; i < 3; ++i)
  {
    const float q = size[i] / spacing[i];
    seeds[i] = (q > 0.0f && q < 2147483647.0f) ? int(q) : 0;
    if (seeds[i] < shape[i] || seeds[i] > shape[i] + 1) return PARS_ERR_INVALID_ARGUMENT;
  }
  *voxels = v;
  return PARS_OK;
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
  if (mode != PARS_FTLE_REGULAR && mode != PARS_FTLE_FRACTIONAL_ANISOTROPY) return PARS_ERR_INVALID_ARGUMENT;
  if (time == 0.0f) return PARS_ERR_INVALID_ARGUMENT;
  // Flow map at the field's own resolution (resolution scale 1): one seed per
  // vertex (seed_generator.cpp:11), so every flow-map voxel is written and the
  // flow-map part of the scratch needs no clearing.
  long long voxels = 0;
  int seeds[3];
  const int32_t geometry = no_alloc_geometry(shape, size, spacing, &voxels, seeds);
  if (geometry != PARS_OK) return geometry;   // PARS_ERR_BUDGET: larger than the static scratch
  step_rule rule;
  try { rule = make_step_rule(integrator, stage_mode, step_size); }
  catch (const error& e) { return e.status; }

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
  if (cudaGetLastError() != cudaSuccess) return PARS_ERR_CUDA;

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
  if (cudaGetLastError() != cudaSuccess) return PARS_ERR_CUDA;

  ftle_args t;
  t.flow = flow; t.nx = shape[0]; t.ny = shape[1]; t.nz = shape[2];
  t.hx = spacing[0]; t.hy = spacing[1]; t.hz = spacing[2];
  t.inverse_time = float(1.0 / fabs(double(time)));
  t.mode = mode;
  t.out = device_ftle;
  launch_ftle_kernel(t, (unsigned)((voxels + 255) / 256), s);
  if (cudaGetLastError() != cudaSuccess) return PARS_ERR_CUDA;
  if (device_steps) steps_to_int64_kernel<<<1, 1, 0, s>>>(counter, device_steps);
  if (cudaGetLastError() != cudaSuccess) return PARS_ERR_CUDA;
  return PARS_OK;
}
#pragma GCC visibility pop
