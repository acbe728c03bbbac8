// CPU restatement of the pars particle-tracing hot path: the ORACLE.
//
// Test infrastructure only.  Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg load this library, and only to check or time against it; the
// product path (pars_gb300, libpars_gpu) never calls it.
//
// Two families of functions:
//  * FP32 restatements that follow the reference's arithmetic operation by
//    operation (no FMA contraction: build with -ffp-contract=off), so that on the
//    same inputs they give bit-identical results to the reference sources
//    compiled against oracle/ref_shim (pinned by tests/test_oracle_golden.py):
//      vector_field::contains / interpolate   pa/source/math/vector_field.cpp:12-48
//      seed_generator::generate               pa/source/stages/seed_generator.cpp:9-21
//      partitioner::set_domain_size           pa/source/stages/partitioner.cpp:8-53
//      particle_tracer round loop + prune     pa/source/stages/particle_tracer.cpp:210-337, 376-409
//      particle_advector::advect              pa/source/stages/particle_advector.cpp:61-141
//      flow_map_generator::generate           pa/source/stages/flow_map_generator.cpp:12-52
//      index_generator::generate              pa/source/stages/index_generator.cpp:10-24
//      color_generator::generate              pa/source/stages/color_generator.cpp:16-98
//  * FP64 oracles of the intended mathematics:
//      true (re-sampled) classical RK4 advection on the same FP32 grid values,
//      FTLE = log(sqrt(lambda_max(J^T J))) / |T| with central differences
//      (one-sided at the borders), the intent of vector_field.cpp:49-93 and
//      ftle_map_generator.cpp:22-60.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace
{
// ---------------------------------------------------------------------------
// Types
// ---------------------------------------------------------------------------
struct vec4 { float v[4]; };

// Layout of pa::particle (pa/include/pa/math/particle.hpp:30-35): Eigen
// Vector4f position (16-byte aligned), three int32, Eigen Vector3i; 48 bytes.
struct alignas(16) particle
{
  float   position[4];
  int32_t remaining_iterations;
  int32_t vector_field_index;
  int32_t original_rank;
  int32_t original_voxel[3];
  int32_t padding[2];
};
static_assert(sizeof(particle) == 48, "particle is 48 bytes");

const vec4 termination_vertex {{-2.0f, -2.0f, -2.0f, 0.0f}};   // integral_curves.hpp:18
const vec4 invalid_vertex     {{-1.0f, -1.0f, -1.0f, 0.0f}};   // integral_curves.hpp:19

inline bool equal(const vec4& a, const vec4& b)
{
  return a.v[0] == b.v[0] && a.v[1] == b.v[1] && a.v[2] == b.v[2] && a.v[3] == b.v[3];
}

struct field
{
  const float* xyz;          // [X][Y][Z][3], C order, z fastest
  int          shape[3];
  float        offset[3];
  float        size[3];
  float        spacing[3];
  const float* at(long long x, long long y, long long z) const
  {
    return xyz + 3 * ((x * shape[1] + y) * (long long)shape[2] + z);
  }
};

// ---------------------------------------------------------------------------
// vector_field::contains / interpolate in FP32 (vector_field.cpp:12-48)
// ---------------------------------------------------------------------------
// contains: per axis s = floor((p - o) / h); inside iff 0 <= s <= shape - 2.
// The reference casts s to size_t (vector_field.cpp:16-17); on x86-64 a negative
// integral s becomes a huge unsigned value, so it counts as outside, and so do
// NaN and out-of-range values.  -0.0 converts to 0 and counts as inside.
inline bool contains(const field& f, const float* p)
{
  for (int i = 0; i < 3; ++i)
  {
    const float s = std::floor((p[i] - f.offset[i]) / f.spacing[i]);
    if (!(s >= 0.0f && s <= float(f.shape[i] - 2))) return false;
  }
  return true;
}

// linear_interpolate (linear_interpolate.hpp:6-10): (1 - w) * a + w * b.
inline float lerp(float a, float b, float w)
{
  const float one_minus = 1.0f - w;
  const float left  = one_minus * a;
  const float right = w * b;
  return left + right;
}

// index = floor((p - o) / h), weight = fmod(p - o, h) / h, corners blended
// along z, then y, then x.
inline void interpolate(const field& f, const float* p, float* out)
{
  int   index[3];
  float weight[3];
  for (int i = 0; i < 3; ++i)
  {
    const float d = p[i] - f.offset[i];
    index [i] = int(std::floor(d / f.spacing[i]));
    weight[i] = std::fmod(d, f.spacing[i]) / f.spacing[i];
  }
  const int x = index[0], y = index[1], z = index[2];
  const float* c000 = f.at(x    , y    , z    );
  const float* c001 = f.at(x    , y    , z + 1);
  const float* c010 = f.at(x    , y + 1, z    );
  const float* c011 = f.at(x    , y + 1, z + 1);
  const float* c100 = f.at(x + 1, y    , z    );
  const float* c101 = f.at(x + 1, y    , z + 1);
  const float* c110 = f.at(x + 1, y + 1, z    );
  const float* c111 = f.at(x + 1, y + 1, z + 1);
  for (int c = 0; c < 3; ++c)
  {
    const float c00 = lerp(c000[c], c001[c], weight[2]);
    const float c01 = lerp(c010[c], c011[c], weight[2]);
    const float c10 = lerp(c100[c], c101[c], weight[2]);
    const float c11 = lerp(c110[c], c111[c], weight[2]);
    const float c0  = lerp(c00, c01, weight[1]);
    const float c1  = lerp(c10, c11, weight[1]);
    out[c] = lerp(c0, c1, weight[0]);
  }
}

// Eigen's isZero() with the default precision: every |v_i| <= 1e-5f.
inline bool is_zero(const float* v)
{
  const float precision = 1e-5f;
  return std::fabs(v[0]) <= precision && std::fabs(v[1]) <= precision && std::fabs(v[2]) <= precision;
}

// ---------------------------------------------------------------------------
// Integrator step with the reference's frozen velocity (particle_tracer.cpp:
// 315-334, particle_advector.cpp:115-130): the right-hand side returns the
// velocity sampled at the step start for every stage.  For the eight steppers
// of integrators.hpp:16-23, with the odeint 1.69 schemes written out from
// their published tableaux (FP32, left to right, b_i = float(p)/float(q)):
//  * explicit RK (euler, runge_kutta4, cash_karp54, dopri5, fehlberg78) and
//    adams_bashforth_moulton<2> (AB2 predictor, trapezoidal corrector):
//      out = 1 * x + (b_1 h) v + ... + (b_s h) v, zero weights included;
//  * modified_midpoint (two substeps, H = h/2):
//      z1 = x + H v,  z2 = x + (2H) v,  out = 0.5 z2 + 0.5 z1 + (0.5 H) v;
//  * adams_bashforth<2>: the first step of a particle is runge_kutta4, later
//    steps out = x + (1.5 h) v_n + (-0.5 h) v_{n-1}; the reference copies the
//    stepper per particle and per tracing call, so the history starts afresh.
// ---------------------------------------------------------------------------
enum integrator_kind { euler = 0, modified_midpoint = 1, runge_kutta_4 = 2, cash_karp_54 = 3, dormand_prince_5 = 4,
                       fehlberg_78 = 5, adams_bashforth_2 = 6, adams_bashforth_moulton_2 = 7 };
enum stage_mode { frozen = 0, resampled = 1 };
enum frozen_method { weighted_sum = 0, midpoint = 1, multistep = 2 };

struct frozen_weights
{
  int   method = weighted_sum;
  int   count = 0;
  float c[16] = {};
};

// Per-particle history of the multistep scheme.
struct frozen_history
{
  float v[3] = {0, 0, 0};
  bool  started = false;
};

frozen_weights make_frozen_weights(int integrator, float h)
{
  frozen_weights w;
  auto fill = [&](std::initializer_list<std::pair<int, int>> b) {
    w.count = 0;
    for (auto& q : b) w.c[w.count++] = (float(q.first) / float(q.second)) * h;
  };
  switch (integrator)
  {
  case euler: w.count = 1; w.c[0] = h; break;
  case modified_midpoint:
  {
    const float H = h / 2.0f;
    w.method = midpoint;
    w.c[0] = H; w.c[1] = 2.0f * H; w.c[2] = 0.5f * H;
    break;
  }
  case cash_karp_54: fill({{37, 378}, {0, 1}, {250, 621}, {125, 594}, {0, 1}, {512, 1771}}); break;
  case dormand_prince_5: fill({{35, 384}, {0, 1}, {500, 1113}, {125, 192}, {-2187, 6784}, {11, 84}}); break;
  case fehlberg_78:
    fill({{41, 840}, {0, 1}, {0, 1}, {0, 1}, {0, 1}, {34, 105}, {9, 35}, {9, 35}, {9, 280}, {9, 280}, {41, 840}, {0, 1}, {0, 1}});
    break;
  case adams_bashforth_moulton_2: w.count = 2; w.c[0] = h * (1.0f / 2.0f); w.c[1] = h * (1.0f / 2.0f); break;
  case adams_bashforth_2:
    fill({{1, 6}, {1, 3}, {1, 3}, {1, 6}});           // first step: runge_kutta4
    w.method = multistep;
    w.c[4] = h * (3.0f / 2.0f);
    w.c[5] = h * (-1.0f / 2.0f);
    break;
  default: fill({{1, 6}, {1, 3}, {1, 3}, {1, 6}}); break;   // runge_kutta_4
  }
  return w;
}

inline void frozen_step(const frozen_weights& w, const float* x, const float* v, float* out, frozen_history& hist)
{
  const float dxdt[4] = {v[0], v[1], v[2], 0.0f};
  if (w.method == midpoint)
  {
    for (int c = 0; c < 4; ++c)
    {
      const float z1 = 1.0f * x[c] + w.c[0] * dxdt[c];
      const float z2 = 1.0f * x[c] + w.c[1] * dxdt[c];
      out[c] = 0.5f * z2 + 0.5f * z1 + w.c[2] * dxdt[c];
    }
    return;
  }
  if (w.method == multistep && hist.started)
  {
    const float previous[4] = {hist.v[0], hist.v[1], hist.v[2], 0.0f};
    for (int c = 0; c < 4; ++c) out[c] = 1.0f * x[c] + w.c[4] * dxdt[c] + w.c[5] * previous[c];
  }
  else
    for (int c = 0; c < 4; ++c)
    {
      float acc = 1.0f * x[c];
      for (int i = 0; i < w.count; ++i) acc = acc + w.c[i] * dxdt[c];
      out[c] = acc;
    }
  if (w.method == multistep)
  {
    for (int c = 0; c < 3; ++c) hist.v[c] = v[c];
    hist.started = true;
  }
}

// ---------------------------------------------------------------------------
// Curves result (one entry per integral_curves batch)
// ---------------------------------------------------------------------------
struct batch
{
  std::vector<vec4>    vertices;
  std::vector<vec4>    colors;
  std::vector<int32_t> indices;
  int                  rank  = 0;
  int                  round = 0;
};
}

struct orc_curves
{
  std::vector<batch> batches;
  long long          steps = 0;
};

namespace
{
// ---------------------------------------------------------------------------
// index_generator::generate (index_generator.cpp:10-24)
// ---------------------------------------------------------------------------
void generate_indices(batch& b)
{
  b.indices.clear();
  const std::size_t n = b.vertices.size();
  for (std::size_t i = 0; i + 1 < n; ++i)
    if (!equal(b.vertices[i], termination_vertex) && !equal(b.vertices[i + 1], termination_vertex))
      b.indices.push_back(int32_t(i));
}

// ---------------------------------------------------------------------------
// color_generator (color_generator.cpp:16-98, coordinates.hpp:8-16)
// ---------------------------------------------------------------------------
// Eigen's Vector4f::normalized(): squared norm reduced as (d0^2 + d2^2) +
// (d1^2 + d3^2) (the SSE packet reduction), then d / sqrt(z) when z > 0.
inline vec4 normalized_difference(const vec4& a, const vec4& b)
{
  vec4 d;
  for (int c = 0; c < 4; ++c) d.v[c] = b.v[c] - a.v[c];
  const float s0 = d.v[0] * d.v[0], s1 = d.v[1] * d.v[1], s2 = d.v[2] * d.v[2], s3 = d.v[3] * d.v[3];
  const float z = (s0 + s2) + (s1 + s3);
  if (z > 0.0f)
  {
    const float r = std::sqrt(z);
    for (int c = 0; c < 4; ++c) d.v[c] = d.v[c] / r;
  }
  return d;
}

inline float clamp01(float x) { return x < 0.0f ? 0.0f : (1.0f < x ? 1.0f : x); }

inline void hue_to_rgba(float hue, float* out)
{
  out[0] = clamp01(std::fabs(6.0f * hue - 3.0f) - 1.0f);
  out[1] = clamp01(2.0f - std::fabs(6.0f * hue - 2.0f));
  out[2] = clamp01(2.0f - std::fabs(6.0f * hue - 4.0f));
  out[3] = 1.0f;
}

// How to_spherical's FP32 atan2 / acos are evaluated: the host libm's
// atan2f / acosf, as the reference calls them (default), or correctly rounded
// (FP64 evaluation rounded to FP32) -- the latter only to attribute colour
// differences to the libms in the tests.
bool correctly_rounded_trig = false;

// to_spherical + correct_range: returns (hue, second) in [0, 1].
inline void spherical_hue(const vec4& t, float& hue, float& second)
{
  const double x = t.v[0], y = t.v[1], zc = t.v[2];
  const float radius = float(std::sqrt(std::pow(x, 2) + std::pow(y, 2) + std::pow(zc, 2)));
  const float ratio = t.v[2] / radius;
  float s1 = correctly_rounded_trig ? float(std::atan2(double(t.v[1]), double(t.v[0]))) : std::atan2(t.v[1], t.v[0]);
  float s2 = correctly_rounded_trig ? float(std::acos(double(ratio))) : std::acos(ratio);
  const float pi = float(M_PI);
  if (s1 <  0.0f) s1 += pi;
  if (s1 >= pi)   s1 -= pi;
  s1 = pi - s1;
  if (s2 <  0.0f) s2 = std::fabs(s2);
  if (s2 >= float(M_PI / 2.0)) s2 = pi - s2;
  hue    = float(s1 / M_PI);
  second = float(s2 / (M_PI / 2.0f));
}

vec4 color_of(const vec4& tangent, int mode, float parameter)
{
  vec4 out;
  if (mode == 4)   // rgb (color_generator.cpp:95-98): (|x|, |z|, |y|, 1)
  {
    out.v[0] = std::fabs(tangent.v[0]);
    out.v[1] = std::fabs(tangent.v[2]);
    out.v[2] = std::fabs(tangent.v[1]);
    out.v[3] = 1.0f;
    return out;
  }
  float hue, second;
  spherical_hue(tangent, hue, second);
  const bool  constant_first = (mode == 0 || mode == 2);   // hsl_constant_s / hsv_constant_s
  const float sat   = constant_first ? parameter : second;
  const float third = constant_first ? second : parameter;
  hue_to_rgba(hue, out.v);
  if (mode == 0 || mode == 1)   // hsl_to_rgba (color_generator.cpp:65-72)
  {
    const float pre = (1.0f - std::fabs(2.0f * third - 1.0f)) * sat;
    for (int c = 0; c < 4; ++c) out.v[c] = (out.v[c] - 0.5f) * pre + third;
  }
  else                          // hsv_to_rgba (color_generator.cpp:73-79)
  {
    for (int c = 0; c < 4; ++c) out.v[c] = ((out.v[c] - 1.0f) * sat + 1.0f) * third;
  }
  out.v[3] = 1.0f;
  return out;
}

// Colours the reference never writes stay NaN (it resizes without initialising).
// Parallel over line segments like the reference's tbb::parallel_for: the
// indices ascend, so the extra write to index + 1 (a curve's last vertex)
// never meets another segment's write.
void generate_colors(batch& b, int mode, float parameter)
{
  const float nan = std::numeric_limits<float>::quiet_NaN();
  b.colors.assign(b.vertices.size(), vec4{{nan, nan, nan, nan}});
  const long long n = static_cast<long long>(b.indices.size());
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i)
  {
    const int32_t index = b.indices[i];
    const vec4 tangent = normalized_difference(b.vertices[index], b.vertices[index + 1]);
    b.colors[index] = color_of(tangent, mode, parameter);
    if (i != n - 1 && b.indices[i + 1] != index + 1) b.colors[index + 1] = b.colors[index];
  }
}

// ---------------------------------------------------------------------------
// One particle of particle_tracer::trace (particle_tracer.cpp:258-336), FP32,
// frozen-velocity step.  Appends the particle's slot contents (seed, steps, and
// the termination vertex) to `out`; returns the number of integrator steps.
// On a block exit, *exit_remaining receives remaining_iterations - i and
// exit_position the out-of-block vertex; otherwise *exit_remaining = -1.
// ---------------------------------------------------------------------------
long long trace_particle(const field& f, const frozen_weights& w, const particle& p, std::vector<vec4>& out,
                         int32_t* exit_remaining, vec4* exit_position)
{
  *exit_remaining = -1;
  vec4 last;
  std::memcpy(last.v, p.position, 16);
  out.push_back(last);
  long long steps = 0;
  frozen_history hist;
  for (long long i = 1; i < (long long)p.remaining_iterations; ++i)
  {
    if (i == (long long)p.remaining_iterations - 1) { out.push_back(termination_vertex); break; }
    if (!contains(f, last.v))
    {
      out.push_back(termination_vertex);
      *exit_remaining = int32_t(p.remaining_iterations - i);
      *exit_position = last;
      break;
    }
    float v[3];
    interpolate(f, last.v, v);
    if (is_zero(v)) { out.push_back(termination_vertex); break; }
    vec4 next;
    frozen_step(w, last.v, v, next.v, hist);
    out.push_back(next);
    last = next;
    ++steps;
  }
  return steps;
}

// compute_round_info (particle_tracer.cpp:210-234) for P particles.
struct round_info
{
  long long maximum_remaining;
  long long particles_per_curve;
  long long curve_count;
};
round_info make_round_info(const std::vector<particle>& particles)
{
  round_info r {0, 0, 0};
  for (auto& p : particles) r.maximum_remaining = std::max<long long>(r.maximum_remaining, p.remaining_iterations);
  const long long max_vertices = std::numeric_limits<int32_t>::max() / 16;
  r.particles_per_curve = max_vertices / r.maximum_remaining;
  r.curve_count = particles.empty() ? 0 : 1 + (long long)particles.size() / r.particles_per_curve;
  return r;
}

// Traces one rank's particle list for one round; appends that round's batches.
// Exits go to `exits` with the face they cross (-1 when no face test holds).
struct exit_record { particle p; int face; };

void trace_round(const field& f, const frozen_weights& w, const std::vector<particle>& particles, int rank, int round,
                 const int* neighbor, std::vector<batch>& batches, std::vector<exit_record>& exits, long long& steps)
{
  if (particles.empty()) return;
  const round_info info = make_round_info(particles);
  std::vector<std::vector<vec4>> per_particle(particles.size());
  std::vector<int32_t>           exit_remaining(particles.size());
  std::vector<vec4>              exit_position(particles.size());
  long long total = 0;
  #pragma omp parallel for schedule(dynamic, 16) reduction(+ : total)
  for (long long i = 0; i < (long long)particles.size(); ++i)
  {
    // Slots the reference leaves as invalid_vertex are removed by prune; so are
    // written vertices that happen to equal it (particle_tracer.cpp:402-409).
    std::vector<vec4> slots;
    total += trace_particle(f, w, particles[i], slots, &exit_remaining[i], &exit_position[i]);
    for (auto& v : slots) if (!equal(v, invalid_vertex)) per_particle[i].push_back(v);
  }
  steps += total;

  const long long first = (long long)batches.size();
  batches.resize(first + info.curve_count);
  for (long long b = first; b < (long long)batches.size(); ++b) { batches[b].rank = rank; batches[b].round = round; }
  for (long long i = 0; i < (long long)particles.size(); ++i)
  {
    const long long b = first + i / info.particles_per_curve;
    batches[b].vertices.insert(batches[b].vertices.end(), per_particle[i].begin(), per_particle[i].end());
  }

  const float minimum[3] = {f.offset[0], f.offset[1], f.offset[2]};
  const float maximum[3] = {f.offset[0] + f.size[0], f.offset[1] + f.size[1], f.offset[2] + f.size[2]};
  for (long long i = 0; i < (long long)particles.size(); ++i)
  {
    if (exit_remaining[i] < 0) continue;
    exit_record e;
    std::memset(&e.p, 0, sizeof(e.p));
    std::memcpy(e.p.position, exit_position[i].v, 16);
    e.p.remaining_iterations = exit_remaining[i];
    e.p.vector_field_index   = -1;
    const float* q = exit_position[i].v;
    // Face order -x, +x, -y, +y, -z, +z: the first face whose strict bound
    // test holds AND whose neighbour exists (particle_tracer.cpp:288-293 chain
    // both conditions in one else-if ladder).  No such face: dropped.
    e.face = -1;
    for (int face = 0; face < 6 && e.face < 0; ++face)
    {
      const int axis = face / 2;
      const bool beyond = (face % 2 == 0) ? (q[axis] < minimum[axis]) : (q[axis] > maximum[axis]);
      if (beyond && neighbor && neighbor[face] >= 0) e.face = face;
    }
    if (e.face >= 0) exits.push_back(e);
  }
}

// partitioner::set_domain_size (partitioner.cpp:24-53) restated.
struct partition
{
  int grid[3];
  int block[3];
};
std::vector<int> prime_factors(int value)   // prime_factorize.hpp:11-32
{
  std::vector<int> factors;
  int d = 2;
  while (d * d <= value)
  {
    if (value % d == 0) { factors.push_back(d); value /= d; }
    else ++d;
  }
  if (value > 1) factors.push_back(value);
  return factors;
}
partition make_partition(int ranks, const int domain[3])
{
  partition p;
  auto factors = prime_factors(ranks);
  int current[3] = {domain[0], domain[1], domain[2]};
  p.grid[0] = p.grid[1] = p.grid[2] = 1;
  while (!factors.empty())
  {
    int dimension = 0;
    for (int i = 0; i < 3; ++i) if (current[i] > current[dimension]) dimension = i;
    current[dimension] /= factors.back();
    p.grid[dimension]  *= factors.back();
    factors.pop_back();
  }
  for (int i = 0; i < 3; ++i) p.block[i] = domain[i] / p.grid[i];
  return p;
}
void unravel(long long index, const int dims[3], int out[3])   // index.hpp:9-19
{
  for (int i = 2; i >= 0; --i) { out[i] = int(index % dims[i]); index /= dims[i]; }
}
long long ravel(const int idx[3], const int dims[3])           // index.hpp:20-27
{
  return ((long long)idx[0] * dims[1] + idx[1]) * dims[2] + idx[2];
}

// ---------------------------------------------------------------------------
// FP64 field sampling on the FP32 grid values (true RK4 oracle)
// ---------------------------------------------------------------------------
// Trilinear interpolation with a consistent cell / weight pair: the cell is the
// floor quotient s and the weight (d - s h) / h lies in [0, 1).  Points outside
// the grid use the cell index clamped to [0, shape-2] and the weight clamped to
// 0 or 1 (constant extension of the boundary values).
inline void interpolate_fp64(const field& f, const double* p, double* out)
{
  long long index[3];
  double    weight[3];
  for (int i = 0; i < 3; ++i)
  {
    const double h = f.spacing[i];
    const double d = p[i] - double(f.offset[i]);
    double s = std::floor(d / h);
    double r = d - s * h;
    if (r < 0.0) { s -= 1.0; r = d - s * h; }
    else if (r >= h) { s += 1.0; r = d - s * h; }
    if (!(s >= 0.0)) { index[i] = 0; weight[i] = 0.0; }
    else if (s > double(f.shape[i] - 2)) { index[i] = f.shape[i] - 2; weight[i] = 1.0; }
    else { index[i] = (long long)s; weight[i] = r / h; }
  }
  const long long x = index[0], y = index[1], z = index[2];
  for (int c = 0; c < 3; ++c)
  {
    auto L = [](double a, double b, double w) { return (1.0 - w) * a + w * b; };
    const double c00 = L(f.at(x, y, z)[c],         f.at(x, y, z + 1)[c],         weight[2]);
    const double c01 = L(f.at(x, y + 1, z)[c],     f.at(x, y + 1, z + 1)[c],     weight[2]);
    const double c10 = L(f.at(x + 1, y, z)[c],     f.at(x + 1, y, z + 1)[c],     weight[2]);
    const double c11 = L(f.at(x + 1, y + 1, z)[c], f.at(x + 1, y + 1, z + 1)[c], weight[2]);
    out[c] = L(L(c00, c01, weight[1]), L(c10, c11, weight[1]), weight[0]);
  }
}
inline bool contains_fp64(const field& f, const double* p)
{
  for (int i = 0; i < 3; ++i)
  {
    const double s = std::floor((p[i] - double(f.offset[i])) / double(f.spacing[i]));
    if (!(s >= 0.0 && s <= double(f.shape[i] - 2))) return false;
  }
  return true;
}
inline bool is_zero_fp64(const double* v)
{
  const double precision = 1e-5;
  return std::fabs(v[0]) <= precision && std::fabs(v[1]) <= precision && std::fabs(v[2]) <= precision;
}
// Explicit tableaux of the other integrators in FP64 (exact fractions):
// modified midpoint (two substeps: z1 = x + h/2 f(x), z2 = x + h f(z1),
// (z2 + z1 + h/2 f(z2)) / 2, as a 3-stage scheme), Cash-Karp 5(4) and
// Dormand-Prince 5 (5th-order weights), Fehlberg 7(8) (8th-order weights).
struct tableau_fp64
{
  int    stages = 0;
  double a[13][13] = {};
  double b[13] = {};
};

tableau_fp64 tableau_for(int integrator)
{
  struct entry { int i, j; double p, q; };
  tableau_fp64 t;
  auto set = [&](int stages, std::initializer_list<entry> a, std::initializer_list<entry> b) {
    t.stages = stages;
    for (const auto& e : a) t.a[e.i][e.j] = e.p / e.q;
    for (const auto& e : b) t.b[e.i] = e.p / e.q;
  };
  switch (integrator)
  {
  case modified_midpoint: set(3, {{1, 0, 1, 2}, {2, 1, 1, 1}}, {{0, 0, 1, 4}, {1, 0, 1, 2}, {2, 0, 1, 4}}); break;
  case cash_karp_54:
    set(6, {{1, 0, 1, 5}, {2, 0, 3, 40}, {2, 1, 9, 40}, {3, 0, 3, 10}, {3, 1, -9, 10}, {3, 2, 6, 5}, {4, 0, -11, 54}, {4, 1, 5, 2},
            {4, 2, -70, 27}, {4, 3, 35, 27}, {5, 0, 1631, 55296}, {5, 1, 175, 512}, {5, 2, 575, 13824}, {5, 3, 44275, 110592},
            {5, 4, 253, 4096}},
        {{0, 0, 37, 378}, {2, 0, 250, 621}, {3, 0, 125, 594}, {5, 0, 512, 1771}});
    break;
  case dormand_prince_5:
    set(6, {{1, 0, 1, 5}, {2, 0, 3, 40}, {2, 1, 9, 40}, {3, 0, 44, 45}, {3, 1, -56, 15}, {3, 2, 32, 9}, {4, 0, 19372, 6561},
            {4, 1, -25360, 2187}, {4, 2, 64448, 6561}, {4, 3, -212, 729}, {5, 0, 9017, 3168}, {5, 1, -355, 33}, {5, 2, 46732, 5247},
            {5, 3, 49, 176}, {5, 4, -5103, 18656}},
        {{0, 0, 35, 384}, {2, 0, 500, 1113}, {3, 0, 125, 192}, {4, 0, -2187, 6784}, {5, 0, 11, 84}});
    break;
  case fehlberg_78:
    set(13, {{1, 0, 2, 27}, {2, 0, 1, 36}, {2, 1, 1, 12}, {3, 0, 1, 24}, {3, 2, 1, 8}, {4, 0, 5, 12}, {4, 2, -25, 16},
             {4, 3, 25, 16}, {5, 0, 1, 20}, {5, 3, 1, 4}, {5, 4, 1, 5}, {6, 0, -25, 108}, {6, 3, 125, 108}, {6, 4, -65, 27},
             {6, 5, 125, 54}, {7, 0, 31, 300}, {7, 4, 61, 225}, {7, 5, -2, 9}, {7, 6, 13, 900}, {8, 0, 2, 1}, {8, 3, -53, 6},
             {8, 4, 704, 45}, {8, 5, -107, 9}, {8, 6, 67, 90}, {8, 7, 3, 1}, {9, 0, -91, 108}, {9, 3, 23, 108},
             {9, 4, -976, 135}, {9, 5, 311, 54}, {9, 6, -19, 60}, {9, 7, 17, 6}, {9, 8, -1, 12}, {10, 0, 2383, 4100},
             {10, 3, -341, 164}, {10, 4, 4496, 1025}, {10, 5, -301, 82}, {10, 6, 2133, 4100}, {10, 7, 45, 82},
             {10, 8, 45, 164}, {10, 9, 18, 41}, {11, 0, 3, 205}, {11, 5, -6, 41}, {11, 6, -3, 205}, {11, 7, -3, 41},
             {11, 8, 3, 41}, {11, 9, 6, 41}, {12, 0, -1777, 4100}, {12, 3, -341, 164}, {12, 4, 4496, 1025},
             {12, 5, -289, 82}, {12, 6, 2193, 4100}, {12, 7, 51, 82}, {12, 8, 33, 164}, {12, 9, 12, 41}, {12, 11, 1, 1}},
        {{5, 0, 34, 105}, {6, 0, 9, 35}, {7, 0, 9, 35}, {8, 0, 9, 280}, {9, 0, 9, 280}, {11, 0, 41, 840}, {12, 0, 41, 840}});
    break;
  default: break;
  }
  return t;
}

// Per-particle history of the two-step Adams schemes in FP64.
struct history_fp64
{
  double v[3] = {0, 0, 0};
  bool   started = false;
};

void rk4_fp64(const field& f, double h, const double* x, const double* k1, double* out);

// One FP64 step.  `mode` frozen: every stage sees k1 (out = x + h k1; the
// two-step Adams-Bashforth scheme x + h (3/2 k1 - 1/2 k_prev) after its RK4
// start).  Re-sampled: each scheme with its stages sampled where they fall.
inline void step_fp64(const field& f, int integrator, int mode, double h, const double* x, const double* k1, double* out,
                      history_fp64& hist)
{
  if (integrator == adams_bashforth_2 || integrator == adams_bashforth_moulton_2)
  {
    double predicted[3];
    if (hist.started) for (int c = 0; c < 3; ++c) predicted[c] = x[c] + h * (1.5 * k1[c] - 0.5 * hist.v[c]);
    else if (mode == frozen) for (int c = 0; c < 3; ++c) predicted[c] = x[c] + h * k1[c];
    else rk4_fp64(f, h, x, k1, predicted);
    for (int c = 0; c < 3; ++c) hist.v[c] = k1[c];
    hist.started = true;
    if (integrator == adams_bashforth_2 || mode == frozen) { std::memcpy(out, predicted, 24); return; }
    double kp[3];
    interpolate_fp64(f, predicted, kp);
    for (int c = 0; c < 3; ++c) out[c] = x[c] + 0.5 * h * (k1[c] + kp[c]);
    return;
  }
  if (integrator == euler || mode == frozen) { for (int c = 0; c < 3; ++c) out[c] = x[c] + h * k1[c]; return; }
  if (integrator != runge_kutta_4)
  {
    const tableau_fp64 t = tableau_for(integrator);
    double k[13][3];
    std::memcpy(k[0], k1, 24);
    for (int s = 1; s < t.stages; ++s)
    {
      double p[3];
      for (int c = 0; c < 3; ++c)
      {
        double acc = 0.0;
        for (int j = 0; j < s; ++j) acc += t.a[s][j] * k[j][c];
        p[c] = x[c] + h * acc;
      }
      interpolate_fp64(f, p, k[s]);
    }
    for (int c = 0; c < 3; ++c)
    {
      double acc = 0.0;
      for (int s = 0; s < t.stages; ++s) acc += t.b[s] * k[s][c];
      out[c] = x[c] + h * acc;
    }
    return;
  }
  rk4_fp64(f, h, x, k1, out);
}

void rk4_fp64(const field& f, double h, const double* x, const double* k1, double* out)
{
  double k2[3], k3[3], k4[3], t[3];
  for (int c = 0; c < 3; ++c) t[c] = x[c] + 0.5 * h * k1[c];
  interpolate_fp64(f, t, k2);
  for (int c = 0; c < 3; ++c) t[c] = x[c] + 0.5 * h * k2[c];
  interpolate_fp64(f, t, k3);
  for (int c = 0; c < 3; ++c) t[c] = x[c] + h * k3[c];
  interpolate_fp64(f, t, k4);
  for (int c = 0; c < 3; ++c) out[c] = x[c] + h / 6.0 * (k1[c] + 2.0 * k2[c] + 2.0 * k3[c] + k4[c]);
}

// Eigenvalues of a symmetric 3x3 matrix by cyclic Jacobi rotations (each
// rotation zeroes one off-diagonal entry; sweeps repeat until the
// off-diagonal part vanishes), accurate to a few ulps of the matrix norm even
// for repeated eigenvalues.  The FTLE oracle uses these.
void eigenvalues_jacobi(const double in[3][3], double lambda[3])
{
  double a[3][3];
  for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) a[r][c] = 0.5 * (in[r][c] + in[c][r]);
  for (int sweep = 0; sweep < 64; ++sweep)
  {
    const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    if (off == 0.0) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q)
      {
        if (a[p][q] == 0.0) continue;
        // rotation angle that zeroes a[p][q]: t = tan(theta), smaller root
        const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k)   // A <- A J (columns p, q)
        {
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k)   // A <- J^T A (rows p, q)
        {
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        a[p][q] = a[q][p] = 0.0;
      }
  }
  for (int i = 0; i < 3; ++i) lambda[i] = a[i][i];
}

double largest_eigenvalue_jacobi(const double in[3][3])
{
  double l[3];
  eigenvalues_jacobi(in, l);
  return std::max(l[0], std::max(l[1], l[2]));
}

// Largest eigenvalue of a symmetric 3x3 matrix (trigonometric closed form,
// O. K. Smith, "Eigenvalues of a symmetric 3x3 matrix", CACM 4(4), 1961).
// Kept as an independent cross-check of the Jacobi eigenvalues.
double largest_eigenvalue(const double a[3][3])
{
  const double p1 = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
  if (p1 == 0.0) return std::max(a[0][0], std::max(a[1][1], a[2][2]));
  const double q  = (a[0][0] + a[1][1] + a[2][2]) / 3.0;
  const double d0 = a[0][0] - q, d1 = a[1][1] - q, d2 = a[2][2] - q;
  const double p2 = d0 * d0 + d1 * d1 + d2 * d2 + 2.0 * p1;
  const double p  = std::sqrt(p2 / 6.0);
  const double b00 = d0 / p, b11 = d1 / p, b22 = d2 / p;
  const double b01 = a[0][1] / p, b02 = a[0][2] / p, b12 = a[1][2] / p;
  const double det = b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02);
  double r = det / 2.0;
  r = r < -1.0 ? -1.0 : (r > 1.0 ? 1.0 : r);
  const double phi = std::acos(r) / 3.0;
  return q + 2.0 * p * std::cos(phi);
}
}

extern "C" {

void orc_set_correctly_rounded_trig(int on) { correctly_rounded_trig = on != 0; }

// ---- curves accessors ------------------------------------------------------
long long orc_curves_batches(const orc_curves* c) { return (long long)c->batches.size(); }
long long orc_curves_steps(const orc_curves* c) { return c->steps; }
long long orc_curves_vertex_count(const orc_curves* c, long long b) { return (long long)c->batches[b].vertices.size(); }
long long orc_curves_index_count(const orc_curves* c, long long b) { return (long long)c->batches[b].indices.size(); }
const float* orc_curves_vertices(const orc_curves* c, long long b) { return c->batches[b].vertices.empty() ? nullptr : c->batches[b].vertices[0].v; }
const float* orc_curves_colors(const orc_curves* c, long long b) { return c->batches[b].colors.empty() ? nullptr : c->batches[b].colors[0].v; }
const int* orc_curves_indices(const orc_curves* c, long long b) { return c->batches[b].indices.empty() ? nullptr : c->batches[b].indices.data(); }
int orc_curves_batch_rank(const orc_curves* c, long long b) { return c->batches[b].rank; }
int orc_curves_batch_round(const orc_curves* c, long long b) { return c->batches[b].round; }
void orc_curves_free(orc_curves* c) { delete c; }

int orc_max_threads()
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n)
{
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// ---- vector_field sampling ---------------------------------------------------
void orc_field_sample(const float* xyz, const int dims[3], const float offset[3], const float size[3], const float spacing[3],
                      const float* positions, long long n, unsigned char* inside, float* velocity)
{
  field f {xyz, {dims[0], dims[1], dims[2]}, {offset[0], offset[1], offset[2]}, {size[0], size[1], size[2]}, {spacing[0], spacing[1], spacing[2]}};
  for (long long i = 0; i < n; ++i)
  {
    inside[i] = contains(f, positions + 4 * i) ? 1 : 0;
    if (inside[i]) interpolate(f, positions + 4 * i, velocity + 3 * i);
    else velocity[3 * i] = velocity[3 * i + 1] = velocity[3 * i + 2] = 0.0f;
  }
}

// ---- seed_generator::generate ----------------------------------------------
long long orc_seed_generate(const float offset[3], const float size[3], const float stride[3], int iterations, int rank, void* out)
{
  int per_dimension[3];
  for (int i = 0; i < 3; ++i) per_dimension[i] = int(size[i] / stride[i]);
  const long long count = (long long)per_dimension[0] * per_dimension[1] * per_dimension[2];
  if (!out) return count;
  particle* particles = static_cast<particle*>(out);
  #pragma omp parallel for schedule(static)
  for (long long index = 0; index < count; ++index)
  {
    int idx[3];
    unravel(index, per_dimension, idx);
    particle& p = particles[index];
    std::memset(&p, 0, sizeof(p));
    for (int i = 0; i < 3; ++i) p.position[i] = offset[i] + stride[i] * float(idx[i]);
    p.position[3] = 0.0f;
    p.remaining_iterations = iterations;
    p.vector_field_index   = -1;
    p.original_rank        = rank;
    for (int i = 0; i < 3; ++i) p.original_voxel[i] = idx[i];
  }
  return count;
}

// ---- partitioner -------------------------------------------------------------
void orc_partition(int ranks, int rank, const int domain[3], int* info)
{
  const partition p = make_partition(ranks, domain);
  int multi[3];
  unravel(rank, p.grid, multi);
  for (int i = 0; i < 3; ++i)
  {
    info[i]      = p.grid[i];
    info[3 + i]  = p.block[i];
    info[6 + i]  = multi[i];
    info[9 + i]  = p.block[i] * multi[i];
    info[12 + i] = p.block[i] + (multi[i] + 1 < p.grid[i] ? 1 : 0);
  }
  for (int face = 0; face < 6; ++face)
  {
    int n[3] = {multi[0], multi[1], multi[2]};
    n[face / 2] += (face % 2 == 0) ? -1 : 1;
    const bool exists = n[face / 2] >= 0 && n[face / 2] < p.grid[face / 2];
    info[15 + face] = exists ? int(ravel(n, p.grid)) : -1;
  }
}

// ---- streamlines, one block --------------------------------------------------
// The reference's round loop on one rank: particles leaving the block have no
// neighbour and are dropped, so one round suffices.  integrator: 0 Euler,
// 2 RK4 (frozen velocity).  color < 0 skips colouring.
orc_curves* orc_trace_single(const float* xyz, const int dims[3], const float offset[3], const float size[3], const float spacing[3],
                             const void* particles_in, long long n, int integrator, float step, int color, float parameter)
{
  field f {xyz, {dims[0], dims[1], dims[2]}, {offset[0], offset[1], offset[2]}, {size[0], size[1], size[2]}, {spacing[0], spacing[1], spacing[2]}};
  const frozen_weights w = make_frozen_weights(integrator, step);
  std::vector<particle> particles(n);
  if (n) std::memcpy(particles.data(), particles_in, n * sizeof(particle));
  auto* result = new orc_curves();
  std::vector<exit_record> exits;
  trace_round(f, w, particles, 0, 0, nullptr, result->batches, exits, result->steps);
  for (auto& b : result->batches)
  {
    if (b.vertices.empty()) continue;
    generate_indices(b);
    if (color >= 0) generate_colors(b, color, parameter);
    else b.colors.clear();
  }
  return result;
}

// ---- streamlines over a partitioned domain -----------------------------------
// One block per rank of a `ranks`-way partition of the domain (partitioner
// restated above); each block holds its +1-ghosted sub-grid.  Every round each
// block traces its particles; particles leaving a block go to the face
// neighbour (dropped at the domain boundary), and the next round's particle
// list of a block is, in order of the sending block's rank, the particles that
// block sent, each sender's particles in their trace order.  Returns batches
// tagged with (rank, round), ordered by round, then rank.
orc_curves* orc_trace_multi(const float* xyz, const int domain[3], const float spacing[3], int ranks,
                            const long long* seed_offsets, const void* seeds_in, int integrator, float step, int color, float parameter)
{
  const partition part = make_partition(ranks, domain);
  const frozen_weights w = make_frozen_weights(integrator, step);
  struct block_data { std::vector<float> xyz; field f; int neighbor[6]; };
  std::vector<block_data> blocks(ranks);
  for (int r = 0; r < ranks; ++r)
  {
    int info[21];
    orc_partition(ranks, r, domain, info);
    auto& b = blocks[r];
    const int gx = info[12], gy = info[13], gz = info[14];
    b.xyz.resize(size_t(gx) * gy * gz * 3);
    for (int x = 0; x < gx; ++x)
      for (int y = 0; y < gy; ++y)
        for (int z = 0; z < gz; ++z)
        {
          const size_t g = (size_t(info[9] + x) * domain[1] + (info[10] + y)) * domain[2] + (info[11] + z);
          const size_t l = (size_t(x) * gy + y) * gz + z;
          for (int c = 0; c < 3; ++c) b.xyz[3 * l + c] = xyz[3 * g + c];
        }
    b.f.xyz = b.xyz.data();
    b.f.shape[0] = gx; b.f.shape[1] = gy; b.f.shape[2] = gz;
    for (int i = 0; i < 3; ++i)
    {
      b.f.spacing[i] = spacing[i];
      b.f.offset[i]  = float(info[9 + i]) * spacing[i];
      b.f.size[i]    = float(part.block[i]) * spacing[i];
    }
    for (int face = 0; face < 6; ++face) b.neighbor[face] = info[15 + face];
  }

  std::vector<std::vector<particle>> current(ranks);
  for (int r = 0; r < ranks; ++r)
  {
    const long long begin = seed_offsets[r], end = seed_offsets[r + 1];
    current[r].resize(end - begin);
    if (end > begin) std::memcpy(current[r].data(), static_cast<const particle*>(seeds_in) + begin, (end - begin) * sizeof(particle));
  }
  auto* result = new orc_curves();
  for (int round = 0;; ++round)
  {
    bool any = false;
    for (auto& c : current) any = any || !c.empty();
    if (!any) break;
    std::vector<std::vector<particle>> next(ranks);
    std::vector<std::vector<exit_record>> exits(ranks);
    for (int r = 0; r < ranks; ++r)
      trace_round(blocks[r].f, w, current[r], r, round, blocks[r].neighbor, result->batches, exits[r], result->steps);
    // Delivery in sender-rank order.
    for (int r = 0; r < ranks; ++r)
      for (auto& e : exits[r])
        next[blocks[r].neighbor[e.face]].push_back(e.p);
    current.swap(next);
  }
  for (auto& b : result->batches)
  {
    if (b.vertices.empty()) continue;
    generate_indices(b);
    if (color >= 0) generate_colors(b, color, parameter);
  }
  return result;
}

// ---- index / colour on one buffer ------------------------------------------
long long orc_index_generate(const float* vertices, long long n, int* indices)
{
  batch b;
  b.vertices.resize(n);
  if (n) std::memcpy(b.vertices.data(), vertices, n * 16);
  generate_indices(b);
  if (indices && !b.indices.empty()) std::memcpy(indices, b.indices.data(), b.indices.size() * 4);
  return (long long)b.indices.size();
}
void orc_color_generate(const float* vertices, long long n, const int* indices, long long n_indices, int mode, float parameter, float* colors)
{
  batch b;
  b.vertices.resize(n);
  if (n) std::memcpy(b.vertices.data(), vertices, n * 16);
  b.indices.assign(indices, indices + n_indices);
  generate_colors(b, mode, parameter);
  if (n) std::memcpy(colors, b.colors.data(), n * 16);
}

// ---- flow map: particle_advector + flow_map_generator, FP32 frozen ----------
// Seeds one particle per voxel of a grid of int(dims * scale) voxels with
// spacing = spacing / scale (flow_map_generator.cpp:23-43) and advects it with
// the reference's rules (particle_advector.cpp:74-139, one block): a particle
// stops with its current position when it leaves the grid, meets a zero
// velocity, or completes iterations - 1 steps.  flow: [X'][Y'][Z'][3].
// Particles first + k * stride (k < count) of the C-order seed list only (a
// bounded sample; stride 1: a contiguous range); returns the steps taken.
long long orc_flow_map(const float* xyz, const int dims[3], const float offset[3], const float size[3], const float spacing[3],
                       int iterations, float scale, int integrator, float step, long long first, long long count,
                       long long stride, float* flow)
{
  field f {xyz, {dims[0], dims[1], dims[2]}, {offset[0], offset[1], offset[2]}, {size[0], size[1], size[2]}, {spacing[0], spacing[1], spacing[2]}};
  const frozen_weights w = make_frozen_weights(integrator, step);
  int fm[3];
  float fm_spacing[3];
  for (int i = 0; i < 3; ++i) { fm[i] = int(float(dims[i]) * scale); fm_spacing[i] = spacing[i] / scale; }
  int per_dimension[3];
  for (int i = 0; i < 3; ++i) per_dimension[i] = int(size[i] / fm_spacing[i]);
  long long steps = 0;
  #pragma omp parallel for schedule(dynamic, 64) reduction(+ : steps)
  for (long long k = 0; k < count; ++k)
  {
    const long long index = first + k * stride;
    int idx[3];
    unravel(index, per_dimension, idx);
    float pos[4];
    for (int i = 0; i < 3; ++i) pos[i] = offset[i] + fm_spacing[i] * float(idx[i]);
    pos[3] = 0.0f;
    bool finished = false;
    frozen_history hist;
    for (long long i = 1; i < iterations; ++i)
    {
      if (!contains(f, pos)) { finished = true; break; }
      float v[3];
      interpolate(f, pos, v);
      if (is_zero(v)) { finished = true; break; }
      float next[4];
      frozen_step(w, pos, v, next, hist);
      std::memcpy(pos, next, 16);
      ++steps;
      if (i + 1 == iterations) { finished = true; break; }
    }
    if (!finished) continue;   // iterations <= 1: the reference never assigns it
    if (idx[0] < fm[0] && idx[1] < fm[1] && idx[2] < fm[2])
      for (int c = 0; c < 3; ++c) flow[3 * ravel(idx, fm) + c] = pos[c];
  }
  return steps;
}

// ---- FP64 advection oracle ---------------------------------------------------
// Advects n positions in FP64 on the FP32 grid values with the reference's
// termination rules (contains / isZero at the step start, at most max_steps
// steps).  mode 0 = frozen velocity, 1 = re-sampled stages (classical RK4).
// When `vertices` is not null it receives, per particle, max_steps + 1 slots
// (xyz, FP64): the start and every step; unused slots are left untouched.
// steps_out receives the steps each particle took.  noise > 0 multiplies each
// new position coordinate by (1 + noise * N(0,1)) (a seeded per-particle
// generator): an ensemble of such runs measures how far rounding at that
// relative level can move an end point, i.e. the problem's conditioning.
void orc_advect_fp64(const float* xyz, const int dims[3], const float offset[3], const float size[3], const float spacing[3],
                     const double* start, long long n, int integrator, int mode, double step, long long max_steps,
                     double* end, long long* steps_out, double* vertices, double noise, unsigned long long seed)
{
  field f {xyz, {dims[0], dims[1], dims[2]}, {offset[0], offset[1], offset[2]}, {size[0], size[1], size[2]}, {spacing[0], spacing[1], spacing[2]}};
  #pragma omp parallel for schedule(dynamic, 16)
  for (long long i = 0; i < n; ++i)
  {
    double x[3] = {start[3 * i], start[3 * i + 1], start[3 * i + 2]};
    double* track = vertices ? vertices + 3 * (max_steps + 1) * i : nullptr;
    if (track) std::memcpy(track, x, 24);
    // splitmix64 stream per particle; Box-Muller normals.
    unsigned long long state = seed * 0x9E3779B97F4A7C15ULL + (unsigned long long)i * 0xD1B54A32D192ED03ULL + 1;
    auto uniform = [&state]() {
      unsigned long long z = (state += 0x9E3779B97F4A7C15ULL);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      z ^= z >> 31;
      return (double(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    long long s = 0;
    history_fp64 hist;
    for (; s < max_steps; ++s)
    {
      if (!contains_fp64(f, x)) break;
      double k1[3];
      interpolate_fp64(f, x, k1);
      if (is_zero_fp64(k1)) break;
      double next[3];
      step_fp64(f, integrator, mode, step, x, k1, next, hist);
      if (noise > 0.0)
        for (int c = 0; c < 3; ++c)
        {
          const double g = std::sqrt(-2.0 * std::log(uniform())) * std::cos(6.283185307179586 * uniform());
          next[c] *= 1.0 + noise * g;
        }
      std::memcpy(x, next, 24);
      if (track) std::memcpy(track + 3 * (s + 1), x, 24);
    }
    std::memcpy(end + 3 * i, x, 24);
    steps_out[i] = s;
  }
}

// ---- FP64 pathline oracle on an unsteady field ----------------------------------
// `slices` grids [slices][X][Y][Z][3] (FP32), slice k at time t0 + k*slice_dt,
// linear in time between slices, constant outside [t0, t_last].  Classical RK4
// in space-time from (start, time_begin) with step h: the step stops when the
// particle leaves the grid (floor quotient outside [0, shape-2]), when |v_i| <=
// 1e-5 at the step start, or after max_steps steps.  Time of step n:
// time_begin + n*h.
void orc_advect_unsteady_fp64(const float* xyz, const int dims[3], int slices, const float offset[3], const float spacing[3],
                              double t0, double slice_dt, const double* start, long long n, double time_begin, double h,
                              long long max_steps, double* end, long long* steps_out)
{
  const long long slice_stride = 3LL * dims[0] * dims[1] * dims[2];
  auto sample = [&](const double* p, double t, double* out) {
    int k = 0;
    double wt = 0.0;
    if (slices > 1)
    {
      const double s = (t - t0) / slice_dt;
      const double fs = std::floor(s);
      if (!(fs >= 0.0)) { k = 0; wt = 0.0; }
      else if (fs >= double(slices - 1)) { k = slices - 2; wt = 1.0; }
      else { k = int(fs); wt = s - fs; }
    }
    field f0 {xyz + k * slice_stride, {dims[0], dims[1], dims[2]}, {offset[0], offset[1], offset[2]}, {0, 0, 0},
              {spacing[0], spacing[1], spacing[2]}};
    double a[3];
    interpolate_fp64(f0, p, a);
    if (slices > 1 && wt != 0.0)
    {
      field f1 = f0;
      f1.xyz = xyz + (k + 1) * slice_stride;
      double b[3];
      interpolate_fp64(f1, p, b);
      for (int c = 0; c < 3; ++c) a[c] = (1.0 - wt) * a[c] + wt * b[c];
    }
    for (int c = 0; c < 3; ++c) out[c] = a[c];
  };
  field shape_only {xyz, {dims[0], dims[1], dims[2]}, {offset[0], offset[1], offset[2]}, {0, 0, 0},
                    {spacing[0], spacing[1], spacing[2]}};
  #pragma omp parallel for schedule(dynamic, 16)
  for (long long i = 0; i < n; ++i)
  {
    double x[3] = {start[3 * i], start[3 * i + 1], start[3 * i + 2]};
    long long s = 0;
    for (; s < max_steps; ++s)
    {
      if (!contains_fp64(shape_only, x)) break;
      const double t = time_begin + double(s) * h;
      double k1[3], k2[3], k3[3], k4[3], tmp[3];
      sample(x, t, k1);
      if (is_zero_fp64(k1)) break;
      for (int c = 0; c < 3; ++c) tmp[c] = x[c] + 0.5 * h * k1[c];
      sample(tmp, t + 0.5 * h, k2);
      for (int c = 0; c < 3; ++c) tmp[c] = x[c] + 0.5 * h * k2[c];
      sample(tmp, t + 0.5 * h, k3);
      for (int c = 0; c < 3; ++c) tmp[c] = x[c] + h * k3[c];
      sample(tmp, t + h, k4);
      for (int c = 0; c < 3; ++c) x[c] += h / 6.0 * (k1[c] + 2.0 * k2[c] + 2.0 * k3[c] + k4[c]);
    }
    std::memcpy(end + 3 * i, x, 24);
    steps_out[i] = s;
  }
}

// ---- FTLE, FP64 intended mathematics -------------------------------------------
// J_ij = d phi_i / d x_j by central differences with denominator 2h_j, one-sided
// at the grid borders (0 along an axis of extent 1); C = J^T J with eigenvalues
// l0, l1, l2.  mode 0 (regular): log(sqrt(max l)) / |T|.  mode 1 (fractional
// anisotropy, ftle_map_generator.cpp:51-54): sqrt(0.5) sqrt((l0 - l1)^2 +
// (l1 - l2)^2 + (l2 - l0)^2) / sqrt(l0^2 + l1^2 + l2^2).  flow: [X][Y][Z][3]
// (FP32), out FP64.
void orc_ftle_fp64(const float* flow, const int dims[3], const float spacing[3], double time, int mode, double* out)
{
  const long long X = dims[0], Y = dims[1], Z = dims[2];
  #pragma omp parallel for schedule(static)
  for (long long x = 0; x < X; ++x)
    for (long long y = 0; y < Y; ++y)
      for (long long z = 0; z < Z; ++z)
      {
        const long long idx[3] = {x, y, z};
        const long long ext[3] = {X, Y, Z};
        double J[3][3];
        for (int j = 0; j < 3; ++j)
        {
          long long lo[3] = {x, y, z}, hi[3] = {x, y, z};
          double denominator;
          if (ext[j] == 1) { for (int i = 0; i < 3; ++i) J[i][j] = 0.0; continue; }
          if (idx[j] == 0)                { hi[j] = 1;              denominator = spacing[j]; }
          else if (idx[j] == ext[j] - 1)  { lo[j] = ext[j] - 2;     denominator = spacing[j]; }
          else                            { lo[j] -= 1; hi[j] += 1; denominator = 2.0 * double(spacing[j]); }
          const float* a = flow + 3 * ((lo[0] * Y + lo[1]) * Z + lo[2]);
          const float* b = flow + 3 * ((hi[0] * Y + hi[1]) * Z + hi[2]);
          for (int i = 0; i < 3; ++i) J[i][j] = (double(b[i]) - double(a[i])) / denominator;
        }
        double C[3][3];
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c)
            C[r][c] = J[0][r] * J[0][c] + J[1][r] * J[1][c] + J[2][r] * J[2][c];
        double l[3];
        eigenvalues_jacobi(C, l);
        double value;
        if (mode == 0) value = std::log(std::sqrt(std::max(l[0], std::max(l[1], l[2])))) / std::fabs(time);
        else
          value = std::sqrt(0.5) *
                  std::sqrt((l[0] - l[1]) * (l[0] - l[1]) + (l[1] - l[2]) * (l[1] - l[2]) + (l[2] - l[0]) * (l[2] - l[0])) /
                  std::sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
        out[(x * Y + y) * Z + z] = value;
      }
}

// Largest eigenvalue of symmetric 3x3 matrices (row-major, 9 doubles each).
void orc_largest_eigenvalue(const double* matrices, long long n, double* out)
{
  for (long long i = 0; i < n; ++i)
  {
    double a[3][3];
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) a[r][c] = matrices[9 * i + 3 * r + c];
    out[i] = largest_eigenvalue_jacobi(a);
  }
}

// The same with the trigonometric closed form (an independent cross-check of
// the Jacobi eigenvalues).
void orc_largest_eigenvalue_closed_form(const double* matrices, long long n, double* out)
{
  for (long long i = 0; i < n; ++i)
  {
    double a[3][3];
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) a[r][c] = matrices[9 * i + 3 * r + c];
    out[i] = largest_eigenvalue(a);
  }
}

}
