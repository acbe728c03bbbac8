// CPU restatement of the ray tracer (test infrastructure only: the oracle the
// GPU ray tracer is checked against, and the CPU baseline of the render
// workload).  It follows the library's definition of the reference's OSPRay
// configuration (pars/source/stages/ray_tracer.cpp:28-253), written here from
// that definition:
//
// * scene: per line index i (segment start vertex g = batch offset + i), a
//   capsule of radius r around (v[g], v[g+1]) -- cylinder plus end spheres --
//   coloured with colour[g] (white without colours); the closest hit is the
//   smallest (distance, g) pair over all capsules with distance > 0;
// * a capsule test shifts the ray origin to the ray's closest approach to the
//   segment start, then takes the cylinder root (inside the segment's extent)
//   and the two sphere roots, nearest first;
// * volume: trilinear samples (cell = floor of (p - offset) / spacing, clamped
//   to the grid, weights clamped to [0, 1], lerp z then y then x) at
//   t_enter + (k + 1/2) dt, dt = min(spacing) / 2, until the box exit or the
//   surface; value v clamped to [0, 1], opacity 0.0001 + 0.0254 v, step alpha
//   1 - sqrt(1 - opacity), grey colour v, front-to-back compositing;
// * shading: base = 0.8 colour; ambient 1; per light l with unit vector L_l
//   towards it and colour (1, 1, 0.8): if n.L > 0, base (n.L) colour_l +
//   0.7 (n.h)^10 colour_l (h = normalize(L + view), only n.h > 0);
// * frame colour clamped to [0, 1] and summed per pixel; the image is the sum
//   over the frames divided by their count, sRGB-encoded to 8 bits (byte q =
//   count of thresholds decode((j + 1/2) / 255), j < 255, at or below the
//   value), alpha 255;
// * camera: fovy 68 degrees, aspect width / height, basis and image plane in
//   FP64 then rounded to FP32; sample (px + jx, py + jy), rows from the top;
//   jitter (1/2, 1/2) for frame 0, else Halton (2, 3) of the frame number.
//
// Every FP32 operation is written in the order the GPU kernel uses and
// compiled without contraction, so the two agree bit for bit.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

namespace
{
struct v3 { float x, y, z; };
inline v3    sub(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline v3    add(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline v3    mul(v3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline v3    unit(v3 a) { const float l = std::sqrt(dot(a, a)); return {a.x / l, a.y / l, a.z / l}; }
inline v3    load(const float* p) { return {p[0], p[1], p[2]}; }

const float inf = std::numeric_limits<float>::infinity();

struct hit { float t = inf; long long g = LLONG_MAX; int part = -1; };

float sphere_entry(v3 o, v3 d, v3 c, float r)
{
  const v3 oc = sub(o, c);
  const float b = dot(d, oc);
  const float h = b * b - (dot(oc, oc) - r * r);
  if (h < 0.0f) return inf;
  return -b - std::sqrt(h);
}

void capsule(v3 o, v3 d, v3 a, v3 b, float r, long long g, hit& best)
{
  const float tc = dot(sub(a, o), d);
  const v3 s = add(o, mul(d, tc));
  float t = inf;
  int part = -1;
  const v3 ba = sub(b, a), sa = sub(s, a);
  const float baba = dot(ba, ba);
  if (baba > 0.0f)
  {
    const float bard = dot(ba, d), baoa = dot(ba, sa), rdoa = dot(d, sa), oaoa = dot(sa, sa);
    const float qa = baba - bard * bard;
    if (qa > 0.0f)
    {
      const float qb = baba * rdoa - baoa * bard;
      const float qc = baba * oaoa - baoa * baoa - r * r * baba;
      const float h = qb * qb - qa * qc;
      if (h >= 0.0f)
      {
        const float u = (-qb - std::sqrt(h)) / qa;
        const float y = baoa + u * bard;
        if (y > 0.0f && y < baba && tc + u > 0.0f) { t = tc + u; part = 0; }
      }
    }
  }
  const float ea = tc + sphere_entry(s, d, a, r);
  if (ea > 0.0f && ea < t) { t = ea; part = 1; }
  const float eb = tc + sphere_entry(s, d, b, r);
  if (eb > 0.0f && eb < t) { t = eb; part = 2; }
  if (part >= 0 && (t < best.t || (t == best.t && g < best.g))) { best.t = t; best.g = g; best.part = part; }
}

// Slab test against [0, t_max] (NaN from 0 * inf ignored, as fminf/fmaxf do).
bool box(v3 o, v3 inv, const float lo[3], const float hi[3], float t_max, float& t_near)
{
  const float tx0 = (lo[0] - o.x) * inv.x, tx1 = (hi[0] - o.x) * inv.x;
  const float ty0 = (lo[1] - o.y) * inv.y, ty1 = (hi[1] - o.y) * inv.y;
  const float tz0 = (lo[2] - o.z) * inv.z, tz1 = (hi[2] - o.z) * inv.z;
  const float tn = std::fmax(std::fmax(std::fmin(tx0, tx1), std::fmin(ty0, ty1)), std::fmax(std::fmin(tz0, tz1), 0.0f));
  const float tf = std::fmin(std::fmin(std::fmax(tx0, tx1), std::fmax(ty0, ty1)), std::fmin(std::fmax(tz0, tz1), t_max));
  t_near = tn;
  return tn <= tf;
}

// A plain median-split BVH over the capsules' padded boxes: it only prunes,
// so the closest (distance, g) pair is the one a test of every capsule gives.
struct bvh
{
  struct node { float lo[3], hi[3]; int left = -1, right = -1, first = 0, count = 0; };
  std::vector<node> nodes;
  std::vector<long long> order;     // prim numbers, leaves are ranges of it
  std::vector<float> plo, phi;      // per prim box

  int build(long long first, long long count, int depth)
  {
    node n;
    for (int i = 0; i < 3; ++i) { n.lo[i] = inf; n.hi[i] = -inf; }
    for (long long k = first; k < first + count; ++k)
      for (int i = 0; i < 3; ++i)
      {
        n.lo[i] = std::min(n.lo[i], plo[3 * order[k] + i]);
        n.hi[i] = std::max(n.hi[i], phi[3 * order[k] + i]);
      }
    const int id = int(nodes.size());
    nodes.push_back(n);
    if (count <= 4 || depth > 48)
    {
      nodes[id].first = int(first);
      nodes[id].count = int(count);
      return id;
    }
    int axis = 0;
    for (int i = 1; i < 3; ++i) if (n.hi[i] - n.lo[i] > n.hi[axis] - n.lo[axis]) axis = i;
    const long long mid = first + count / 2;
    std::nth_element(order.begin() + first, order.begin() + mid, order.begin() + first + count, [&](long long a, long long b) {
      return plo[3 * a + axis] + phi[3 * a + axis] < plo[3 * b + axis] + phi[3 * b + axis];
    });
    const int l = build(first, mid - first, depth + 1);
    const int r = build(mid, first + count - mid, depth + 1);
    nodes[id].left = l;
    nodes[id].right = r;
    return id;
  }
};

struct scene
{
  const float* v;            // float4 vertices
  const float* c;            // float4 colours or nullptr
  const long long* prim;     // segment start vertex per prim
  long long prims;
  float r;
  bvh tree;
  const float* vol;
  int n[3];
  float vo[3], vh[3], vhi[3], dt;
};

hit closest(const scene& S, v3 o, v3 d, v3 inv)
{
  hit best;
  if (S.prims <= 0) return best;
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp)
  {
    const auto& n = S.tree.nodes[stack[--sp]];
    float tn;
    if (!box(o, inv, n.lo, n.hi, best.t, tn)) continue;
    if (n.left < 0)
    {
      for (int k = n.first; k < n.first + n.count; ++k)
      {
        const long long p = S.tree.order[k];
        const long long g = S.prim[p];
        capsule(o, d, load(S.v + 4 * g), load(S.v + 4 * (g + 1)), S.r, g, best);
      }
      continue;
    }
    stack[sp++] = n.left;
    stack[sp++] = n.right;
  }
  return best;
}

inline float lerp(float a, float b, float w) { return a + w * (b - a); }

float sample(const scene& S, v3 p)
{
  const float qx = (p.x - S.vo[0]) / S.vh[0], qy = (p.y - S.vo[1]) / S.vh[1], qz = (p.z - S.vo[2]) / S.vh[2];
  const float fx = std::fmin(std::fmax(std::floor(qx), 0.0f), float(S.n[0] - 2));
  const float fy = std::fmin(std::fmax(std::floor(qy), 0.0f), float(S.n[1] - 2));
  const float fz = std::fmin(std::fmax(std::floor(qz), 0.0f), float(S.n[2] - 2));
  const float wx = std::fmin(std::fmax(qx - fx, 0.0f), 1.0f), wy = std::fmin(std::fmax(qy - fy, 0.0f), 1.0f),
              wz = std::fmin(std::fmax(qz - fz, 0.0f), 1.0f);
  const long long ix = (long long)fx, iy = (long long)fy, iz = (long long)fz;
  const long long sy = S.n[2], sx = (long long)S.n[1] * S.n[2];
  const float* c = S.vol + ix * sx + iy * sy + iz;
  const float c00 = lerp(c[0], c[1], wz), c01 = lerp(c[sy], c[sy + 1], wz);
  const float c10 = lerp(c[sx], c[sx + 1], wz), c11 = lerp(c[sx + sy], c[sx + sy + 1], wz);
  return lerp(lerp(c00, c01, wy), lerp(c10, c11, wy), wx);
}

void camera(const float pos[3], const float fwd[3], const float up[3], int w, int h, v3& corner, v3& du, v3& dv)
{
  const double pi = 3.14159265358979323846;
  double f[3] = {fwd[0], fwd[1], fwd[2]};
  const double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  for (auto& x : f) x /= fl;
  double u[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
  const double ul = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  for (auto& x : u) x /= ul;
  const double v[3] = {u[1] * f[2] - u[2] * f[1], u[2] * f[0] - u[0] * f[2], u[0] * f[1] - u[1] * f[0]};
  const double sy = 2.0 * std::tan(68.0 * pi / 360.0), sx = sy * double(w) / double(h);
  corner = {float(f[0] - 0.5 * sx * u[0] - 0.5 * sy * v[0]), float(f[1] - 0.5 * sx * u[1] - 0.5 * sy * v[1]),
            float(f[2] - 0.5 * sx * u[2] - 0.5 * sy * v[2])};
  du = {float(sx * u[0]), float(sx * u[1]), float(sx * u[2])};
  dv = {float(sy * v[0]), float(sy * v[1]), float(sy * v[2])};
}

void jitter(long long frame, float& jx, float& jy)
{
  if (frame == 0) { jx = jy = 0.5f; return; }
  double x = 0.0, f = 0.5;
  for (long long i = frame; i > 0; i /= 2, f *= 0.5) x += f * double(i % 2);
  double y = 0.0, g = 1.0 / 3.0;
  for (long long i = frame; i > 0; i /= 3, g /= 3.0) y += g * double(i % 3);
  jx = float(x);
  jy = float(y);
}
}  // namespace

extern "C" {

// Adds `frames` frames (numbered first_frame ...) to accum (width*height*4
// floats: r, g, b sums and the frame count) and, when rgba is not NULL,
// writes the encoded image of accum.  vertices / colors: float4 arrays;
// prim_vertex: the start vertex of each capsule's segment.  volume may be
// NULL.  Returns 0.
int orc_render(const float* vertices, const float* colors, const long long* prim_vertex, long long prims, float radius,
               const float* volume, const int* vshape, const float* voffset, const float* vspacing, const float* position,
               const float* forward, const float* up, int width, int height, long long first_frame, int frames, float* accum,
               unsigned char* rgba)
{
  scene S {};
  S.v = vertices; S.c = colors; S.prim = prim_vertex; S.prims = prims; S.r = radius; S.vol = volume;
  if (prims > 0)
  {
    float big = 0.0f;
    for (long long k = 0; k < prims; ++k)
      for (int e = 0; e < 2; ++e)
        for (int i = 0; i < 3; ++i) big = std::max(big, std::fabs(vertices[4 * (prim_vertex[k] + e) + i]));
    const float pad = radius + (radius + big) * (1.0f / 65536.0f);
    S.tree.plo.resize(3 * prims);
    S.tree.phi.resize(3 * prims);
    for (long long k = 0; k < prims; ++k)
      for (int i = 0; i < 3; ++i)
      {
        const float a = vertices[4 * prim_vertex[k] + i], b = vertices[4 * (prim_vertex[k] + 1) + i];
        S.tree.plo[3 * k + i] = std::min(a, b) - pad;
        S.tree.phi[3 * k + i] = std::max(a, b) + pad;
      }
    S.tree.order.resize(prims);
    std::iota(S.tree.order.begin(), S.tree.order.end(), 0LL);
    S.tree.build(0, prims, 0);
  }
  if (volume)
  {
    for (int i = 0; i < 3; ++i)
    {
      S.n[i] = vshape[i];
      S.vo[i] = voffset[i];
      S.vh[i] = vspacing[i];
      S.vhi[i] = voffset[i] + float(vshape[i] - 1) * vspacing[i];
    }
    S.dt = 0.5f * std::min(vspacing[0], std::min(vspacing[1], vspacing[2]));
  }
  v3 corner, du, dv;
  camera(position, forward, up, width, height, corner, du, dv);
  const v3 o = load(position);
  v3 light[2];
  const double dirs[2][3] = {{1.0, 1.0, -0.5}, {-1.0, 0.0, 0.5}};
  for (int l = 0; l < 2; ++l)
  {
    const double len = std::sqrt(dirs[l][0] * dirs[l][0] + dirs[l][1] * dirs[l][1] + dirs[l][2] * dirs[l][2]);
    light[l] = {float(-dirs[l][0] / len), float(-dirs[l][1] / len), float(-dirs[l][2] / len)};
  }
  const v3 light_color = {1.0f, 1.0f, 0.8f};
  std::vector<float> jx(frames), jy(frames);
  for (int f = 0; f < frames; ++f) jitter(first_frame + f, jx[f], jy[f]);

  #pragma omp parallel for schedule(dynamic, 4)
  for (int py = 0; py < height; ++py)
    for (int px = 0; px < width; ++px)
    {
      float* acc = accum + 4 * ((long long)py * width + px);
      for (int f = 0; f < frames; ++f)
      {
        const float sx = (float(px) + jx[f]) / float(width);
        const float sy = 1.0f - (float(py) + jy[f]) / float(height);
        const v3 r = {corner.x + sx * du.x + sy * dv.x, corner.y + sx * du.y + sy * dv.y, corner.z + sx * du.z + sy * dv.z};
        const v3 d = unit(r);
        const v3 inv = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
        const hit h = closest(S, o, d, inv);
        float cr = 0.0f, cg = 0.0f, cb = 0.0f, alpha = 0.0f;
        if (volume)
        {
          float t_enter;
          if (box(o, inv, S.vo, S.vhi, inf, t_enter))
          {
            const float tx = std::fmax((S.vo[0] - o.x) * inv.x, (S.vhi[0] - o.x) * inv.x);
            const float ty = std::fmax((S.vo[1] - o.y) * inv.y, (S.vhi[1] - o.y) * inv.y);
            const float tz = std::fmax((S.vo[2] - o.z) * inv.z, (S.vhi[2] - o.z) * inv.z);
            const float t_exit = std::fmin(std::fmin(std::fmin(tx, ty), tz), h.t);
            for (int k = 0; k < (1 << 22); ++k)
            {
              const float t = t_enter + (float(k) + 0.5f) * S.dt;
              if (!(t < t_exit)) break;
              const float value = std::fmin(std::fmax(sample(S, add(o, mul(d, t))), 0.0f), 1.0f);
              const float opacity = 0.0001f + value * 0.0254f;
              const float a = 1.0f - std::sqrt(1.0f - opacity);
              const float w = (1.0f - alpha) * a;
              cr = cr + w * value; cg = cg + w * value; cb = cb + w * value;
              alpha = alpha + w;
            }
          }
        }
        if (h.part >= 0)
        {
          const v3 a = load(vertices + 4 * h.g), b = load(vertices + 4 * (h.g + 1));
          const v3 p = add(o, mul(d, h.t));
          v3 n;
          if (h.part == 1) n = sub(p, a);
          else if (h.part == 2) n = sub(p, b);
          else
          {
            const v3 ba = sub(b, a), pa = sub(p, a);
            n = sub(pa, mul(ba, dot(pa, ba) / dot(ba, ba)));
          }
          n = unit(n);
          const v3 view = {-d.x, -d.y, -d.z};
          v3 base = {0.8f, 0.8f, 0.8f};
          if (colors) base = {0.8f * colors[4 * h.g], 0.8f * colors[4 * h.g + 1], 0.8f * colors[4 * h.g + 2]};
          v3 out = mul(base, 1.0f);
          for (int l = 0; l < 2; ++l)
          {
            const float ndl = dot(n, light[l]);
            if (ndl <= 0.0f) continue;
            out = add(out, {base.x * ndl * light_color.x, base.y * ndl * light_color.y, base.z * ndl * light_color.z});
            const float ndh = dot(n, unit(add(light[l], view)));
            if (ndh > 0.0f)
            {
              const float x2 = ndh * ndh, x4 = x2 * x2, x8 = x4 * x4, s = 0.7f * (x8 * x2);
              out = add(out, {s * light_color.x, s * light_color.y, s * light_color.z});
            }
          }
          const float w = 1.0f - alpha;
          cr = cr + w * out.x; cg = cg + w * out.y; cb = cb + w * out.z;
        }
        acc[0] = acc[0] + std::fmin(std::fmax(cr, 0.0f), 1.0f);
        acc[1] = acc[1] + std::fmin(std::fmax(cg, 0.0f), 1.0f);
        acc[2] = acc[2] + std::fmin(std::fmax(cb, 0.0f), 1.0f);
        acc[3] = acc[3] + 1.0f;
      }
    }

  if (rgba)
  {
    float thresholds[255];
    for (int q = 0; q < 255; ++q)
    {
      const double s = (q + 0.5) / 255.0;
      thresholds[q] = float(s <= 0.04045 ? s / 12.92 : std::pow((s + 0.055) / 1.055, 2.4));
    }
    const long long pixels = (long long)width * height;
    for (long long p = 0; p < pixels; ++p)
    {
      const float count = accum[4 * p + 3];
      for (int ch = 0; ch < 3; ++ch)
      {
        const float value = count > 0.0f ? accum[4 * p + ch] / count : 0.0f;
        int q = 0;
        while (q < 255 && value >= thresholds[q]) ++q;
        rgba[4 * p + ch] = (unsigned char)q;
      }
      rgba[4 * p + 3] = 255;
    }
  }
  return 0;
}

}  // extern "C"
