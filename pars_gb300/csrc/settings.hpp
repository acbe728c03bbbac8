// The request message of pars_service: proto3 `pars.settings`
// (pars/proto/settings.proto:5-27), decoded from its binary wire form without
// libprotobuf.  Unknown fields are skipped; repeated scalars are accepted both
// packed and unpacked, as the proto3 wire format requires.
#pragma once

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace pars
{
struct settings
{
  std::string          mode;                               // 1
  std::string          volume_type;                        // 2
  std::string          dataset_filepath;                   // 3
  std::vector<int32_t> seed_generation_stride;             // 4
  int32_t              seed_generation_iterations = 0;     // 5
  std::string          particle_tracing_integrator;        // 6
  float                particle_tracing_step_size = 0.0f;  // 7
  bool                 particle_tracing_load_balance = false;  // 8
  std::string          color_generation_mode;              // 9
  float                color_generation_free_parameter = 0.0f; // 10
  std::vector<float>   raytracing_camera_position;         // 11
  std::vector<float>   raytracing_camera_forward;          // 12
  std::vector<float>   raytracing_camera_up;               // 13
  std::vector<int32_t> raytracing_image_size;              // 14
  float                raytracing_streamline_radius = 0.0f;    // 15
  int32_t              raytracing_iterations = 0;          // 16
};

namespace wire
{
struct reader
{
  const uint8_t* p;
  const uint8_t* end;
  bool           ok = true;

  uint64_t varint()
  {
    uint64_t value = 0;
    for (int shift = 0; shift < 64; shift += 7)
    {
      if (p >= end) { ok = false; return 0; }
      const uint8_t byte = *p++;
      value |= uint64_t(byte & 0x7f) << shift;
      if (!(byte & 0x80)) return value;
    }
    ok = false;
    return 0;
  }
  uint32_t fixed32()
  {
    if (end - p < 4) { ok = false; return 0; }
    uint32_t v = uint32_t(p[0]) | uint32_t(p[1]) << 8 | uint32_t(p[2]) << 16 | uint32_t(p[3]) << 24;
    p += 4;
    return v;
  }
  bool skip(int wire_type)
  {
    switch (wire_type)
    {
    case 0: varint(); return ok;
    case 1: if (end - p < 8) return ok = false; p += 8; return true;
    case 2: { const uint64_t n = varint(); if (!ok || uint64_t(end - p) < n) return ok = false; p += n; return true; }
    case 5: if (end - p < 4) return ok = false; p += 4; return true;
    default: return ok = false;
    }
  }
};

inline float as_float(uint32_t bits) { float f; std::memcpy(&f, &bits, 4); return f; }
}

// Decodes `bytes` into `out`; returns false (with a message) on malformed input.
inline bool decode_settings(const uint8_t* bytes, std::size_t length, settings& out, std::string& error)
{
  wire::reader r {bytes, bytes + length};
  auto string_field = [&](std::string& s) {
    const uint64_t n = r.varint();
    if (!r.ok || uint64_t(r.end - r.p) < n) { r.ok = false; return; }
    s.assign(reinterpret_cast<const char*>(r.p), std::size_t(n));
    r.p += n;
  };
  auto int32s = [&](int wire_type, std::vector<int32_t>& v) {
    if (wire_type == 0) { v.push_back(int32_t(r.varint())); return; }
    if (wire_type != 2) { r.ok = false; return; }
    const uint64_t n = r.varint();
    if (!r.ok || uint64_t(r.end - r.p) < n) { r.ok = false; return; }
    wire::reader inner {r.p, r.p + n};
    while (inner.ok && inner.p < inner.end) v.push_back(int32_t(inner.varint()));
    r.ok = inner.ok;
    r.p += n;
  };
  auto floats = [&](int wire_type, std::vector<float>& v) {
    if (wire_type == 5) { v.push_back(wire::as_float(r.fixed32())); return; }
    if (wire_type != 2) { r.ok = false; return; }
    const uint64_t n = r.varint();
    if (!r.ok || uint64_t(r.end - r.p) < n || n % 4) { r.ok = false; return; }
    wire::reader inner {r.p, r.p + n};
    while (inner.ok && inner.p < inner.end) v.push_back(wire::as_float(inner.fixed32()));
    r.p += n;
  };
  while (r.ok && r.p < r.end)
  {
    const uint64_t key = r.varint();
    if (!r.ok) break;
    const int field = int(key >> 3), type = int(key & 7);
    auto expect = [&](int wanted) { if (type != wanted) r.ok = false; return r.ok; };
    switch (field)
    {
    case 1:  if (expect(2)) string_field(out.mode); break;
    case 2:  if (expect(2)) string_field(out.volume_type); break;
    case 3:  if (expect(2)) string_field(out.dataset_filepath); break;
    case 4:  int32s(type, out.seed_generation_stride); break;
    case 5:  if (expect(0)) out.seed_generation_iterations = int32_t(r.varint()); break;
    case 6:  if (expect(2)) string_field(out.particle_tracing_integrator); break;
    case 7:  if (expect(5)) out.particle_tracing_step_size = wire::as_float(r.fixed32()); break;
    case 8:  if (expect(0)) out.particle_tracing_load_balance = r.varint() != 0; break;
    case 9:  if (expect(2)) string_field(out.color_generation_mode); break;
    case 10: if (expect(5)) out.color_generation_free_parameter = wire::as_float(r.fixed32()); break;
    case 11: floats(type, out.raytracing_camera_position); break;
    case 12: floats(type, out.raytracing_camera_forward); break;
    case 13: floats(type, out.raytracing_camera_up); break;
    case 14: int32s(type, out.raytracing_image_size); break;
    case 15: if (expect(5)) out.raytracing_streamline_radius = wire::as_float(r.fixed32()); break;
    case 16: if (expect(0)) out.raytracing_iterations = int32_t(r.varint()); break;
    default: r.skip(type); break;
    }
  }
  if (!r.ok) { error = "malformed settings message"; return false; }
  return true;
}
}
