// The request message of pars_service: proto3 `pars.settings`
// (pars/proto/settings.proto:5-27), decoded from its binary wire form without
// libprotobuf.  Unknown fields are skipped; repeated scalars are accepted both
// packed and unpacked, as the proto3 wire format requires.  Also the encoder
// and the JSON form the reference's benchmark reads (service.cpp:72-77).
#pragma once

#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
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

// ---- encoder ------------------------------------------------------------------
// The binary message as a proto3 serializer writes it: fields in number order,
// scalars equal to their default omitted, repeated scalars packed.
inline std::vector<uint8_t> encode_settings(const settings& s)
{
  std::vector<uint8_t> out;
  auto varint = [&](uint64_t v) { while (v >= 0x80) { out.push_back(uint8_t(v | 0x80)); v >>= 7; } out.push_back(uint8_t(v)); };
  auto key = [&](int field, int wire_type) { varint(uint64_t(field) << 3 | uint64_t(wire_type)); };
  auto fixed = [&](float f) { uint32_t b; std::memcpy(&b, &f, 4); for (int i = 0; i < 4; ++i) out.push_back(uint8_t(b >> (8 * i))); };
  auto string_field = [&](int field, const std::string& v) {
    if (v.empty()) return;
    key(field, 2); varint(v.size()); out.insert(out.end(), v.begin(), v.end());
  };
  auto int32_field = [&](int field, int32_t v) { if (v) { key(field, 0); varint(uint64_t(int64_t(v))); } };
  auto float_field = [&](int field, float v) {
    uint32_t b; std::memcpy(&b, &v, 4);
    if (b) { key(field, 5); fixed(v); }          // -0.0 is not the default and is written
  };
  auto int32s = [&](int field, const std::vector<int32_t>& v) {
    if (v.empty()) return;
    std::vector<uint8_t> body;
    std::swap(body, out);
    for (int32_t x : v) varint(uint64_t(int64_t(x)));
    std::swap(body, out);
    key(field, 2); varint(body.size()); out.insert(out.end(), body.begin(), body.end());
  };
  auto floats = [&](int field, const std::vector<float>& v) {
    if (v.empty()) return;
    key(field, 2); varint(4 * v.size());
    for (float x : v) fixed(x);
  };
  string_field(1, s.mode);
  string_field(2, s.volume_type);
  string_field(3, s.dataset_filepath);
  int32s(4, s.seed_generation_stride);
  int32_field(5, s.seed_generation_iterations);
  string_field(6, s.particle_tracing_integrator);
  float_field(7, s.particle_tracing_step_size);
  if (s.particle_tracing_load_balance) { key(8, 0); varint(1); }
  string_field(9, s.color_generation_mode);
  float_field(10, s.color_generation_free_parameter);
  floats(11, s.raytracing_camera_position);
  floats(12, s.raytracing_camera_forward);
  floats(13, s.raytracing_camera_up);
  int32s(14, s.raytracing_image_size);
  float_field(15, s.raytracing_streamline_radius);
  int32_field(16, s.raytracing_iterations);
  return out;
}

// ---- JSON (the benchmark's settings files, service.cpp:72-77) ---------------------
// The proto3 JSON mapping of `settings` as JsonStringToMessage reads it with
// default options: keys are the field names or their lowerCamelCase JSON names,
// unknown keys are errors, null leaves a field at its default, int32 and float
// values may be numbers or numeric strings ("NaN", "Infinity", "-Infinity" for
// floats), int32 values must be integral and in range.
namespace json
{
struct value
{
  enum kind_type { null_value, boolean, number, text, array, object } kind = null_value;
  bool                                        b = false;
  double                                      n = 0.0;
  std::string                                 s;
  std::vector<value>                          items;
  std::vector<std::pair<std::string, value>>  members;
};

struct parser
{
  const char* p;
  const char* end;
  std::string error;
  int         depth = 0;

  void space() { while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p; }
  bool fail(const char* what) { if (error.empty()) error = what; return false; }

  bool literal(const char* word)
  {
    const std::size_t n = std::strlen(word);
    if (std::size_t(end - p) < n || std::memcmp(p, word, n) != 0) return fail("invalid literal");
    p += n;
    return true;
  }

  static void utf8(std::string& out, uint32_t c)
  {
    if (c < 0x80) out.push_back(char(c));
    else if (c < 0x800) { out.push_back(char(0xC0 | (c >> 6))); out.push_back(char(0x80 | (c & 0x3F))); }
    else if (c < 0x10000) { out.push_back(char(0xE0 | (c >> 12))); out.push_back(char(0x80 | ((c >> 6) & 0x3F))); out.push_back(char(0x80 | (c & 0x3F))); }
    else { out.push_back(char(0xF0 | (c >> 18))); out.push_back(char(0x80 | ((c >> 12) & 0x3F))); out.push_back(char(0x80 | ((c >> 6) & 0x3F))); out.push_back(char(0x80 | (c & 0x3F))); }
  }

  bool hex4(uint32_t& v)
  {
    if (end - p < 4) return fail("truncated escape");
    v = 0;
    for (int i = 0; i < 4; ++i)
    {
      const char c = *p++;
      v <<= 4;
      if (c >= '0' && c <= '9') v |= uint32_t(c - '0');
      else if (c >= 'a' && c <= 'f') v |= uint32_t(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') v |= uint32_t(c - 'A' + 10);
      else return fail("invalid escape");
    }
    return true;
  }

  bool string(std::string& out)
  {
    if (p >= end || *p != '"') return fail("expected a string");
    ++p;
    while (p < end && *p != '"')
    {
      const char c = *p++;
      if (static_cast<unsigned char>(c) < 0x20) return fail("control character in a string");
      if (c != '\\') { out.push_back(c); continue; }
      if (p >= end) return fail("truncated escape");
      const char e = *p++;
      switch (e)
      {
      case '"': out.push_back('"'); break;
      case '\\': out.push_back('\\'); break;
      case '/': out.push_back('/'); break;
      case 'b': out.push_back('\b'); break;
      case 'f': out.push_back('\f'); break;
      case 'n': out.push_back('\n'); break;
      case 'r': out.push_back('\r'); break;
      case 't': out.push_back('\t'); break;
      case 'u':
      {
        uint32_t c1;
        if (!hex4(c1)) return false;
        if (c1 >= 0xD800 && c1 < 0xDC00)
        {
          uint32_t c2;
          if (end - p < 2 || p[0] != '\\' || p[1] != 'u') return fail("unpaired surrogate");
          p += 2;
          if (!hex4(c2) || c2 < 0xDC00 || c2 >= 0xE000) return fail("unpaired surrogate");
          c1 = 0x10000 + ((c1 - 0xD800) << 10) + (c2 - 0xDC00);
        }
        utf8(out, c1);
        break;
      }
      default: return fail("invalid escape");
      }
    }
    if (p >= end) return fail("unterminated string");
    ++p;
    return true;
  }

  bool number(double& out)
  {
    const char* start = p;
    if (p < end && *p == '-') ++p;
    if (p >= end || !(*p >= '0' && *p <= '9')) return fail("invalid number");
    if (*p == '0') ++p;
    else while (p < end && *p >= '0' && *p <= '9') ++p;
    if (p < end && *p == '.')
    {
      ++p;
      if (p >= end || !(*p >= '0' && *p <= '9')) return fail("invalid number");
      while (p < end && *p >= '0' && *p <= '9') ++p;
    }
    if (p < end && (*p == 'e' || *p == 'E'))
    {
      ++p;
      if (p < end && (*p == '+' || *p == '-')) ++p;
      if (p >= end || !(*p >= '0' && *p <= '9')) return fail("invalid number");
      while (p < end && *p >= '0' && *p <= '9') ++p;
    }
    out = std::strtod(std::string(start, p).c_str(), nullptr);
    return true;
  }

  bool parse(value& v)
  {
    if (++depth > 64) return fail("nested too deeply");
    space();
    if (p >= end) return fail("unexpected end");
    bool ok = true;
    switch (*p)
    {
    case '{':
    {
      v.kind = value::object;
      ++p;
      space();
      if (p < end && *p == '}') { ++p; break; }
      for (;;)
      {
        space();
        std::pair<std::string, value> m;
        if (!string(m.first)) return false;
        space();
        if (p >= end || *p != ':') return fail("expected ':'");
        ++p;
        if (!parse(m.second)) return false;
        v.members.push_back(std::move(m));
        space();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == '}') { ++p; break; }
        return fail("expected ',' or '}'");
      }
      break;
    }
    case '[':
    {
      v.kind = value::array;
      ++p;
      space();
      if (p < end && *p == ']') { ++p; break; }
      for (;;)
      {
        value item;
        if (!parse(item)) return false;
        v.items.push_back(std::move(item));
        space();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == ']') { ++p; break; }
        return fail("expected ',' or ']'");
      }
      break;
    }
    case '"': v.kind = value::text; ok = string(v.s); break;
    case 't': v.kind = value::boolean; v.b = true; ok = literal("true"); break;
    case 'f': v.kind = value::boolean; v.b = false; ok = literal("false"); break;
    case 'n': v.kind = value::null_value; ok = literal("null"); break;
    default: v.kind = value::number; ok = number(v.n); break;
    }
    --depth;
    return ok;
  }
};

inline bool to_double(const value& v, double& out)
{
  if (v.kind == value::number) { out = v.n; return true; }
  if (v.kind != value::text) return false;
  if (v.s == "NaN") { out = std::numeric_limits<double>::quiet_NaN(); return true; }
  if (v.s == "Infinity") { out = std::numeric_limits<double>::infinity(); return true; }
  if (v.s == "-Infinity") { out = -std::numeric_limits<double>::infinity(); return true; }
  json::parser q {v.s.c_str(), v.s.c_str() + v.s.size()};
  return q.number(out) && q.p == q.end;
}

inline bool to_int32(const value& v, int32_t& out)
{
  double d;
  if (!to_double(v, d) || !(d == std::floor(d)) || d < -2147483648.0 || d > 2147483647.0) return false;
  out = int32_t(d);
  return true;
}

inline bool to_float(const value& v, float& out)
{
  double d;
  if (!to_double(v, d)) return false;
  if (std::isfinite(d) && std::fabs(d) > double(std::numeric_limits<float>::max())) return false;
  out = float(d);
  return true;
}
}

// Reads the JSON form of `settings` into `out`.
inline bool settings_from_json(const char* text, std::size_t length, settings& out, std::string& error)
{
  json::parser q {text, text + length};
  json::value root;
  if (!q.parse(root)) { error = "invalid JSON: " + q.error; return false; }
  q.space();
  if (q.p != q.end) { error = "invalid JSON: trailing characters"; return false; }
  if (root.kind != json::value::object) { error = "settings JSON must be an object"; return false; }
  auto camel = [](const std::string& name) {
    std::string c;
    bool up = false;
    for (char ch : name) { if (ch == '_') { up = true; continue; } c.push_back(up ? char(std::toupper(static_cast<unsigned char>(ch))) : ch); up = false; }
    return c;
  };
  static const char* names[] = {"mode", "volume_type", "dataset_filepath", "seed_generation_stride", "seed_generation_iterations",
                                "particle_tracing_integrator", "particle_tracing_step_size", "particle_tracing_load_balance",
                                "color_generation_mode", "color_generation_free_parameter", "raytracing_camera_position",
                                "raytracing_camera_forward", "raytracing_camera_up", "raytracing_image_size",
                                "raytracing_streamline_radius", "raytracing_iterations"};
  for (const auto& m : root.members)
  {
    int field = -1;
    for (int i = 0; i < 16 && field < 0; ++i)
      if (m.first == names[i] || m.first == camel(names[i])) field = i + 1;
    if (field < 0) { error = "unknown settings field '" + m.first + "'"; return false; }
    const json::value& v = m.second;
    if (v.kind == json::value::null_value) continue;
    bool ok = true;
    auto text = [&](std::string& target) { if (v.kind != json::value::text) ok = false; else target = v.s; };
    auto int32s = [&](std::vector<int32_t>& target) {
      if (v.kind != json::value::array) { ok = false; return; }
      target.clear();
      for (const auto& item : v.items) { int32_t x; if (!json::to_int32(item, x)) { ok = false; return; } target.push_back(x); }
    };
    auto floats = [&](std::vector<float>& target) {
      if (v.kind != json::value::array) { ok = false; return; }
      target.clear();
      for (const auto& item : v.items) { float x; if (!json::to_float(item, x)) { ok = false; return; } target.push_back(x); }
    };
    switch (field)
    {
    case 1: text(out.mode); break;
    case 2: text(out.volume_type); break;
    case 3: text(out.dataset_filepath); break;
    case 4: int32s(out.seed_generation_stride); break;
    case 5: ok = json::to_int32(v, out.seed_generation_iterations); break;
    case 6: text(out.particle_tracing_integrator); break;
    case 7: ok = json::to_float(v, out.particle_tracing_step_size); break;
    case 8:
      if (v.kind == json::value::boolean) out.particle_tracing_load_balance = v.b;
      else if (v.kind == json::value::text && (v.s == "true" || v.s == "false")) out.particle_tracing_load_balance = v.s == "true";
      else ok = false;
      break;
    case 9: text(out.color_generation_mode); break;
    case 10: ok = json::to_float(v, out.color_generation_free_parameter); break;
    case 11: floats(out.raytracing_camera_position); break;
    case 12: floats(out.raytracing_camera_forward); break;
    case 13: floats(out.raytracing_camera_up); break;
    case 14: int32s(out.raytracing_image_size); break;
    case 15: ok = json::to_float(v, out.raytracing_streamline_radius); break;
    case 16: ok = json::to_int32(v, out.raytracing_iterations); break;
    }
    if (!ok) { error = "invalid value for settings field '" + m.first + "'"; return false; }
  }
  return true;
}
}
