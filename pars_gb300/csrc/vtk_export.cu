// Polyline export of integral curves: the counterpart of
// data_io::save_integral_curves (pa/source/stages/data_io.cpp:142-196), which
// writes the curves with VTK's XML writer when the mode contains "export".
// VTK is not part of this library; the file is VTK XML PolyData (.vtp, one
// piece, raw appended data), which VTK and ParaView readers open directly.
//
// Content, as the reference assembles it: every vertex that is not the
// termination vertex becomes a point (batches in order), with its colour's
// (r, g, b) x 255 as bytes ("Colors", the point scalars); a polyline holds the
// points of one run and is emitted when a termination vertex ends a run that
// has points -- an open run carries over from one batch to the next, and a run
// that no termination vertex ends is not emitted (its points stay).  So the
// lines are consecutive ranges of the point list.  Colour bytes are rounded to
// nearest and clamped to [0, 255]; NaN (a colour the reference never writes)
// becomes 0.
#include "context.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace pars
{
namespace
{
struct polylines
{
  std::vector<float>   points;     // xyz per point
  std::vector<uint8_t> colors;     // rgb per point
  std::vector<int64_t> ends;       // one past the last point of each line
  int64_t              open = 0;   // points of the run not ended yet
};

uint8_t color_byte(float c)
{
  const float v = c * 255.0f;
  if (!(v > 0.0f)) return 0;       // also NaN
  if (v >= 255.0f) return 255;
  return uint8_t(std::floor(double(v) + 0.5));
}

void add_batch(polylines& p, const float* vertices, const float* colors, int64_t n)
{
  for (int64_t i = 0; i < n; ++i)
  {
    const float* v = vertices + 4 * i;
    if (v[0] == -2.0f && v[1] == -2.0f && v[2] == -2.0f && v[3] == 0.0f)    // termination vertex
    {
      if (p.open > 0) p.ends.push_back(int64_t(p.points.size() / 3));
      p.open = 0;
      continue;
    }
    p.points.insert(p.points.end(), {v[0], v[1], v[2]});
    const float* c = colors ? colors + 4 * i : nullptr;
    p.colors.insert(p.colors.end(), {c ? color_byte(c[0]) : uint8_t(0), c ? color_byte(c[1]) : uint8_t(0),
                                     c ? color_byte(c[2]) : uint8_t(0)});
    ++p.open;
  }
}

void write_vtp(const char* path, const polylines& p)
{
  PARS_REQUIRE(path, "path is required");
  const int64_t npoints = int64_t(p.points.size() / 3), nlines = int64_t(p.ends.size());
  const int64_t connected = nlines ? p.ends.back() : 0;
  std::vector<int64_t> connectivity(static_cast<std::size_t>(connected));
  for (int64_t i = 0; i < connected; ++i) connectivity[i] = i;
  const uint64_t sizes[4] = {uint64_t(p.colors.size()), uint64_t(p.points.size()) * 4, uint64_t(connected) * 8,
                             uint64_t(nlines) * 8};
  uint64_t offsets[4];
  uint64_t at = 0;
  for (int k = 0; k < 4; ++k) { offsets[k] = at; at += 8 + sizes[k]; }
  std::string head;
  head += "<?xml version=\"1.0\"?>\n";
  head += "<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n";
  head += "  <PolyData>\n";
  head += "    <Piece NumberOfPoints=\"" + std::to_string(npoints) + "\" NumberOfVerts=\"0\" NumberOfLines=\"" +
          std::to_string(nlines) + "\" NumberOfStrips=\"0\" NumberOfPolys=\"0\">\n";
  head += "      <PointData Scalars=\"Colors\">\n";
  head += "        <DataArray type=\"UInt8\" Name=\"Colors\" NumberOfComponents=\"3\" format=\"appended\" offset=\"" +
          std::to_string(offsets[0]) + "\"/>\n";
  head += "      </PointData>\n";
  head += "      <Points>\n";
  head += "        <DataArray type=\"Float32\" Name=\"Points\" NumberOfComponents=\"3\" format=\"appended\" offset=\"" +
          std::to_string(offsets[1]) + "\"/>\n";
  head += "      </Points>\n";
  head += "      <Lines>\n";
  head += "        <DataArray type=\"Int64\" Name=\"connectivity\" format=\"appended\" offset=\"" + std::to_string(offsets[2]) + "\"/>\n";
  head += "        <DataArray type=\"Int64\" Name=\"offsets\" format=\"appended\" offset=\"" + std::to_string(offsets[3]) + "\"/>\n";
  head += "      </Lines>\n";
  head += "    </Piece>\n";
  head += "  </PolyData>\n";
  head += "  <AppendedData encoding=\"raw\">\n   _";
  std::FILE* f = std::fopen(path, "wb");
  if (!f) throw error(PARS_ERR_INVALID_ARGUMENT, std::string("cannot create ") + path);
  bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
  const void* data[4] = {p.colors.data(), p.points.data(), connectivity.data(), p.ends.data()};
  for (int k = 0; k < 4 && ok; ++k)
  {
    ok = std::fwrite(&sizes[k], 8, 1, f) == 1;
    if (ok && sizes[k]) ok = std::fwrite(data[k], 1, std::size_t(sizes[k]), f) == sizes[k];
  }
  const char tail[] = "\n  </AppendedData>\n</VTKFile>\n";
  ok = ok && std::fwrite(tail, 1, sizeof(tail) - 1, f) == sizeof(tail) - 1;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) throw error(PARS_ERR_INVALID_ARGUMENT, std::string("writing ") + path + " failed");
}
}  // namespace
}  // namespace pars

using pars::error;

#pragma GCC visibility push(default)
extern "C" {

int32_t pars_gpu_export_vtk(const char* path, int64_t batches, const int64_t* vertex_counts, const float* const* vertices,
                            const float* const* colors)
{
  try
  {
    PARS_REQUIRE(batches >= 0 && (batches == 0 || (vertex_counts && vertices)), "curve arrays are required");
    pars::polylines p;
    for (int64_t b = 0; b < batches; ++b)
    {
      PARS_REQUIRE(vertex_counts[b] >= 0 && (vertex_counts[b] == 0 || vertices[b]), "vertices are required");
      pars::add_batch(p, vertices[b], colors ? colors[b] : nullptr, vertex_counts[b]);
    }
    pars::write_vtp(path, p);
    return PARS_OK;
  }
  catch (const error& e) { return e.status; }
  catch (const std::bad_alloc&) { return PARS_ERR_OUT_OF_MEMORY; }
  catch (...) { return PARS_ERR_STATE; }
}

int32_t pars_gpu_curves_export_vtk(pars_gpu_context* ctx, const char* path)
{
  return pars::run_guarded(ctx, [&] {
    auto& c = ctx->curves;
    pars::polylines p;
    std::vector<float> vertices, colors;
    for (const auto& b : c.batches)
    {
      vertices.resize(std::size_t(b.vertex_count) * 4);
      colors.resize(c.colored ? std::size_t(b.vertex_count) * 4 : 0);
      if (b.vertex_count)
      {
        PARS_CUDA(cudaMemcpyAsync(vertices.data(), c.vertices.as<float4>() + b.vertex_offset, sizeof(float4) * b.vertex_count,
                                  cudaMemcpyDeviceToHost, ctx->stream));
        if (c.colored)
          PARS_CUDA(cudaMemcpyAsync(colors.data(), c.colors.as<float4>() + b.vertex_offset, sizeof(float4) * b.vertex_count,
                                    cudaMemcpyDeviceToHost, ctx->stream));
        PARS_CUDA(cudaStreamSynchronize(ctx->stream));
      }
      pars::add_batch(p, vertices.data(), c.colored ? colors.data() : nullptr, b.vertex_count);
    }
    pars::write_vtp(path, p);
  });
}

}  // extern "C"
#pragma GCC visibility pop
