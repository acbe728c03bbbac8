// Field files: the counterpart of pa::data_io (pa/source/stages/data_io.cpp)
// for a raw binary container, since HDF5 is not part of this library.
//
// A "pars raw" file holds one dataset: a 64-byte header (magic "PARSRAW1",
// uint32 components -- 3 for a vector field like the reference's "vectors"
// dataset, 1 for a scalar field like its volume datasets --, uint32 0, int64
// shape[3], float spacing[3] -- the file's "spacing" attribute --, zero
// padding) followed by FP32 data [shape0][shape1][shape2][components], little
// endian, z fastest: the layout data_io's hyperslab reads return
// (data_io.cpp:76-81, 90-106).
//
// Loading a rank's block follows load_vector_field / load_scalar_field: the
// partitioner's ghosted block is read, the spacing is divided by its maximum
// (data_io.cpp:108-111), offset = voxel offset x spacing, size = block size
// x spacing (:113-114).  A vector block streams from the file through two
// pinned staging buffers into device memory (reads of one chunk overlap the
// copy of the previous one), then packs to the float4 field layout on the GPU.
// save_ftle writes one rank's FTLE block into a file of the whole domain
// (save_ftle_field, data_io.cpp:117-140), creating it when missing.
#include "context.hpp"

#include <cerrno>
#include <cstdio>
#include <cstring>
#include <fcntl.h>
#include <string>
#include <sys/stat.h>
#include <unistd.h>

namespace pars
{
namespace
{
constexpr char        raw_magic[8] = {'P', 'A', 'R', 'S', 'R', 'A', 'W', '1'};
constexpr std::size_t raw_header = 64;
constexpr std::size_t chunk_bytes = std::size_t(64) << 20;

struct raw_info
{
  uint32_t components = 0;
  int64_t  shape[3] = {0, 0, 0};
  float    spacing[3] = {1, 1, 1};
};

struct file_handle
{
  int fd = -1;
  ~file_handle() { if (fd >= 0) ::close(fd); }
};

void read_exact(int fd, void* out, std::size_t bytes, uint64_t offset)
{
  auto* p = static_cast<char*>(out);
  while (bytes)
  {
    const ssize_t n = ::pread(fd, p, bytes, off_t(offset));
    if (n < 0 && errno == EINTR) continue;
    if (n <= 0) throw error(PARS_ERR_INVALID_ARGUMENT, "field file is shorter than its header says");
    p += n;
    bytes -= std::size_t(n);
    offset += uint64_t(n);
  }
}

void write_exact(int fd, const void* in, std::size_t bytes, uint64_t offset)
{
  auto* p = static_cast<const char*>(in);
  while (bytes)
  {
    const ssize_t n = ::pwrite(fd, p, bytes, off_t(offset));
    if (n < 0 && errno == EINTR) continue;
    if (n <= 0) throw error(PARS_ERR_INVALID_ARGUMENT, std::string("writing the field file failed: ") + std::strerror(errno));
    p += n;
    bytes -= std::size_t(n);
    offset += uint64_t(n);
  }
}

void open_file(file_handle& f, const char* path, int flags)
{
  PARS_REQUIRE(path, "path is required");
  f.fd = ::open(path, flags, 0644);
  if (f.fd < 0)
    throw error(errno == ENOENT ? PARS_ERR_NOT_FOUND : PARS_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path + ": " + std::strerror(errno));
}

raw_info read_header(int fd)
{
  unsigned char h[raw_header];
  read_exact(fd, h, raw_header, 0);
  PARS_REQUIRE(std::memcmp(h, raw_magic, 8) == 0, "not a pars raw field file");
  raw_info info;
  std::memcpy(&info.components, h + 8, 4);
  std::memcpy(info.shape, h + 16, 24);
  std::memcpy(info.spacing, h + 40, 12);
  PARS_REQUIRE(info.components == 1 || info.components == 3, "field files hold 1 or 3 components");
  for (int i = 0; i < 3; ++i)
  {
    PARS_REQUIRE(info.shape[i] >= 1 && info.shape[i] < (1LL << 31), "field file shape out of range");
    PARS_REQUIRE(info.spacing[i] > 0.0f, "field file spacing must be positive");
  }
  // each extent is below 2^31, so the first product fits; the second must be checked
  const uint64_t plane = uint64_t(info.shape[0]) * uint64_t(info.shape[1]);
  PARS_REQUIRE(uint64_t(info.shape[2]) <= (uint64_t(1) << 58) / plane, "field file shape out of range");
  struct stat st {};
  PARS_REQUIRE(::fstat(fd, &st) == 0, "cannot stat the field file");
  const uint64_t need = raw_header + plane * uint64_t(info.shape[2]) * info.components * 4;
  PARS_REQUIRE(uint64_t(st.st_size) >= need, "field file is shorter than its header says");
  return info;
}

void write_header(int fd, const raw_info& info)
{
  unsigned char h[raw_header] = {};
  std::memcpy(h, raw_magic, 8);
  std::memcpy(h + 8, &info.components, 4);
  std::memcpy(h + 16, info.shape, 24);
  std::memcpy(h + 40, info.spacing, 12);
  write_exact(fd, h, raw_header, 0);
}

// The rank's ghosted block as data_io reads it, with its placement.
struct block_geometry
{
  pars_partition_info part;
  int32_t             offset[3], extent[3];   // voxels: first, count (ghosted)
  float               spacing[3], origin[3], size[3];
};

block_geometry block_of(const raw_info& info, int32_t ranks, int32_t rank)
{
  PARS_REQUIRE(ranks >= 1 && rank >= 0 && rank < ranks, "rank out of range");
  const int32_t domain[3] = {int32_t(info.shape[0]), int32_t(info.shape[1]), int32_t(info.shape[2])};
  block_geometry g {};
  const int32_t status = pars_gpu_partition(ranks, rank, domain, &g.part);
  if (status != PARS_OK) throw error(status, "partition failed");
  float largest = info.spacing[0];
  for (int i = 1; i < 3; ++i) largest = std::max(largest, info.spacing[i]);
  for (int i = 0; i < 3; ++i)
  {
    g.offset[i] = g.part.offset[i];
    g.extent[i] = g.part.ghosted_block_size[i];
    PARS_REQUIRE(g.offset[i] + g.extent[i] <= domain[i], "block exceeds the dataset");
    g.spacing[i] = info.spacing[i] / largest;                     // data_io.cpp:110-111
    g.origin[i] = float(g.part.offset[i]) * g.spacing[i];         // :113
    g.size[i] = float(g.part.block_size[i]) * g.spacing[i];       // :114
  }
  return g;
}

// Calls sink(x, y, data, floats) for each (x, y) run of the block along z, in
// order, reading runs that are contiguous in the file together.
template <typename sink_type>
void read_block(int fd, const raw_info& info, const int32_t offset[3], const int32_t extent[3], char* staging,
                std::size_t staging_bytes, sink_type&& sink)
{
  const uint64_t nc = info.components;
  const uint64_t run = uint64_t(extent[2]) * nc * 4;                       // bytes of one z-run
  const bool full_rows = extent[2] == info.shape[2];
  PARS_REQUIRE(run <= staging_bytes, "a z-run of the block exceeds the staging buffer");
  for (int64_t x = 0; x < extent[0]; ++x)
  {
    int64_t y = 0;
    while (y < extent[1])
    {
      // runs that follow each other in the file: whole rows (and whole planes)
      int64_t rows = 1;
      if (full_rows)
      {
        rows = std::min<int64_t>(extent[1] - y, int64_t(staging_bytes / run));
        if (rows < 1) rows = 1;
      }
      const uint64_t first = raw_header + (((uint64_t(offset[0]) + x) * info.shape[1] + uint64_t(offset[1]) + y) * info.shape[2] +
                                           uint64_t(offset[2])) * nc * 4;
      read_exact(fd, staging, std::size_t(run * rows), first);
      sink(x, y, staging, std::size_t(rows * extent[2] * nc));
      y += rows;
    }
  }
}
}  // namespace
}  // namespace pars

using pars::error;

#pragma GCC visibility push(default)
extern "C" {

int32_t pars_gpu_raw_info(const char* path, int32_t* components, int64_t shape[3], float spacing[3])
{
  try
  {
    pars::file_handle f;
    pars::open_file(f, path, O_RDONLY);
    const auto info = pars::read_header(f.fd);
    if (components) *components = int32_t(info.components);
    for (int i = 0; i < 3; ++i)
    {
      if (shape) shape[i] = info.shape[i];
      if (spacing) spacing[i] = info.spacing[i];
    }
    return PARS_OK;
  }
  catch (const error& e) { return e.status; }
  catch (...) { return PARS_ERR_STATE; }
}

int32_t pars_gpu_raw_write(const char* path, int32_t components, const int64_t shape[3], const float spacing[3], const float* data)
{
  try
  {
    PARS_REQUIRE((components == 1 || components == 3) && shape && spacing && data, "components, shape, spacing and data are required");
    pars::raw_info info;
    info.components = uint32_t(components);
    for (int i = 0; i < 3; ++i)
    {
      PARS_REQUIRE(shape[i] >= 1 && shape[i] < (1LL << 31) && spacing[i] > 0.0f, "shape or spacing out of range");
      info.shape[i] = shape[i];
      info.spacing[i] = spacing[i];
    }
    const uint64_t plane = uint64_t(shape[0]) * uint64_t(shape[1]);
    PARS_REQUIRE(uint64_t(shape[2]) <= (uint64_t(1) << 58) / plane, "shape out of range");
    pars::file_handle f;
    pars::open_file(f, path, O_WRONLY | O_CREAT | O_TRUNC);
    pars::write_header(f.fd, info);
    pars::write_exact(f.fd, data, std::size_t(plane * uint64_t(shape[2]) * uint64_t(components)) * 4, pars::raw_header);
    return PARS_OK;
  }
  catch (const error& e) { return e.status; }
  catch (...) { return PARS_ERR_STATE; }
}

int32_t pars_gpu_scalar_load(const char* path, int32_t ranks, int32_t rank, float* values, int32_t shape[3], float offset[3],
                             float spacing[3], float size[3])
{
  try
  {
    pars::file_handle f;
    pars::open_file(f, path, O_RDONLY);
    const auto info = pars::read_header(f.fd);
    PARS_REQUIRE(info.components == 1, "not a scalar field file");
    const auto g = pars::block_of(info, ranks, rank);
    for (int i = 0; i < 3; ++i)
    {
      if (shape) shape[i] = g.extent[i];
      if (offset) offset[i] = g.origin[i];
      if (spacing) spacing[i] = g.spacing[i];
      if (size) size[i] = g.size[i];
    }
    if (!values) return PARS_OK;
    const std::size_t staging = std::max<std::size_t>(pars::chunk_bytes, std::size_t(g.extent[2]) * 4);
    std::vector<char> buffer(staging);
    pars::read_block(f.fd, info, g.offset, g.extent, buffer.data(), staging,
                     [&](int64_t x, int64_t y, const char* data, std::size_t floats) {
                       std::memcpy(values + (uint64_t(x) * g.extent[1] + uint64_t(y)) * g.extent[2], data, floats * 4);
                     });
    return PARS_OK;
  }
  catch (const error& e) { return e.status; }
  catch (const std::bad_alloc&) { return PARS_ERR_OUT_OF_MEMORY; }
  catch (...) { return PARS_ERR_STATE; }
}

int32_t pars_gpu_field_load(pars_gpu_context* ctx, const char* path, int32_t ranks, int32_t rank, int32_t* field,
                            pars_partition_info* partition)
{
  if (!ctx || !field) return PARS_ERR_INVALID_ARGUMENT;
  char* pinned[2] = {nullptr, nullptr};
  cudaEvent_t copied[2] = {nullptr, nullptr};
  cudaStream_t stream = nullptr;
  float* device_xyz = nullptr;
  int32_t status = PARS_OK;
  try
  {
    pars::file_handle f;
    pars::open_file(f, path, O_RDONLY);
    const auto info = pars::read_header(f.fd);
    PARS_REQUIRE(info.components == 3, "not a vector field file");
    const auto g = pars::block_of(info, ranks, rank);
    for (int i = 0; i < 3; ++i) PARS_REQUIRE(g.extent[i] >= 2, "every block extent must be >= 2");
    if (partition) *partition = g.part;
    PARS_CUDA(cudaSetDevice(ctx->device));
    const uint64_t floats = uint64_t(g.extent[0]) * g.extent[1] * g.extent[2] * 3;
    PARS_CUDA(cudaMalloc(&device_xyz, floats * 4));
    PARS_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    const std::size_t staging = std::max<std::size_t>(pars::chunk_bytes, std::size_t(g.extent[2]) * 12);
    for (int b = 0; b < 2; ++b)
    {
      PARS_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&pinned[b]), staging, cudaHostAllocDefault));
      PARS_CUDA(cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming));
      PARS_CUDA(cudaEventRecord(copied[b], stream));
    }
    // Reads alternate between the two staging buffers: a buffer is refilled
    // only after its previous copy to the device has finished.
    int which = 0;
    char* chunk_start = pinned[0];
    uint64_t chunk_dst = 0, chunk_fill = 0;
    auto flush = [&] {
      if (!chunk_fill) return;
      PARS_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(device_xyz) + chunk_dst, chunk_start, chunk_fill, cudaMemcpyHostToDevice, stream));
      PARS_CUDA(cudaEventRecord(copied[which], stream));
      which ^= 1;
      PARS_CUDA(cudaEventSynchronize(copied[which]));
      chunk_start = pinned[which];
      chunk_dst += chunk_fill;
      chunk_fill = 0;
    };
    // runs arrive in device order; gather them into the current buffer
    std::vector<char> run_buffer(staging);
    pars::read_block(f.fd, info, g.offset, g.extent, run_buffer.data(), staging,
                     [&](int64_t, int64_t, const char* data, std::size_t n) {
                       const uint64_t bytes = uint64_t(n) * 4;
                       if (chunk_fill + bytes > staging) flush();
                       std::memcpy(chunk_start + chunk_fill, data, bytes);
                       chunk_fill += bytes;
                     });
    flush();
    PARS_CUDA(cudaStreamSynchronize(stream));
    const int32_t shape[3] = {g.extent[0], g.extent[1], g.extent[2]};
    status = pars_gpu_field_upload_device(ctx, device_xyz, shape, g.origin, g.size, g.spacing, field);
  }
  catch (const error& e) { status = e.status; }
  catch (const std::bad_alloc&) { status = PARS_ERR_OUT_OF_MEMORY; }
  catch (...) { status = PARS_ERR_STATE; }
  if (stream) cudaStreamSynchronize(stream);
  for (int b = 0; b < 2; ++b)
  {
    if (pinned[b]) cudaFreeHost(pinned[b]);
    if (copied[b]) cudaEventDestroy(copied[b]);
  }
  if (stream) cudaStreamDestroy(stream);
  if (device_xyz) cudaFree(device_xyz);
  return status;
}

int32_t pars_gpu_ftle_save(const char* path, const int32_t domain[3], const int32_t offset[3], const int32_t shape[3],
                           const float* values, const float spacing[3])
{
  try
  {
    PARS_REQUIRE(domain && offset && shape && values, "domain, offset, shape and values are required");
    for (int i = 0; i < 3; ++i)
      PARS_REQUIRE(domain[i] >= 1 && offset[i] >= 0 && shape[i] >= 1 && offset[i] + shape[i] <= domain[i], "block outside the domain");
    pars::file_handle f;
    struct stat st {};
    const bool exists = ::stat(path ? path : "", &st) == 0;
    pars::open_file(f, path, O_RDWR | O_CREAT);
    pars::raw_info info;
    if (exists && st.st_size > 0)
    {
      info = pars::read_header(f.fd);
      PARS_REQUIRE(info.components == 1 && info.shape[0] == domain[0] && info.shape[1] == domain[1] && info.shape[2] == domain[2],
                   "the existing file holds another dataset");
    }
    else
    {
      info.components = 1;
      for (int i = 0; i < 3; ++i)
      {
        info.shape[i] = domain[i];
        info.spacing[i] = spacing ? spacing[i] : 1.0f;
      }
      pars::write_header(f.fd, info);
      const uint64_t total = pars::raw_header + uint64_t(domain[0]) * domain[1] * domain[2] * 4;
      PARS_REQUIRE(::ftruncate(f.fd, off_t(total)) == 0, "cannot size the FTLE file");
    }
    for (int64_t x = 0; x < shape[0]; ++x)
      for (int64_t y = 0; y < shape[1]; ++y)
      {
        const uint64_t at = pars::raw_header + ((uint64_t(offset[0] + x) * domain[1] + uint64_t(offset[1] + y)) * domain[2] + offset[2]) * 4;
        pars::write_exact(f.fd, values + (uint64_t(x) * shape[1] + uint64_t(y)) * shape[2], std::size_t(shape[2]) * 4, at);
      }
    return PARS_OK;
  }
  catch (const error& e) { return e.status; }
  catch (...) { return PARS_ERR_STATE; }
}

}  // extern "C"
#pragma GCC visibility pop
