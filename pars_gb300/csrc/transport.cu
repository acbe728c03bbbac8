// The service's transport: pars_service's ZeroMQ PAIR socket
// (pars/source/service.cpp:20-69), spoken without libzmq.
//
// The reference binds a PAIR socket, receives one binary `settings` message
// at a time, runs the pipeline and sends back the serialised `image`.  Here a
// TCP listener accepts one peer at a time and speaks ZMTP 3.0 (ZeroMQ RFC 23)
// with the NULL security mechanism as a PAIR socket:
//   greeting   10-octet signature (0xFF, 8 x 0x00, 0x7F), version 3.0, the
//              mechanism name "NULL" padded to 20 octets, as-server, 31
//              octets of filler — 64 octets each way, ours sent first;
//   handshake  each side sends a READY command whose metadata names its
//              socket type ("Socket-Type" = "PAIR"); the peer's must be PAIR;
//   traffic    frames: a flags octet (bit 0 more frames follow, bit 1 the
//              size is 8 octets big-endian rather than 1, bit 2 command),
//              the size, the body; a message is its frames up to the first
//              without "more".  PING commands (ZMTP 3.1 peers) get a PONG
//              carrying the ping's context; other commands are ignored.
// Each received message is submitted to the service as a request, and the
// reply is the request's `image` message (pars_gpu_image_encode; width and
// height 0 when the request produced no image or failed), as the reference
// replies with ray_tracer::serialize for every request.
//
// Host code only (POSIX sockets); no CUDA call of its own.
#include <arpa/inet.h>
#include <netinet/in.h>
#include <netinet/tcp.h>
#include <strings.h>
#include <sys/socket.h>
#include <unistd.h>

#include <cerrno>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pars_gpu.h"

namespace
{
struct transport_error
{
  int32_t     status;
  std::string message;
};

void write_all(int fd, const uint8_t* data, std::size_t n)
{
  while (n > 0)
  {
    const ssize_t k = ::send(fd, data, n, MSG_NOSIGNAL);
    if (k < 0 && errno == EINTR) continue;
    if (k <= 0) throw transport_error{PARS_ERR_STATE, "send failed: " + std::string(std::strerror(errno))};
    data += k;
    n -= std::size_t(k);
  }
}

// Reads exactly n octets; false when the peer closed before the first one.
bool read_all(int fd, uint8_t* data, std::size_t n)
{
  std::size_t got = 0;
  while (got < n)
  {
    const ssize_t k = ::recv(fd, data + got, n - got, 0);
    if (k < 0 && errno == EINTR) continue;
    if (k == 0 && got == 0) return false;
    if (k <= 0) throw transport_error{PARS_ERR_STATE, "connection lost in the middle of a frame"};
    got += std::size_t(k);
  }
  return true;
}

void send_frame(int fd, uint8_t flags, const uint8_t* body, std::size_t n)
{
  std::vector<uint8_t> head;
  if (n <= 255) { head = {flags, uint8_t(n)}; }
  else
  {
    head.push_back(uint8_t(flags | 0x02));
    for (int i = 7; i >= 0; --i) head.push_back(uint8_t(uint64_t(n) >> (8 * i)));
  }
  write_all(fd, head.data(), head.size());
  if (n) write_all(fd, body, n);
}

// One frame: its flags and body; false when the peer closed between frames.
bool read_frame(int fd, uint8_t& flags, std::vector<uint8_t>& body)
{
  if (!read_all(fd, &flags, 1)) return false;
  uint64_t n = 0;
  if (flags & 0x02)
  {
    uint8_t s[8];
    if (!read_all(fd, s, 8)) throw transport_error{PARS_ERR_STATE, "connection lost in a frame header"};
    for (int i = 0; i < 8; ++i) n = (n << 8) | s[i];
  }
  else
  {
    uint8_t s;
    if (!read_all(fd, &s, 1)) throw transport_error{PARS_ERR_STATE, "connection lost in a frame header"};
    n = s;
  }
  if (n > (uint64_t(1) << 32)) throw transport_error{PARS_ERR_INVALID_ARGUMENT, "frame larger than 4 GiB"};
  body.resize(std::size_t(n));
  if (n && !read_all(fd, body.data(), std::size_t(n))) throw transport_error{PARS_ERR_STATE, "connection lost in a frame body"};
  return true;
}

void send_command(int fd, const std::string& name, const std::vector<uint8_t>& data)
{
  std::vector<uint8_t> body;
  body.push_back(uint8_t(name.size()));
  body.insert(body.end(), name.begin(), name.end());
  body.insert(body.end(), data.begin(), data.end());
  send_frame(fd, 0x04, body.data(), body.size());
}

// READY metadata: name (1-octet length) and value (4-octet big-endian length).
std::vector<uint8_t> property(const std::string& name, const std::string& value)
{
  std::vector<uint8_t> out;
  out.push_back(uint8_t(name.size()));
  out.insert(out.end(), name.begin(), name.end());
  const uint32_t n = uint32_t(value.size());
  for (int i = 3; i >= 0; --i) out.push_back(uint8_t(n >> (8 * i)));
  out.insert(out.end(), value.begin(), value.end());
  return out;
}

// The value of a READY property, or "" when absent.
std::string ready_property(const std::vector<uint8_t>& body, std::size_t at, const std::string& wanted)
{
  while (at < body.size())
  {
    const std::size_t name_length = body[at++];
    if (at + name_length + 4 > body.size()) break;
    const std::string name(body.begin() + long(at), body.begin() + long(at + name_length));
    at += name_length;
    const uint32_t value_length = (uint32_t(body[at]) << 24) | (uint32_t(body[at + 1]) << 16) | (uint32_t(body[at + 2]) << 8) | body[at + 3];
    at += 4;
    if (at + value_length > body.size()) break;
    if (name.size() == wanted.size() && strncasecmp(name.c_str(), wanted.c_str(), name.size()) == 0)
      return std::string(body.begin() + long(at), body.begin() + long(at + value_length));
    at += value_length;
  }
  return "";
}

void greet(int fd)
{
  uint8_t ours[64] = {0xFF, 0, 0, 0, 0, 0, 0, 0, 0, 0x7F, 3, 0, 'N', 'U', 'L', 'L'};
  ours[32] = 1;   // as-server
  write_all(fd, ours, sizeof(ours));
  uint8_t theirs[64];
  if (!read_all(fd, theirs, sizeof(theirs))) throw transport_error{PARS_ERR_STATE, "the peer closed during the greeting"};
  if (theirs[0] != 0xFF || theirs[9] != 0x7F) throw transport_error{PARS_ERR_INVALID_ARGUMENT, "not a ZMTP peer (signature)"};
  if (theirs[10] < 3) throw transport_error{PARS_ERR_UNSUPPORTED, "ZMTP version below 3"};
  if (std::memcmp(theirs + 12, "NULL", 4) != 0 || theirs[16] != 0)
    throw transport_error{PARS_ERR_UNSUPPORTED, "only the NULL security mechanism is supported"};
  send_command(fd, "READY", property("Socket-Type", "PAIR"));
  uint8_t flags = 0;
  std::vector<uint8_t> body;
  if (!read_frame(fd, flags, body)) throw transport_error{PARS_ERR_STATE, "the peer closed during the handshake"};
  if (!(flags & 0x04) || body.size() < 6 || body[0] != 5 || std::memcmp(body.data() + 1, "READY", 5) != 0)
    throw transport_error{PARS_ERR_INVALID_ARGUMENT, "expected the peer's READY command"};
  const std::string type = ready_property(body, 6, "Socket-Type");
  if (type != "PAIR") throw transport_error{PARS_ERR_INVALID_ARGUMENT, "the peer is a " + type + " socket, not PAIR"};
}

// The next message (its frames' bodies joined); false when the peer closed.
bool read_message(int fd, std::vector<uint8_t>& message)
{
  message.clear();
  for (;;)
  {
    uint8_t flags = 0;
    std::vector<uint8_t> body;
    if (!read_frame(fd, flags, body))
    {
      if (message.empty()) return false;
      throw transport_error{PARS_ERR_STATE, "connection lost in the middle of a message"};
    }
    if (flags & 0x04)
    {
      // PING (ZMTP 3.1): 2-octet TTL, then a context that the PONG echoes
      if (body.size() >= 7 && body[0] == 4 && std::memcmp(body.data() + 1, "PING", 4) == 0)
        send_command(fd, "PONG", std::vector<uint8_t>(body.begin() + 7, body.end()));
      continue;
    }
    message.insert(message.end(), body.begin(), body.end());
    if (!(flags & 0x01)) return true;
  }
}

// The service's reply to one request: its `image` message.
std::vector<uint8_t> reply_for(pars_gpu_service* service, const std::vector<uint8_t>& request)
{
  int32_t size[2] = {0, 0};
  std::vector<uint8_t> rgba;
  int64_t ticket = 0;
  if (pars_gpu_service_submit(service, request.data(), int64_t(request.size()), &ticket) == PARS_OK)
  {
    int32_t state = 0;
    if (pars_gpu_service_wait(service, ticket, -1, &state) == PARS_OK &&
        pars_gpu_service_result_image(service, ticket, nullptr, size) == PARS_OK && size[0] > 0 && size[1] > 0)
    {
      rgba.resize(std::size_t(size[0]) * std::size_t(size[1]) * 4);
      if (pars_gpu_service_result_image(service, ticket, rgba.data(), size) != PARS_OK) { rgba.clear(); size[0] = size[1] = 0; }
    }
    else size[0] = size[1] = 0;
    pars_gpu_service_release(service, ticket);
  }
  int64_t length = 0;
  if (pars_gpu_image_encode(size, rgba.data(), int64_t(rgba.size()), nullptr, 0, &length) != PARS_OK)
    throw transport_error{PARS_ERR_STATE, "image encoding failed"};
  std::vector<uint8_t> out(static_cast<std::size_t>(length));
  if (pars_gpu_image_encode(size, rgba.data(), int64_t(rgba.size()), out.data(), length, &length) != PARS_OK)
    throw transport_error{PARS_ERR_STATE, "image encoding failed"};
  return out;
}
}

#pragma GCC visibility push(default)
extern "C" {

int32_t pars_gpu_transport_listen(const char* address, int32_t port, int32_t* bound_port, int64_t* listener)
{
  if (!address || !listener || port < 0 || port > 65535) return PARS_ERR_INVALID_ARGUMENT;
  sockaddr_in a {};
  a.sin_family = AF_INET;
  a.sin_port = htons(uint16_t(port));
  if (inet_pton(AF_INET, address, &a.sin_addr) != 1) return PARS_ERR_INVALID_ARGUMENT;
  const int fd = ::socket(AF_INET, SOCK_STREAM, 0);
  if (fd < 0) return PARS_ERR_STATE;
  const int on = 1;
  ::setsockopt(fd, SOL_SOCKET, SO_REUSEADDR, &on, sizeof(on));
  if (::bind(fd, reinterpret_cast<sockaddr*>(&a), sizeof(a)) != 0 || ::listen(fd, 4) != 0) { ::close(fd); return PARS_ERR_STATE; }
  if (bound_port)
  {
    socklen_t n = sizeof(a);
    ::getsockname(fd, reinterpret_cast<sockaddr*>(&a), &n);
    *bound_port = ntohs(a.sin_port);
  }
  *listener = fd;
  return PARS_OK;
}

int32_t pars_gpu_transport_close(int64_t listener)
{
  if (listener < 0) return PARS_ERR_INVALID_ARGUMENT;
  return ::close(int(listener)) == 0 ? PARS_OK : PARS_ERR_STATE;
}

int32_t pars_gpu_service_serve(pars_gpu_service* service, int64_t listener, int64_t max_requests, int64_t* served)
{
  if (!service || listener < 0) return PARS_ERR_INVALID_ARGUMENT;
  int64_t count = 0;
  if (served) *served = 0;
  const int fd = ::accept(int(listener), nullptr, nullptr);
  if (fd < 0) return PARS_ERR_STATE;
  const int on = 1;
  ::setsockopt(fd, IPPROTO_TCP, TCP_NODELAY, &on, sizeof(on));
  int32_t status = PARS_OK;
  try
  {
    greet(fd);
    std::vector<uint8_t> request;
    while ((max_requests <= 0 || count < max_requests) && read_message(fd, request))
    {
      const std::vector<uint8_t> reply = reply_for(service, request);
      send_frame(fd, 0x00, reply.data(), reply.size());
      ++count;
      if (served) *served = count;
    }
  }
  catch (const transport_error& e) { status = e.status; }
  ::close(fd);
  return status;
}

}
#pragma GCC visibility pop
