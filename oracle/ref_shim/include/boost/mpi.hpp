// Minimal in-process stand-in for the Boost.MPI calls of the reference hot path:
// communicator rank/size/barrier/isend/recv, request::wait, gather, broadcast,
// all_to_all and environment.  A default-constructed communicator is a world of
// one rank.  pars_shim::world(n) builds a world of n ranks that run as threads
// of one process; communicator(world, rank) is that rank's endpoint.  Messages
// are copied into per-(source, destination, tag) FIFO queues, so isend never
// blocks and request::wait has nothing to wait for; recv blocks until a
// matching message arrives (bounded: it throws after a time limit rather than
// hanging).
//
// This is test infrastructure for the oracle build only.
#ifndef PARS_SHIM_BOOST_MPI_HPP
#define PARS_SHIM_BOOST_MPI_HPP

#include <any>
#include <chrono>
#include <condition_variable>
#include <cstddef>
#include <deque>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <tuple>
#include <vector>

namespace pars_shim
{
class world
{
public:
  explicit world(int size) : size_(size) {}
  int size() const { return size_; }

  void push(int source, int destination, int tag, std::any message)
  {
    std::lock_guard<std::mutex> lock(mutex_);
    queues_[std::make_tuple(source, destination, tag)].push_back(std::move(message));
    ready_.notify_all();
  }
  std::any pop(int source, int destination, int tag)
  {
    std::unique_lock<std::mutex> lock(mutex_);
    auto key = std::make_tuple(source, destination, tag);
    const bool arrived = ready_.wait_for(lock, std::chrono::seconds(600), [&] {
      auto it = queues_.find(key);
      return it != queues_.end() && !it->second.empty();
    });
    if (!arrived) throw std::runtime_error("in-process MPI stand-in: recv timed out");
    auto& queue = queues_[key];
    std::any message = std::move(queue.front());
    queue.pop_front();
    return message;
  }
  void barrier()
  {
    std::unique_lock<std::mutex> lock(mutex_);
    const long generation = barrier_generation_;
    if (++barrier_count_ == size_)
    {
      barrier_count_ = 0;
      ++barrier_generation_;
      ready_.notify_all();
      return;
    }
    const bool released = ready_.wait_for(lock, std::chrono::seconds(600), [&] { return barrier_generation_ != generation; });
    if (!released) throw std::runtime_error("in-process MPI stand-in: barrier timed out");
  }

private:
  int                                                   size_;
  std::mutex                                            mutex_;
  std::condition_variable                               ready_;
  std::map<std::tuple<int, int, int>, std::deque<std::any>> queues_;
  int                                                   barrier_count_      = 0;
  long                                                  barrier_generation_ = 0;
};
}

namespace boost { namespace mpi {

namespace threading { enum level { single, funneled, serialized, multiple }; }

class environment
{
public:
  environment() = default;
  explicit environment(threading::level) {}
};

class request
{
public:
  void wait() {}
};

struct status {};

class communicator
{
public:
  communicator() : world_(std::make_shared<pars_shim::world>(1)), rank_(0) {}
  communicator(std::shared_ptr<pars_shim::world> world, int rank) : world_(std::move(world)), rank_(rank) {}

  int  rank   () const { return rank_; }
  int  size   () const { return world_->size(); }
  void barrier() const { world_->barrier(); }

  template <typename value_type>
  request isend(int destination, int tag, const value_type& value) const
  {
    world_->push(rank_, destination, tag, std::any(value));
    return request();
  }
  template <typename value_type>
  status recv(int source, int tag, value_type& value) const
  {
    value = std::any_cast<value_type>(world_->pop(source, rank_, tag));
    return status();
  }

private:
  std::shared_ptr<pars_shim::world> world_;
  int                               rank_;
};

namespace detail_shim { enum collective_tag { gather_tag = -101, broadcast_tag = -102, all_to_all_tag = -103 }; }

template <typename value_type>
void gather(const communicator& comm, const value_type& value, std::vector<value_type>& out, int root)
{
  if (comm.rank() != root) { comm.isend(root, detail_shim::gather_tag, value); return; }
  out.assign(comm.size(), value_type());
  for (int source = 0; source < comm.size(); ++source)
    if (source == root) out[source] = value;
    else comm.recv(source, detail_shim::gather_tag, out[source]);
}

template <typename value_type>
void broadcast(const communicator& comm, value_type& value, int root)
{
  if (comm.rank() == root)
  {
    for (int destination = 0; destination < comm.size(); ++destination)
      if (destination != root) comm.isend(destination, detail_shim::broadcast_tag, value);
    return;
  }
  comm.recv(root, detail_shim::broadcast_tag, value);
}

template <typename value_type>
void all_to_all(const communicator& comm, const std::vector<value_type>& in, std::vector<value_type>& out)
{
  out.assign(comm.size(), value_type());
  for (int destination = 0; destination < comm.size(); ++destination)
    if (destination != comm.rank()) comm.isend(destination, detail_shim::all_to_all_tag, in[destination]);
  for (int source = 0; source < comm.size(); ++source)
    if (source == comm.rank()) out[source] = in[source];
    else comm.recv(source, detail_shim::all_to_all_tag, out[source]);
}

}}

#endif
