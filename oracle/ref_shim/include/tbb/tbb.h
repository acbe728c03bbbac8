// Minimal stand-in for the parts of Intel TBB 2019 that the reference hot path
// uses: parallel_for over an index range or a blocked_range3d, blocked_range3d,
// concurrent_hash_map with a locking accessor, mutex with scoped_lock and
// task_scheduler_init.  Work is spread over OpenMP threads.  When several
// threads run as in-process MPI ranks, pars_shim::set_serial(true) makes every
// parallel_for on that thread run serially so the ranks do not oversubscribe
// the host.
//
// This is test infrastructure for the oracle build only.
#ifndef PARS_SHIM_TBB_H
#define PARS_SHIM_TBB_H

#include <cstddef>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <utility>

namespace pars_shim
{
inline bool& serial_flag() { static thread_local bool flag = false; return flag; }
inline void  set_serial(bool value) { serial_flag() = value; }
inline bool  serial() { return serial_flag(); }
}

namespace tbb
{
template <typename value_type>
class blocked_range
{
public:
  blocked_range() = default;
  blocked_range(value_type begin, value_type end) : begin_(begin), end_(end) {}
  value_type begin() const { return begin_; }
  value_type end  () const { return end_;   }
  value_type size () const { return end_ - begin_; }
  bool       empty() const { return !(begin_ < end_); }
private:
  value_type begin_ {};
  value_type end_   {};
};

template <typename value_type>
class blocked_range3d
{
public:
  blocked_range3d(value_type page_begin, value_type page_end,
                  value_type row_begin , value_type row_end ,
                  value_type col_begin , value_type col_end )
  : pages_(page_begin, page_end), rows_(row_begin, row_end), cols_(col_begin, col_end) {}
  blocked_range3d(const blocked_range<value_type>& pages, const blocked_range<value_type>& rows, const blocked_range<value_type>& cols)
  : pages_(pages), rows_(rows), cols_(cols) {}
  const blocked_range<value_type>& pages() const { return pages_; }
  const blocked_range<value_type>& rows () const { return rows_;  }
  const blocked_range<value_type>& cols () const { return cols_;  }
private:
  blocked_range<value_type> pages_, rows_, cols_;
};

// parallel_for(first, last, step, body): body(index) for index in [first, last) by step.
template <typename index_type, typename function_type>
void parallel_for(index_type first, index_type last, index_type step, const function_type& body)
{
  if (!(first < last)) return;
  const long long count = static_cast<long long>((last - first + step - 1) / step);
  if (pars_shim::serial())
  {
    for (long long k = 0; k < count; ++k) body(static_cast<index_type>(first + static_cast<index_type>(k) * step));
    return;
  }
  #pragma omp parallel for schedule(dynamic, 16)
  for (long long k = 0; k < count; ++k)
    body(static_cast<index_type>(first + static_cast<index_type>(k) * step));
}

// parallel_for(range3d, body): the page (outermost) axis is split into chunks.
template <typename value_type, typename function_type>
void parallel_for(const blocked_range3d<value_type>& range, const function_type& body)
{
  const value_type p0 = range.pages().begin(), p1 = range.pages().end();
  if (!(p0 < p1)) return;
  const long long count = static_cast<long long>(p1 - p0);
  if (pars_shim::serial())
  {
    body(range);
    return;
  }
  #pragma omp parallel for schedule(dynamic, 1)
  for (long long k = 0; k < count; ++k)
  {
    const value_type page = static_cast<value_type>(p0 + static_cast<value_type>(k));
    body(blocked_range3d<value_type>(blocked_range<value_type>(page, page + 1), range.rows(), range.cols()));
  }
}

class mutex
{
public:
  class scoped_lock
  {
  public:
    explicit scoped_lock(mutex& m) : lock_(m.mutex_) {}
  private:
    std::unique_lock<std::mutex> lock_;
  };
private:
  std::mutex mutex_;
};

// Ordered map guarded by one mutex; an accessor holds the lock while it is alive.
template <typename key_type, typename mapped_type>
class concurrent_hash_map
{
public:
  using map_type   = std::map<key_type, mapped_type>;
  using value_type = typename map_type::value_type;

  class accessor
  {
  public:
    value_type* operator->() const { return item_; }
    value_type& operator* () const { return *item_; }
    void        release   ()       { item_ = nullptr; if (lock_.owns_lock()) lock_.unlock(); }
  private:
    friend class concurrent_hash_map;
    std::unique_lock<std::mutex> lock_;
    value_type*                  item_ = nullptr;
  };

  concurrent_hash_map() : mutex_(std::make_unique<std::mutex>()) {}
  concurrent_hash_map(const concurrent_hash_map& that) : map_(that.map_), mutex_(std::make_unique<std::mutex>()) {}
  concurrent_hash_map(concurrent_hash_map&& temp) noexcept : map_(std::move(temp.map_)), mutex_(std::make_unique<std::mutex>()) {}
  concurrent_hash_map& operator=(const concurrent_hash_map& that) { map_ = that.map_; return *this; }
  concurrent_hash_map& operator=(concurrent_hash_map&& temp) noexcept { map_ = std::move(temp.map_); return *this; }

  bool find(accessor& result, const key_type& key)
  {
    result.release();
    result.lock_ = std::unique_lock<std::mutex>(*mutex_);
    auto it = map_.find(key);
    if (it == map_.end()) { result.lock_.unlock(); return false; }
    result.item_ = &*it;
    return true;
  }
  template <typename... args_type>
  bool emplace(args_type&&... args)
  {
    std::lock_guard<std::mutex> lock(*mutex_);
    return map_.emplace(std::forward<args_type>(args)...).second;
  }
  std::size_t size () const { return map_.size(); }
  bool        empty() const { return map_.empty(); }
  typename map_type::iterator       begin()       { return map_.begin(); }
  typename map_type::iterator       end  ()       { return map_.end();   }
  typename map_type::const_iterator begin() const { return map_.begin(); }
  typename map_type::const_iterator end  () const { return map_.end();   }

private:
  map_type                    map_;
  std::unique_ptr<std::mutex> mutex_;
};

class task_scheduler_init
{
public:
  explicit task_scheduler_init(int = -1) {}
};
}

#endif
