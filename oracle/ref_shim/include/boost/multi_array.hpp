// Minimal stand-in for boost::multi_array as the reference hot path uses it:
// C-order (last index fastest) storage, resize(boost::extents[a][b][c]) or
// resize(std::array), shape(), operator()(std::array), chained operator[],
// data() and num_elements().
//
// This is test infrastructure for the oracle build only.
#ifndef PARS_SHIM_BOOST_MULTI_ARRAY_HPP
#define PARS_SHIM_BOOST_MULTI_ARRAY_HPP

#include <array>
#include <cstddef>
#include <vector>

namespace boost
{
namespace detail_shim
{
template <std::size_t count>
struct extent_list
{
  std::array<std::size_t, count> sizes {};
  extent_list<count + 1> operator[](long long size) const
  {
    extent_list<count + 1> result;
    for (std::size_t i = 0; i < count; ++i) result.sizes[i] = sizes[i];
    result.sizes[count] = static_cast<std::size_t>(size);
    return result;
  }
};

// A view of the sub-array below the first `depth` fixed indices.
template <typename element, std::size_t remaining>
struct sub_array
{
  element*           base;
  const std::size_t* strides;
  sub_array<element, remaining - 1> operator[](std::size_t index) const
  {
    return sub_array<element, remaining - 1>{base + index * strides[0], strides + 1};
  }
};
template <typename element>
struct sub_array<element, 1>
{
  element*           base;
  const std::size_t* strides;
  element& operator[](std::size_t index) const { return base[index]; }
};
}

static const detail_shim::extent_list<0> extents {};

template <typename element, std::size_t dimensions>
class multi_array
{
public:
  using value_type = element;
  using index      = long long;
  using size_type  = std::size_t;

  multi_array() { shape_.fill(0); strides_.fill(0); }
  template <std::size_t count>
  explicit multi_array(const detail_shim::extent_list<count>& extents) : multi_array() { resize(extents); }

  template <std::size_t count>
  multi_array& resize(const detail_shim::extent_list<count>& extents)
  {
    static_assert(count == dimensions, "extent count must match the array rank");
    set_shape(extents.sizes);
    return *this;
  }
  template <typename integer_type>
  multi_array& resize(const std::array<integer_type, dimensions>& sizes)
  {
    std::array<std::size_t, dimensions> converted;
    for (std::size_t i = 0; i < dimensions; ++i) converted[i] = static_cast<std::size_t>(sizes[i]);
    set_shape(converted);
    return *this;
  }

  const std::size_t* shape       () const { return shape_.data(); }
  std::size_t        num_elements() const { return data_.size();  }
  element*           data        ()       { return data_.data();  }
  const element*     data        () const { return data_.data();  }

  template <typename integer_type>
  element&       operator()(const std::array<integer_type, dimensions>& indices)       { return data_[offset(indices)]; }
  template <typename integer_type>
  const element& operator()(const std::array<integer_type, dimensions>& indices) const { return data_[offset(indices)]; }

  detail_shim::sub_array<element, dimensions - 1> operator[](std::size_t index)
  {
    return detail_shim::sub_array<element, dimensions - 1>{data_.data() + index * strides_[0], strides_.data() + 1};
  }
  detail_shim::sub_array<const element, dimensions - 1> operator[](std::size_t index) const
  {
    return detail_shim::sub_array<const element, dimensions - 1>{data_.data() + index * strides_[0], strides_.data() + 1};
  }

private:
  void set_shape(const std::array<std::size_t, dimensions>& sizes)
  {
    shape_ = sizes;
    std::size_t total = 1;
    for (std::size_t i = dimensions; i-- > 0;) { strides_[i] = total; total *= shape_[i]; }
    data_.assign(total, element());
  }
  template <typename integer_type>
  std::size_t offset(const std::array<integer_type, dimensions>& indices) const
  {
    std::size_t result = 0;
    for (std::size_t i = 0; i < dimensions; ++i) result += static_cast<std::size_t>(indices[i]) * strides_[i];
    return result;
  }

  std::array<std::size_t, dimensions> shape_;
  std::array<std::size_t, dimensions> strides_;
  std::vector<element>                data_;
};
}

#endif
