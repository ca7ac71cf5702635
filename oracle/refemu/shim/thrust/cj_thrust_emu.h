// Minimal stand-in for the Thrust calls on the reference's parse path
// (cujson/parse_standard_json.cu:1163,1245,1254,1537,1540,1546 and
// cujson/parse_json_lines.cu:865,885,890,1029,1032,1038): sequential
// exclusive/inclusive scans, transform_if and a stable sort by key over a zip
// of value arrays, with Thrust's documented results.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <algorithm>
#include <cstddef>
#include <iterator>
#include <numeric>
#include <tuple>
#include <vector>

namespace thrust {

struct par_t {};
namespace cuda { inline constexpr par_t par{}; }
inline constexpr par_t host{};
inline constexpr par_t device{};

template <typename It> using iterator_traits = std::iterator_traits<It>;

template <typename T> inline T* raw_pointer_cast(T* p) { return p; }
template <typename T> using device_ptr = T*;

template <typename T>
struct device_vector : std::vector<T> {
    using std::vector<T>::vector;
};
template <typename T>
struct host_vector : std::vector<T> {
    using std::vector<T>::vector;
};

template <typename InIt, typename OutIt>
inline OutIt copy(InIt first, InIt last, OutIt out) { return std::copy(first, last, out); }

template <typename T>
struct counting_iterator {
    using iterator_category = std::random_access_iterator_tag;
    using value_type = T;
    using difference_type = std::ptrdiff_t;
    using pointer = const T*;
    using reference = T;
    T v;
    T operator*() const { return v; }
    T operator[](difference_type i) const { return (T)(v + i); }
    counting_iterator operator+(difference_type i) const { return {(T)(v + i)}; }
    counting_iterator& operator++() { ++v; return *this; }
    difference_type operator-(const counting_iterator& o) const { return (difference_type)v - (difference_type)o.v; }
    bool operator!=(const counting_iterator& o) const { return v != o.v; }
    bool operator==(const counting_iterator& o) const { return v == o.v; }
};
template <typename T> inline counting_iterator<T> make_counting_iterator(T v) { return {v}; }

template <typename... P> inline std::tuple<P...> make_tuple(P... p) { return std::tuple<P...>(p...); }
template <typename Tup>
struct zip_iterator {
    Tup t;
};
template <typename Tup> inline zip_iterator<Tup> make_zip_iterator(Tup t) { return {t}; }

// result[i] = init + in[0] + ... + in[i-1]  (init = value_type{})
template <typename In, typename Out>
inline Out exclusive_scan(par_t, In first, In last, Out result)
{
    using V = typename std::iterator_traits<In>::value_type;
    V acc = V{};
    const std::ptrdiff_t n = last - first;
    for (std::ptrdiff_t i = 0; i < n; i++) {
        const V x = first[i];
        result[i] = acc;
        acc = (V)(acc + x);
    }
    return result + n;
}

// result[i] = in[0] + ... + in[i]
template <typename In, typename Out>
inline Out inclusive_scan(par_t, In first, In last, Out result)
{
    using V = typename std::iterator_traits<In>::value_type;
    V acc = V{};
    const std::ptrdiff_t n = last - first;
    for (std::ptrdiff_t i = 0; i < n; i++) {
        acc = (V)(acc + first[i]);
        result[i] = acc;
    }
    return result + n;
}

// result[i] = op(in[i]) where pred(stencil[i])
template <typename In, typename St, typename Out, typename Op, typename Pr>
inline Out transform_if(par_t, In first, In last, St stencil, Out result, Op op, Pr pred)
{
    const std::ptrdiff_t n = last - first;
    for (std::ptrdiff_t i = 0; i < n; i++)
        if (pred(stencil[i])) result[i] = op(first[i]);
    return result + n;
}

namespace detail {
template <typename Ptr>
inline void permute(Ptr p, const std::vector<std::size_t>& idx)
{
    using V = typename std::iterator_traits<Ptr>::value_type;
    std::vector<V> tmp(idx.size());
    for (std::size_t i = 0; i < idx.size(); i++) tmp[i] = p[idx[i]];
    for (std::size_t i = 0; i < idx.size(); i++) p[i] = tmp[i];
}
}  // namespace detail

// keys sorted ascending, equal keys keep their order; every value array of
// the zip moves with its key
template <typename K, typename... P>
inline void stable_sort_by_key(par_t, K kfirst, K klast, zip_iterator<std::tuple<P...>> values)
{
    const std::size_t n = (std::size_t)(klast - kfirst);
    std::vector<std::size_t> idx(n);
    std::iota(idx.begin(), idx.end(), (std::size_t)0);
    std::stable_sort(idx.begin(), idx.end(), [&](std::size_t a, std::size_t b) { return kfirst[a] < kfirst[b]; });
    detail::permute(kfirst, idx);
    std::apply([&](auto... p) { (detail::permute(p, idx), ...); }, values.t);
}

}  // namespace thrust
