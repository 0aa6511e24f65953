// Minimal stand-in for boost::iterator_range, boost::make_iterator_range,
// boost::begin/end and boost::counting_iterator / counting_range, limited to
// what the reference's simulation headers use.  Written from the documented
// Boost.Range interface.
//
// Test infrastructure only: used to compile the reference's own sources into
// oracle/_ref; nothing in the product includes it.
#ifndef ORACLE_SHIM_BOOST_RANGE_HPP
#define ORACLE_SHIM_BOOST_RANGE_HPP

#include <cstddef>
#include <iterator>

namespace boost {

template <typename Int>
class counting_iterator {
public:
    using value_type = Int;
    using reference = Int;
    using difference_type = std::ptrdiff_t;
    using pointer = const Int*;
    using iterator_category = std::random_access_iterator_tag;

    counting_iterator() = default;
    explicit counting_iterator(Int v)
    : v_{v} { }

    Int operator*() const { return v_; }
    counting_iterator& operator++() {
        ++v_;
        return *this;
    }
    counting_iterator operator++(int) {
        auto t = *this;
        ++v_;
        return t;
    }
    counting_iterator& operator--() {
        --v_;
        return *this;
    }
    counting_iterator& operator+=(difference_type d) {
        v_ += static_cast<Int>(d);
        return *this;
    }
    counting_iterator operator+(difference_type d) const { return counting_iterator{v_ + static_cast<Int>(d)}; }
    difference_type operator-(const counting_iterator& o) const { return v_ - o.v_; }
    Int operator[](difference_type d) const { return v_ + static_cast<Int>(d); }
    bool operator==(const counting_iterator& o) const { return v_ == o.v_; }
    bool operator!=(const counting_iterator& o) const { return v_ != o.v_; }
    bool operator<(const counting_iterator& o) const { return v_ < o.v_; }

private:
    Int v_{};
};

template <typename Iter>
class iterator_range {
public:
    using iterator = Iter;
    using const_iterator = Iter;

    iterator_range() = default;
    iterator_range(Iter b, Iter e)
    : b_{b}
    , e_{e} { }

    Iter begin() const { return b_; }
    Iter end() const { return e_; }
    bool empty() const { return b_ == e_; }
    std::ptrdiff_t size() const { return std::distance(b_, e_); }

    friend bool operator==(const iterator_range& a, const iterator_range& b) {
        return a.b_ == b.b_ && a.e_ == b.e_;
    }
    friend bool operator!=(const iterator_range& a, const iterator_range& b) { return !(a == b); }

private:
    Iter b_{};
    Iter e_{};
};

template <typename Iter>
iterator_range<Iter> make_iterator_range(Iter b, Iter e) {
    return {b, e};
}

template <typename Range>
auto begin(const Range& r) {
    return r.begin();
}

template <typename Range>
auto end(const Range& r) {
    return r.end();
}

template <typename Int>
iterator_range<counting_iterator<Int>> counting_range(Int b, Int e) {
    return {counting_iterator<Int>{b}, counting_iterator<Int>{e}};
}

}  // namespace boost

#endif
