// Minimal stand-in for the part of Boost.Iterator's iterator_facade that the
// reference headers use (forward traversal only).  Written from the documented
// interface: the derived class supplies increment(), dereference() and
// equal(other), and grants access through iterator_core_access.
//
// Test infrastructure only: used to compile the reference's own sources into
// oracle/_ref; nothing in the product includes it.
#ifndef ORACLE_SHIM_BOOST_ITERATOR_FACADE_HPP
#define ORACLE_SHIM_BOOST_ITERATOR_FACADE_HPP

#include <cstddef>
#include <iterator>

namespace boost {

struct forward_traversal_tag { };

class iterator_core_access {
public:
    template <typename D>
    static void increment(D& d) { d.increment(); }
    template <typename D>
    static auto dereference(const D& d) { return d.dereference(); }
    template <typename D>
    static bool equal(const D& a, const D& b) { return a.equal(b); }
};

template <typename Derived, typename Value, typename Traversal, typename Reference = Value&>
class iterator_facade {
public:
    using value_type = Value;
    using reference = Reference;
    using difference_type = std::ptrdiff_t;
    using pointer = void;
    using iterator_category = std::forward_iterator_tag;

    Reference operator*() const { return iterator_core_access::dereference(self()); }

    Derived& operator++() {
        iterator_core_access::increment(self());
        return self();
    }

    Derived operator++(int) {
        Derived tmp = self();
        ++*this;
        return tmp;
    }

    friend bool operator==(const Derived& a, const Derived& b) {
        return iterator_core_access::equal(a, b);
    }
    friend bool operator!=(const Derived& a, const Derived& b) { return !(a == b); }

private:
    Derived& self() { return static_cast<Derived&>(*this); }
    const Derived& self() const { return static_cast<const Derived&>(*this); }
};

}  // namespace boost

#endif
