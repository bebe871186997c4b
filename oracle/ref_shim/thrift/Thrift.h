// Minimal stand-in for Apache Thrift's <thrift/Thrift.h>.
//
// TEST INFRASTRUCTURE ONLY.  It lets the reference's Thrift-generated plan
// types (gen-cpp/calciteserver_types.*) compile so that the oracle can build
// PlanResult objects in memory and hand them to the reference's own
// executor.  Nothing here serialises: the protocol calls the generated
// read/write code makes are stubs that throw if ever reached.  Written for
// this shim; none of it is Thrift library code.
#pragma once

#include <cstdint>
#include <exception>
#include <iterator>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace apache {
namespace thrift {

class TException : public std::exception {
public:
    TException() = default;
    explicit TException(const std::string &m) : msg_(m) {}
    const char *what() const noexcept override { return msg_.c_str(); }

private:
    std::string msg_;
};

// Walks parallel arrays of enum values and names as (value, name) pairs; the
// generated code builds its VALUES_TO_NAMES maps from a range of these.
class TEnumIterator {
public:
    using iterator_category = std::forward_iterator_tag;
    using value_type = std::pair<int, const char *>;
    using difference_type = std::ptrdiff_t;
    using pointer = const value_type *;
    using reference = value_type;

    TEnumIterator(int n, int *values, const char **names) : n_(n), values_(values), names_(names) {}
    TEnumIterator &operator++()
    {
        ++values_;
        ++names_;
        --n_;
        return *this;
    }
    TEnumIterator operator++(int)
    {
        TEnumIterator t = *this;
        ++*this;
        return t;
    }
    bool operator==(const TEnumIterator &o) const { return n_ == o.n_ || (n_ <= 0 && o.n_ <= 0); }
    bool operator!=(const TEnumIterator &o) const { return !(*this == o); }
    value_type operator*() const { return value_type(*values_, *names_); }

private:
    int n_;
    int *values_;
    const char **names_;
};

}  // namespace thrift
}  // namespace apache
