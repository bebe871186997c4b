// Minimal stand-in for <thrift/TToString.h> (test infrastructure; see
// thrift/Thrift.h): to_string of values, lists and generated structs for the
// generated printTo code.
#pragma once

#include <sstream>
#include <string>
#include <vector>

#include "Thrift.h"

namespace apache {
namespace thrift {

template <typename T>
std::string to_string(const T &v)
{
    std::ostringstream o;
    o << v;
    return o.str();
}

template <typename T>
std::string to_string(const std::vector<T> &v)
{
    std::ostringstream o;
    o << "[";
    for (size_t i = 0; i < v.size(); i++) o << (i ? ", " : "") << to_string(v[i]);
    o << "]";
    return o.str();
}

}  // namespace thrift
}  // namespace apache
