// Minimal stand-in for <thrift/TBase.h> (test infrastructure; see thrift/Thrift.h).
#pragma once

#include "Thrift.h"
#include "protocol/TProtocol.h"

namespace apache {
namespace thrift {

class TBase {
public:
    virtual ~TBase() = default;
    virtual uint32_t read(protocol::TProtocol *iprot) = 0;
    virtual uint32_t write(protocol::TProtocol *oprot) const = 0;
};

}  // namespace thrift
}  // namespace apache
