// Minimal stand-in for <thrift/TDispatchProcessor.h> (test infrastructure;
// see thrift/Thrift.h): the base classes the generated service header
// derives from, declared so it compiles.  No service runs in the oracle.
#pragma once

#include <memory>
#include <string>

#include "Thrift.h"
#include "protocol/TProtocol.h"

namespace apache {
namespace thrift {

struct TConnectionInfo {
    std::shared_ptr<protocol::TProtocol> input, output;
};

class TProcessor {
public:
    virtual ~TProcessor() = default;
};

class TDispatchProcessor : public TProcessor {
protected:
    virtual bool dispatchCall(protocol::TProtocol *in, protocol::TProtocol *out, const std::string &fname,
                              int32_t seqid, void *callContext) = 0;
};

class TProcessorFactory {
public:
    virtual ~TProcessorFactory() = default;
    virtual std::shared_ptr<TProcessor> getProcessor(const TConnectionInfo &info) = 0;
};

}  // namespace thrift
}  // namespace apache
