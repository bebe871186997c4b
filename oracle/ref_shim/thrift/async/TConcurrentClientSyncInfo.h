// Minimal stand-in for <thrift/async/TConcurrentClientSyncInfo.h> (test
// infrastructure; see thrift/Thrift.h).
#pragma once

namespace apache {
namespace thrift {
namespace async {

class TConcurrentClientSyncInfo {};

}  // namespace async
}  // namespace thrift
}  // namespace apache
