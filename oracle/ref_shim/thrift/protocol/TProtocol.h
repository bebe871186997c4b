// Minimal stand-in for <thrift/protocol/TProtocol.h> (test infrastructure;
// see thrift/Thrift.h).  The oracle never serialises a plan: every read and
// write call throws.
#pragma once

#include <cstdint>
#include <string>

#include "../Thrift.h"

namespace apache {
namespace thrift {
namespace protocol {

enum TType {
    T_STOP = 0, T_VOID = 1, T_BOOL = 2, T_BYTE = 3, T_I08 = 3, T_I16 = 6, T_I32 = 8, T_U64 = 9, T_I64 = 10,
    T_DOUBLE = 4, T_STRING = 11, T_UTF7 = 11, T_STRUCT = 12, T_MAP = 13, T_SET = 14, T_LIST = 15, T_UUID = 16
};

class TProtocolException : public TException {
public:
    enum TProtocolExceptionType { UNKNOWN = 0, INVALID_DATA = 1, NEGATIVE_SIZE = 2, SIZE_LIMIT = 3, BAD_VERSION = 4,
                                  NOT_IMPLEMENTED = 5, DEPTH_LIMIT = 6 };
    explicit TProtocolException(TProtocolExceptionType) : TException("thrift protocol (oracle shim)") {}
};

class TProtocol {
    [[noreturn]] static uint32_t no() { throw TException("the oracle's Thrift shim does not serialise"); }

public:
    uint32_t readStructBegin(std::string &) { no(); }
    uint32_t readStructEnd() { no(); }
    uint32_t readFieldBegin(std::string &, TType &, int16_t &) { no(); }
    uint32_t readFieldEnd() { no(); }
    uint32_t readListBegin(TType &, uint32_t &) { no(); }
    uint32_t readListEnd() { no(); }
    uint32_t readBool(bool &) { no(); }
    uint32_t readI32(int32_t &) { no(); }
    uint32_t readI64(int64_t &) { no(); }
    uint32_t readString(std::string &) { no(); }
    uint32_t skip(TType) { no(); }
    uint32_t writeStructBegin(const char *) { no(); }
    uint32_t writeStructEnd() { no(); }
    uint32_t writeFieldBegin(const char *, TType, int16_t) { no(); }
    uint32_t writeFieldEnd() { no(); }
    uint32_t writeFieldStop() { no(); }
    uint32_t writeListBegin(TType, uint32_t) { no(); }
    uint32_t writeListEnd() { no(); }
    uint32_t writeBool(bool) { no(); }
    uint32_t writeI32(int32_t) { no(); }
    uint32_t writeI64(int64_t) { no(); }
    uint32_t writeString(const std::string &) { no(); }
};

struct TInputRecursionTracker {
    explicit TInputRecursionTracker(TProtocol &) {}
};
struct TOutputRecursionTracker {
    explicit TOutputRecursionTracker(TProtocol &) {}
};

}  // namespace protocol
}  // namespace thrift
}  // namespace apache
