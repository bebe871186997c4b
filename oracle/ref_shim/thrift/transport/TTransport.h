// Minimal stand-in for <thrift/transport/TTransport.h> (test infrastructure; see thrift/Thrift.h).
#pragma once

#include "../Thrift.h"
