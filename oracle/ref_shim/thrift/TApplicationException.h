// Minimal stand-in for <thrift/TApplicationException.h> (test infrastructure; see thrift/Thrift.h).
#pragma once

#include "Thrift.h"
