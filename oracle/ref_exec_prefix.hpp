// Included before every translation unit of the reference-executor checker
// (TEST INFRASTRUCTURE ONLY; build_oracle.py passes it with -include).
// The reference's common.hpp fixes PERFORMANCE_MEASUREMENT_ACTIVE 1, in which
// execute_ddor_plan writes no result; the checker needs its correctness mode
// (0: the executor saves the result rows).  REF_EXEC_SEGMENT_SIZE, when the
// recipe defines it, replaces SEGMENT_SIZE (2^28 rows) so that small inputs
// span several segments.  common.hpp is include-guarded, so these values
// hold for every file that includes it afterwards.
#include "common.hpp"
#undef PERFORMANCE_MEASUREMENT_ACTIVE
#define PERFORMANCE_MEASUREMENT_ACTIVE 0
#ifdef REF_EXEC_SEGMENT_SIZE
#undef SEGMENT_SIZE
#define SEGMENT_SIZE ((uint64_t)(REF_EXEC_SEGMENT_SIZE))
#endif
