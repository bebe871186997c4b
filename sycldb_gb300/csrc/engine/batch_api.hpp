// Internal interface between the executor (engine.cpp) and the request server
// (server.cpp): batches of plans built on memory and streams that the caller
// owns, for one eager run each.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sycldb_gpu.h"

namespace sdb {

// Every executor failure: an sdb_status and a message.
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

// What a set of plans needs, from a sizing pass (the plans recorded against
// addresses that are never dereferenced).  Sizes of plans recorded one after
// the other add up: arena and zeroed bytes of a batch are the sums over its
// plans, its result staging too.
struct BatchSize {
    uint64_t arena = 0;     // arena bytes
    uint64_t zero = 0;      // zeroed-region bytes
    uint64_t staging = 0;   // result region bytes (on the device, and its pinned mirror)
    std::vector<sdb_chain_desc> chains;  // the aggregating chains (addresses of the sizing pass)
};

// The streams and events of one server slot: work goes on `main`, each plan's
// work on side[p % side.size()] between fork and join events.
struct SlotStreams {
    cudaStream_t main = nullptr;
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> join;  // one per side stream
    cudaEvent_t fork = nullptr;
};

// Sizing pass over `plans` (throws Error on a bad plan).  Touches no device.
BatchSize batch_size(sdb_engine *eng, const std::vector<std::string> &plans);

// Device bytes the chain batch of `chains` takes (also the pinned bytes its
// tables are staged in).
size_t batch_chain_bytes(const std::vector<sdb_chain_desc> &chains);

// Records `plans` (sized by `z`, which must be the sum of their sizing passes
// with the chains concatenated) against the device region dev[0, dev_bytes)
// -- arena, then zeroed region, then result region (every plan's count and
// result columns), then chain-batch tables, each rounded up to 256 bytes --
// and the pinned region pinned[0, pinned_bytes) -- chain-batch tables, then
// the result region's mirror -- and enqueues the whole batch on the slot's
// streams.  Returns the batch; its results are read with batch_take_result
// once the work on ss.main has completed.
sdb_batch *batch_launch_external(sdb_engine *eng, const std::vector<std::string> &plans, const BatchSize &z,
                                 char *dev, size_t dev_bytes, char *pinned, size_t pinned_bytes,
                                 const SlotStreams &ss);

// Plan p's result (caller frees it with sdb_result_free).
sdb_result *batch_take_result(const sdb_batch *b, size_t p);

// Fact chains the batch runs in paired passes (shared scans).
int batch_paired_chains(const sdb_batch *b);

void batch_destroy(sdb_batch *b);

// Runs one plan with the engine's plain path (sdb_engine_execute).
sdb_result *execute_plain(sdb_engine *eng, const std::string &plan);

// Device bytes of the engine's own arena and zeroed region (what a plain
// execution can use at most).
uint64_t engine_memory_bytes(const sdb_engine *eng);

}  // namespace sdb
