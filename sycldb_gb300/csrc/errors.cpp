// Status codes, the per-thread last-error message and the device error word.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sycldb_gpu.h"

namespace {
thread_local std::string g_last_error;
std::atomic<unsigned long long> g_launches{0};
std::mutex g_readers_mu;
std::vector<unsigned long long (*)(cudaStream_t)> &readers()
{
    static std::vector<unsigned long long (*)(cudaStream_t)> r;
    return r;
}
}  // namespace

int sdb_set_error(int status, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

void sdb_count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int sdb_check_launch(const char *what)
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return sdb_set_error(SDB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return SDB_OK;
}

namespace sdb {
int device_sms()
{
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cache[kMaxDevices];  // 0: not queried yet
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
    if (dev >= kMaxDevices) dev = kMaxDevices - 1;
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 152;  // GB300's count, as a default when the query fails
    }
    cache[dev].store(n, std::memory_order_relaxed);
    return n;
}
}  // namespace sdb

void sdb_errors_add_reader(unsigned long long (*reader)(cudaStream_t))
{
    std::lock_guard<std::mutex> lk(g_readers_mu);
    readers().push_back(reader);
}

extern "C" {

const char *sdb_last_error(void) { return g_last_error.c_str(); }

const char *sdb_version(void) { return "sycldb-gb300 0.1 (sm_103a)"; }

uint64_t sdb_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

size_t sdb_abi_sizeof(const char *type_name)
{
    if (!type_name) return 0;
    std::string t(type_name);
    if (t == "sdb_operand") return sizeof(sdb_operand);
    if (t == "sdb_chain_op") return sizeof(sdb_chain_op);
    if (t == "sdb_chain_desc") return sizeof(sdb_chain_desc);
    if (t == "sdb_engine_config") return sizeof(sdb_engine_config);
    if (t == "sdb_batch_stats") return sizeof(sdb_batch_stats);
    if (t == "sdb_server_config") return sizeof(sdb_server_config);
    if (t == "sdb_server_stats") return sizeof(sdb_server_stats);
    return 0;
}

int sdb_device_errors(uint64_t *count, sdb_stream_t stream)
{
    if (!count) return sdb_set_error(SDB_ERR_INVALID, "sdb_device_errors: count is NULL");
    unsigned long long total = 0;
    std::lock_guard<std::mutex> lk(g_readers_mu);
    for (auto r : readers()) total += r((cudaStream_t)stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return sdb_set_error(SDB_ERR_CUDA, "sdb_device_errors: %s", cudaGetErrorString(e));
    *count = total;
    return SDB_OK;
}

}  // extern "C"
