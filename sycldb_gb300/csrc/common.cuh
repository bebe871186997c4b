// Device helpers shared by the operator kernels and the fused chain kernel.
//
// The arithmetic follows the reference kernels exactly:
//   compare()   kernels/selection.hpp:61-81
//   logical()   kernels/selection.hpp:83-96  (NONE returns the new value)
//   binop()     kernels/aggregation.hpp:19-35 (int32, wrapping)
//   HASH()      kernels/join.hpp:11-15       ((x - min) % len, identity in range)
//   slot()      kernels/aggregation.hpp:315-321
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "sycldb_gpu.h"

namespace sdb {

// SM count of the calling thread's current device, queried once per device
// (errors.cpp); every grid of the library is sized from it.
int device_sms();

__host__ __device__ __forceinline__ bool compare(int cmp, int32_t a, int32_t b)
{
    switch (cmp) {
    case SDB_EQ: return a == b;
    case SDB_NE: return a != b;
    case SDB_LT: return a < b;
    case SDB_LE: return a <= b;
    case SDB_GT: return a > b;
    case SDB_GE: return a >= b;
    default: return false;
    }
}

__host__ __device__ __forceinline__ bool logical(int logic, bool a, bool b)
{
    switch (logic) {
    case SDB_AND: return a && b;
    case SDB_OR: return a || b;
    case SDB_NONE: return b;
    default: return false;
    }
}

// 4-row bit masks: bit j is row j of a 4-row group.
__host__ __device__ __forceinline__ uint32_t logical4(int logic, uint32_t a, uint32_t b)
{
    switch (logic) {
    case SDB_AND: return a & b;
    case SDB_OR: return a | b;
    case SDB_NONE: return b;
    default: return 0u;
    }
}

__host__ __device__ __forceinline__ int32_t binop(int32_t a, int32_t b, int op)
{
    switch (op) {
    case SDB_MUL: return (int32_t)((uint32_t)a * (uint32_t)b);
    case SDB_DIV:
        if (b == 0) return 0;
        if (a == INT32_MIN && b == -1) return INT32_MIN;
        return a / b;
    case SDB_ADD: return (int32_t)((uint32_t)a + (uint32_t)b);
    case SDB_SUB: return (int32_t)((uint32_t)a - (uint32_t)b);
    default: return 0;
    }
}

// HASH(x, len, min) = (x - min) % len in int.  Returns -1 when len == 0.
__host__ __device__ __forceinline__ int64_t ht_slot(int32_t x, int32_t len, int32_t mn)
{
    int32_t d = (int32_t)((uint32_t)x - (uint32_t)mn);
    if (len == 0) return -1;
    if (len == -1) return 0;
    return (int64_t)(d % len);
}

// ---- open-addressing join tables (sparse key ranges) -------------------------
// A join table over keys [min, max] whose range is much wider than the build
// side's rows is kept as 2^lg slots of linear probing instead of one entry
// per key of the range (the reference's direct-address HASH).  A slot's
// 32-bit word is tag << 1 | flag with tag = key - min + 1 (range < 2^31, so
// the tag fits 31 bits; word 0 = empty slot); a key/value table pairs the
// word with the value (int2 {word, value}).  Inserts claim an empty slot
// with atomicCAS; a key's flag and value are then stored as the direct
// table stores them (the reference's unordered writes), so probes see the
// same hits and values as with the direct table.  Tables are sized at least
// twice the build side's rows, so an insert always finds a slot; every
// probe loop is still bounded by the slot count.
__host__ __device__ __forceinline__ uint32_t oa_tag(int32_t key, int32_t mn)
{
    return (uint32_t)key - (uint32_t)mn + 1u;
}

__host__ __device__ __forceinline__ uint32_t oa_home(uint32_t tag, int lg)
{
    return (tag * 2654435761u) >> (32 - lg);
}

// Looks tag up in a table of 2^lg slots whose words are STRIDE words apart
// (1: keys table, 2: key/value table).  Returns the slot, or -1 when the key
// is absent.
template <int STRIDE>
__device__ __forceinline__ int64_t oa_find(const uint32_t *words, int lg, uint32_t tag)
{
    const uint32_t mask = (uint32_t)((1ull << lg) - 1);
    uint32_t h = oa_home(tag, lg);
    for (uint64_t i = 0; i <= mask; i++) {
        const uint32_t w = __ldg(words + (uint64_t)h * STRIDE);
        if (w == 0) return -1;
        if ((w >> 1) == tag) return (int64_t)h;
        h = (h + 1) & mask;
    }
    return -1;
}

// Writes (tag, live) into the table: a live row claims the key's slot (or
// its empty home run) and sets its flag, a dead row clears the flag of a key
// already present (absent reads as a miss already).  Returns the slot
// written (the caller stores a live row's value there), -1 when nothing was
// written, -2 when the table had no free slot (sized too small).
template <int STRIDE>
__device__ __forceinline__ int64_t oa_put(uint32_t *words, int lg, uint32_t tag, bool live)
{
    const uint32_t mask = (uint32_t)((1ull << lg) - 1);
    const uint32_t want = (tag << 1) | (live ? 1u : 0u);
    uint32_t h = oa_home(tag, lg);
    for (uint64_t i = 0; i <= mask; i++) {
        uint32_t *p = words + (uint64_t)h * STRIDE;
        uint32_t w = *p;
        if (w == 0) {
            if (!live) return -1;
            w = atomicCAS(p, 0u, want);
            if (w == 0) return (int64_t)h;
        }
        if ((w >> 1) == tag) {
            atomicExch(p, want);
            return (int64_t)h;
        }
        h = (h + 1) & mask;
    }
    return -2;
}

// Group-by slot: hash = sum_j (k_j - min_j) * mult_j in wrapping int, then
// `hash %= prod_ranges` with hash converted to uint64 and the result stored
// back into an int.
__host__ __device__ __forceinline__ int64_t group_slot(uint32_t hash, uint64_t P)
{
    // same value as the general form below: a non-negative hash below P is
    // its own slot (every key tuple inside its ranges), and a non-negative
    // hash needs only a 32-bit remainder when P fits 32 bits
    if ((int32_t)hash >= 0) {
        if ((uint64_t)hash < P) return (int64_t)hash;
        if (P <= 0xffffffffull) return (int64_t)(hash % (uint32_t)P);
    }
    return (int64_t)(int32_t)(uint32_t)((uint64_t)(int64_t)(int32_t)hash % P);
}

__host__ __device__ __forceinline__ uint64_t widen(int32_t v)
{
    return (uint64_t)(int64_t)v;
}

__host__ __device__ inline bool aligned(const void *p, uintptr_t a)
{
    return p == nullptr || (reinterpret_cast<uintptr_t>(p) % a) == 0;
}

// Grid for a grid-stride loop over `work` items of `threads` threads each.
inline unsigned grid_for(uint64_t work, int threads, int blocks_per_sm = 8)
{
    uint64_t b = (work + threads - 1) / threads;
    uint64_t cap = (uint64_t)device_sms() * blocks_per_sm;
    if (b > cap) b = cap;
    if (b == 0) b = 1;
    return (unsigned)b;
}

}  // namespace sdb

// Host-side error plumbing shared by all translation units (errors.cpp).
int sdb_set_error(int status, const char *fmt, ...);
// Counts one kernel launch and checks it; sdb_count_launches adds the
// extra launches of entry points that launch several kernels.
int sdb_check_launch(const char *what);
void sdb_count_launches(unsigned n);
void sdb_errors_add_reader(unsigned long long (*reader)(cudaStream_t));
