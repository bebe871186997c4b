// Counter-based synthetic data for the star schema, identical on host and
// device: value(seed, stream, row) depends only on its arguments, so any
// thread count, any device and any row range produce the same columns.
#pragma once

#include <cstdint>

namespace sdb {

// SplitMix64 finaliser (Steele, Lea, Flood: "Fast splittable pseudorandom
// number generators", OOPSLA 2014).
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__host__ __device__ __forceinline__ uint64_t stream_key(uint64_t seed, uint64_t stream)
{
    return splitmix64(seed ^ (stream * 0xD1B54A32D192ED03ull));
}

// Uniform integer in [lo, hi] (inclusive): the high 32 random bits scaled by
// the span with a multiply-shift.
__host__ __device__ __forceinline__ int32_t uniform_from_key(uint64_t key, uint64_t row, int32_t lo, int32_t hi)
{
    uint64_t r = splitmix64(key + row);
    uint64_t span = (uint64_t)((int64_t)hi - (int64_t)lo) + 1u;
    return (int32_t)((int64_t)lo + (int64_t)(((r >> 32) * span) >> 32));
}

// Days since 1970-01-01 -> (y, m, d) in the proleptic Gregorian calendar
// (the era/day-of-era method of H. Hinnant, "chrono-Compatible Low-Level Date
// Algorithms").
__host__ __device__ __forceinline__ void civil_from_days(int64_t z, int32_t &y, int32_t &m, int32_t &d)
{
    z += 719468;
    const int64_t era = (z >= 0 ? z : z - 146096) / 146097;
    const int64_t doe = z - era * 146097;
    const int64_t yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
    const int64_t doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
    const int64_t mp = (5 * doy + 2) / 153;
    d = (int32_t)(doy - (153 * mp + 2) / 5 + 1);
    m = (int32_t)(mp < 10 ? mp + 3 : mp - 9);
    y = (int32_t)(yoe + era * 400 + (m <= 2 ? 1 : 0));
}

constexpr int64_t kDay1992 = 8035;  // 1992-01-01 in days since 1970-01-01

// YYYYMMDD of the day `day` counted from 1992-01-01.
__host__ __device__ __forceinline__ int32_t datekey_of_day(int64_t day)
{
    int32_t y, m, d;
    civil_from_days(kDay1992 + day, y, m, d);
    return y * 10000 + m * 100 + d;
}

}  // namespace sdb
