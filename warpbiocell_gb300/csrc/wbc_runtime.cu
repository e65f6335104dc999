// Library plumbing: error bookkeeping, version, device count, the multi-block int32 scan used by
// the hash-grid binning and the division slots, and the test hooks of the random streams.
#include <atomic>
#include <cstdio>
#include <cstring>

#include "wbc_common.cuh"

namespace wbc {

namespace {
thread_local char g_error[512] = "no error";
std::atomic<int64_t> g_launches{0};
}

void set_error(const char* where, cudaError_t err) {
    std::snprintf(g_error, sizeof(g_error), "%s: %s (%s)", where, cudaGetErrorString(err), cudaGetErrorName(err));
}

void set_error_msg(const char* msg) { std::snprintf(g_error, sizeof(g_error), "%s", msg); }

int check_launch(const char* where, int64_t launches) {
    g_launches.fetch_add(launches, std::memory_order_relaxed);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_error(where, err);
        return WBC_ERR_CUDA;
    }
    return WBC_OK;
}

// ---- scan --------------------------------------------------------------------------------------
// Tile = kScanThreads x kScanItems consecutive elements. Phase 1 reduces every tile to one
// partial; phase 2 (one block) turns the partials into exclusive tile offsets with a running
// carry, so any number of tiles works; phase 3 rescans each tile from its offset. Pure integer
// work, so the result does not depend on the launch shape.
int64_t scan_partials_count(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

__global__ void scan_reduce_tiles(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ partials) {
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
    int32_t vals[kScanItems];
    load_items(in, base, n, vals);
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) s += vals[k];
    int32_t total;
    block_exclusive(s, &total);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

__global__ void scan_partials(int32_t* __restrict__ partials, int64_t tiles, int32_t* __restrict__ total_out) {
    int32_t carry = 0;
    for (int64_t base = 0; base < tiles; base += kScanThreads) {
        int64_t idx = base + threadIdx.x;
        int32_t v = idx < tiles ? partials[idx] : 0;
        int32_t chunk_total;
        int32_t ex = block_exclusive(v, &chunk_total);
        if (idx < tiles) partials[idx] = carry + ex;
        carry += chunk_total;
    }
    if (threadIdx.x == 0) {
        partials[tiles] = carry;
        if (total_out) *total_out = carry;
    }
}

__global__ void scan_tiles(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t n,
                           const int32_t* __restrict__ partials, bool inclusive) {
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
    int32_t vals[kScanItems];
    load_items(in, base, n, vals);
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) s += vals[k];
    int32_t total;
    int32_t run = block_exclusive(s, &total) + partials[blockIdx.x];
    int32_t res[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (inclusive) run += vals[k];
        res[k] = run;
        if (!inclusive) run += vals[k];
    }
    store_items(out, base, n, res);
}

int scan_i32(const int32_t* in, int32_t* out, int64_t n, bool inclusive, int32_t* partials, int32_t* total,
             cudaStream_t stream) {
    if (n <= 0) {
        if (total) {
            cudaError_t err = cudaMemsetAsync(total, 0, sizeof(int32_t), stream);
            if (err != cudaSuccess) {
                set_error("scan: cudaMemsetAsync", err);
                return WBC_ERR_CUDA;
            }
        }
        return WBC_OK;
    }
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    scan_reduce_tiles<<<static_cast<unsigned>(tiles), kScanThreads, 0, stream>>>(in, n, partials);
    scan_partials<<<1, kScanThreads, 0, stream>>>(partials, tiles, total);
    scan_tiles<<<static_cast<unsigned>(tiles), kScanThreads, 0, stream>>>(in, out, n, partials, inclusive);
    return check_launch("scan_i32", 3);
}

// ---- random-stream test hooks ----------------------------------------------------------------------
__global__ void k_rng_init(int32_t seed, uint32_t* __restrict__ rng_state, int64_t capacity) {
    int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < capacity) rng_state[i] = rng_start(seed, static_cast<uint32_t>(i));
}

__global__ void k_rng_uniform(int32_t n, int32_t draws, uint32_t* __restrict__ rng_state, float* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = rng_state[i];
    const uint32_t inc = rng_increment(static_cast<uint32_t>(i));
    for (int k = 0; k < draws; ++k) out[static_cast<int64_t>(i) * draws + k] = randf(s, inc);
    rng_state[i] = s;
}

__global__ void k_rng_sphere(int32_t n, uint32_t* __restrict__ rng_state, float* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = rng_state[i];
    float x, y, z;
    unit_sphere(s, rng_increment(static_cast<uint32_t>(i)), x, y, z);
    rng_state[i] = s;
    out[3 * static_cast<int64_t>(i) + 0] = x;
    out[3 * static_cast<int64_t>(i) + 1] = y;
    out[3 * static_cast<int64_t>(i) + 2] = z;
}

__global__ void k_expf(int32_t n, const float* __restrict__ x, float* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = wbc_expf(x[i]);
}

__global__ void k_div(int32_t n, const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = div_rn(a[i], b[i]);
}

__device__ __forceinline__ bool same_result(float x, float y) {
    return __float_as_uint(x) == __float_as_uint(y) || (x != x && y != y);
}

__device__ __forceinline__ void note_mismatch(unsigned long long* count, uint32_t* first, float a, float b) {
    if (atomicAdd(count, 1ull) == 0ull) {
        first[0] = __float_as_uint(a);
        first[1] = __float_as_uint(b);
    }
}

// Every b = +-1.m * 2^e, e in [e_lo, e_hi]: the refined reciprocal against IEEE 1 / b.
__global__ void k_recip_exhaustive(int32_t e_lo, int32_t e_hi, unsigned long long* count, uint32_t* first) {
    const int64_t total = static_cast<int64_t>(e_hi - e_lo + 1) << 23;
    for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const uint32_t e = static_cast<uint32_t>(e_lo + static_cast<int32_t>(t >> 23) + 127);
        const uint32_t bits = (e << 23) | static_cast<uint32_t>(t & 0x7fffff);
        for (uint32_t sign = 0; sign < 2; ++sign) {
            const float b = __uint_as_float(bits | (sign << 31));
            if (!same_result(recip_rn_estimate(b), __fdiv_rn(1.0f, b))) note_mismatch(count, first, 1.0f, b);
        }
    }
}

// Seeded operand pairs of four kinds against IEEE a / b: raw bit patterns (every class, including
// zeros, subnormals, infinities and NaN), operands with exponents in [-40, 40], exact products
// a = q b, and quotients within a few ulp of a rounding midpoint (a = RN(b m), m a midpoint).
__global__ void k_div_random(uint32_t seed, int64_t pairs, unsigned long long* count, uint32_t* first) {
    for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < pairs;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t st = rng_start(seed, static_cast<uint32_t>(t) ^ static_cast<uint32_t>(t >> 32) * 0x85EBCA6Bu);
        const uint32_t inc = rng_increment(static_cast<uint32_t>(t));
        const uint32_t kind = static_cast<uint32_t>(t & 3);
        const uint32_t r1 = rng_next(st, inc), r2 = rng_next(st, inc), r3 = rng_next(st, inc);
        float a, b;
        if (kind == 0) {
            a = __uint_as_float(r1);
            b = __uint_as_float(r2);
        } else {
            const uint32_t ea = 127 - 40 + (r3 % 81), eb = 127 - 40 + ((r3 >> 8) % 81);
            a = __uint_as_float((r1 & 0x807fffffu) | (ea << 23));
            b = __uint_as_float((r2 & 0x807fffffu) | (eb << 23));
            if (kind == 2) {
                a = __fmul_rn(a, b);
            } else if (kind == 3) {
                // m = 1.m' + half an ulp of a 24-bit significand: a midpoint in [1, 2)
                const float m_lo = __uint_as_float((127u << 23) | (r1 & 0x7fffffu));
                const double mid = static_cast<double>(m_lo) + 0x1p-24;
                a = __double2float_rn(mid * static_cast<double>(b));
                const int nudge = static_cast<int>((r3 >> 24) & 7) - 3;
                a = __uint_as_float(__float_as_uint(a) + nudge);
            }
        }
        if (!same_result(div_rn(a, b), __fdiv_rn(a, b))) note_mismatch(count, first, a, b);
    }
}

}  // namespace wbc

using namespace wbc;

extern "C" {

int wbc_version(void) { return 1; }

const char* wbc_last_error(void) { return g_error; }

int64_t wbc_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int wbc_device_count(void) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return count;
}

size_t wbc_scan_workspace_bytes(int64_t n) {
    return static_cast<size_t>(scan_partials_count(n < 1 ? 1 : n)) * sizeof(int32_t);
}

int wbc_rng_init(int32_t seed, uint32_t* rng_state, int64_t capacity, void* stream) {
    if (capacity < 0 || (capacity > 0 && !rng_state)) return WBC_ERR_INVALID;
    if (capacity == 0) return WBC_OK;
    k_rng_init<<<grid_for(capacity), kThreads, 0, as_stream(stream)>>>(seed, rng_state, capacity);
    return check_launch("wbc_rng_init");
}

int wbc_rng_uniform(int32_t n, int32_t draws, uint32_t* rng_state, float* out, void* stream) {
    if (n < 0 || draws < 0 || (n > 0 && (!rng_state || !out))) return WBC_ERR_INVALID;
    if (n == 0 || draws == 0) return WBC_OK;
    k_rng_uniform<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, draws, rng_state, out);
    return check_launch("wbc_rng_uniform");
}

int wbc_rng_sphere(int32_t n, uint32_t* rng_state, float* out_xyz, void* stream) {
    if (n < 0 || (n > 0 && (!rng_state || !out_xyz))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_rng_sphere<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, rng_state, out_xyz);
    return check_launch("wbc_rng_sphere");
}

int wbc_div_batch(int32_t n, const float* a, const float* b, float* out, void* stream) {
    if (n < 0 || (n > 0 && (!a || !b || !out))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_div<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, a, b, out);
    return check_launch("wbc_div_batch");
}

int wbc_div_check(int32_t mode, int32_t e_lo, int32_t e_hi, uint32_t seed, int64_t pairs,
                  unsigned long long* mismatches, uint32_t* first_bad, void* stream) {
    if (!mismatches || !first_bad || mode < 0 || mode > 1) return WBC_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    if (mode == 0) {
        if (e_lo < -126 || e_hi > 127 || e_lo > e_hi) return WBC_ERR_INVALID;
        k_recip_exhaustive<<<4096, 256, 0, s>>>(e_lo, e_hi, mismatches, first_bad);
    } else {
        if (pairs < 0) return WBC_ERR_INVALID;
        if (pairs == 0) return WBC_OK;
        k_div_random<<<4096, 256, 0, s>>>(seed, pairs, mismatches, first_bad);
    }
    return check_launch("wbc_div_check");
}

int wbc_expf_batch(int32_t n, const float* x, float* out, void* stream) {
    if (n < 0 || (n > 0 && (!x || !out))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_expf<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, x, out);
    return check_launch("wbc_expf_batch");
}

}  // extern "C"
