// Lifecycle: per-cell death / state / division intent, the prefix-sum slot allocation and the
// daughter placement, plus the state census.
//
// Reference: kernels/cell_kernels.py:68-208 and cells/lifecycle.py:96-179. Draw order per living
// cell: the death draw is always consumed; the division draw only when the cell may divide
// (cell_kernels.py:115-154). Every draw comes from the cell's own stream (wbc_common.cuh), so the
// decisions depend on the seed and the cell's history only; probabilities use the project's
// exp (wbc_expf), so the oracle reproduces every decision bit for bit.
#include <mutex>

#include "wbc_bodies.cuh"

namespace wbc {

__global__ void k_lifecycle_decide(wbc_lifecycle_params p, int32_t n, int32_t* __restrict__ cell_state,
                                   float* __restrict__ age, const int32_t* __restrict__ neighbor_count,
                                   const float* __restrict__ oxygen_local, const float* __restrict__ glucose_local,
                                   const int32_t* __restrict__ fate_flags, uint32_t* __restrict__ rng_state,
                                   int32_t* __restrict__ divide_flag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        lifecycle_cell(p, i, cell_state, age, neighbor_count, oxygen_local, glucose_local, fate_flags, rng_state,
                       divide_flag);
}

__global__ void k_place_daughters(int32_t count, float placement_factor, const int32_t* __restrict__ divide_flag,
                                  const int32_t* __restrict__ division_offset, float* __restrict__ position,
                                  float* __restrict__ radius, int32_t* __restrict__ cell_state,
                                  int32_t* __restrict__ cell_type, float* __restrict__ age,
                                  float* __restrict__ oxygen_local, float* __restrict__ glucose_local,
                                  uint32_t* __restrict__ rng_state, float* __restrict__ velocity,
                                  int32_t* __restrict__ neighbor_count, int32_t* __restrict__ fate_flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count || divide_flag[i] == 0) return;
    place_daughter(i, count, placement_factor, division_offset, position, radius, cell_state, cell_type, age,
                   oxygen_local, glucose_local, rng_state, velocity, neighbor_count, fate_flags);
}

__global__ void k_count_states(int32_t n, const int32_t* __restrict__ cell_state, int32_t* __restrict__ counts) {
    __shared__ int32_t local[4];
    if (threadIdx.x < 4) local[threadIdx.x] = 0;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int s = cell_state[i];
        if (s >= 0 && s < 4) atomicAdd(local + s, 1);
    }
    __syncthreads();
    if (threadIdx.x < 4 && local[threadIdx.x]) atomicAdd(counts + threadIdx.x, local[threadIdx.x]);
}

}  // namespace wbc

using namespace wbc;

extern "C" {

int wbc_lifecycle_decide(const wbc_lifecycle_params* p, int32_t n, int32_t* cell_state, float* age,
                         const int32_t* neighbor_count, const float* oxygen_local, const float* glucose_local,
                         const int32_t* fate_flags, uint32_t* rng_state, int32_t* divide_flag, void* stream) {
    if (!p || n < 0 ||
        (n > 0 && (!cell_state || !age || !neighbor_count || !oxygen_local || !glucose_local || !fate_flags ||
                   !rng_state || !divide_flag)))
        return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_lifecycle_decide<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(
        *p, n, cell_state, age, neighbor_count, oxygen_local, glucose_local, fate_flags, rng_state, divide_flag);
    return check_launch("wbc_lifecycle_decide");
}

int wbc_division_scan(int32_t n, const int32_t* divide_flag, int32_t* division_offset, int32_t* total_out,
                      void* workspace, size_t workspace_bytes, void* stream) {
    if (n < 0 || (n > 0 && (!divide_flag || !division_offset)) || !workspace) return WBC_ERR_INVALID;
    if (workspace_bytes < wbc_scan_workspace_bytes(n)) return WBC_ERR_WORKSPACE;
    return scan_i32(divide_flag, division_offset, n, true, static_cast<int32_t*>(workspace), total_out,
                    as_stream(stream));
}

}  // extern "C"

// ---- allocation-free division scan ----------------------------------------------------------------
// For callers that cannot allocate device memory themselves, the scan's tile partials live in
// this file-scope array instead of a caller-provided workspace. Every GPU that loads the library
// holds it (32,772 bytes) until the process exits. Host code must not pass the symbol itself to a
// kernel (on the host it names a stand-in, not device memory): its device address is looked up
// once per device, with that device current, and cached.
namespace wbc {
namespace {
constexpr int64_t kNoAllocPartials = WBC_NOALLOC_SCAN_MAX_CELLS / kScanTileItems + 1;
static __device__ __align__(256) int32_t g_noalloc_partials[kNoAllocPartials];
static_assert(WBC_NOALLOC_SCAN_MAX_CELLS % kScanTileItems == 0, "whole tiles");

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
int32_t* g_noalloc_ptr[kMaxDevices] = {};

int noalloc_partials(int32_t** out) {
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) {
        set_error("wbc_division_scan_noalloc: cudaGetDevice", err);
        return WBC_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        set_error_msg("wbc_division_scan_noalloc: device index beyond the supported range");
        return WBC_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        err = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (err != cudaSuccess || !p) {
            set_error("wbc_division_scan_noalloc: cudaGetSymbolAddress", err);
            return WBC_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = static_cast<int32_t*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return WBC_OK;
}
}  // namespace
}  // namespace wbc

extern "C" {

int wbc_division_scan_noalloc(int32_t n, const int32_t* divide_flag, int32_t* division_offset, int32_t* total_out,
                              void* stream) {
    if (n < 0 || (n > 0 && (!divide_flag || !division_offset))) return WBC_ERR_INVALID;
    if (n > WBC_NOALLOC_SCAN_MAX_CELLS) {
        set_error_msg("wbc_division_scan_noalloc: n exceeds WBC_NOALLOC_SCAN_MAX_CELLS (33,554,432 cells); "
                      "use wbc_division_scan with a caller-provided workspace");
        return WBC_ERR_INVALID;
    }
    int32_t* partials = nullptr;
    int rc = noalloc_partials(&partials);
    if (rc != WBC_OK) return rc;
    return scan_i32(divide_flag, division_offset, n, true, partials, total_out, as_stream(stream));
}

int wbc_place_daughters(int32_t count, float placement_factor, const int32_t* divide_flag,
                        const int32_t* division_offset, float* position, float* radius, int32_t* cell_state,
                        int32_t* cell_type, float* age, float* oxygen_local, float* glucose_local,
                        uint32_t* rng_state, float* velocity, int32_t* neighbor_count, int32_t* fate_flags,
                        void* stream) {
    if (count < 0 || (count > 0 && (!divide_flag || !division_offset || !position || !radius || !cell_state ||
                                     !cell_type || !age || !oxygen_local || !glucose_local || !rng_state ||
                                     !velocity || !neighbor_count || !fate_flags)))
        return WBC_ERR_INVALID;
    if (count == 0) return WBC_OK;
    k_place_daughters<<<grid_for(count), kThreads, 0, as_stream(stream)>>>(
        count, placement_factor, divide_flag, division_offset, position, radius, cell_state, cell_type, age,
        oxygen_local, glucose_local, rng_state, velocity, neighbor_count, fate_flags);
    return check_launch("wbc_place_daughters");
}

int wbc_count_states(int32_t n, const int32_t* cell_state, int32_t* counts, void* stream) {
    if (n < 0 || !counts || (n > 0 && !cell_state)) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_count_states<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, cell_state, counts);
    return check_launch("wbc_count_states");
}

}  // extern "C"
