// Lifecycle: per-cell death / state / division intent, the prefix-sum slot allocation and the
// daughter placement, plus the state census.
//
// Reference: kernels/cell_kernels.py:68-208 and cells/lifecycle.py:96-179. Draw order per living
// cell: the death draw is always consumed; the division draw only when the cell may divide
// (cell_kernels.py:115-154). Every draw comes from the cell's own stream (wbc_common.cuh), so the
// decisions depend on the seed and the cell's history only; probabilities use the project's
// exp (wbc_expf), so the oracle reproduces every decision bit for bit.
#include <mutex>

#include "wbc_common.cuh"

namespace wbc {

__device__ __forceinline__ float oxygen_factor(float o, float hypoxia_threshold, float death_threshold) {
    if (o >= hypoxia_threshold) return 1.0f;
    if (o <= death_threshold) return 0.0f;
    return (o - death_threshold) / (hypoxia_threshold - death_threshold);
}

__global__ void k_lifecycle_decide(wbc_lifecycle_params p, int32_t n, int32_t* __restrict__ cell_state,
                                   float* __restrict__ age, const int32_t* __restrict__ neighbor_count,
                                   const float* __restrict__ oxygen_local, const float* __restrict__ glucose_local,
                                   const int32_t* __restrict__ fate_flags, uint32_t* __restrict__ rng_state,
                                   int32_t* __restrict__ divide_flag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    divide_flag[i] = 0;
    if (cell_state[i] == WBC_STATE_DEAD) return;

    age[i] = age[i] + p.dt;
    uint32_t rng = rng_state[i];
    const uint32_t inc = rng_increment(static_cast<uint32_t>(i));
    const float o = oxygen_local[i];
    const float g = glucose_local[i];
    const int flags = p.phenotype_model == 1 ? fate_flags[i] : 0;

    bool lethal = o < p.death_threshold;
    if (p.necrosis_requires_glucose != 0) lethal = lethal && (g < p.glucose_death_threshold);
    float rate = p.death_rate;
    if (lethal) rate = fmaxf(p.death_rate, p.anoxic_death_rate);
    if (flags & WBC_FATE_NECROSIS) rate = fmaxf(rate, p.necrosis_rate);
    if (flags & WBC_FATE_APOPTOSIS) rate = fmaxf(rate, p.apoptosis_rate);
    const float p_death = 1.0f - wbc_expf(-rate * p.dt);
    if (randf(rng, inc) < p_death) {
        cell_state[i] = WBC_STATE_DEAD;
        rng_state[i] = rng;
        return;
    }

    const bool crowded = neighbor_count[i] >= p.inhibition_threshold;
    bool may_divide = !crowded;
    float factor = 1.0f;
    if (p.phenotype_model == 1) {
        may_divide = may_divide && (flags & WBC_FATE_PROLIFERATION) != 0 && (flags & WBC_FATE_GROWTH_ARREST) == 0;
    } else {
        factor = oxygen_factor(o, p.hypoxia_threshold, p.death_threshold) *
                 oxygen_factor(g, p.glucose_threshold, p.glucose_death_threshold);
    }

    if (o < p.hypoxia_threshold)
        cell_state[i] = WBC_STATE_HYPOXIC;
    else if (may_divide)
        cell_state[i] = WBC_STATE_PROLIFERATIVE;
    else
        cell_state[i] = WBC_STATE_QUIESCENT;

    if (may_divide) {
        const float p_divide = 1.0f - wbc_expf(-p.division_rate * factor * p.dt);
        if (randf(rng, inc) < p_divide) divide_flag[i] = 1;
    }
    rng_state[i] = rng;
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
    const int j = count + division_offset[i] - 1;

    uint32_t rng = rng_state[i];
    float dx, dy, dz;
    unit_sphere(rng, rng_increment(static_cast<uint32_t>(i)), dx, dy, dz);
    rng_state[i] = rng;

    const float scale = 0.5f * placement_factor * radius[i];
    const float hx = dx * scale, hy = dy * scale, hz = dz * scale;
    const int64_t pi = 3 * static_cast<int64_t>(i), pj = 3 * static_cast<int64_t>(j);
    const float x = position[pi], y = position[pi + 1], z = position[pi + 2];
    position[pi] = x - hx;
    position[pi + 1] = y - hy;
    position[pi + 2] = z - hz;
    position[pj] = x + hx;
    position[pj + 1] = y + hy;
    position[pj + 2] = z + hz;

    radius[j] = radius[i];
    cell_state[j] = cell_state[i];
    cell_type[j] = cell_type[i];
    age[j] = 0.0f;
    oxygen_local[j] = oxygen_local[i];
    glucose_local[j] = glucose_local[i];
    velocity[pj] = 0.0f;
    velocity[pj + 1] = 0.0f;
    velocity[pj + 2] = 0.0f;
    neighbor_count[j] = 0;
    fate_flags[j] = fate_flags[i];
    // rng_state[j] was set for every slot when the population was created and stays as it is.
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
__device__ __align__(256) int32_t g_noalloc_partials[kNoAllocPartials];
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
