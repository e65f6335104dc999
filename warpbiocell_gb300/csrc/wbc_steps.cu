// Many contact steps in one cooperative launch, and their reverse (the hand-written adjoint's
// mechanics), for the adjoint model's K steps and its checkpointed segments.
//
// Each step is the plain path's binning + contact substep (wbc_grid_build followed by
// wbc_contact_substep): bucket counts, exclusive scan of the counts, scatter, in-bucket ordering by
// slot, then the contact and Euler step, with the same per-cell bodies (wbc_bodies.cuh) and so the
// same bits as the separate launches. Phases are separated by a grid barrier over the
// co-resident blocks of the launch; loops over cells and buckets are block-strided. A step's grid
// can be kept in a history slot of the workspace, so that the reverse pass (wbc_adjoint_steps)
// finds the grid of x_t without rebuilding it.
//
// With compensated positions (a low-order part beside each float position) the same steps keep the
// trajectory to about 48 bits, for the adjoint model, whose stiffness derivative is sensitive to
// single roundings of the positions.
//
// Every barrier wait is bounded in time (2 s of the GPU's global timer); on timeout the launch
// raises its abort flag, every block leaves, and the host gets WBC_ERR_TIMEOUT.
#include <algorithm>
#include <mutex>

#include "wbc_bodies.cuh"

namespace wbc {
namespace {

constexpr int kStepThreads = kScanThreads;  // 512: the block scan's width
constexpr int kMaxStepBlocks = 1024;
constexpr unsigned long long kStepWaitNs = 2000000000ull;

struct __align__(128) StepSync {
    unsigned int abort;
    int status;
    int pad[30];
    unsigned int flags[kMaxStepBlocks];
};

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned int* p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Arrive at the next epoch and wait for every block of the launch; false when aborted.
__device__ __forceinline__ bool step_barrier(StepSync* sy, unsigned int& epoch) {
    epoch += 1;
    __syncthreads();
    if (threadIdx.x == 0) st_release(sy->flags + blockIdx.x, epoch);
    int aborted = 0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
        unsigned polls = 0;
        unsigned long long start = 0;
        while (static_cast<int>(ld_acquire(sy->flags + b) - epoch) < 0) {
            if ((++polls & 255u) == 0u) {
                if (ld_acquire(&sy->abort) != 0u) {
                    aborted = 1;
                    break;
                }
                const unsigned long long t = now_ns();
                if (start == 0) {
                    start = t;
                } else if (t - start > kStepWaitNs) {
                    atomicExch(&sy->abort, 1u);
                    aborted = 1;
                    break;
                }
            }
        }
    }
    return __syncthreads_or(aborted) == 0;
}

// The grid of one step: bucket counts and starts, sorted ids and (x, y, z, r).
struct GridSlot {
    int32_t* count;
    int32_t* start;
    int32_t* sorted_id;
    float4* sorted_xyzr;
};

struct StepsArgs {
    BucketMap map;
    int32_t n, steps;
    float query_radius, rate, dt;
    float* position;
    const float* radius;
    float* velocity;
    int32_t* neighbor_count;
    int32_t* cell_bucket;
    int32_t* cell_rank;
    int32_t* scatter;
    int32_t* partials;  // tiles + 1
    int64_t buckets;
    int64_t tiles;
    // slot s: count / start at slot_ints + s * 2 * buckets, ids / xyzr at ids + s * capacity
    int32_t* slot_ints;
    int32_t* slot_ids;
    float4* slot_xyzr;
    int64_t capacity;
    int32_t slots;       // history slots; with history == 0 two slots are used in turn
    int32_t history;     // 1: step t builds into slot t (steps <= slots)
    int32_t last_build_only;  // 1: the last step builds its grid but does not move the cells
    float* checkpoints;  // optional: x_t before step t for t % every == 0, at checkpoints + (t / every) * 3n
    int32_t every;
    StepSync* sync;
    float* position_lo;     // compensated positions (NULL: plain float positions)
    float* checkpoints_lo;  // their low parts, as checkpoints
    float4* slot_lo;        // slot s: sorted low parts at slot_lo + s * capacity
};

__device__ __forceinline__ float4* slot_lo_of(const StepsArgs& a, int s) {
    return a.slot_lo + static_cast<int64_t>(s) * a.capacity;
}

__device__ __forceinline__ GridSlot slot_of(const StepsArgs& a, int s) {
    GridSlot g;
    g.count = a.slot_ints + static_cast<int64_t>(s) * 2 * a.buckets;
    g.start = g.count + a.buckets;
    g.sorted_id = a.slot_ids + static_cast<int64_t>(s) * a.capacity;
    g.sorted_xyzr = a.slot_xyzr + static_cast<int64_t>(s) * a.capacity;
    return g;
}

__device__ __forceinline__ int slot_for(const StepsArgs& a, int t) { return a.history ? t : (t & 1); }

// ---- compensated positions -------------------------------------------------------------------------
// With a low-order part (position = hi + lo, both float) the steps keep the trajectory to about
// 48 bits: pair differences are taken as (hi_i - hi_j) + (lo_i - lo_j), and the Euler step adds
// v dt to (hi, lo) with Knuth's TwoSum (D. Knuth, TAOCP vol. 2, sec. 4.2.2) and a renormalisation,
// so no rounding of the position is lost. Forces stay in float. Binning uses hi.

__device__ __forceinline__ void add_compensated(float& hi, float& lo, float delta) {
    const float s = hi + delta;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (delta - bb);  // hi + delta = s + e exactly
    const float l2 = lo + e;
    const float h2 = s + l2;
    lo = l2 - (h2 - s);
    hi = h2;
}

__device__ __forceinline__ void order_cell_compensated(int i, const float* __restrict__ position,
                                                       const float* __restrict__ position_lo,
                                                       const float* __restrict__ radius,
                                                       const int32_t* __restrict__ cell_bucket,
                                                       const int32_t* __restrict__ bucket_start,
                                                       const int32_t* __restrict__ bucket_count,
                                                       const int32_t* __restrict__ scatter, int32_t* __restrict__ sorted_id,
                                                       float4* __restrict__ sorted_xyzr, float4* __restrict__ sorted_lo) {
    bin_order_cell(i, position, radius, cell_bucket, bucket_start, bucket_count, scatter, sorted_id, sorted_xyzr);
    const int b = cell_bucket[i];
    const int s = bucket_start[b];
    const int c = bucket_count[b];
    int rank = 0;
    for (int u = s; u < s + c; ++u) rank += scatter[u] < i ? 1 : 0;
    const float* l = position_lo + 3 * static_cast<int64_t>(i);
    sorted_lo[s + rank] = make_float4(l[0], l[1], l[2], 0.0f);
}

// contact_slot with compensated positions.
__device__ __forceinline__ void contact_slot_compensated(BucketMap map, int t, const int32_t* __restrict__ bucket_start,
                                                         const int32_t* __restrict__ bucket_count,
                                                         const int32_t* __restrict__ sorted_id,
                                                         const float4* __restrict__ sorted_xyzr,
                                                         const float4* __restrict__ sorted_lo, float query_radius,
                                                         float rate, float dt, float* __restrict__ position,
                                                         float* __restrict__ position_lo, float* __restrict__ velocity,
                                                         int32_t* __restrict__ neighbor_count) {
    const float4 me = sorted_xyzr[t];
    const float4 ml = sorted_lo[t];
    const int i = sorted_id[t];
    const int cx = map.coord(me.x), cy = map.coord(me.y), cz = map.coord(me.z);
    const float cut2 = cutoff_squared_above(query_radius);
    float vx = 0.0f, vy = 0.0f, vz = 0.0f;
    int count = 0;
    for (int ox = -1; ox <= 1; ++ox)
        for (int oy = -1; oy <= 1; ++oy)
            for (int oz = -1; oz <= 1; ++oz) {
                const int b = map.bucket(cx + ox, cy + oy, cz + oz);
                const int s = bucket_start[b];
                const int e = s + bucket_count[b];
                for (int u = s; u < e; ++u) {
                    if (u == t) continue;
                    const float4 q = sorted_xyzr[u];
                    const float4 ql = sorted_lo[u];
                    const float dx = (me.x - q.x) + (ml.x - ql.x);
                    const float dy = (me.y - q.y) + (ml.y - ql.y);
                    const float dz = (me.z - q.z) + (ml.z - ql.z);
                    const float d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 >= cut2) continue;
                    const float d = sqrtf(d2);
                    if (d < query_radius) {
                        ++count;
                        const float overlap = me.w + q.w - d;
                        if (overlap > 0.0f && d > 1.0e-6f) {
                            const float f = rate * overlap / d;
                            vx = vx + f * dx;
                            vy = vy + f * dy;
                            vz = vz + f * dz;
                        }
                    }
                }
            }
    const int64_t o = 3 * static_cast<int64_t>(i);
    velocity[o + 0] = vx;
    velocity[o + 1] = vy;
    velocity[o + 2] = vz;
    neighbor_count[i] = count;
    float hx = me.x, hy = me.y, hz = me.z, lx = ml.x, ly = ml.y, lz = ml.z;
    add_compensated(hx, lx, vx * dt);
    add_compensated(hy, ly, vy * dt);
    add_compensated(hz, lz, vz * dt);
    position[o + 0] = hx;
    position[o + 1] = hy;
    position[o + 2] = hz;
    position_lo[o + 0] = lx;
    position_lo[o + 1] = ly;
    position_lo[o + 2] = lz;
}

// adjoint_contact_slot (wbc_bodies.cuh) with compensated positions.
__device__ __forceinline__ float adjoint_slot_compensated(BucketMap map, int t, const int32_t* __restrict__ bucket_start,
                                                          const int32_t* __restrict__ bucket_count,
                                                          const int32_t* __restrict__ sorted_id,
                                                          const float4* __restrict__ sorted_xyzr,
                                                          const float4* __restrict__ sorted_lo, float query_radius,
                                                          float rate, float dt, const float* __restrict__ lambda_in,
                                                          float* __restrict__ lambda_out) {
    const float4 me = sorted_xyzr[t];
    const float4 ml = sorted_lo[t];
    const int i = sorted_id[t];
    const float lix = lambda_in[3 * static_cast<int64_t>(i)], liy = lambda_in[3 * static_cast<int64_t>(i) + 1],
                liz = lambda_in[3 * static_cast<int64_t>(i) + 2];
    const int cx = map.coord(me.x), cy = map.coord(me.y), cz = map.coord(me.z);
    const float cut2 = cutoff_squared_above(query_radius);
    float gx = 0.0f, gy = 0.0f, gz = 0.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
    for (int ox = -1; ox <= 1; ++ox)
        for (int oy = -1; oy <= 1; ++oy)
            for (int oz = -1; oz <= 1; ++oz) {
                const int b = map.bucket(cx + ox, cy + oy, cz + oz);
                const int s = bucket_start[b];
                const int e = s + bucket_count[b];
                for (int u = s; u < e; ++u) {
                    if (u == t) continue;
                    const float4 q = sorted_xyzr[u];
                    const float4 ql = sorted_lo[u];
                    const float dx = (me.x - q.x) + (ml.x - ql.x);
                    const float dy = (me.y - q.y) + (ml.y - ql.y);
                    const float dz = (me.z - q.z) + (ml.z - ql.z);
                    const float d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 >= cut2) continue;
                    const float d = sqrtf(d2);
                    if (!(d < query_radius)) continue;
                    const float R = me.w + q.w;
                    if (!(R - d > 0.0f && d > 1.0e-6f)) continue;
                    const float inv_d = 1.0f / d;
                    const float a = R * inv_d - 1.0f;
                    ux += a * dx;
                    uy += a * dy;
                    uz += a * dz;
                    const int j = sorted_id[u];
                    const float ldx = lix - lambda_in[3 * static_cast<int64_t>(j)];
                    const float ldy = liy - lambda_in[3 * static_cast<int64_t>(j) + 1];
                    const float ldz = liz - lambda_in[3 * static_cast<int64_t>(j) + 2];
                    const float proj = R * inv_d * inv_d * inv_d * (dx * ldx + dy * ldy + dz * ldz);
                    gx += a * ldx - proj * dx;
                    gy += a * ldy - proj * dy;
                    gz += a * ldz - proj * dz;
                }
            }
    const float f = dt * rate;
    const int64_t o = 3 * static_cast<int64_t>(i);
    lambda_out[o] = lix + f * gx;
    lambda_out[o + 1] = liy + f * gy;
    lambda_out[o + 2] = liz + f * gz;
    return lix * ux + liy * uy + liz * uz;
}

template <bool COMP>
__global__ void __launch_bounds__(kStepThreads) k_contact_steps(StepsArgs a) {
    unsigned int epoch = 0;
    const int64_t gtid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t gthreads = static_cast<int64_t>(gridDim.x) * blockDim.x;
    bool ok = true;
    {
        const GridSlot g0 = slot_of(a, slot_for(a, 0));
        for (int64_t b = gtid; b < a.buckets; b += gthreads) g0.count[b] = 0;
    }
    ok = step_barrier(a.sync, epoch);
    for (int t = 0; ok && t < a.steps; ++t) {
        const GridSlot g = slot_of(a, slot_for(a, t));
        // x_t to its checkpoint; counts; the next step's counts cleared
        if (a.checkpoints && t % a.every == 0) {
            float* cp = a.checkpoints + static_cast<int64_t>(t / a.every) * 3 * a.n;
            for (int64_t q = gtid; q < 3 * static_cast<int64_t>(a.n); q += gthreads) cp[q] = a.position[q];
            if (COMP) {
                float* cl = a.checkpoints_lo + static_cast<int64_t>(t / a.every) * 3 * a.n;
                for (int64_t q = gtid; q < 3 * static_cast<int64_t>(a.n); q += gthreads) cl[q] = a.position_lo[q];
            }
        }
        for (int64_t i = gtid; i < a.n; i += gthreads)
            bin_assign_cell(a.map, static_cast<int>(i), a.position, g.count, a.cell_bucket, a.cell_rank);
        if (t + 1 < a.steps) {
            const GridSlot gn = slot_of(a, slot_for(a, t + 1));
            for (int64_t b = gtid; b < a.buckets; b += gthreads) gn.count[b] = 0;
        }
        if (!(ok = step_barrier(a.sync, epoch))) break;
        // exclusive scan of the counts: tile sums, their offsets, then each tile from its offset
        for (int64_t tile = blockIdx.x; tile < a.tiles; tile += gridDim.x) {
            const int64_t base = tile * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
            int32_t s = 0;
#pragma unroll
            for (int k = 0; k < kScanItems; ++k)
                if (base + k < a.buckets) s += g.count[base + k];
            int32_t total;
            block_exclusive(s, &total);
            if (threadIdx.x == 0) a.partials[tile] = total;
        }
        if (!(ok = step_barrier(a.sync, epoch))) break;
        if (blockIdx.x == 0) {
            int32_t carry = 0;
            for (int64_t base = 0; base < a.tiles; base += kScanThreads) {
                const int64_t idx = base + threadIdx.x;
                const int32_t v = idx < a.tiles ? a.partials[idx] : 0;
                int32_t chunk_total;
                const int32_t ex = block_exclusive(v, &chunk_total);
                if (idx < a.tiles) a.partials[idx] = carry + ex;
                carry += chunk_total;
            }
        }
        if (!(ok = step_barrier(a.sync, epoch))) break;
        for (int64_t tile = blockIdx.x; tile < a.tiles; tile += gridDim.x) {
            const int64_t base = tile * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
            int32_t vals[kScanItems];
            int32_t s = 0;
#pragma unroll
            for (int k = 0; k < kScanItems; ++k) {
                vals[k] = base + k < a.buckets ? g.count[base + k] : 0;
                s += vals[k];
            }
            int32_t total;
            int32_t run = block_exclusive(s, &total) + a.partials[tile];
#pragma unroll
            for (int k = 0; k < kScanItems; ++k) {
                if (base + k < a.buckets) g.start[base + k] = run;
                run += vals[k];
            }
        }
        if (!(ok = step_barrier(a.sync, epoch))) break;
        for (int64_t i = gtid; i < a.n; i += gthreads)
            bin_scatter_cell(static_cast<int>(i), a.cell_bucket, a.cell_rank, g.start, a.scatter);
        if (!(ok = step_barrier(a.sync, epoch))) break;
        for (int64_t i = gtid; i < a.n; i += gthreads) {
            if (COMP)
                order_cell_compensated(static_cast<int>(i), a.position, a.position_lo, a.radius, a.cell_bucket,
                                       g.start, g.count, a.scatter, g.sorted_id, g.sorted_xyzr,
                                       slot_lo_of(a, slot_for(a, t)));
            else
                bin_order_cell(static_cast<int>(i), a.position, a.radius, a.cell_bucket, g.start, g.count, a.scatter,
                               g.sorted_id, g.sorted_xyzr);
        }
        if (!(ok = step_barrier(a.sync, epoch))) break;
        if (a.last_build_only && t + 1 == a.steps) break;
        for (int64_t q = gtid; q < a.n; q += gthreads) {
            if (COMP)
                contact_slot_compensated(a.map, static_cast<int>(q), g.start, g.count, g.sorted_id, g.sorted_xyzr,
                                         slot_lo_of(a, slot_for(a, t)), a.query_radius, a.rate, a.dt, a.position,
                                         a.position_lo, a.velocity, a.neighbor_count);
            else
                contact_slot<false>(a.map, static_cast<int>(q), g.start, g.count, g.sorted_id, g.sorted_xyzr,
                                    a.query_radius, a.rate, a.dt, a.position, a.velocity, a.neighbor_count);
        }
        if (!(ok = step_barrier(a.sync, epoch))) break;
    }
    if (!ok && blockIdx.x == 0 && threadIdx.x == 0) a.sync->status = 1;
}

struct AdjointStepsArgs {
    BucketMap map;
    int32_t n, steps;
    float query_radius, rate, dt;
    float* lambda;      // dL/dx_steps on entry, dL/dx_0 on return
    float* lambda_tmp;  // ping-pong buffer
    double* rate_dot;   // += sum_t sum_i lambda_{t+1,i} . v_i(x_t) / rate
    int32_t* slot_ints;
    int32_t* slot_ids;
    float4* slot_xyzr;
    int64_t buckets, capacity;
    StepSync* sync;
    const float4* slot_lo;  // compensated positions' low parts per slot (NULL: plain positions)
};

// The reverse of `steps` contact steps whose grids sit in history slots 0 .. steps - 1.
template <bool COMP>
__global__ void __launch_bounds__(kStepThreads) k_adjoint_steps(AdjointStepsArgs a) {
    __shared__ double s_sum[kStepThreads / 32];
    unsigned int epoch = 0;
    const int64_t gtid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t gthreads = static_cast<int64_t>(gridDim.x) * blockDim.x;
    double acc = 0.0;
    bool ok = true;
    for (int t = a.steps - 1; t >= 0; --t) {
        const int32_t* count = a.slot_ints + static_cast<int64_t>(t) * 2 * a.buckets;
        const int32_t* start = count + a.buckets;
        const int32_t* ids = a.slot_ids + static_cast<int64_t>(t) * a.capacity;
        const float4* xyzr = a.slot_xyzr + static_cast<int64_t>(t) * a.capacity;
        // step t reads lambda_{t+1} and writes lambda_t: into `lambda` for even t, so that step 0
        // leaves dL/dx_0 there (the host puts dL/dx_steps in the buffer step steps - 1 reads)
        const bool into_main = (t % 2) == 0;
        const float* in = into_main ? a.lambda_tmp : a.lambda;
        float* out = into_main ? a.lambda : a.lambda_tmp;
        for (int64_t q = gtid; q < a.n; q += gthreads) {
            int cell;
            if (COMP)
                acc += static_cast<double>(adjoint_slot_compensated(a.map, static_cast<int>(q), start, count, ids, xyzr,
                                                                    a.slot_lo + static_cast<int64_t>(t) * a.capacity,
                                                                    a.query_radius, a.rate, a.dt, in, out));
            else
                acc += static_cast<double>(adjoint_contact_slot(a.map, static_cast<int>(q), start, count, ids, xyzr,
                                                                a.query_radius, a.rate, a.dt, in, out, &cell));
        }
        if (!(ok = step_barrier(a.sync, epoch))) break;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
    if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double total = 0.0;
        for (int w = 0; w < kStepThreads / 32; ++w) total += s_sum[w];
        atomicAdd(a.rate_dot, total);
        if (!ok) a.sync->status = 1;
    }
}

struct StepsLayout {
    size_t sync, partials, ints, ids, xyzr, lo, bytes;
};

StepsLayout steps_layout(int64_t buckets, int64_t capacity, int slots) {
    auto up = [](size_t v) { return (v + 255) / 256 * 256; };
    StepsLayout L{};
    const int64_t tiles = (buckets + kScanTile - 1) / kScanTile;
    L.sync = 0;
    L.partials = up(sizeof(StepSync));
    L.ints = L.partials + up((tiles + 1) * sizeof(int32_t));
    L.ids = L.ints + up(static_cast<size_t>(slots) * 2 * buckets * sizeof(int32_t));
    L.xyzr = L.ids + up(static_cast<size_t>(slots) * capacity * sizeof(int32_t));
    L.lo = L.xyzr + up(static_cast<size_t>(slots) * capacity * sizeof(float4));
    L.bytes = L.lo + up(static_cast<size_t>(slots) * capacity * sizeof(float4));
    return L;
}

int step_blocks(const void* fn) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kStepThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return std::min(kMaxStepBlocks, sms * std::min(per_sm, 2));
}

BucketMap steps_map(const wbc_neighbor_grid* g) {
    BucketMap m;
    m.inv_edge = 1.0f / (g->cell_size * 1.0009765625f);
    m.dim = g->dim;
    return m;
}

int read_status(StepSync* sync, cudaStream_t s, const char* where) {
    int status = 0;
    cudaError_t err = cudaMemcpyAsync(&status, &sync->status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) {
        set_error(where, err);
        return WBC_ERR_CUDA;
    }
    if (status != 0) {
        set_error_msg("a grid barrier of the contact steps timed out");
        return WBC_ERR_TIMEOUT;
    }
    return WBC_OK;
}

}  // namespace
}  // namespace wbc

using namespace wbc;

extern "C" {

size_t wbc_contact_steps_workspace_bytes(int32_t dim, int64_t capacity, int32_t slots) {
    if (dim < 3 || capacity < 0 || slots < 2) return 0;
    const int64_t buckets = static_cast<int64_t>(dim) * dim * dim;
    return steps_layout(buckets, capacity, slots).bytes;
}

int wbc_contact_steps(const wbc_neighbor_grid* grid, int32_t n, float query_radius, float rate, float dt,
                      int32_t steps, float* position, float* position_lo, const float* radius, float* velocity,
                      int32_t* neighbor_count, float* checkpoints, float* checkpoints_lo, int32_t checkpoint_every,
                      int32_t slots, int32_t history, int32_t last_build_only, void* workspace,
                      size_t workspace_bytes, int32_t sync_status, void* stream) {
    if (!grid || n < 0 || n > grid->capacity || steps < 0 || slots < 2 || !workspace ||
        (n > 0 && (!position || !radius || !velocity || !neighbor_count)) || (history && steps > slots) ||
        (checkpoints && checkpoint_every < 1) || !grid->cell_bucket || !grid->cell_rank || !grid->scatter ||
        (position_lo && checkpoints && !checkpoints_lo))
        return WBC_ERR_INVALID;
    if (!(query_radius <= grid->cell_size)) {
        set_error_msg("wbc_contact_steps: query_radius exceeds the grid's cell_size");
        return WBC_ERR_INVALID;
    }
    const int64_t buckets = static_cast<int64_t>(grid->dim) * grid->dim * grid->dim;
    const StepsLayout L = steps_layout(buckets, grid->capacity, slots);
    if (workspace_bytes < L.bytes || reinterpret_cast<uintptr_t>(workspace) % 256 != 0) return WBC_ERR_WORKSPACE;
    if (steps == 0 || n == 0) return WBC_OK;
    const int64_t tiles = (buckets + kScanTile - 1) / kScanTile;
    char* base = static_cast<char*>(workspace);
    StepsArgs a{};
    a.map = steps_map(grid);
    a.n = n;
    a.steps = steps;
    a.query_radius = query_radius;
    a.rate = rate;
    a.dt = dt;
    a.position = position;
    a.radius = radius;
    a.velocity = velocity;
    a.neighbor_count = neighbor_count;
    a.cell_bucket = grid->cell_bucket;
    a.cell_rank = grid->cell_rank;
    a.scatter = grid->scatter;
    a.partials = reinterpret_cast<int32_t*>(base + L.partials);
    a.buckets = buckets;
    a.tiles = tiles;
    a.slot_ints = reinterpret_cast<int32_t*>(base + L.ints);
    a.slot_ids = reinterpret_cast<int32_t*>(base + L.ids);
    a.slot_xyzr = reinterpret_cast<float4*>(base + L.xyzr);
    a.capacity = grid->capacity;
    a.slots = slots;
    a.history = history ? 1 : 0;
    a.last_build_only = last_build_only ? 1 : 0;
    a.checkpoints = checkpoints;
    a.every = checkpoint_every > 0 ? checkpoint_every : 1;
    a.sync = reinterpret_cast<StepSync*>(base + L.sync);
    a.position_lo = position_lo;
    a.checkpoints_lo = checkpoints_lo;
    a.slot_lo = reinterpret_cast<float4*>(base + L.lo);
    cudaStream_t s = as_stream(stream);
    const void* fn = position_lo ? reinterpret_cast<const void*>(k_contact_steps<true>)
                                 : reinterpret_cast<const void*>(k_contact_steps<false>);
    const int blocks = step_blocks(fn);
    if (blocks < 1) {
        set_error_msg("wbc_contact_steps: the kernel does not fit on an SM");
        return WBC_ERR_CUDA;
    }
    cudaError_t err = cudaMemsetAsync(a.sync, 0, sizeof(StepSync), s);
    if (err != cudaSuccess) {
        set_error("wbc_contact_steps: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    void* params[] = {&a};
    err = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kStepThreads), params, 0, s);
    if (err != cudaSuccess) {
        set_error("wbc_contact_steps: cudaLaunchCooperativeKernel", err);
        return WBC_ERR_CUDA;
    }
    const int rc = check_launch("wbc_contact_steps", 1);
    if (rc != WBC_OK || !sync_status) return rc;
    return read_status(a.sync, s, "wbc_contact_steps: reading the status");
}

int wbc_adjoint_steps(const wbc_neighbor_grid* grid, int32_t n, float query_radius, float rate, float dt,
                      int32_t steps, int32_t compensated, float* lambda, float* lambda_tmp, double* rate_dot,
                      int32_t slots, void* workspace, size_t workspace_bytes, int32_t sync_status, void* stream) {
    if (!grid || n < 0 || n > grid->capacity || steps < 0 || steps > slots || slots < 2 || !workspace ||
        !rate_dot || (n > 0 && (!lambda || !lambda_tmp)) || lambda == lambda_tmp)
        return WBC_ERR_INVALID;
    const int64_t buckets = static_cast<int64_t>(grid->dim) * grid->dim * grid->dim;
    const StepsLayout L = steps_layout(buckets, grid->capacity, slots);
    if (workspace_bytes < L.bytes || reinterpret_cast<uintptr_t>(workspace) % 256 != 0) return WBC_ERR_WORKSPACE;
    if (steps == 0 || n == 0) return WBC_OK;
    char* base = static_cast<char*>(workspace);
    AdjointStepsArgs a{};
    a.map = steps_map(grid);
    a.n = n;
    a.steps = steps;
    a.query_radius = query_radius;
    a.rate = rate;
    a.dt = dt;
    a.lambda = lambda;
    a.lambda_tmp = lambda_tmp;
    a.rate_dot = rate_dot;
    a.slot_ints = reinterpret_cast<int32_t*>(base + L.ints);
    a.slot_ids = reinterpret_cast<int32_t*>(base + L.ids);
    a.slot_xyzr = reinterpret_cast<float4*>(base + L.xyzr);
    a.buckets = buckets;
    a.capacity = grid->capacity;
    a.sync = reinterpret_cast<StepSync*>(base + L.sync);
    a.slot_lo = compensated ? reinterpret_cast<const float4*>(base + L.lo) : nullptr;
    cudaStream_t s = as_stream(stream);
    const void* fn = compensated ? reinterpret_cast<const void*>(k_adjoint_steps<true>)
                                 : reinterpret_cast<const void*>(k_adjoint_steps<false>);
    const int blocks = step_blocks(fn);
    if (blocks < 1) {
        set_error_msg("wbc_adjoint_steps: the kernel does not fit on an SM");
        return WBC_ERR_CUDA;
    }
    // The first reverse step reads lambda_{steps}: it must sit in the buffer the kernel reads first.
    if ((steps - 1) % 2 == 0) {
        cudaError_t err = cudaMemcpyAsync(lambda_tmp, lambda, 3 * static_cast<size_t>(n) * sizeof(float),
                                          cudaMemcpyDeviceToDevice, s);
        if (err != cudaSuccess) {
            set_error("wbc_adjoint_steps: cudaMemcpyAsync", err);
            return WBC_ERR_CUDA;
        }
    }
    cudaError_t err = cudaMemsetAsync(a.sync, 0, sizeof(StepSync), s);
    if (err != cudaSuccess) {
        set_error("wbc_adjoint_steps: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    void* params[] = {&a};
    err = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kStepThreads), params, 0, s);
    if (err != cudaSuccess) {
        set_error("wbc_adjoint_steps: cudaLaunchCooperativeKernel", err);
        return WBC_ERR_CUDA;
    }
    const int rc = check_launch("wbc_adjoint_steps", 1);
    if (rc != WBC_OK || !sync_status) return rc;
    return read_status(a.sync, s, "wbc_adjoint_steps: reading the status");
}

}  // extern "C"
