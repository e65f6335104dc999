// Batched coupled steps: many independent spheroids (each with its own population, hash grid and
// oxygen grid) advanced together, one launch per stage for the whole batch.
//
// Every launch walks a static work list (chunks of 256 cells over each instance's capacity,
// chunks of 256 nodes, scan tiles over each instance's buckets or slots); a block finds its
// instance by a binary search over the per-instance chunk offsets, reads the instance's cell count
// from device memory and runs the same per-thread body as the single-population kernel
// (wbc_bodies.cuh), so every instance's results are bit-identical to a plain run of it. Nothing
// here reads a count back to the host, so a whole step can be captured in a CUDA graph: a
// division that would overflow an instance's capacity is not placed and sets that instance's
// status instead of raising.
#include <algorithm>
#include <cstring>
#include <vector>

#include "wbc_bodies.cuh"

namespace wbc {

constexpr int kChunk = 256;

// The device plan: the instance descriptors, then the work-list offsets, then scan scratch.
struct BatchPlan {
    const wbc_batch_instance* inst;
    const int32_t* cell_first;    // [n + 1] cell chunks
    const int32_t* node_first;    // [n + 1] node chunks
    const int32_t* bucket_first;  // [n + 1] scan tiles over buckets
    const int32_t* slot_first;    // [n + 1] scan tiles over slots (division scan)
    int32_t* bucket_partials;     // [bucket tiles + n]
    int32_t* slot_partials;       // [slot tiles + n]
    int32_t* totals;              // [n] daughters per instance this step
    int32_t n;
};

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct PlanLayout {
    size_t inst, cell_first, node_first, bucket_first, slot_first, bucket_partials, slot_partials, totals, bytes;
};

static int64_t buckets_of(const wbc_batch_instance& b) {
    return static_cast<int64_t>(b.grid.dim) * b.grid.dim * b.grid.dim;
}

static int64_t nodes_of(const wbc_batch_instance& b) {
    return static_cast<int64_t>(b.geom.nx) * b.geom.ny * b.geom.nz;
}

static PlanLayout plan_layout(int n, int32_t bucket_tiles, int32_t slot_tiles) {
    PlanLayout L{};
    size_t off = 0;
    L.inst = off;
    off = align_up(off + n * sizeof(wbc_batch_instance), 256);
    L.cell_first = off;
    off += (n + 1) * sizeof(int32_t);
    L.node_first = off;
    off += (n + 1) * sizeof(int32_t);
    L.bucket_first = off;
    off += (n + 1) * sizeof(int32_t);
    L.slot_first = off;
    off = align_up(off + (n + 1) * sizeof(int32_t), 256);
    L.bucket_partials = off;
    off = align_up(off + (static_cast<size_t>(bucket_tiles) + n) * sizeof(int32_t), 256);
    L.slot_partials = off;
    off = align_up(off + (static_cast<size_t>(slot_tiles) + n) * sizeof(int32_t), 256);
    L.totals = off;
    off = align_up(off + n * sizeof(int32_t), 256);
    L.bytes = off;
    return L;
}

static bool offsets(int n, const wbc_batch_instance* insts, std::vector<int32_t>& cell, std::vector<int32_t>& node,
                    std::vector<int32_t>& bucket, std::vector<int32_t>& slot) {
    cell.assign(n + 1, 0);
    node.assign(n + 1, 0);
    bucket.assign(n + 1, 0);
    slot.assign(n + 1, 0);
    for (int b = 0; b < n; ++b) {
        const int64_t c = (insts[b].capacity + kChunk - 1) / kChunk;
        const int64_t d = (nodes_of(insts[b]) + kChunk - 1) / kChunk;
        const int64_t t = (buckets_of(insts[b]) + kScanTile - 1) / kScanTile;
        const int64_t u = (insts[b].capacity + kScanTile - 1) / kScanTile;
        const int64_t lim = 0x7fffffff;
        if (cell[b] + c > lim || node[b] + d > lim || bucket[b] + t > lim || slot[b] + u > lim) return false;
        cell[b + 1] = static_cast<int32_t>(cell[b] + c);
        node[b + 1] = static_cast<int32_t>(node[b] + d);
        bucket[b + 1] = static_cast<int32_t>(bucket[b] + t);
        slot[b + 1] = static_cast<int32_t>(slot[b] + u);
    }
    return true;
}

__device__ __forceinline__ int find_item(const int32_t* first, int n, int x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= x)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ BucketMap map_of(const wbc_neighbor_grid& g) {
    BucketMap m;
    m.inv_edge = 1.0f / (g.cell_size * 1.0009765625f);  // as make_map() rounds it on the host
    m.dim = g.dim;
    return m;
}

// ---- per-cell stages ----------------------------------------------------------------------------
// The cell work list: chunk c is slots [(c - cell_first[b]) * 256, + 256) of instance b.
#define WBC_CELL_LOOP                                                          \
    for (int c = blockIdx.x; c < P.cell_first[P.n]; c += gridDim.x) {          \
        const int b = find_item(P.cell_first, P.n, c);                         \
        const int i = (c - P.cell_first[b]) * kChunk + static_cast<int>(threadIdx.x); \
        const wbc_batch_instance& I = P.inst[b];                               \
        if (i >= counts[b]) continue;

__global__ void __launch_bounds__(kChunk) k_b_bin_assign(BatchPlan P, const int32_t* __restrict__ counts) {
    WBC_CELL_LOOP
        bin_assign_cell(map_of(I.grid), i, I.position, I.grid.bucket_count, I.grid.cell_bucket, I.grid.cell_rank);
    }
}

__global__ void __launch_bounds__(kChunk) k_b_bin_scatter(BatchPlan P, const int32_t* __restrict__ counts) {
    WBC_CELL_LOOP
        bin_scatter_cell(i, I.grid.cell_bucket, I.grid.cell_rank, I.grid.bucket_start, I.grid.scatter);
    }
}

__global__ void __launch_bounds__(kChunk) k_b_bin_order(BatchPlan P, const int32_t* __restrict__ counts) {
    WBC_CELL_LOOP
        bin_order_cell(i, I.position, I.radius, I.grid.cell_bucket, I.grid.bucket_start, I.grid.bucket_count,
                       I.grid.scatter, I.grid.sorted_id, reinterpret_cast<float4*>(I.grid.sorted_xyzr));
    }
}

__global__ void __launch_bounds__(kChunk) k_b_contact(BatchPlan P, const int32_t* __restrict__ counts) {
    WBC_CELL_LOOP
        const BucketMap map = map_of(I.grid);
        const int32_t* bucket_start = I.grid.bucket_start;
        const int32_t* bucket_count = I.grid.bucket_count;
        const int32_t* sorted_id = I.grid.sorted_id;
        const float4* sorted_xyzr = reinterpret_cast<const float4*>(I.grid.sorted_xyzr);
        const float query_radius = I.query_radius, rate = I.contact_rate, dt = I.contact_dt;
        float* position = I.position;
        float* velocity = I.velocity;
        int32_t* neighbor_count = I.neighbor_count;
        contact_slot(map, i, bucket_start, bucket_count, sorted_id, sorted_xyzr, query_radius, rate, dt, position,
                     velocity, neighbor_count);
    }
}

// An instance's 32-bit accumulator (the layout of wbc_deposit32): low words, wrap counts, carry.
struct Acc32 {
    uint32_t* lo;
    uint32_t* count;
    uint32_t* carry;
};
__device__ __forceinline__ Acc32 acc32_of(const wbc_batch_instance& I) {
    const int64_t nodes = static_cast<int64_t>(I.geom.nx) * I.geom.ny * I.geom.nz;
    uint32_t* lo = static_cast<uint32_t*>(I.accumulator);
    return Acc32{lo, lo + 4 * nodes, lo + 8 * nodes};
}

__global__ void __launch_bounds__(kChunk) k_b_deposit(BatchPlan P, const int32_t* __restrict__ counts) {
    WBC_CELL_LOOP
        const Acc32 A = acc32_of(I);
        deposit32_cell(I.geom, i, I.position, I.cell_state, A.lo, A.count, A.carry);
    }
}

__global__ void __launch_bounds__(kChunk) k_b_sample(BatchPlan P, const int32_t* __restrict__ counts) {
    WBC_CELL_LOOP
        sample_cell(I.geom, I.field, i, I.position, I.oxygen_local);
    }
}

__global__ void __launch_bounds__(kChunk) k_b_lifecycle_decide(BatchPlan P, const int32_t* __restrict__ counts) {
    WBC_CELL_LOOP
        lifecycle_cell(I.lifecycle, i, I.cell_state, I.age, I.neighbor_count, I.oxygen_local, I.glucose_local,
                       I.fate_flags, I.rng_state, I.divide_flag);
    }
}

// Daughters of an instance are placed only if they fit its capacity; otherwise its status says so.
__global__ void __launch_bounds__(kChunk) k_b_place(BatchPlan P, const int32_t* __restrict__ counts) {
    WBC_CELL_LOOP
        const int count = counts[b];
        if (I.divide_flag[i] != 0 && count + P.totals[b] <= I.capacity)
            place_daughter(i, count, I.placement_factor, I.division_offset, I.position, I.radius, I.cell_state,
                           I.cell_type, I.age, I.oxygen_local, I.glucose_local, I.rng_state, I.velocity,
                           I.neighbor_count, I.fate_flags);
    }
}

__global__ void k_b_commit(BatchPlan P, int32_t* __restrict__ counts, int32_t* __restrict__ status) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P.n) return;
    const int total = P.totals[b];
    if (counts[b] + total <= P.inst[b].capacity) {
        counts[b] += total;
    } else if (status) {
        status[b] = WBC_ERR_CAPACITY;
    }
}

#undef WBC_CELL_LOOP

// ---- per-node stage --------------------------------------------------------------------------------
// Zeroes every instance's low words, and its wrap counts when its previous deposit wrapped.
__global__ void __launch_bounds__(kChunk) k_b_clear32(BatchPlan P) {
    for (int c = blockIdx.x; c < P.node_first[P.n]; c += gridDim.x) {
        const int b = find_item(P.node_first, P.n, c);
        const wbc_batch_instance& I = P.inst[b];
        const int64_t nodes = static_cast<int64_t>(I.geom.nx) * I.geom.ny * I.geom.nz;
        const int64_t node = static_cast<int64_t>(c - P.node_first[b]) * kChunk + threadIdx.x;
        if (node >= nodes) continue;
        const Acc32 A = acc32_of(I);
        const bool wrapped = *A.carry != 0u;
#pragma unroll
        for (int st = 0; st < 4; ++st) {
            A.lo[st * nodes + node] = 0u;
            if (wrapped) A.count[st * nodes + node] = 0u;
        }
    }
}

// Clears the carry flags once every clear has read them.
__global__ void k_b_reset_carry(BatchPlan P) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < P.n) *acc32_of(P.inst[b]).carry = 0u;
}

// The solver's combined uptake density of every instance from its deposit; the per-state densities
// are left to be converted from the same sums when they are read.
__global__ void __launch_bounds__(kChunk) k_b_convert(BatchPlan P) {
    for (int c = blockIdx.x; c < P.node_first[P.n]; c += gridDim.x) {
        const int b = find_item(P.node_first, P.n, c);
        const wbc_batch_instance& I = P.inst[b];
        const int64_t nodes = static_cast<int64_t>(I.geom.nx) * I.geom.ny * I.geom.nz;
        const int64_t node = static_cast<int64_t>(c - P.node_first[b]) * kChunk + threadIdx.x;
        if (node >= nodes) continue;
        const Acc32 A = acc32_of(I);
        convert32_node(nodes, node, A.lo, A.count, *A.carry != 0u, I.inv_voxel_volume, nullptr, I.uptake_weights[0],
                       I.uptake_weights[1], I.uptake_weights[2], I.uptake_weights[3], I.uptake_density);
    }
}

// ---- segmented scans ----------------------------------------------------------------------------
// Each instance's segment: in[0, n) -> out (exclusive for buckets, inclusive for divisions), its
// tile partials at partials + first[b] + b, and optionally its total.
struct Segment {
    const int32_t* in;
    int32_t* out;
    int64_t n;
    int32_t* partials;
    int32_t* total;
};

struct BucketSegments {
    static constexpr bool kInclusive = false;
    __device__ static const int32_t* first(const BatchPlan& P) { return P.bucket_first; }
    __device__ static Segment get(const BatchPlan& P, const int32_t*, int b) {
        const wbc_batch_instance& I = P.inst[b];
        const int64_t n = static_cast<int64_t>(I.grid.dim) * I.grid.dim * I.grid.dim;
        return Segment{I.grid.bucket_count, I.grid.bucket_start, n, P.bucket_partials + P.bucket_first[b] + b,
                       nullptr};
    }
};

struct DivisionSegments {
    static constexpr bool kInclusive = true;
    __device__ static const int32_t* first(const BatchPlan& P) { return P.slot_first; }
    __device__ static Segment get(const BatchPlan& P, const int32_t* counts, int b) {
        const wbc_batch_instance& I = P.inst[b];
        return Segment{I.divide_flag, I.division_offset, counts[b], P.slot_partials + P.slot_first[b] + b,
                       P.totals + b};
    }
};

template <class S>
__global__ void __launch_bounds__(kScanThreads) k_b_scan_reduce(BatchPlan P, const int32_t* __restrict__ counts) {
    const int32_t* first = S::first(P);
    for (int t = blockIdx.x; t < first[P.n]; t += gridDim.x) {
        const int b = find_item(first, P.n, t);
        const Segment g = S::get(P, counts, b);
        const int local = t - first[b];
        const int64_t base = static_cast<int64_t>(local) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
        int32_t vals[kScanItems];
        load_items(g.in, base, g.n, vals);
        int32_t s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) s += vals[k];
        int32_t total;
        block_exclusive(s, &total);
        if (threadIdx.x == 0) g.partials[local] = total;
    }
}

// One block per instance: exclusive offsets of its tiles, its total after them.
template <class S>
__global__ void __launch_bounds__(kScanThreads) k_b_scan_partials(BatchPlan P, const int32_t* __restrict__ counts) {
    const int32_t* first = S::first(P);
    for (int b = blockIdx.x; b < P.n; b += gridDim.x) {
        const Segment g = S::get(P, counts, b);
        const int tiles = first[b + 1] - first[b];
        int32_t carry = 0;
        for (int base = 0; base < tiles; base += kScanThreads) {
            const int idx = base + threadIdx.x;
            const int32_t v = idx < tiles ? g.partials[idx] : 0;
            int32_t chunk_total;
            const int32_t ex = block_exclusive(v, &chunk_total);
            if (idx < tiles) g.partials[idx] = carry + ex;
            carry += chunk_total;
        }
        if (threadIdx.x == 0) {
            g.partials[tiles] = carry;
            if (g.total) *g.total = carry;
        }
        __syncthreads();
    }
}

template <class S>
__global__ void __launch_bounds__(kScanThreads) k_b_scan_apply(BatchPlan P, const int32_t* __restrict__ counts) {
    const int32_t* first = S::first(P);
    for (int t = blockIdx.x; t < first[P.n]; t += gridDim.x) {
        const int b = find_item(first, P.n, t);
        const Segment g = S::get(P, counts, b);
        const int local = t - first[b];
        const int64_t base = static_cast<int64_t>(local) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
        int32_t vals[kScanItems];
        load_items(g.in, base, g.n, vals);
        int32_t s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) s += vals[k];
        int32_t total;
        int32_t run = block_exclusive(s, &total) + g.partials[local];
        int32_t res[kScanItems];
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (S::kInclusive) run += vals[k];
            res[k] = run;
            if (!S::kInclusive) run += vals[k];
        }
        store_items(g.out, base, g.n, res);
    }
}

// Zeroes every instance's bucket counts (one scan tile's worth per block).
__global__ void __launch_bounds__(kScanThreads) k_b_clear_buckets(BatchPlan P) {
    for (int t = blockIdx.x; t < P.bucket_first[P.n]; t += gridDim.x) {
        const int b = find_item(P.bucket_first, P.n, t);
        const wbc_batch_instance& I = P.inst[b];
        const int64_t n = static_cast<int64_t>(I.grid.dim) * I.grid.dim * I.grid.dim;
        const int64_t base = static_cast<int64_t>(t - P.bucket_first[b]) * kScanTile;
        for (int k = threadIdx.x; k < kScanTile; k += kScanThreads)
            if (base + k < n) I.grid.bucket_count[base + k] = 0;
    }
}

static BatchPlan plan_of(const wbc_batch* b) {
    const int n = b->instances;
    const PlanLayout L = plan_layout(n, b->bucket_tiles, b->slot_tiles);
    char* base = static_cast<char*>(b->device_plan);
    BatchPlan P;
    P.inst = reinterpret_cast<const wbc_batch_instance*>(base + L.inst);
    P.cell_first = reinterpret_cast<const int32_t*>(base + L.cell_first);
    P.node_first = reinterpret_cast<const int32_t*>(base + L.node_first);
    P.bucket_first = reinterpret_cast<const int32_t*>(base + L.bucket_first);
    P.slot_first = reinterpret_cast<const int32_t*>(base + L.slot_first);
    P.bucket_partials = reinterpret_cast<int32_t*>(base + L.bucket_partials);
    P.slot_partials = reinterpret_cast<int32_t*>(base + L.slot_partials);
    P.totals = reinterpret_cast<int32_t*>(base + L.totals);
    P.n = n;
    return P;
}

static bool batch_ok(const wbc_batch* b) { return b && b->instances > 0 && b->device_plan; }

static unsigned grid_of(int32_t work) { return static_cast<unsigned>(work > 0 ? work : 1); }

}  // namespace wbc

using namespace wbc;

extern "C" {

size_t wbc_batch_plan_bytes(int32_t n, const wbc_batch_instance* insts) {
    if (n <= 0 || !insts) return 0;
    std::vector<int32_t> cell, node, bucket, slot;
    if (!offsets(n, insts, cell, node, bucket, slot)) return 0;
    return plan_layout(n, bucket[n], slot[n]).bytes;
}

int wbc_batch_prepare(int32_t n, const wbc_batch_instance* insts, void* plan, size_t plan_bytes, wbc_batch* out,
                      void* stream) {
    if (n <= 0 || !insts || !plan || !out) return WBC_ERR_INVALID;
    for (int b = 0; b < n; ++b) {
        const wbc_batch_instance& I = insts[b];
        if (I.capacity < 0 || I.grid.dim < 3 || I.grid.dim > 1290 || !(I.grid.cell_size > 0.0f) ||
            I.grid.capacity < I.capacity || !(I.query_radius <= I.grid.cell_size) || I.contact_substeps < 1 ||
            I.geom.nx < 2 || I.geom.ny < 2 || I.geom.nz < 2 || !I.accumulator || !I.uptake_density || !I.field ||
            reinterpret_cast<uintptr_t>(I.accumulator) % 16 != 0) {
            set_error_msg("wbc_batch_prepare: invalid instance description");
            return WBC_ERR_INVALID;
        }
    }
    std::vector<int32_t> cell, node, bucket, slot;
    if (!offsets(n, insts, cell, node, bucket, slot)) {
        set_error_msg("wbc_batch_prepare: work list too long");
        return WBC_ERR_INVALID;
    }
    const PlanLayout L = plan_layout(n, bucket[n], slot[n]);
    if (plan_bytes < L.bytes) return WBC_ERR_WORKSPACE;
    std::vector<char> host(L.bytes, 0);
    std::memcpy(host.data() + L.inst, insts, n * sizeof(wbc_batch_instance));
    std::memcpy(host.data() + L.cell_first, cell.data(), (n + 1) * sizeof(int32_t));
    std::memcpy(host.data() + L.node_first, node.data(), (n + 1) * sizeof(int32_t));
    std::memcpy(host.data() + L.bucket_first, bucket.data(), (n + 1) * sizeof(int32_t));
    std::memcpy(host.data() + L.slot_first, slot.data(), (n + 1) * sizeof(int32_t));
    cudaStream_t s = as_stream(stream);
    cudaError_t err = cudaMemcpyAsync(plan, host.data(), L.bytes, cudaMemcpyHostToDevice, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);  // `host` goes out of scope
    if (err != cudaSuccess) {
        set_error("wbc_batch_prepare: copying the plan", err);
        return WBC_ERR_CUDA;
    }
    out->instances = n;
    out->device_plan = plan;
    out->cell_chunks = cell[n];
    out->node_chunks = node[n];
    out->bucket_tiles = bucket[n];
    out->slot_tiles = slot[n];
    int substeps = insts[0].contact_substeps;
    for (int b = 1; b < n; ++b) substeps = std::max(substeps, insts[b].contact_substeps);
    out->max_substeps = substeps;
    return WBC_OK;
}

int wbc_batch_grid_build(const wbc_batch* b, const int32_t* counts, void* stream) {
    if (!batch_ok(b) || !counts) return WBC_ERR_INVALID;
    const BatchPlan P = plan_of(b);
    cudaStream_t s = as_stream(stream);
    k_b_clear_buckets<<<grid_of(b->bucket_tiles), kScanThreads, 0, s>>>(P);
    k_b_bin_assign<<<grid_of(b->cell_chunks), kChunk, 0, s>>>(P, counts);
    k_b_scan_reduce<BucketSegments><<<grid_of(b->bucket_tiles), kScanThreads, 0, s>>>(P, counts);
    k_b_scan_partials<BucketSegments><<<grid_of(b->instances), kScanThreads, 0, s>>>(P, counts);
    k_b_scan_apply<BucketSegments><<<grid_of(b->bucket_tiles), kScanThreads, 0, s>>>(P, counts);
    k_b_bin_scatter<<<grid_of(b->cell_chunks), kChunk, 0, s>>>(P, counts);
    k_b_bin_order<<<grid_of(b->cell_chunks), kChunk, 0, s>>>(P, counts);
    return check_launch("wbc_batch_grid_build", 7);
}

int wbc_batch_contact(const wbc_batch* b, const int32_t* counts, void* stream) {
    if (!batch_ok(b) || !counts) return WBC_ERR_INVALID;
    k_b_contact<<<grid_of(b->cell_chunks), kChunk, 0, as_stream(stream)>>>(plan_of(b), counts);
    return check_launch("wbc_batch_contact");
}

int wbc_batch_deposit(const wbc_batch* b, const int32_t* counts, void* stream) {
    if (!batch_ok(b) || !counts) return WBC_ERR_INVALID;
    const BatchPlan P = plan_of(b);
    cudaStream_t s = as_stream(stream);
    k_b_clear32<<<grid_of(b->node_chunks), kChunk, 0, s>>>(P);
    k_b_reset_carry<<<grid_of((b->instances + 127) / 128), 128, 0, s>>>(P);
    k_b_deposit<<<grid_of(b->cell_chunks), kChunk, 0, s>>>(P, counts);
    k_b_convert<<<grid_of(b->node_chunks), kChunk, 0, s>>>(P);
    return check_launch("wbc_batch_deposit", 4);
}

int wbc_batch_sample(const wbc_batch* b, const int32_t* counts, void* stream) {
    if (!batch_ok(b) || !counts) return WBC_ERR_INVALID;
    k_b_sample<<<grid_of(b->cell_chunks), kChunk, 0, as_stream(stream)>>>(plan_of(b), counts);
    return check_launch("wbc_batch_sample");
}

int wbc_batch_lifecycle(const wbc_batch* b, int32_t* counts, int32_t* status, void* stream) {
    if (!batch_ok(b) || !counts) return WBC_ERR_INVALID;
    const BatchPlan P = plan_of(b);
    cudaStream_t s = as_stream(stream);
    k_b_lifecycle_decide<<<grid_of(b->cell_chunks), kChunk, 0, s>>>(P, counts);
    k_b_scan_reduce<DivisionSegments><<<grid_of(b->slot_tiles), kScanThreads, 0, s>>>(P, counts);
    k_b_scan_partials<DivisionSegments><<<grid_of(b->instances), kScanThreads, 0, s>>>(P, counts);
    k_b_scan_apply<DivisionSegments><<<grid_of(b->slot_tiles), kScanThreads, 0, s>>>(P, counts);
    k_b_place<<<grid_of(b->cell_chunks), kChunk, 0, s>>>(P, counts);
    k_b_commit<<<grid_of((b->instances + 127) / 128), 128, 0, s>>>(P, counts, status);
    return check_launch("wbc_batch_lifecycle", 6);
}

}  // extern "C"
