// Hash-grid binning and the fused contact substep (neighbour count + overlap repulsion + Euler
// integration).
//
// Binning: a counting sort of the active slots into dim^3 hashed buckets of edge
// cell_size * (1 + 2^-10) (the 0.1% widening keeps every pair closer than cell_size in adjacent
// buckets despite the rounding of x / edge). Within a bucket the slots are put in ascending
// order, so the order in which a cell visits its candidates — 27 buckets in (x, y, z) offset
// order, ascending slot inside each — is fixed by the positions alone. That fixes the float
// summation order of the velocity, which is what lets the CPU oracle reproduce positions bit
// for bit and keeps same-device runs bitwise reproducible.
//
// Reference: spatial/neighbors.py:33-37 (HashGrid build over the active prefix) and
// kernels/mechanics_kernels.py:26-67 (contact_velocities, integrate_positions).
#include "wbc_bodies.cuh"

namespace wbc {

// Host-side: the bucket edge and its inverse, rounded exactly as the oracle rounds them.
static BucketMap make_map(float cell_size, int dim) {
    float edge = cell_size * 1.0009765625f;
    BucketMap m;
    m.inv_edge = 1.0f / edge;
    m.dim = dim;
    return m;
}

__global__ void k_bin_assign(BucketMap map, int32_t n, const float* __restrict__ position,
                             int32_t* __restrict__ bucket_count, int32_t* __restrict__ cell_bucket,
                             int32_t* __restrict__ cell_rank) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) bin_assign_cell(map, i, position, bucket_count, cell_bucket, cell_rank);
}

__global__ void k_bin_scatter(int32_t n, const int32_t* __restrict__ cell_bucket, const int32_t* __restrict__ cell_rank,
                              const int32_t* __restrict__ bucket_start, int32_t* __restrict__ scatter) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) bin_scatter_cell(i, cell_bucket, cell_rank, bucket_start, scatter);
}

__global__ void k_bin_order(int32_t n, const float* __restrict__ position, const float* __restrict__ radius,
                            const int32_t* __restrict__ cell_bucket, const int32_t* __restrict__ bucket_start,
                            const int32_t* __restrict__ bucket_count, const int32_t* __restrict__ scatter,
                            int32_t* __restrict__ sorted_id, float4* __restrict__ sorted_xyzr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        bin_order_cell(i, position, radius, cell_bucket, bucket_start, bucket_count, scatter, sorted_id, sorted_xyzr);
}

// One thread per sorted slot t (so a warp works on neighbouring cells and shares buckets).
template <bool REGION>
__global__ void __launch_bounds__(256) k_contact(BucketMap map, int32_t n, const int32_t* __restrict__ bucket_start,
                                                 const int32_t* __restrict__ bucket_count,
                                                 const int32_t* __restrict__ sorted_id,
                                                 const float4* __restrict__ sorted_xyzr, float query_radius, float rate,
                                                 float dt, float* __restrict__ position, float* __restrict__ velocity,
                                                 int32_t* __restrict__ neighbor_count, wbc_tissue_region region) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n)
        contact_slot<REGION>(map, t, bucket_start, bucket_count, sorted_id, sorted_xyzr, query_radius, rate, dt,
                             position, velocity, neighbor_count, &region);
}

// Trilinear signed distance at each cell, positions clamped to the grid (geometry_kernels.py:46-56).
__global__ void k_sample_sdf(wbc_tissue_region R, int32_t n, const float* __restrict__ position,
                             float* __restrict__ out) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const float* p = position + 3 * static_cast<int64_t>(c);
    int i0, j0, k0;
    float fx, fy, fz;
    region_cell(R.geom, p[0], p[1], p[2], i0, j0, k0, fx, fy, fz);
    out[c] = region_sample(R.geom, R.sdf, 1, i0, j0, k0, fx, fy, fz);
}

static bool grid_ok(const wbc_neighbor_grid* g) {
    return g && g->dim >= 3 && g->dim <= 1290 && g->cell_size > 0.0f && g->bucket_count && g->bucket_start &&
           g->cell_bucket && g->cell_rank && g->scatter && g->sorted_id && g->sorted_xyzr && g->scan_partials;
}

}  // namespace wbc

using namespace wbc;

extern "C" {

int wbc_grid_build(const wbc_neighbor_grid* grid, int32_t n, const float* position, const float* radius,
                   void* stream) {
    if (!grid_ok(grid) || n < 0 || n > grid->capacity || (n > 0 && (!position || !radius))) return WBC_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const int64_t buckets = static_cast<int64_t>(grid->dim) * grid->dim * grid->dim;
    cudaError_t err = cudaMemsetAsync(grid->bucket_count, 0, buckets * sizeof(int32_t), s);
    if (err != cudaSuccess) {
        set_error("wbc_grid_build: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    if (n == 0) return scan_i32(grid->bucket_count, grid->bucket_start, buckets, false, grid->scan_partials, nullptr, s);
    BucketMap map = make_map(grid->cell_size, grid->dim);
    k_bin_assign<<<grid_for(n), kThreads, 0, s>>>(map, n, position, grid->bucket_count, grid->cell_bucket,
                                                  grid->cell_rank);
    int rc = scan_i32(grid->bucket_count, grid->bucket_start, buckets, false, grid->scan_partials, nullptr, s);
    if (rc != WBC_OK) return rc;
    k_bin_scatter<<<grid_for(n), kThreads, 0, s>>>(n, grid->cell_bucket, grid->cell_rank, grid->bucket_start,
                                                   grid->scatter);
    k_bin_order<<<grid_for(n), kThreads, 0, s>>>(n, position, radius, grid->cell_bucket, grid->bucket_start,
                                                 grid->bucket_count, grid->scatter, grid->sorted_id,
                                                 reinterpret_cast<float4*>(grid->sorted_xyzr));
    return check_launch("wbc_grid_build", 3);
}

int wbc_contact_substep(const wbc_neighbor_grid* grid, int32_t n, float query_radius, float rate, float dt,
                        float* position, float* velocity, int32_t* neighbor_count, void* stream) {
    if (!grid_ok(grid) || n < 0 || n > grid->capacity || (n > 0 && (!position || !velocity || !neighbor_count)))
        return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    if (!(query_radius <= grid->cell_size)) {
        set_error_msg("wbc_contact_substep: query_radius exceeds the grid's cell_size");
        return WBC_ERR_INVALID;
    }
    BucketMap map = make_map(grid->cell_size, grid->dim);
    k_contact<false><<<grid_for(n), 256, 0, as_stream(stream)>>>(
        map, n, grid->bucket_start, grid->bucket_count, grid->sorted_id,
        reinterpret_cast<const float4*>(grid->sorted_xyzr), query_radius, rate, dt, position, velocity,
        neighbor_count, wbc_tissue_region{});
    return check_launch("wbc_contact_substep");
}

static bool region_ok(const wbc_tissue_region* r) {
    return r && r->sdf && r->gradient && r->geom.nx >= 2 && r->geom.ny >= 2 && r->geom.nz >= 2 && r->wall_rate >= 0.0f;
}

int wbc_contact_substep_region(const wbc_neighbor_grid* grid, int32_t n, float query_radius, float rate, float dt,
                               const wbc_tissue_region* region, float* position, float* velocity,
                               int32_t* neighbor_count, void* stream) {
    if (!grid_ok(grid) || !region_ok(region) || n < 0 || n > grid->capacity ||
        (n > 0 && (!position || !velocity || !neighbor_count)))
        return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    if (!(query_radius <= grid->cell_size)) {
        set_error_msg("wbc_contact_substep_region: query_radius exceeds the grid's cell_size");
        return WBC_ERR_INVALID;
    }
    BucketMap map = make_map(grid->cell_size, grid->dim);
    k_contact<true><<<grid_for(n), 256, 0, as_stream(stream)>>>(
        map, n, grid->bucket_start, grid->bucket_count, grid->sorted_id,
        reinterpret_cast<const float4*>(grid->sorted_xyzr), query_radius, rate, dt, position, velocity,
        neighbor_count, *region);
    return check_launch("wbc_contact_substep_region");
}

int wbc_sample_sdf(const wbc_tissue_region* region, int32_t n, const float* position, float* out, void* stream) {
    if (!region_ok(region) || n < 0 || (n > 0 && (!position || !out))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_sample_sdf<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(*region, n, position, out);
    return check_launch("wbc_sample_sdf");
}

}  // extern "C"
