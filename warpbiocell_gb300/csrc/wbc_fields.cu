// Cell <-> grid transfer and the Michaelis-Menten reaction-diffusion solver.
//
//   deposit    int64 fixed-point trilinear weights, atomically added (order independent, so the
//              accumulator is bit-exact whatever the thread order)        field_kernels.py:78-116
//   convert    acc / 2^24 / dx^3 per state, optional per-species combination and clearing of the
//              accumulator in the same pass                             field_kernels.py:119-142
//   sample     clamped trilinear interpolation at the cells             field_kernels.py:153-182
//   SOR        red-black colour half-sweeps, in place                   field_kernels.py:185-212
//   residual   max-norm of the dimensionless residual, block-reduced    field_kernels.py:215-243
//   FTCS       explicit reference step (validation only)                field_kernels.py:246-273
//
// Layout: fields are float[nx][ny][nz] with k fastest; the int64 accumulator is int64[4][nodes], the
// 32-bit one uint32 low words [4][nodes], uint32 wrap counts [4][nodes] and a carry flag.
// Every float expression is evaluated in the reference's order (no contraction, see
// wbc_common.cuh), so the field after a given number of sweeps is bit-identical to the oracle's.
#include <algorithm>

#include "wbc_bodies.cuh"

namespace wbc {

__global__ void k_deposit(wbc_grid_geometry g, int32_t n, const float* __restrict__ position,
                          const int32_t* __restrict__ cell_state, unsigned long long* __restrict__ acc) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) deposit_cell(g, c, position, cell_state, acc);
}

__global__ void k_convert(int64_t nodes, long long* __restrict__ acc, float inv_vol, float* __restrict__ density,
                          float w0, float w1, float w2, float w3, float* __restrict__ combined, int clear) {
    int64_t node = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (node < nodes) convert_node(nodes, node, acc, inv_vol, density, w0, w1, w2, w3, combined, clear);
}

// ---- 32-bit deposit with an exact carry -------------------------------------------------------------
// The same integer sums as the int64 accumulator, in half the bytes. Each state layer is a uint32
// low word per node, and the low words are added to in aligned pairs (words 2m and 2m+1) by 64-bit
// atomics: the two z-corners k0, k0+1 of a cell's (i, j) column are adjacent words, so when the
// first is even one atomic adds both (otherwise two, each adding to one half of a pair). A 64-bit
// add carries out of the even word into the odd one and out of the pair altogether; the first
// wrap increments the even word's count c[2m], the second the odd word's count c[2m+1]. With those
// counts the exact sums are
//     S[2m]   = low[2m]   + 2^32 c[2m]
//     S[2m+1] = low[2m+1] + 2^32 c[2m+1] - c[2m]
// (the pair's 64-bit total is S[2m] + 2^32 S[2m+1] = low + 2^64 c[2m+1]). A carry flag records
// whether any add wrapped; without one the low words are the sums (a node would need
// contributions worth 256 whole cells for a wrap). The cells are visited in the order given (the
// hash grid's, so that a warp's cells are neighbours in space and their atomics hit nearby lines).
// (Combining the lanes' additions first, by warp matching or in a shared-memory tile, was slower:
// at about half a cell per grid cell a node receives only a few contributions, which rarely
// share a warp or a block.)

// Streaming multiprocessors of the current device (cached per device).
static int sm_count() {
    static int cache[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152;
    if (cache[dev] == 0) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = sms > 0 ? sms : 152;
    }
    return cache[dev];
}

// Zeroes the low words, and the wrap counts when the previous deposit wrapped (otherwise they are
// zero already); `words` is a multiple of 4, the buffers are 16-byte aligned.
__global__ void k_deposit32_clear(int64_t words, uint4* __restrict__ lo, uint4* __restrict__ count,
                                  const uint32_t* __restrict__ carry) {
    const bool wrapped = *carry != 0u;
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    const int64_t quads = words / 4;
    for (int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; q < quads;
         q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        lo[q] = zero;
        if (wrapped) count[q] = zero;
    }
}

__global__ void k_deposit32(wbc_grid_geometry g, int32_t n, const float* __restrict__ position,
                            const int32_t* __restrict__ cell_state, const int32_t* __restrict__ order,
                            uint32_t* __restrict__ lo, uint32_t* __restrict__ count, uint32_t* __restrict__ carry) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) deposit32_cell(g, order ? order[t] : t, position, cell_state, lo, count, carry);
}

// density_s = S_s / 2^24 * inv_vol per state, as convert_node, with S_s the exact sum of the paired
// low words and their wrap counts (the formula above k_deposit32_clear).
__global__ void k_convert32(int64_t nodes, const uint32_t* __restrict__ lo, const uint32_t* __restrict__ count,
                            const uint32_t* __restrict__ carry, float inv_vol, float* __restrict__ density, float w0,
                            float w1, float w2, float w3, float* __restrict__ combined) {
    const int64_t node = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (node < nodes) convert32_node(nodes, node, lo, count, *carry != 0u, inv_vol, density, w0, w1, w2, w3, combined);
}

__global__ void k_combine(int64_t nodes, float w0, float w1, float w2, float w3, const float* __restrict__ density,
                          float* __restrict__ out) {
    int64_t node = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (node >= nodes) return;
    out[node] = w0 * density[node] + w1 * density[nodes + node] + w2 * density[2 * nodes + node] +
                w3 * density[3 * nodes + node];
}

__global__ void k_sample(wbc_grid_geometry g, const float* __restrict__ field, int32_t n,
                         const float* __restrict__ position, float* __restrict__ out) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) sample_cell(g, field, c, position, out);
}

// ---- SOR -----------------------------------------------------------------------------------------
__device__ __forceinline__ bool on_dirichlet_face(const wbc_sor_params& p, int i, int j, int k) {
    if (p.bc_x == 0 && (i == 0 || i == p.nx - 1)) return true;
    if (p.bc_y == 0 && (j == 0 || j == p.ny - 1)) return true;
    if (p.bc_z == 0 && (k == 0 || k == p.nz - 1)) return true;
    return false;
}

// Sum of the six neighbours, mirrored at every edge (only reached on Neumann faces).
__device__ __forceinline__ float neighbor_sum(const float* __restrict__ f, const wbc_sor_params& p, int i, int j,
                                              int k) {
    const int im = i - 1 < 0 ? 1 : i - 1;
    const int ip = i + 1 > p.nx - 1 ? p.nx - 2 : i + 1;
    const int jm = j - 1 < 0 ? 1 : j - 1;
    const int jp = j + 1 > p.ny - 1 ? p.ny - 2 : j + 1;
    const int km = k - 1 < 0 ? 1 : k - 1;
    const int kp = k + 1 > p.nz - 1 ? p.nz - 2 : k + 1;
    const int64_t sx = static_cast<int64_t>(p.ny) * p.nz;
    const int64_t sy = p.nz;
    const int64_t row = j * sy;
    const int64_t base = i * sx;
    return f[im * sx + row + k] + f[ip * sx + row + k] + f[base + jm * sy + k] + f[base + jp * sy + k] +
           f[base + row + km] + f[base + row + kp];
}

__device__ __forceinline__ float production_at(const wbc_sor_params& p, const float* __restrict__ production,
                                               const float* __restrict__ source, int64_t idx) {
    const float prod = production ? production[idx] : 0.0f;
    if (!p.has_source) return prod * 1.0f;
    const float v = source[idx];
    return prod * div_rn(v, p.source_k + v);
}

// One colour: thread (i, j, m) updates k = 2m + ((colour + i + j) & 1).
__global__ void k_sor_colour(wbc_sor_params p, int colour, const int32_t* __restrict__ fixed,
                             const float* __restrict__ density, const float* __restrict__ production,
                             const float* __restrict__ source, float* __restrict__ field) {
    const int half = (p.nz + 1) >> 1;
    int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = static_cast<int64_t>(p.nx) * p.ny * half;
    if (t >= total) return;
    const int m = static_cast<int>(t % half);
    const int64_t ij = t / half;
    const int j = static_cast<int>(ij % p.ny);
    const int i = static_cast<int>(ij / p.ny);
    const int k = 2 * m + ((colour + i + j) & 1);
    if (k >= p.nz) return;
    const int64_t idx = (static_cast<int64_t>(i) * p.ny + j) * p.nz + k;
    if ((fixed && fixed[idx] != 0) || on_dirichlet_face(p, i, j, k)) return;
    const float o = field[idx];
    const float c = div_rn(density[idx] * p.uptake_max, p.michaelis_k + o);
    const float prod = production_at(p, production, source, idx);
    const float gs = div_rn(neighbor_sum(field, p, i, j, k) + p.dx2_over_D * prod, 6.0f + p.dx2_over_D * c);
    field[idx] = fmaxf((1.0f - p.omega) * o + p.omega * gs, 0.0f);
}

__global__ void k_residual(wbc_sor_params p, const int32_t* __restrict__ fixed, const float* __restrict__ density,
                           const float* __restrict__ production, const float* __restrict__ source,
                           const float* __restrict__ field, unsigned int* __restrict__ residual_bits) {
    const int64_t nodes = static_cast<int64_t>(p.nx) * p.ny * p.nz;
    int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    float val = 0.0f;
    if (idx < nodes) {
        const int k = static_cast<int>(idx % p.nz);
        const int64_t ij = idx / p.nz;
        const int j = static_cast<int>(ij % p.ny);
        const int i = static_cast<int>(ij / p.ny);
        if ((!fixed || fixed[idx] == 0) && !on_dirichlet_face(p, i, j, k)) {
            const float o = field[idx];
            const float c = div_rn(density[idx] * p.uptake_max, p.michaelis_k + o);
            const float prod = production_at(p, production, source, idx);
            const float r = neighbor_sum(field, p, i, j, k) + p.dx2_over_D * prod - (6.0f + p.dx2_over_D * c) * o;
            val = div_rn(fabsf(r), fmaxf(6.0f * o, p.reference));
        }
    }
    // Max of non-negative floats = max of their bit patterns; NaN (0x7fc00000) dominates.
    unsigned int bits = __float_as_uint(val);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, d));
    __shared__ unsigned int warp_max[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_max[warp] = bits;
    __syncthreads();
    if (warp == 0) {
        bits = lane < (blockDim.x >> 5) ? warp_max[lane] : 0u;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, d));
        if (lane == 0) atomicMax(residual_bits, bits);
    }
}

__global__ void k_ftcs(wbc_sor_params p, float dt, const int32_t* __restrict__ fixed, const float* __restrict__ density,
                       const float* __restrict__ production, const float* __restrict__ source,
                       const float* __restrict__ in, float* __restrict__ out) {
    const int64_t nodes = static_cast<int64_t>(p.nx) * p.ny * p.nz;
    int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= nodes) return;
    const int k = static_cast<int>(idx % p.nz);
    const int64_t ij = idx / p.nz;
    const int j = static_cast<int>(ij % p.ny);
    const int i = static_cast<int>(ij / p.ny);
    const float o = in[idx];
    if (fixed[idx] != 0 || on_dirichlet_face(p, i, j, k)) {
        out[idx] = o;
        return;
    }
    const float D_over_dx2 = p.dx2_over_D;
    const float lap = D_over_dx2 * (neighbor_sum(in, p, i, j, k) - 6.0f * o);
    const float uptake = density[idx] * p.uptake_max * o / (p.michaelis_k + o);
    const float prod = production_at(p, production, source, idx);
    out[idx] = o + dt * (lap - uptake + prod);
}

static bool geom_ok(const wbc_grid_geometry* g) { return g && g->nx >= 2 && g->ny >= 2 && g->nz >= 2; }

static bool sor_ok(const wbc_sor_params* p) { return p && p->nx >= 3 && p->ny >= 3 && p->nz >= 3; }

}  // namespace wbc

using namespace wbc;

extern "C" {

int wbc_deposit(const wbc_grid_geometry* geom, int32_t n, const float* position, const int32_t* cell_state,
                int64_t* accumulator, void* stream) {
    if (!geom_ok(geom) || n < 0 || !accumulator || (n > 0 && (!position || !cell_state))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_deposit<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(*geom, n, position, cell_state,
                                                               reinterpret_cast<unsigned long long*>(accumulator));
    return check_launch("wbc_deposit");
}

int wbc_density_convert(int64_t nodes, int64_t* accumulator, float inv_voxel_volume, float* density,
                        const float* weights4, float* combined, int32_t clear, void* stream) {
    if (nodes < 0 || !accumulator || (combined && !weights4)) return WBC_ERR_INVALID;
    if (nodes == 0) return WBC_OK;
    float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (weights4)
        for (int s = 0; s < 4; ++s) w[s] = weights4[s];
    k_convert<<<grid_for(nodes), kThreads, 0, as_stream(stream)>>>(nodes, reinterpret_cast<long long*>(accumulator),
                                                                   inv_voxel_volume, density, w[0], w[1], w[2], w[3],
                                                                   combined, clear);
    return check_launch("wbc_density_convert");
}

int wbc_density_combine(int64_t nodes, const float* weights4, const float* density, float* out, void* stream) {
    if (nodes < 0 || !weights4 || (nodes > 0 && (!density || !out))) return WBC_ERR_INVALID;
    if (nodes == 0) return WBC_OK;
    k_combine<<<grid_for(nodes), kThreads, 0, as_stream(stream)>>>(nodes, weights4[0], weights4[1], weights4[2],
                                                                   weights4[3], density, out);
    return check_launch("wbc_density_combine");
}

int wbc_sample(const wbc_grid_geometry* geom, const float* field, int32_t n, const float* position, float* out,
               void* stream) {
    if (!geom_ok(geom) || n < 0 || (n > 0 && (!field || !position || !out))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_sample<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(*geom, field, n, position, out);
    return check_launch("wbc_sample");
}

int wbc_sor_sweeps(const wbc_sor_params* p, int32_t sweeps, const int32_t* fixed, const float* density,
                   const float* production, const float* source, float* field, float* residual_out, void* stream) {
    if (!sor_ok(p) || sweeps < 0 || !density || !field || (p->has_source && !source))
        return WBC_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const int64_t nodes = static_cast<int64_t>(p->nx) * p->ny * p->nz;
    const int64_t half_nodes = static_cast<int64_t>(p->nx) * p->ny * ((p->nz + 1) >> 1);
    for (int sweep = 0; sweep < sweeps; ++sweep) {
        for (int colour = 0; colour < 2; ++colour)
            k_sor_colour<<<grid_for(half_nodes), kThreads, 0, s>>>(*p, colour, fixed, density, production, source,
                                                                   field);
    }
    if (residual_out) {
        cudaError_t err = cudaMemsetAsync(residual_out, 0, sizeof(float), s);
        if (err != cudaSuccess) {
            set_error("wbc_sor_sweeps: cudaMemsetAsync", err);
            return WBC_ERR_CUDA;
        }
        k_residual<<<grid_for(nodes), kThreads, 0, s>>>(*p, fixed, density, production, source, field,
                                                        reinterpret_cast<unsigned int*>(residual_out));
    }
    return check_launch("wbc_sor_sweeps", 2 * static_cast<int64_t>(sweeps) + (residual_out ? 1 : 0));
}

int wbc_ftcs_step(const wbc_sor_params* p, float dt, const int32_t* fixed, const float* density,
                  const float* production, const float* source, const float* field_in, float* field_out,
                  void* stream) {
    if (!sor_ok(p) || !fixed || !density || !field_in || !field_out || (p->has_source && !source))
        return WBC_ERR_INVALID;
    const int64_t nodes = static_cast<int64_t>(p->nx) * p->ny * p->nz;
    k_ftcs<<<grid_for(nodes), kThreads, 0, as_stream(stream)>>>(*p, dt, fixed, density, production, source, field_in,
                                                                field_out);
    return check_launch("wbc_ftcs_step");
}


size_t wbc_deposit32_bytes(int64_t nodes) {
    // low words, high words ([4][nodes] uint32 each), then the carry flag
    return nodes < 0 ? 0 : static_cast<size_t>(8 * 4 * nodes + 256);
}

int wbc_deposit32(const wbc_grid_geometry* geom, int32_t n, const float* position, const int32_t* cell_state,
                  const int32_t* order, void* accumulator, size_t accumulator_bytes, void* stream) {
    if (!geom_ok(geom) || n < 0 || !accumulator || (n > 0 && (!position || !cell_state))) return WBC_ERR_INVALID;
    const int64_t nodes = static_cast<int64_t>(geom->nx) * geom->ny * geom->nz;
    if (accumulator_bytes < wbc_deposit32_bytes(nodes) || reinterpret_cast<uintptr_t>(accumulator) % 16 != 0)
        return WBC_ERR_WORKSPACE;
    if (4 * nodes >= (1ll << 32) - 1) {
        set_error_msg("wbc_deposit32: more than 2^32 - 2 state-node words");
        return WBC_ERR_INVALID;
    }
    uint32_t* lo = static_cast<uint32_t*>(accumulator);
    uint32_t* count = lo + 4 * nodes;
    uint32_t* carry = count + 4 * nodes;
    cudaStream_t s = as_stream(stream);
    const int64_t words = 4 * nodes;
    const int64_t want = (words / 4 + kThreads - 1) / kThreads;
    const unsigned blocks = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(want, 4 * sm_count())));
    k_deposit32_clear<<<blocks, kThreads, 0, s>>>(words, reinterpret_cast<uint4*>(lo), reinterpret_cast<uint4*>(count),
                                                  carry);
    cudaError_t err = cudaMemsetAsync(carry, 0, sizeof(uint32_t), s);
    if (err != cudaSuccess) {
        set_error("wbc_deposit32: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    if (n > 0) k_deposit32<<<grid_for(n), kThreads, 0, s>>>(*geom, n, position, cell_state, order, lo, count, carry);
    return check_launch("wbc_deposit32", n > 0 ? 2 : 1);
}

int wbc_convert32(int64_t nodes, const void* accumulator, float inv_voxel_volume, float* density,
                  const float* weights4, float* combined, void* stream) {
    if (nodes < 0 || !accumulator || (combined && !weights4)) return WBC_ERR_INVALID;
    if (nodes == 0) return WBC_OK;
    const uint32_t* lo = static_cast<const uint32_t*>(accumulator);
    const uint32_t* count = lo + 4 * nodes;
    const uint32_t* carry = count + 4 * nodes;
    float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (weights4)
        for (int k = 0; k < 4; ++k) w[k] = weights4[k];
    k_convert32<<<grid_for(nodes), kThreads, 0, as_stream(stream)>>>(nodes, lo, count, carry, inv_voxel_volume, density,
                                                                     w[0], w[1], w[2], w[3], combined);
    return check_launch("wbc_convert32");
}

}  // extern "C"
