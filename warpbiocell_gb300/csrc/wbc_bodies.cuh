// Per-thread bodies of the per-cell and per-node kernels, shared by the single-population kernels
// and the batched ones (wbc_batch.cu), so both run the same arithmetic in the same order.
#pragma once

#include "wbc_common.cuh"

namespace wbc {

constexpr float kFixedOne = 16777216.0f;  // 2^24

struct BucketMap {
    float inv_edge;
    int dim;

    __device__ __forceinline__ int coord(float x) const {
        float q = x * inv_edge;
        q = fminf(fmaxf(q, -1.0e9f), 1.0e9f);
        return static_cast<int>(floorf(q));
    }
    __device__ __forceinline__ int wrap(int c) const {
        int m = c % dim;
        return m < 0 ? m + dim : m;
    }
    __device__ __forceinline__ int bucket(int cx, int cy, int cz) const {
        return (wrap(cx) * dim + wrap(cy)) * dim + wrap(cz);
    }
};

__device__ __forceinline__ void bin_assign_cell(BucketMap map, int i, const float* __restrict__ position,
                                                int32_t* __restrict__ bucket_count, int32_t* __restrict__ cell_bucket,
                                                int32_t* __restrict__ cell_rank) {
    const float* p = position + 3 * static_cast<int64_t>(i);
    int b = map.bucket(map.coord(p[0]), map.coord(p[1]), map.coord(p[2]));
    cell_bucket[i] = b;
    cell_rank[i] = atomicAdd(bucket_count + b, 1);
}

__device__ __forceinline__ void bin_scatter_cell(int i, const int32_t* __restrict__ cell_bucket,
                                                 const int32_t* __restrict__ cell_rank,
                                                 const int32_t* __restrict__ bucket_start, int32_t* __restrict__ scatter) {
    scatter[bucket_start[cell_bucket[i]] + cell_rank[i]] = i;
}

// Each slot finds its place among the members of its bucket in ascending slot order.
__device__ __forceinline__ void bin_order_cell(int i, const float* __restrict__ position,
                                               const float* __restrict__ radius, const int32_t* __restrict__ cell_bucket,
                                               const int32_t* __restrict__ bucket_start,
                                               const int32_t* __restrict__ bucket_count,
                                               const int32_t* __restrict__ scatter, int32_t* __restrict__ sorted_id,
                                               float4* __restrict__ sorted_xyzr) {
    const int b = cell_bucket[i];
    const int s = bucket_start[b];
    const int c = bucket_count[b];
    int rank = 0;
    for (int u = s; u < s + c; ++u) rank += scatter[u] < i ? 1 : 0;
    const float* p = position + 3 * static_cast<int64_t>(i);
    sorted_id[s + rank] = i;
    sorted_xyzr[s + rank] = make_float4(p[0], p[1], p[2], radius[i]);
}

// Tissue-region confinement (kernels/geometry_kernels.py:59-79): with phi the trilinear signed
// distance at the cell (negative inside, position clamped to the grid), p = phi + r; if p > 0 the
// velocity loses wall_rate * p / |n| * n, n the trilinear node gradient of the distance.
__device__ __forceinline__ float region_sample(const wbc_grid_geometry& g, const float* __restrict__ f, int stride,
                                              int i0, int j0, int k0, float fx, float fy, float fz) {
    const int64_t sy = g.nz, sx = static_cast<int64_t>(g.ny) * g.nz;
    const int64_t b = i0 * sx + j0 * sy + k0;
    auto at = [&](int64_t node) { return f[node * stride]; };
    const float c00 = at(b) * (1.0f - fx) + at(b + sx) * fx;
    const float c10 = at(b + sy) * (1.0f - fx) + at(b + sx + sy) * fx;
    const float c01 = at(b + 1) * (1.0f - fx) + at(b + sx + 1) * fx;
    const float c11 = at(b + sy + 1) * (1.0f - fx) + at(b + sx + sy + 1) * fx;
    return (c00 * (1.0f - fy) + c10 * fy) * (1.0f - fz) + (c01 * (1.0f - fy) + c11 * fy) * fz;
}

__device__ __forceinline__ void region_cell(const wbc_grid_geometry& g, float x, float y, float z, int& i0, int& j0,
                                            int& k0, float& fx, float& fy, float& fz) {
    const float ux = fminf(fmaxf((x - g.origin_x) * g.inv_dx, 0.0f), static_cast<float>(g.nx - 1));
    const float uy = fminf(fmaxf((y - g.origin_y) * g.inv_dx, 0.0f), static_cast<float>(g.ny - 1));
    const float uz = fminf(fmaxf((z - g.origin_z) * g.inv_dx, 0.0f), static_cast<float>(g.nz - 1));
    i0 = min(static_cast<int>(floorf(ux)), g.nx - 2);
    j0 = min(static_cast<int>(floorf(uy)), g.ny - 2);
    k0 = min(static_cast<int>(floorf(uz)), g.nz - 2);
    fx = ux - static_cast<float>(i0);
    fy = uy - static_cast<float>(j0);
    fz = uz - static_cast<float>(k0);
}

__device__ __forceinline__ void confine(const wbc_tissue_region& R, float x, float y, float z, float radius,
                                        float& vx, float& vy, float& vz) {
    int i0, j0, k0;
    float fx, fy, fz;
    region_cell(R.geom, x, y, z, i0, j0, k0, fx, fy, fz);
    const float penetration = region_sample(R.geom, R.sdf, 1, i0, j0, k0, fx, fy, fz) + radius;
    if (penetration <= 0.0f) return;
    const float nx = region_sample(R.geom, R.gradient, 3, i0, j0, k0, fx, fy, fz);
    const float ny = region_sample(R.geom, R.gradient + 1, 3, i0, j0, k0, fx, fy, fz);
    const float nz = region_sample(R.geom, R.gradient + 2, 3, i0, j0, k0, fx, fy, fz);
    const float length = sqrtf(nx * nx + ny * ny + nz * nz);
    if (length < 1.0e-8f) return;
    const float s = R.wall_rate * penetration / length;
    vx = vx - s * nx;
    vy = vy - s * ny;
    vz = vz - s * nz;
}

// ---- 32-bit deposit with exact wrap counts (wbc_deposit32, the batched deposit) -------------------
// Low words [4][nodes] added to in aligned pairs (2m, 2m+1) by 64-bit atomics; a wrap out of the
// even word increments count[2m], a wrap out of the pair count[2m+1], and any wrap sets *carry:
//     S[2m] = low[2m] + 2^32 count[2m],   S[2m+1] = low[2m+1] + 2^32 count[2m+1] - count[2m].

// adds `add` (low half to word `even`, high half to word `even` + 1) and counts the wraps
__device__ __forceinline__ void add_pair32(uint32_t* lo, uint32_t* count, uint32_t* carry, int64_t even,
                                           unsigned long long add) {
    const unsigned long long old = atomicAdd(reinterpret_cast<unsigned long long*>(lo + even), add);
    const bool low_wrap = ((old & 0xffffffffull) + (add & 0xffffffffull)) >> 32;
    const bool pair_wrap = old + add < old;
    if (low_wrap) atomicAdd(count + even, 1u);
    if (pair_wrap) atomicAdd(count + even + 1, 1u);
    if (low_wrap || pair_wrap) atomicOr(carry, 1u);
}

// Cell c's trilinear weights (the cell rule and weights of deposit_cell, kernels/field_kernels.py:
// 78-116) into the 32-bit accumulator: for each (i, j) column of its corners one pair add when the
// word of corner k0 is even, else two (4 * nodes is even, so both pairs lie inside the array).
__device__ __forceinline__ void deposit32_cell(const wbc_grid_geometry& g, int c, const float* __restrict__ position,
                                               const int32_t* __restrict__ cell_state, uint32_t* lo, uint32_t* count,
                                               uint32_t* carry) {
    const int64_t nodes = static_cast<int64_t>(g.nx) * g.ny * g.nz;
    const int s = cell_state[c];
    const float* p = position + 3 * static_cast<int64_t>(c);
    const float ux = (p[0] - g.origin_x) * g.inv_dx;
    const float uy = (p[1] - g.origin_y) * g.inv_dx;
    const float uz = (p[2] - g.origin_z) * g.inv_dx;
    const int i0 = static_cast<int>(floorf(ux));
    const int j0 = static_cast<int>(floorf(uy));
    const int k0 = static_cast<int>(floorf(uz));
    if (!(s >= 0 && s < 4 && i0 >= 0 && j0 >= 0 && k0 >= 0 && i0 + 1 < g.nx && j0 + 1 < g.ny && k0 + 1 < g.nz))
        return;
    const float fx = ux - static_cast<float>(i0);
    const float fy = uy - static_cast<float>(j0);
    const float fz = uz - static_cast<float>(k0);
#pragma unroll
    for (int di = 0; di < 2; ++di) {
        const float wx = di == 0 ? 1.0f - fx : fx;
#pragma unroll
        for (int dj = 0; dj < 2; ++dj) {
            const float wy = dj == 0 ? 1.0f - fy : fy;
            const float w0 = wx * wy * (1.0f - fz);
            const float w1 = wx * wy * fz;
            const unsigned long long q0 = static_cast<unsigned int>(static_cast<int>(w0 * kFixedOne + 0.5f));
            const unsigned long long q1 = static_cast<unsigned int>(static_cast<int>(w1 * kFixedOne + 0.5f));
            const int64_t key = s * nodes + (static_cast<int64_t>(i0 + di) * g.ny + (j0 + dj)) * g.nz + k0;
            if ((key & 1) == 0) {
                add_pair32(lo, count, carry, key, q0 | (q1 << 32));
            } else {
                add_pair32(lo, count, carry, key - 1, q0 << 32);
                add_pair32(lo, count, carry, key + 1, q1);
            }
        }
    }
}

// One node's per-state densities S_s / 2^24 * inv_vol (convert_node's expression; `density` may be
// null) and their combination `combined` = sum_s w_s density_s (may be null).
__device__ __forceinline__ void convert32_node(int64_t nodes, int64_t node, const uint32_t* __restrict__ lo,
                                               const uint32_t* __restrict__ count, bool wrapped, float inv_vol,
                                               float* __restrict__ density, float w0, float w1, float w2, float w3,
                                               float* __restrict__ combined) {
    float d[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int64_t w = s * nodes + node;
        long long a = static_cast<long long>(lo[w]);
        if (wrapped) {
            a += static_cast<long long>(count[w]) << 32;
            if (w & 1) a -= static_cast<long long>(count[w - 1]);
        }
        d[s] = static_cast<float>(a) / kFixedOne * inv_vol;
        if (density) density[s * nodes + node] = d[s];
    }
    if (combined) combined[node] = w0 * d[0] + w1 * d[1] + w2 * d[2] + w3 * d[3];
}

// A float at or above r * r (r > 0): RN(r * r) raised by one ulp. A candidate whose squared
// distance d2 reaches it has sqrt(d2) >= r exactly, so the correctly rounded sqrtf(d2) is >= r too
// (rounding is monotonic and r is a float), and the test d < r fails: the candidate is skipped
// before its square root, with the same outcome. (r * r = inf gives NaN, which skips nothing.)
__device__ __forceinline__ float cutoff_squared_above(float r) {
    return __int_as_float(__float_as_int(__fmul_rn(r, r)) + 1);
}

// Sorted slot t: neighbour count, overlap-repulsion velocity (plus the region's push when REGION)
// and the Euler step of its cell.
template <bool REGION = false>
__device__ __forceinline__ void contact_slot(BucketMap map, int t, const int32_t* __restrict__ bucket_start,
                                             const int32_t* __restrict__ bucket_count,
                                             const int32_t* __restrict__ sorted_id,
                                             const float4* __restrict__ sorted_xyzr, float query_radius, float rate,
                                             float dt, float* __restrict__ position, float* __restrict__ velocity,
                                             int32_t* __restrict__ neighbor_count,
                                             const wbc_tissue_region* region = nullptr) {
    const float4 me = sorted_xyzr[t];
    const int i = sorted_id[t];
    const int cx = map.coord(me.x), cy = map.coord(me.y), cz = map.coord(me.z);
    const float cut2 = cutoff_squared_above(query_radius);
    float vx = 0.0f, vy = 0.0f, vz = 0.0f;
    int count = 0;
    for (int ox = -1; ox <= 1; ++ox) {
        for (int oy = -1; oy <= 1; ++oy) {
            for (int oz = -1; oz <= 1; ++oz) {
                const int b = map.bucket(cx + ox, cy + oy, cz + oz);
                const int s = bucket_start[b];
                const int e = s + bucket_count[b];
                for (int u = s; u < e; ++u) {
                    if (u == t) continue;
                    const float4 q = sorted_xyzr[u];
                    const float dx = me.x - q.x;
                    const float dy = me.y - q.y;
                    const float dz = me.z - q.z;
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
        }
    }
    if (REGION) confine(*region, me.x, me.y, me.z, me.w, vx, vy, vz);
    const int64_t o = 3 * static_cast<int64_t>(i);
    velocity[o + 0] = vx;
    velocity[o + 1] = vy;
    velocity[o + 2] = vz;
    neighbor_count[i] = count;
    position[o + 0] = me.x + vx * dt;
    position[o + 1] = me.y + vy * dt;
    position[o + 2] = me.z + vz * dt;
}

// The reverse of one contact step for sorted slot t (cell i, returned in *cell) of the grid built
// at x_t: lambda_out_i = lambda_in_i + dt (J^T lambda_in)_i with (J^T lambda)_i = rate sum_j A_ij
// (lambda_i - lambda_j), A_ij = (R/d - 1) I - R e e^T / d^3 (e = x_i - x_j, R = r_i + r_j), over the
// same candidates and conditions as contact_slot. Returns lambda_in_i . v_i(x_t) / rate, the cell's
// term of dL/drate.
__device__ __forceinline__ float adjoint_contact_slot(BucketMap map, int t, const int32_t* __restrict__ bucket_start,
                                                      const int32_t* __restrict__ bucket_count,
                                                      const int32_t* __restrict__ sorted_id,
                                                      const float4* __restrict__ sorted_xyzr, float query_radius,
                                                      float rate, float dt, const float* __restrict__ lambda_in,
                                                      float* __restrict__ lambda_out, int* cell) {
    const float4 me = sorted_xyzr[t];
    const int i = sorted_id[t];
    const float lix = lambda_in[3 * static_cast<int64_t>(i)], liy = lambda_in[3 * static_cast<int64_t>(i) + 1],
                liz = lambda_in[3 * static_cast<int64_t>(i) + 2];
    const int cx = map.coord(me.x), cy = map.coord(me.y), cz = map.coord(me.z);
    const float cut2 = cutoff_squared_above(query_radius);
    float gx = 0.0f, gy = 0.0f, gz = 0.0f;  // sum_j A_ij (lambda_i - lambda_j) / rate
    float ux = 0.0f, uy = 0.0f, uz = 0.0f;  // v_i / rate
    for (int ox = -1; ox <= 1; ++ox) {
        for (int oy = -1; oy <= 1; ++oy) {
            for (int oz = -1; oz <= 1; ++oz) {
                const int b = map.bucket(cx + ox, cy + oy, cz + oz);
                const int s = bucket_start[b];
                const int e = s + bucket_count[b];
                for (int u = s; u < e; ++u) {
                    if (u == t) continue;
                    const float4 q = sorted_xyzr[u];
                    const float dx = me.x - q.x;
                    const float dy = me.y - q.y;
                    const float dz = me.z - q.z;
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
        }
    }
    const float f = dt * rate;
    const int64_t o = 3 * static_cast<int64_t>(i);
    lambda_out[o] = lix + f * gx;
    lambda_out[o + 1] = liy + f * gy;
    lambda_out[o + 2] = liz + f * gz;
    *cell = i;
    return lix * ux + liy * uy + liz * uz;
}

__device__ __forceinline__ void deposit_cell(const wbc_grid_geometry& g, int c, const float* __restrict__ position,
                                             const int32_t* __restrict__ cell_state,
                                             unsigned long long* __restrict__ acc) {
    const int s = cell_state[c];
    if (s < 0 || s >= 4) return;
    const float* p = position + 3 * static_cast<int64_t>(c);
    const float ux = (p[0] - g.origin_x) * g.inv_dx;
    const float uy = (p[1] - g.origin_y) * g.inv_dx;
    const float uz = (p[2] - g.origin_z) * g.inv_dx;
    const int i0 = static_cast<int>(floorf(ux));
    const int j0 = static_cast<int>(floorf(uy));
    const int k0 = static_cast<int>(floorf(uz));
    if (i0 < 0 || j0 < 0 || k0 < 0) return;
    if (i0 + 1 >= g.nx || j0 + 1 >= g.ny || k0 + 1 >= g.nz) return;
    const float fx = ux - static_cast<float>(i0);
    const float fy = uy - static_cast<float>(j0);
    const float fz = uz - static_cast<float>(k0);
    const int64_t nodes = static_cast<int64_t>(g.nx) * g.ny * g.nz;
    unsigned long long* layer = acc + s * nodes;
#pragma unroll
    for (int di = 0; di < 2; ++di) {
        const float wx = di == 0 ? 1.0f - fx : fx;
#pragma unroll
        for (int dj = 0; dj < 2; ++dj) {
            const float wy = dj == 0 ? 1.0f - fy : fy;
#pragma unroll
            for (int dk = 0; dk < 2; ++dk) {
                const float wz = dk == 0 ? 1.0f - fz : fz;
                const float w = wx * wy * wz;
                const int q = static_cast<int>(w * kFixedOne + 0.5f);
                const int64_t node = (static_cast<int64_t>(i0 + di) * g.ny + (j0 + dj)) * g.nz + (k0 + dk);
                atomicAdd(layer + node, static_cast<unsigned long long>(static_cast<long long>(q)));
            }
        }
    }
}

__device__ __forceinline__ void convert_node(int64_t nodes, int64_t node, long long* __restrict__ acc, float inv_vol,
                                             float* __restrict__ density, float w0, float w1, float w2, float w3,
                                             float* __restrict__ combined, int clear) {
    float d[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const long long a = acc[s * nodes + node];
        d[s] = static_cast<float>(a) / kFixedOne * inv_vol;
        if (density) density[s * nodes + node] = d[s];
        if (clear) acc[s * nodes + node] = 0;
    }
    if (combined) combined[node] = w0 * d[0] + w1 * d[1] + w2 * d[2] + w3 * d[3];
}

__device__ __forceinline__ void sample_cell(const wbc_grid_geometry& g, const float* __restrict__ field, int c,
                                            const float* __restrict__ position, float* __restrict__ out) {
    const float* p = position + 3 * static_cast<int64_t>(c);
    const float ux = (p[0] - g.origin_x) * g.inv_dx;
    const float uy = (p[1] - g.origin_y) * g.inv_dx;
    const float uz = (p[2] - g.origin_z) * g.inv_dx;
    const float cx = fminf(fmaxf(ux, 0.0f), static_cast<float>(g.nx - 1));
    const float cy = fminf(fmaxf(uy, 0.0f), static_cast<float>(g.ny - 1));
    const float cz = fminf(fmaxf(uz, 0.0f), static_cast<float>(g.nz - 1));
    const int i0 = min(static_cast<int>(floorf(cx)), g.nx - 2);
    const int j0 = min(static_cast<int>(floorf(cy)), g.ny - 2);
    const int k0 = min(static_cast<int>(floorf(cz)), g.nz - 2);
    const float fx = cx - static_cast<float>(i0);
    const float fy = cy - static_cast<float>(j0);
    const float fz = cz - static_cast<float>(k0);
    const int64_t sy = g.nz, sx = static_cast<int64_t>(g.ny) * g.nz;
    const int64_t b = i0 * sx + j0 * sy + k0;
    const float gx = 1.0f - fx;
    const float c00 = field[b] * gx + field[b + sx] * fx;
    const float c10 = field[b + sy] * gx + field[b + sx + sy] * fx;
    const float c01 = field[b + 1] * gx + field[b + sx + 1] * fx;
    const float c11 = field[b + sy + 1] * gx + field[b + sx + sy + 1] * fx;
    const float c0 = c00 * (1.0f - fy) + c10 * fy;
    const float c1 = c01 * (1.0f - fy) + c11 * fy;
    out[c] = c0 * (1.0f - fz) + c1 * fz;
}

__device__ __forceinline__ float oxygen_factor(float o, float hypoxia_threshold, float death_threshold) {
    if (o >= hypoxia_threshold) return 1.0f;
    if (o <= death_threshold) return 0.0f;
    return (o - death_threshold) / (hypoxia_threshold - death_threshold);
}

__device__ __forceinline__ void lifecycle_cell(const wbc_lifecycle_params& p, int i, int32_t* __restrict__ cell_state,
                                               float* __restrict__ age, const int32_t* __restrict__ neighbor_count,
                                               const float* __restrict__ oxygen_local,
                                               const float* __restrict__ glucose_local,
                                               const int32_t* __restrict__ fate_flags, uint32_t* __restrict__ rng_state,
                                               int32_t* __restrict__ divide_flag) {
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

// Parent slot i (with divide_flag set) of a population of `count` cells places its daughter.
__device__ __forceinline__ void place_daughter(int i, int32_t count, float placement_factor,
                                               const int32_t* __restrict__ division_offset, float* __restrict__ position,
                                               float* __restrict__ radius, int32_t* __restrict__ cell_state,
                                               int32_t* __restrict__ cell_type, float* __restrict__ age,
                                               float* __restrict__ oxygen_local, float* __restrict__ glucose_local,
                                               uint32_t* __restrict__ rng_state, float* __restrict__ velocity,
                                               int32_t* __restrict__ neighbor_count, int32_t* __restrict__ fate_flags) {
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

}  // namespace wbc
