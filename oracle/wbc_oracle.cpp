// wbc_oracle.cpp — CPU restatement of WarpBioCell's coupled cell step, used ONLY as test
// infrastructure: the parity tests, the smoke check and the CPU baseline of the benchmark call it
// as the checker. Nothing in the product links, imports or falls back to it.
//
// Every function restates one reference kernel (paths inside Gennappio/WarpBioCell,
// src/warpbiocell/...) with the same float operations in the same order. Compiled with
// -ffp-contract=off (no fused multiply-add), so with IEEE float arithmetic it reproduces the
// GPU library bit for bit wherever the GPU's result is order independent or its order is
// fixed (integer deposits, neighbour counts, lifecycle decisions, network states, SOR sweeps,
// and, because the neighbour traversal order is canonical, positions). The *_f64 variants are
// the FP64 re-runs the tolerances are measured against.
//
// The project's random streams, exp, log and unit-sphere sampling are defined by their published
// methods (see the function comments) and written here independently of the CUDA sources; the
// parity tests compare the two.
//
// Parallelism: OpenMP over cells or grid planes; every result is independent of the thread count
// (integer atomics, per-cell outputs, red-black colours).
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---- random streams (project definition) ----------------------------------------------------------
// MurmurHash3 fmix32 finaliser (Appleby, public domain) over a Weyl sequence with a per-slot odd
// increment: SplitMix-style (Steele, Lea & Flood, OOPSLA 2014).
inline uint32_t fmix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
inline uint32_t rng_start(int32_t seed, uint32_t slot) {
    return fmix32(static_cast<uint32_t>(seed) ^ fmix32(slot * 0x9E3779B9u + 0x6A09E667u));
}
inline uint32_t rng_increment(uint32_t slot) { return fmix32(slot + 0xBB67AE85u) | 1u; }
inline float randf(uint32_t& state, uint32_t inc) {
    state += inc;
    return static_cast<float>(fmix32(state) >> 8) * (1.0f / 16777216.0f);
}

inline float bits_to_float(uint32_t b) {
    float f;
    std::memcpy(&f, &b, sizeof f);
    return f;
}
inline uint32_t float_to_bits(float f) {
    uint32_t b;
    std::memcpy(&b, &f, sizeof b);
    return b;
}
inline float pow2i(int n) { return bits_to_float(static_cast<uint32_t>(n + 127) << 23); }

// exp: Cody & Waite reduction (1980) with ln2 = 0.693145751953125 + 1.4286068203e-6, degree-7
// Taylor polynomial in Horner form, 2^n from exponent bits.
float proj_expf(float x) {
    if (!(x == x)) return x;
    if (x > 88.72283935546875f) return bits_to_float(0x7f800000u);
    if (x < -103.97208404541015625f) return 0.0f;
    const float log2e = 1.44269502162933349609375f;
    const float ln2_hi = 0.693145751953125f;
    const float ln2_lo = 1.42860682030941723212e-06f;
    const float magic = 12582912.0f;
    float t = x * log2e;
    float kf = (t + magic) - magic;
    int n = static_cast<int>(kf);
    float r = (x - kf * ln2_hi) - kf * ln2_lo;
    float p = 1.98412698412698412698e-4f;
    p = p * r + 1.38888888888888888889e-3f;
    p = p * r + 8.33333333333333333333e-3f;
    p = p * r + 4.16666666666666666667e-2f;
    p = p * r + 1.66666666666666666667e-1f;
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    if (n > 127) return (p * pow2i(n - 1)) * 2.0f;
    if (n < -126) return (p * pow2i(n + 64)) * pow2i(-64);
    return p * pow2i(n);
}

// log: x = m 2^e, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh((m-1)/(m+1)) by its odd series to s^11.
float proj_logf(float x) {
    if (!(x > 0.0f)) return x == 0.0f ? -bits_to_float(0x7f800000u) : bits_to_float(0x7fc00000u);
    if (x == bits_to_float(0x7f800000u)) return x;
    int e = 0;
    if (x < 1.17549435e-38f) {
        x = x * 16777216.0f;
        e = -24;
    }
    uint32_t bits = float_to_bits(x);
    e += static_cast<int>((bits >> 23) & 0xff) - 127;
    float m = bits_to_float((bits & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421353816986083984375f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 9.09090909090909090909e-2f;
    p = p * s2 + 1.11111111111111111111e-1f;
    p = p * s2 + 1.42857142857142857143e-1f;
    p = p * s2 + 2.0e-1f;
    p = p * s2 + 3.33333333333333333333e-1f;
    p = p * s2 + 1.0f;
    const float log_m = 2.0f * s * p;
    const float ef = static_cast<float>(e);
    return (ef * 0.693145751953125f + log_m) + ef * 1.42860682030941723212e-06f;
}

// Marsaglia (1972): rejection in the unit disc, at most 64 attempts, then +z.
void unit_sphere(uint32_t& state, uint32_t inc, float& x, float& y, float& z) {
    for (int attempt = 0; attempt < 64; ++attempt) {
        float a = 2.0f * randf(state, inc) - 1.0f;
        float b = 2.0f * randf(state, inc) - 1.0f;
        float s = a * a + b * b;
        if (s < 1.0f && s > 0.0f) {
            float t = 2.0f * std::sqrt(1.0f - s);
            x = a * t;
            y = b * t;
            z = 1.0f - 2.0f * s;
            return;
        }
    }
    x = 0.0f;
    y = 0.0f;
    z = 1.0f;
}

// ---- hashed buckets (the neighbour traversal order) ------------------------------------------------
// Bucket edge cell_size * (1 + 2^-10); cell coordinate floor(x / edge) clamped to +-1e9, wrapped
// mod dim. A cell visits the 27 buckets around its own in (x, y, z) offset order, slots ascending
// inside each bucket (spatial/neighbors.py:33-37 defines what is indexed: the prefix [0, n)).
struct Buckets {
    int dim = 0;
    float inv_edge = 0.0f;
    std::vector<int32_t> start, count, ids;

    int coord(float x) const {
        float q = x * inv_edge;
        q = std::fmin(std::fmax(q, -1.0e9f), 1.0e9f);
        return static_cast<int>(std::floor(q));
    }
    int wrap(int c) const {
        int m = c % dim;
        return m < 0 ? m + dim : m;
    }
    int bucket(int cx, int cy, int cz) const { return (wrap(cx) * dim + wrap(cy)) * dim + wrap(cz); }

    void build(int n, const float* pos, float cell_size, int dim_) {
        dim = dim_;
        float edge = cell_size * 1.0009765625f;
        inv_edge = 1.0f / edge;
        const size_t nb = static_cast<size_t>(dim) * dim * dim;
        count.assign(nb, 0);
        start.assign(nb, 0);
        std::vector<int32_t> key(n);
        for (int i = 0; i < n; ++i) {
            key[i] = bucket(coord(pos[3 * i]), coord(pos[3 * i + 1]), coord(pos[3 * i + 2]));
            count[key[i]]++;
        }
        int32_t run = 0;
        for (size_t b = 0; b < nb; ++b) {
            start[b] = run;
            run += count[b];
        }
        ids.assign(n, 0);
        std::vector<int32_t> fill(start);
        for (int i = 0; i < n; ++i) ids[fill[key[i]]++] = i;  // ascending slots: stable
    }
};

template <typename T>
inline T tsqrt(T v) {
    return std::sqrt(v);
}

// Tissue region for the confinement push (kernels/geometry_kernels.py:14-79): signed distance and
// node gradient (x, y, z per node) on a grid, sampled trilinearly with positions clamped to it.
struct Region {
    int32_t nx, ny, nz;
    float ox, oy, oz, inv_dx;
    const float* sdf;
    const float* gradient;
    float wall_rate;
};

// Trilinear sample of the region's SDF / gradient grid (kernels/geometry_kernels.py:16-44).
inline float region_sample(const Region& R, const float* f, int stride, int i0, int j0, int k0, float fx, float fy,
                           float fz) {
    auto at = [&](int i, int j, int k) { return f[((static_cast<int64_t>(i) * R.ny + j) * R.nz + k) * stride]; };
    const float c00 = at(i0, j0, k0) * (1.0f - fx) + at(i0 + 1, j0, k0) * fx;
    const float c10 = at(i0, j0 + 1, k0) * (1.0f - fx) + at(i0 + 1, j0 + 1, k0) * fx;
    const float c01 = at(i0, j0, k0 + 1) * (1.0f - fx) + at(i0 + 1, j0, k0 + 1) * fx;
    const float c11 = at(i0, j0 + 1, k0 + 1) * (1.0f - fx) + at(i0 + 1, j0 + 1, k0 + 1) * fx;
    return (c00 * (1.0f - fy) + c10 * fy) * (1.0f - fz) + (c01 * (1.0f - fy) + c11 * fy) * fz;
}

// Wall push of a cell outside the tissue region (kernels/geometry_kernels.py:59-79).
inline void confine(const Region& R, float x, float y, float z, float radius, float& vx, float& vy, float& vz) {
    const float ux = std::min(std::max((x - R.ox) * R.inv_dx, 0.0f), static_cast<float>(R.nx - 1));
    const float uy = std::min(std::max((y - R.oy) * R.inv_dx, 0.0f), static_cast<float>(R.ny - 1));
    const float uz = std::min(std::max((z - R.oz) * R.inv_dx, 0.0f), static_cast<float>(R.nz - 1));
    const int i0 = std::min(static_cast<int>(std::floor(ux)), R.nx - 2);
    const int j0 = std::min(static_cast<int>(std::floor(uy)), R.ny - 2);
    const int k0 = std::min(static_cast<int>(std::floor(uz)), R.nz - 2);
    const float fx = ux - static_cast<float>(i0), fy = uy - static_cast<float>(j0), fz = uz - static_cast<float>(k0);
    const float penetration = region_sample(R, R.sdf, 1, i0, j0, k0, fx, fy, fz) + radius;
    if (penetration <= 0.0f) return;
    const float nx = region_sample(R, R.gradient, 3, i0, j0, k0, fx, fy, fz);
    const float ny = region_sample(R, R.gradient + 1, 3, i0, j0, k0, fx, fy, fz);
    const float nz = region_sample(R, R.gradient + 2, 3, i0, j0, k0, fx, fy, fz);
    const float length = std::sqrt(nx * nx + ny * ny + nz * nz);
    if (length < 1.0e-8f) return;
    const float s = R.wall_rate * penetration / length;
    vx = vx - s * nx;
    vy = vy - s * ny;
    vz = vz - s * nz;
}

// contact_velocities + integrate_positions (kernels/mechanics_kernels.py:26-67), fused: every
// velocity is computed from the positions at the start of the substep; with a region (float
// only), the confinement push of cells/mechanics.py:95-102 before the Euler step.
template <typename T>
void contact_substep(int n, T* pos, const T* radius, const float* bin_pos, float cell_size, int dim,
                     T query_radius, T rate, T dt, T* velocity, int32_t* neighbor_count,
                     const Region* region = nullptr) {
    Buckets bk;
    bk.build(n, bin_pos, cell_size, dim);
    std::vector<T> x0(pos, pos + 3 * static_cast<size_t>(n));
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        const T xi = x0[3 * i], yi = x0[3 * i + 1], zi = x0[3 * i + 2], ri = radius[i];
        const int cx = bk.coord(bin_pos[3 * i]), cy = bk.coord(bin_pos[3 * i + 1]), cz = bk.coord(bin_pos[3 * i + 2]);
        T vx = 0, vy = 0, vz = 0;
        int cnt = 0;
        for (int ox = -1; ox <= 1; ++ox)
            for (int oy = -1; oy <= 1; ++oy)
                for (int oz = -1; oz <= 1; ++oz) {
                    const int b = bk.bucket(cx + ox, cy + oy, cz + oz);
                    const int s = bk.start[b], e = s + bk.count[b];
                    for (int u = s; u < e; ++u) {
                        const int j = bk.ids[u];
                        if (j == i) continue;
                        const T dx = xi - x0[3 * j];
                        const T dy = yi - x0[3 * j + 1];
                        const T dz = zi - x0[3 * j + 2];
                        const T d = tsqrt<T>(dx * dx + dy * dy + dz * dz);
                        if (d < query_radius) {
                            ++cnt;
                            const T overlap = ri + radius[j] - d;
                            if (overlap > T(0) && d > T(1.0e-6f)) {
                                const T f = rate * overlap / d;
                                vx = vx + f * dx;
                                vy = vy + f * dy;
                                vz = vz + f * dz;
                            }
                        }
                    }
                }
        if constexpr (std::is_same<T, float>::value) {
            if (region) confine(*region, xi, yi, zi, ri, vx, vy, vz);
        }
        velocity[3 * i] = vx;
        velocity[3 * i + 1] = vy;
        velocity[3 * i + 2] = vz;
        neighbor_count[i] = cnt;
        pos[3 * i] = xi + vx * dt;
        pos[3 * i + 1] = yi + vy * dt;
        pos[3 * i + 2] = zi + vz * dt;
    }
}

// ---- field kernels (kernels/field_kernels.py) --------------------------------------------------------
struct SorParams {
    int32_t nx, ny, nz, bc_x, bc_y, bc_z;
    float omega, dx2_over_D, uptake_max, michaelis_k, reference;
    int32_t has_source;
    float source_k;
};

inline bool dirichlet_face(const SorParams& p, int i, int j, int k) {
    if (p.bc_x == 0 && (i == 0 || i == p.nx - 1)) return true;
    if (p.bc_y == 0 && (j == 0 || j == p.ny - 1)) return true;
    if (p.bc_z == 0 && (k == 0 || k == p.nz - 1)) return true;
    return false;
}

template <typename T>
inline T neighbor_sum(const T* f, const SorParams& p, int i, int j, int k) {
    const int im = i - 1 < 0 ? 1 : i - 1;
    const int ip = i + 1 > p.nx - 1 ? p.nx - 2 : i + 1;
    const int jm = j - 1 < 0 ? 1 : j - 1;
    const int jp = j + 1 > p.ny - 1 ? p.ny - 2 : j + 1;
    const int km = k - 1 < 0 ? 1 : k - 1;
    const int kp = k + 1 > p.nz - 1 ? p.nz - 2 : k + 1;
    auto at = [&](int a, int b, int c) { return f[(static_cast<int64_t>(a) * p.ny + b) * p.nz + c]; };
    return at(im, j, k) + at(ip, j, k) + at(i, jm, k) + at(i, jp, k) + at(i, j, km) + at(i, j, kp);
}

template <typename T>
inline T production_at(const SorParams& p, const T* production, const T* source, int64_t idx) {
    const T prod = production ? production[idx] : T(0);
    if (!p.has_source) return prod * T(1);
    const T v = source[idx];
    return prod * (v / (T(p.source_k) + v));
}

template <typename T>
void sor_sweeps(const SorParams& p, int sweeps, const int32_t* fixed, const T* density, const T* production,
                const T* source, T* field, T* residual_out) {
    const T omega = p.omega, h = p.dx2_over_D, um = p.uptake_max, K = p.michaelis_k;
    for (int sweep = 0; sweep < sweeps; ++sweep) {
        for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static)
            for (int i = 0; i < p.nx; ++i)
                for (int j = 0; j < p.ny; ++j)
                    for (int k = (colour + i + j) & 1; k < p.nz; k += 2) {
                        const int64_t idx = (static_cast<int64_t>(i) * p.ny + j) * p.nz + k;
                        if (fixed[idx] != 0 || dirichlet_face(p, i, j, k)) continue;
                        const T o = field[idx];
                        const T c = density[idx] * um / (K + o);
                        const T prod = production_at<T>(p, production, source, idx);
                        const T gs = (neighbor_sum<T>(field, p, i, j, k) + h * prod) / (T(6) + h * c);
                        const T v = (T(1) - omega) * o + omega * gs;
                        field[idx] = std::fmax(v, T(0));
                    }
        }
    }
    if (residual_out) {
        T res = 0;
#pragma omp parallel for schedule(static) reduction(max : res)
        for (int i = 0; i < p.nx; ++i)
            for (int j = 0; j < p.ny; ++j)
                for (int k = 0; k < p.nz; ++k) {
                    const int64_t idx = (static_cast<int64_t>(i) * p.ny + j) * p.nz + k;
                    if (fixed[idx] != 0 || dirichlet_face(p, i, j, k)) continue;
                    const T o = field[idx];
                    const T c = density[idx] * um / (K + o);
                    const T prod = production_at<T>(p, production, source, idx);
                    const T r = neighbor_sum<T>(field, p, i, j, k) + h * prod - (T(6) + h * c) * o;
                    const T v = std::fabs(r) / std::fmax(T(6) * o, T(p.reference));
                    if (v > res || v != v) res = v;
                }
        *residual_out = res;
    }
}

// kernels/field_kernels.py:153-182 (clamped trilinear, lerp x then y then z)
template <typename T>
void sample(int nx, int ny, int nz, T ox, T oy, T oz, T inv_dx, const T* field, int n, const T* pos, T* out) {
#pragma omp parallel for schedule(static)
    for (int c = 0; c < n; ++c) {
        const T ux = (pos[3 * c] - ox) * inv_dx;
        const T uy = (pos[3 * c + 1] - oy) * inv_dx;
        const T uz = (pos[3 * c + 2] - oz) * inv_dx;
        const T cx = std::fmin(std::fmax(ux, T(0)), T(nx - 1));
        const T cy = std::fmin(std::fmax(uy, T(0)), T(ny - 1));
        const T cz = std::fmin(std::fmax(uz, T(0)), T(nz - 1));
        const int i0 = std::min(static_cast<int>(std::floor(cx)), nx - 2);
        const int j0 = std::min(static_cast<int>(std::floor(cy)), ny - 2);
        const int k0 = std::min(static_cast<int>(std::floor(cz)), nz - 2);
        const T fx = cx - T(i0), fy = cy - T(j0), fz = cz - T(k0);
        auto at = [&](int a, int b, int d) { return field[(static_cast<int64_t>(a) * ny + b) * nz + d]; };
        const T gx = T(1) - fx;
        const T c00 = at(i0, j0, k0) * gx + at(i0 + 1, j0, k0) * fx;
        const T c10 = at(i0, j0 + 1, k0) * gx + at(i0 + 1, j0 + 1, k0) * fx;
        const T c01 = at(i0, j0, k0 + 1) * gx + at(i0 + 1, j0, k0 + 1) * fx;
        const T c11 = at(i0, j0 + 1, k0 + 1) * gx + at(i0 + 1, j0 + 1, k0 + 1) * fx;
        const T c0 = c00 * (T(1) - fy) + c10 * fy;
        const T c1 = c01 * (T(1) - fy) + c11 * fy;
        out[c] = c0 * (T(1) - fz) + c1 * fz;
    }
}

// ---- Boolean networks (kernels/network_kernels.py) ------------------------------------------------
struct Program {
    int32_t n_nodes, n_words, n_ops, n_updatable;
    const int32_t *ops, *args, *start, *length, *updatable;
};

// get_bit / set_bit on the packed words (kernels/network_kernels.py:35-47).
inline uint64_t get_bit(const uint64_t* w, int idx) { return (w[idx >> 6] >> (idx & 63)) & 1ull; }
inline void set_bit(uint64_t* w, int idx, uint64_t v) {
    const uint64_t mask = 1ull << (idx & 63);
    w[idx >> 6] = v ? (w[idx >> 6] | mask) : (w[idx >> 6] & ~mask);
}

// Postfix program of one node on a one-word bit stack (kernels/network_kernels.py:50-78).
uint64_t eval_program(const Program& p, int node, const uint64_t* s) {
    uint64_t stack = 0;
    const int b = p.start[node], len = p.length[node];
    for (int k = 0; k < len; ++k) {
        const int op = p.ops[b + k], a = p.args[b + k];
        if (op == 0) {
            stack = (stack << 1) | get_bit(s, a);
        } else if (op == 4) {
            stack = (stack << 1) | static_cast<uint64_t>(static_cast<int64_t>(a));
        } else if (op == 1) {
            stack ^= 1ull;
        } else if (op == 2) {
            const uint64_t top = stack & 1ull;
            stack >>= 1;
            stack = (stack & ~1ull) | ((stack & 1ull) & top);
        } else if (op == 3) {
            const uint64_t top = stack & 1ull;
            stack >>= 1;
            stack = (stack & ~1ull) | ((stack & 1ull) | top);
        }
    }
    return stack & 1ull;
}

// Transition rate of one node in the MaBoSS chain (kernels/network_kernels.py:178-245).
inline float node_rate(uint64_t on, uint64_t logic, int node, const float* ut, const float* uf, const float* dt_,
                       const float* df) {
    if (on == 0ull) return logic ? ut[node] : uf[node];
    return logic ? dt_[node] : df[node];
}

}  // namespace

extern "C" {

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

// cells/state.py:25-28
void orc_rng_init(int32_t seed, uint32_t* state, int64_t capacity) {
    for (int64_t i = 0; i < capacity; ++i) state[i] = rng_start(seed, static_cast<uint32_t>(i));
}

// Draws from the project's own streams, as wp.randf / wp.sample_unit_sphere_surface are used at
// kernels/cell_kernels.py:129,151,183 (Warp's generator itself is not restated).
void orc_rng_uniform(int32_t n, int32_t draws, uint32_t* state, float* out) {
    for (int i = 0; i < n; ++i) {
        const uint32_t inc = rng_increment(static_cast<uint32_t>(i));
        for (int k = 0; k < draws; ++k) out[static_cast<int64_t>(i) * draws + k] = randf(state[i], inc);
    }
}

void orc_rng_sphere(int32_t n, uint32_t* state, float* out) {
    for (int i = 0; i < n; ++i) unit_sphere(state[i], rng_increment(static_cast<uint32_t>(i)), out[3 * i], out[3 * i + 1], out[3 * i + 2]);
}

// The project's exp / log (wp.exp at kernels/cell_kernels.py:128,150).
void orc_expf(int32_t n, const float* x, float* out) {
    for (int i = 0; i < n; ++i) out[i] = proj_expf(x[i]);
}

void orc_logf(int32_t n, const float* x, float* out) {
    for (int i = 0; i < n; ++i) out[i] = proj_logf(x[i]);
}

// spatial/neighbors.py:33-37 + kernels/mechanics_kernels.py:26-67
void orc_contact_substep_f32(int32_t n, float* pos, const float* radius, float cell_size, int32_t dim, float query_radius,
                             float rate, float dt, float* velocity, int32_t* neighbor_count) {
    std::vector<float> bin_pos(pos, pos + 3 * static_cast<size_t>(n));
    contact_substep<float>(n, pos, radius, bin_pos.data(), cell_size, dim, query_radius, rate, dt, velocity,
                           neighbor_count);
}

// The contact substep with the confinement push (cells/mechanics.py:75-110, kernels/geometry_kernels.py:59-79).
void orc_contact_substep_region_f32(int32_t n, float* pos, const float* radius, float cell_size, int32_t dim,
                                    float query_radius, float rate, float dt, int32_t rnx, int32_t rny, int32_t rnz,
                                    float rox, float roy, float roz, float rinv_dx, const float* sdf,
                                    const float* gradient, float wall_rate, float* velocity, int32_t* neighbor_count) {
    const Region R{rnx, rny, rnz, rox, roy, roz, rinv_dx, sdf, gradient, wall_rate};
    std::vector<float> bin_pos(pos, pos + 3 * static_cast<size_t>(n));
    contact_substep<float>(n, pos, radius, bin_pos.data(), cell_size, dim, query_radius, rate, dt, velocity,
                           neighbor_count, &R);
}

// FP64 re-run: same pairs and order (buckets from the float32 image of the positions).
void orc_contact_substep_f64(int32_t n, double* pos, const double* radius, float cell_size, int32_t dim,
                             double query_radius, double rate, double dt, double* velocity, int32_t* neighbor_count) {
    std::vector<float> bin_pos(3 * static_cast<size_t>(n));
    for (size_t q = 0; q < bin_pos.size(); ++q) bin_pos[q] = static_cast<float>(pos[q]);
    contact_substep<double>(n, pos, radius, bin_pos.data(), cell_size, dim, query_radius, rate, dt, velocity,
                            neighbor_count);
}

// kernels/field_kernels.py:78-116
void orc_deposit(int32_t nx, int32_t ny, int32_t nz, float ox, float oy, float oz, float inv_dx, int32_t n,
                 const float* pos, const int32_t* state, int64_t* acc) {
    const int64_t nodes = static_cast<int64_t>(nx) * ny * nz;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < n; ++c) {
        const int s = state[c];
        if (s < 0 || s >= 4) continue;
        const float ux = (pos[3 * c] - ox) * inv_dx;
        const float uy = (pos[3 * c + 1] - oy) * inv_dx;
        const float uz = (pos[3 * c + 2] - oz) * inv_dx;
        const int i0 = static_cast<int>(std::floor(ux));
        const int j0 = static_cast<int>(std::floor(uy));
        const int k0 = static_cast<int>(std::floor(uz));
        if (i0 < 0 || j0 < 0 || k0 < 0) continue;
        if (i0 + 1 >= nx || j0 + 1 >= ny || k0 + 1 >= nz) continue;
        const float fx = ux - static_cast<float>(i0);
        const float fy = uy - static_cast<float>(j0);
        const float fz = uz - static_cast<float>(k0);
        for (int di = 0; di < 2; ++di) {
            const float wx = di == 0 ? 1.0f - fx : fx;
            for (int dj = 0; dj < 2; ++dj) {
                const float wy = dj == 0 ? 1.0f - fy : fy;
                for (int dk = 0; dk < 2; ++dk) {
                    const float wz = dk == 0 ? 1.0f - fz : fz;
                    const float w = wx * wy * wz;
                    const int q = static_cast<int>(w * 16777216.0f + 0.5f);
                    const int64_t node = (static_cast<int64_t>(i0 + di) * ny + (j0 + dj)) * nz + (k0 + dk);
#pragma omp atomic
                    acc[s * nodes + node] += q;
                }
            }
        }
    }
}

// kernels/field_kernels.py:119-142
void orc_density_convert(int64_t nodes, const int64_t* acc, float inv_vol, float* density, const float* w,
                         float* combined) {
#pragma omp parallel for schedule(static)
    for (int64_t node = 0; node < nodes; ++node) {
        float d[4];
        for (int s = 0; s < 4; ++s) {
            d[s] = static_cast<float>(acc[s * nodes + node]) / 16777216.0f * inv_vol;
            if (density) density[s * nodes + node] = d[s];
        }
        if (combined) combined[node] = w[0] * d[0] + w[1] * d[1] + w[2] * d[2] + w[3] * d[3];
    }
}

void orc_sample_f32(int32_t nx, int32_t ny, int32_t nz, float ox, float oy, float oz, float inv_dx, const float* field,
                    int32_t n, const float* pos, float* out) {
    sample<float>(nx, ny, nz, ox, oy, oz, inv_dx, field, n, pos, out);
}

void orc_sample_f64(int32_t nx, int32_t ny, int32_t nz, double ox, double oy, double oz, double inv_dx,
                    const double* field, int32_t n, const double* pos, double* out) {
    sample<double>(nx, ny, nz, ox, oy, oz, inv_dx, field, n, pos, out);
}

// kernels/field_kernels.py:185-243 as launched by fields/diffusion.py:103-120
void orc_sor_sweeps_f32(const SorParams* p, int32_t sweeps, const int32_t* fixed, const float* density,
                        const float* production, const float* source, float* field, float* residual_out) {
    sor_sweeps<float>(*p, sweeps, fixed, density, production, source, field, residual_out);
}

void orc_sor_sweeps_f64(const SorParams* p, int32_t sweeps, const int32_t* fixed, const double* density,
                        const double* production, const double* source, double* field, double* residual_out) {
    sor_sweeps<double>(*p, sweeps, fixed, density, production, source, field, residual_out);
}

// kernels/field_kernels.py:246-273 (p->dx2_over_D carries D/dx^2)
void orc_ftcs_step_f32(const SorParams* p, float dt, const int32_t* fixed, const float* density,
                       const float* production, const float* source, const float* in, float* out) {
    const float D_over_dx2 = p->dx2_over_D;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < p->nx; ++i)
        for (int j = 0; j < p->ny; ++j)
            for (int k = 0; k < p->nz; ++k) {
                const int64_t idx = (static_cast<int64_t>(i) * p->ny + j) * p->nz + k;
                const float o = in[idx];
                if (fixed[idx] != 0 || dirichlet_face(*p, i, j, k)) {
                    out[idx] = o;
                    continue;
                }
                const float lap = D_over_dx2 * (neighbor_sum<float>(in, *p, i, j, k) - 6.0f * o);
                const float uptake = density[idx] * p->uptake_max * o / (p->michaelis_k + o);
                const float prod = production_at<float>(*p, production, source, idx);
                out[idx] = o + dt * (lap - uptake + prod);
            }
}

// ---- lifecycle (kernels/cell_kernels.py:68-208, cells/lifecycle.py:135-179) -----------------------------
struct LifecycleParams {
    float dt, death_rate, anoxic_death_rate, division_rate;
    int32_t inhibition_threshold;
    float hypoxia_threshold, death_threshold, glucose_threshold, glucose_death_threshold;
    int32_t necrosis_requires_glucose, phenotype_model;
    float apoptosis_rate, necrosis_rate;
};

static inline float oxygen_factor(float o, float hyp, float death) {
    if (o >= hyp) return 1.0f;
    if (o <= death) return 0.0f;
    return (o - death) / (hyp - death);
}

// kernels/cell_kernels.py:77-154 as launched by cells/lifecycle.py:96-132
void orc_lifecycle_decide(const LifecycleParams* pp, int32_t n, int32_t* cell_state, float* age,
                          const int32_t* neighbor_count, const float* oxygen_local, const float* glucose_local,
                          const int32_t* fate_flags, uint32_t* rng_state, int32_t* divide_flag) {
    const LifecycleParams& p = *pp;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        divide_flag[i] = 0;
        if (cell_state[i] == 3) continue;
        age[i] = age[i] + p.dt;
        uint32_t rng = rng_state[i];
        const uint32_t inc = rng_increment(static_cast<uint32_t>(i));
        const float o = oxygen_local[i], g = glucose_local[i];
        const int flags = p.phenotype_model == 1 ? fate_flags[i] : 0;
        bool lethal = o < p.death_threshold;
        if (p.necrosis_requires_glucose != 0) lethal = lethal && (g < p.glucose_death_threshold);
        float rate = p.death_rate;
        if (lethal) rate = std::fmax(p.death_rate, p.anoxic_death_rate);
        if (flags & 8) rate = std::fmax(rate, p.necrosis_rate);
        if (flags & 2) rate = std::fmax(rate, p.apoptosis_rate);
        const float p_death = 1.0f - proj_expf(-rate * p.dt);
        if (randf(rng, inc) < p_death) {
            cell_state[i] = 3;
            rng_state[i] = rng;
            continue;
        }
        const bool crowded = neighbor_count[i] >= p.inhibition_threshold;
        bool may_divide = !crowded;
        float factor = 1.0f;
        if (p.phenotype_model == 1)
            may_divide = may_divide && (flags & 1) != 0 && (flags & 4) == 0;
        else
            factor = oxygen_factor(o, p.hypoxia_threshold, p.death_threshold) *
                     oxygen_factor(g, p.glucose_threshold, p.glucose_death_threshold);
        if (o < p.hypoxia_threshold)
            cell_state[i] = 2;
        else if (may_divide)
            cell_state[i] = 0;
        else
            cell_state[i] = 1;
        if (may_divide) {
            const float p_divide = 1.0f - proj_expf(-p.division_rate * factor * p.dt);
            if (randf(rng, inc) < p_divide) divide_flag[i] = 1;
        }
        rng_state[i] = rng;
    }
}

// warp.utils.array_scan(inclusive=True) as used at cells/lifecycle.py:146; returns the total.
int32_t orc_division_scan(int32_t n, const int32_t* flags, int32_t* offsets) {
    int32_t run = 0;
    for (int i = 0; i < n; ++i) {
        run += flags[i];
        offsets[i] = run;
    }
    return run;
}

// kernels/cell_kernels.py:157-200
void orc_place_daughters(int32_t count, float placement_factor, const int32_t* divide_flag, const int32_t* division_offset,
                         float* position, float* radius, int32_t* cell_state, int32_t* cell_type, float* age,
                         float* oxygen_local, float* glucose_local, uint32_t* rng_state, float* velocity,
                         int32_t* neighbor_count, int32_t* fate_flags) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < count; ++i) {
        if (divide_flag[i] == 0) continue;
        const int j = count + division_offset[i] - 1;
        uint32_t rng = rng_state[i];
        float dx, dy, dz;
        unit_sphere(rng, rng_increment(static_cast<uint32_t>(i)), dx, dy, dz);
        rng_state[i] = rng;
        const float scale = 0.5f * placement_factor * radius[i];
        const float hx = dx * scale, hy = dy * scale, hz = dz * scale;
        const float x = position[3 * i], y = position[3 * i + 1], z = position[3 * i + 2];
        position[3 * i] = x - hx;
        position[3 * i + 1] = y - hy;
        position[3 * i + 2] = z - hz;
        position[3 * j] = x + hx;
        position[3 * j + 1] = y + hy;
        position[3 * j + 2] = z + hz;
        radius[j] = radius[i];
        cell_state[j] = cell_state[i];
        cell_type[j] = cell_type[i];
        age[j] = 0.0f;
        oxygen_local[j] = oxygen_local[i];
        glucose_local[j] = glucose_local[i];
        velocity[3 * j] = 0.0f;
        velocity[3 * j + 1] = 0.0f;
        velocity[3 * j + 2] = 0.0f;
        neighbor_count[j] = 0;
        fate_flags[j] = fate_flags[i];
    }
}

// kernels/cell_kernels.py:203-208
void orc_count_states(int32_t n, const int32_t* cell_state, int32_t* counts) {
    for (int i = 0; i < n; ++i)
        if (cell_state[i] >= 0 && cell_state[i] < 4) counts[cell_state[i]]++;
}

// ---- networks -----------------------------------------------------------------------------------------
// kernels/network_kernels.py:81-95
void orc_network_initialize(const Program* p, int32_t n, const float* p_on, uint32_t* rng_state, uint64_t* states) {
    for (int c = 0; c < n; ++c) {
        uint32_t rng = rng_state[c];
        const uint32_t inc = rng_increment(static_cast<uint32_t>(c));
        uint64_t* w = states + static_cast<int64_t>(c) * p->n_words;
        for (int q = 0; q < p->n_words; ++q) w[q] = 0;
        for (int i = 0; i < p->n_nodes; ++i)
            if (randf(rng, inc) < p_on[i]) set_bit(w, i, 1);
        rng_state[c] = rng;
    }
}

// kernels/network_kernels.py:98-132
void orc_network_clamp_inputs(int32_t n, int32_t n_words, int32_t n_clamps, const int32_t* node, const int32_t* source,
                              const float* threshold, const int32_t* above, const float* oxygen, const float* glucose,
                              const float* extra_a, const float* extra_b, uint64_t* states) {
    for (int c = 0; c < n; ++c) {
        uint64_t* w = states + static_cast<int64_t>(c) * n_words;
        for (int k = 0; k < n_clamps; ++k) {
            float value = 0.0f;
            if (source[k] == 0) value = oxygen[c];
            else if (source[k] == 1) value = glucose[c];
            else if (source[k] == 2) value = extra_a[c];
            else if (source[k] == 3) value = extra_b[c];
            bool on;
            if (source[k] == 4) on = threshold[k] > 0.0f;
            else if (above[k] != 0) on = value > threshold[k];
            else on = value < threshold[k];
            set_bit(w, node[k], on ? 1 : 0);
        }
    }
}

// kernels/network_kernels.py:157-175 (every updatable node from the old state)
void orc_network_update_sync(const Program* p, int32_t n, int32_t sweeps, uint64_t* states) {
#pragma omp parallel for schedule(static)
    for (int c = 0; c < n; ++c) {
        uint64_t* w = states + static_cast<int64_t>(c) * p->n_words;
        for (int s = 0; s < sweeps; ++s) {
            uint64_t next[4] = {0, 0, 0, 0};
            for (int q = 0; q < p->n_words; ++q) next[q] = w[q];
            for (int k = 0; k < p->n_updatable; ++k) {
                const int node = p->updatable[k];
                set_bit(next, node, eval_program(*p, node, w));
            }
            for (int q = 0; q < p->n_words; ++q) w[q] = next[q];
        }
    }
}

// kernels/network_kernels.py:135-154
void orc_network_update_async(const Program* p, int32_t n, int32_t n_updates, uint32_t* rng_state, uint64_t* states) {
#pragma omp parallel for schedule(static)
    for (int c = 0; c < n; ++c) {
        uint64_t* w = states + static_cast<int64_t>(c) * p->n_words;
        uint32_t rng = rng_state[c];
        const uint32_t inc = rng_increment(static_cast<uint32_t>(c));
        const int m = p->n_updatable;
        for (int k = 0; k < n_updates; ++k) {
            const int pick = std::min(static_cast<int>(randf(rng, inc) * static_cast<float>(m)), m - 1);
            const int node = p->updatable[pick];
            set_bit(w, node, eval_program(*p, node, w));
        }
        rng_state[c] = rng;
    }
}

// kernels/network_kernels.py:178-245
void orc_network_update_maboss(const Program* p, int32_t n, float duration, int32_t max_events, const float* ut,
                               const float* uf, const float* dt_, const float* df, uint32_t* rng_state,
                               uint64_t* states) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int c = 0; c < n; ++c) {
        uint64_t* w = states + static_cast<int64_t>(c) * p->n_words;
        uint32_t rng = rng_state[c];
        const uint32_t inc = rng_increment(static_cast<uint32_t>(c));
        const int m = p->n_updatable;
        float t = 0.0f;
        for (int event = 0; event < max_events; ++event) {
            float total = 0.0f;
            for (int k = 0; k < m; ++k) {
                const int node = p->updatable[k];
                total += node_rate(get_bit(w, node), eval_program(*p, node, w), node, ut, uf, dt_, df);
            }
            if (total <= 0.0f) break;
            const float u1 = std::fmax(randf(rng, inc), 1.0e-12f);
            const float tau = -proj_logf(u1) / total;
            if (t + tau > duration) break;
            t += tau;
            const float target = randf(rng, inc) * total;
            float acc = 0.0f;
            int chosen = -1;
            for (int k = 0; k < m; ++k) {
                if (chosen >= 0) break;
                const int node = p->updatable[k];
                const float r = node_rate(get_bit(w, node), eval_program(*p, node, w), node, ut, uf, dt_, df);
                acc += r;
                if (acc >= target && r > 0.0f) chosen = node;
            }
            if (chosen < 0) chosen = p->updatable[m - 1];
            set_bit(w, chosen, 1ull - get_bit(w, chosen));
        }
        rng_state[c] = rng;
    }
}

// kernels/network_kernels.py:248-268
void orc_network_read_fates(int32_t n, int32_t n_words, int32_t np, int32_t na, int32_t ng, int32_t nn,
                            const uint64_t* states, int32_t* fate_flags) {
    for (int c = 0; c < n; ++c) {
        const uint64_t* w = states + static_cast<int64_t>(c) * n_words;
        int flags = 0;
        if (np >= 0 && get_bit(w, np)) flags |= 1;
        if (na >= 0 && get_bit(w, na)) flags |= 2;
        if (ng >= 0 && get_bit(w, ng)) flags |= 4;
        if (nn >= 0 && get_bit(w, nn)) flags |= 8;
        fate_flags[c] = flags;
    }
}

// kernels/network_kernels.py:271-284
void orc_network_inherit(int32_t count_before, int32_t n_words, const int32_t* divide_flag,
                         const int32_t* division_offset, uint64_t* states) {
    for (int i = 0; i < count_before; ++i) {
        if (divide_flag[i] == 0) continue;
        const int j = count_before + division_offset[i] - 1;
        for (int q = 0; q < n_words; ++q) states[static_cast<int64_t>(j) * n_words + q] = states[static_cast<int64_t>(i) * n_words + q];
    }
}

// kernels/network_kernels.py:287-302
void orc_network_count_on(int32_t n, int32_t n_words, int32_t n_query, const int32_t* nodes, int32_t living_only,
                          const int32_t* cell_state, const uint64_t* states, int32_t* counts) {
    for (int c = 0; c < n; ++c) {
        if (living_only != 0 && cell_state[c] == 3) continue;
        const uint64_t* w = states + static_cast<int64_t>(c) * n_words;
        for (int k = 0; k < n_query; ++k)
            if (nodes[k] >= 0 && get_bit(w, nodes[k])) counts[k]++;
    }
}

// ---- FP64 forward of the adjoint model (finite-difference reference) ------------------------------------
// K contact steps in double, the per-cell uptake deposit with exact (unquantised) trilinear
// weights, and the steady Michaelis-Menten field in double with double parameters, Dirichlet
// faces at `boundary`, red-black SOR (omega) until max |r| / max(6 u, boundary) < tolerance.
// The GPU model quantises the deposit weights to 2^-24; the reference does not, so central
// differences of its loss measure the derivative of the exact model.
int32_t orc_adjoint_forward_f64(int32_t n, double* pos, const double* radius, const double* vmax, float cell_size,
                                int32_t dim, double query_radius, double rate, double dt, int32_t steps, int32_t nx,
                                int32_t ny, int32_t nz, const double* origin, double dx, double diffusion,
                                double michaelis_k, double boundary, double omega, double tolerance,
                                int32_t max_sweeps, double* field) {
    std::vector<double> vel(3 * static_cast<size_t>(n));
    std::vector<int32_t> nc(n);
    for (int32_t t = 0; t < steps; ++t)
        orc_contact_substep_f64(n, pos, radius, cell_size, dim, query_radius, rate, dt, vel.data(), nc.data());
    const int64_t nodes = static_cast<int64_t>(nx) * ny * nz;
    std::vector<double> U(nodes, 0.0);
    const double inv_dx = 1.0 / dx, inv_vol = inv_dx * inv_dx * inv_dx;
    for (int32_t c = 0; c < n; ++c) {
        const double ux = (pos[3 * c] - origin[0]) * inv_dx, uy = (pos[3 * c + 1] - origin[1]) * inv_dx,
                     uz = (pos[3 * c + 2] - origin[2]) * inv_dx;
        const int i0 = static_cast<int>(std::floor(ux)), j0 = static_cast<int>(std::floor(uy)),
                  k0 = static_cast<int>(std::floor(uz));
        if (i0 < 0 || j0 < 0 || k0 < 0 || i0 + 1 >= nx || j0 + 1 >= ny || k0 + 1 >= nz) continue;
        const double fx = ux - i0, fy = uy - j0, fz = uz - k0;
        for (int di = 0; di < 2; ++di)
            for (int dj = 0; dj < 2; ++dj)
                for (int dk = 0; dk < 2; ++dk) {
                    const double w = (di ? fx : 1.0 - fx) * (dj ? fy : 1.0 - fy) * (dk ? fz : 1.0 - fz);
                    U[(static_cast<int64_t>(i0 + di) * ny + (j0 + dj)) * nz + (k0 + dk)] += w * vmax[c] * inv_vol;
                }
    }
    const double h = dx * dx / diffusion;
    for (int64_t a = 0; a < nodes; ++a) field[a] = boundary;
    auto interior = [&](int i, int j, int k) { return i > 0 && j > 0 && k > 0 && i < nx - 1 && j < ny - 1 && k < nz - 1; };
    const double ref = boundary > 0.0 ? boundary : 1.0;
    int32_t sweeps = 0;
    while (sweeps < max_sweeps) {
        for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static)
            for (int i = 1; i < nx - 1; ++i)
                for (int j = 1; j < ny - 1; ++j)
                    for (int k = 1 + ((colour + i + j + 1) & 1); k < nz - 1; k += 2) {
                        const int64_t a = (static_cast<int64_t>(i) * ny + j) * nz + k;
                        const double o = field[a];
                        const double nb = field[a - static_cast<int64_t>(ny) * nz] + field[a + static_cast<int64_t>(ny) * nz] +
                                          field[a - nz] + field[a + nz] + field[a - 1] + field[a + 1];
                        const double gs = nb / (6.0 + h * U[a] / (michaelis_k + o));
                        field[a] = std::max((1.0 - omega) * o + omega * gs, 0.0);
                    }
        }
        ++sweeps;
        if (sweeps % 20 != 0) continue;
        double res = 0.0;
#pragma omp parallel for reduction(max : res) schedule(static)
        for (int i = 1; i < nx - 1; ++i)
            for (int j = 1; j < ny - 1; ++j)
                for (int k = 1; k < nz - 1; ++k) {
                    if (!interior(i, j, k)) continue;
                    const int64_t a = (static_cast<int64_t>(i) * ny + j) * nz + k;
                    const double o = field[a];
                    const double nb = field[a - static_cast<int64_t>(ny) * nz] + field[a + static_cast<int64_t>(ny) * nz] +
                                      field[a - nz] + field[a + nz] + field[a - 1] + field[a + 1];
                    const double r = nb - (6.0 + h * U[a] / (michaelis_k + o)) * o;
                    // nodes at the clamp (o = 0 with a negative unclamped update) are settled
                    if (o == 0.0 && r <= 0.0) continue;
                    res = std::max(res, std::fabs(r) / std::max(6.0 * o, ref));
                }
        if (res < tolerance) break;
    }
    return sweeps;
}

// ---- FP64 reverse of the contact steps (checks of the GPU adjoint) --------------------------------------
// The contact law of contact_substep, v_i = rate sum_j (R/d - 1) e_ij over the pairs with d < query
// radius, R - d > 0 and d > 1e-6, in double, from the positions after `steps` FP64 steps; the reverse
// sweep lambda_t = lambda_{t+1} + dt J(x_t)^T lambda_{t+1} with (J^T lambda)_i = rate sum_j A_ij
// (lambda_i - lambda_j), A_ij = (R/d - 1) I - R e e^T / d^3, and dL/drate = dt sum_t lambda_{t+1} .
// v(x_t) / rate. On entry `lambda` holds dL/dx_K; on return dL/dx_0. Pairs come from the buckets of
// the float32 image of the positions, as orc_contact_substep_f64.
void orc_adjoint_contact_f64(int32_t n, const double* pos0, const double* radius, float cell_size, int32_t dim,
                             double query_radius, double rate, double dt, int32_t steps, double* lambda,
                             double* d_rate) {
    const size_t n3 = 3 * static_cast<size_t>(n);
    std::vector<double> traj(n3 * static_cast<size_t>(steps > 0 ? steps : 1));
    std::vector<double> pos(pos0, pos0 + n3), vel(n3);
    std::vector<int32_t> nc(n);
    for (int32_t t = 0; t < steps; ++t) {
        std::copy(pos.begin(), pos.end(), traj.begin() + n3 * t);
        orc_contact_substep_f64(n, pos.data(), radius, cell_size, dim, query_radius, rate, dt, vel.data(), nc.data());
    }
    std::vector<double> lam(lambda, lambda + n3), out(n3);
    std::vector<float> bin(n3);
    double total = 0.0;
    for (int32_t t = steps - 1; t >= 0; --t) {
        const double* x = traj.data() + n3 * t;
        for (size_t q = 0; q < n3; ++q) bin[q] = static_cast<float>(x[q]);
        Buckets bk;
        bk.build(n, bin.data(), cell_size, dim);
        double step_dot = 0.0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : step_dot)
        for (int i = 0; i < n; ++i) {
            const int cx = bk.coord(bin[3 * i]), cy = bk.coord(bin[3 * i + 1]), cz = bk.coord(bin[3 * i + 2]);
            double g[3] = {0, 0, 0}, u[3] = {0, 0, 0};
            for (int ox = -1; ox <= 1; ++ox)
                for (int oy = -1; oy <= 1; ++oy)
                    for (int oz = -1; oz <= 1; ++oz) {
                        const int b = bk.bucket(cx + ox, cy + oy, cz + oz);
                        for (int s = bk.start[b], e = s + bk.count[b]; s < e; ++s) {
                            const int j = bk.ids[s];
                            if (j == i) continue;
                            const double e3[3] = {x[3 * i] - x[3 * j], x[3 * i + 1] - x[3 * j + 1],
                                                  x[3 * i + 2] - x[3 * j + 2]};
                            const double d = std::sqrt(e3[0] * e3[0] + e3[1] * e3[1] + e3[2] * e3[2]);
                            if (!(d < query_radius)) continue;
                            const double R = radius[i] + radius[j];
                            if (!(R - d > 0.0 && d > 1.0e-6)) continue;
                            const double a = R / d - 1.0;
                            const double l[3] = {lam[3 * i] - lam[3 * j], lam[3 * i + 1] - lam[3 * j + 1],
                                                 lam[3 * i + 2] - lam[3 * j + 2]};
                            const double proj = R / (d * d * d) * (e3[0] * l[0] + e3[1] * l[1] + e3[2] * l[2]);
                            for (int c = 0; c < 3; ++c) {
                                u[c] += a * e3[c];
                                g[c] += a * l[c] - proj * e3[c];
                            }
                        }
                    }
            for (int c = 0; c < 3; ++c) out[3 * i + c] = lam[3 * i + c] + dt * rate * g[c];
            step_dot += lam[3 * i] * u[0] + lam[3 * i + 1] * u[1] + lam[3 * i + 2] * u[2];
        }
        total += step_dot;
        lam.swap(out);
    }
    std::copy(lam.begin(), lam.end(), lambda);
    *d_rate = dt * total;
}

// Contact pairs (i < j with d < query radius, R - d > 0 and d > 1e-6) present at a step of one FP64
// trajectory but not of the other, summed over the steps: trajectories from the same start with
// contact rates rate_a and rate_b. Counts where a finite difference in the rate steps over the
// force law's kink at contact onset.
int64_t orc_contact_crossings_f64(int32_t n, const double* pos0, const double* radius, float cell_size, int32_t dim,
                                  double query_radius, double rate_a, double rate_b, double dt, int32_t steps) {
    const size_t n3 = 3 * static_cast<size_t>(n);
    std::vector<double> pa(pos0, pos0 + n3), pb(pos0, pos0 + n3), vel(n3);
    std::vector<int32_t> nc(n);
    std::vector<float> ba(n3), bb(n3);
    int64_t crossings = 0;
    auto pairs_of = [&](const Buckets& bk, const std::vector<float>& bin, const std::vector<double>& x, int i,
                        std::vector<int32_t>& out) {
        out.clear();
        const int cx = bk.coord(bin[3 * i]), cy = bk.coord(bin[3 * i + 1]), cz = bk.coord(bin[3 * i + 2]);
        for (int ox = -1; ox <= 1; ++ox)
            for (int oy = -1; oy <= 1; ++oy)
                for (int oz = -1; oz <= 1; ++oz) {
                    const int b = bk.bucket(cx + ox, cy + oy, cz + oz);
                    for (int s = bk.start[b], e = s + bk.count[b]; s < e; ++s) {
                        const int j = bk.ids[s];
                        if (j <= i) continue;
                        const double dx = x[3 * i] - x[3 * j], dy = x[3 * i + 1] - x[3 * j + 1],
                                     dz = x[3 * i + 2] - x[3 * j + 2];
                        const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
                        if (d < query_radius && radius[i] + radius[j] - d > 0.0 && d > 1.0e-6) out.push_back(j);
                    }
                }
        std::sort(out.begin(), out.end());
    };
    for (int32_t t = 0; t <= steps; ++t) {
        for (size_t q = 0; q < n3; ++q) {
            ba[q] = static_cast<float>(pa[q]);
            bb[q] = static_cast<float>(pb[q]);
        }
        Buckets ka, kb;
        ka.build(n, ba.data(), cell_size, dim);
        kb.build(n, bb.data(), cell_size, dim);
        int64_t step_count = 0;
#pragma omp parallel reduction(+ : step_count)
        {
            std::vector<int32_t> la, lb;
#pragma omp for schedule(dynamic, 256)
            for (int i = 0; i < n; ++i) {
                pairs_of(ka, ba, pa, i, la);
                pairs_of(kb, bb, pb, i, lb);
                size_t x = 0, y = 0;
                while (x < la.size() || y < lb.size()) {
                    if (y == lb.size() || (x < la.size() && la[x] < lb[y])) {
                        ++step_count;
                        ++x;
                    } else if (x == la.size() || lb[y] < la[x]) {
                        ++step_count;
                        ++y;
                    } else {
                        ++x;
                        ++y;
                    }
                }
            }
        }
        crossings += step_count;
        if (t == steps) break;
        orc_contact_substep_f64(n, pa.data(), radius, cell_size, dim, query_radius, rate_a, dt, vel.data(), nc.data());
        orc_contact_substep_f64(n, pb.data(), radius, cell_size, dim, query_radius, rate_b, dt, vel.data(), nc.data());
    }
    return crossings;
}

// FP64 field half of the adjoint (Dirichlet faces on every side, the adjoint model's boundary): for
// the steady field u of orc_adjoint_forward_f64 (cells at `pos`, capacities `vmax`) and dL/du = g,
// solves (6 + h kappa_a) mu_a - sum_nb mu_nb = g_a (kappa_a = U_a K / (K + u_a)^2; mu = 0 on the faces
// and where u_a = 0) by red-black SOR in double to a max residual below `tolerance` relative to
// max(6 |mu|, |g|), then forms sums = {dL/dK, dL/dD, dL/dO_b}, dL/dVmax_i = -h inv_vol sum_a w_a(x_i)
// phi_a (phi_a = mu_a u_a / (K + u_a)) and adds -h inv_vol Vmax_i grad_x sum_a w_a(x) phi_a to grad_x.
// Returns the sweeps run.
int32_t orc_adjoint_field_f64(int32_t nx, int32_t ny, int32_t nz, const double* origin, double dx, double diffusion,
                              double michaelis_k, int32_t n, const double* pos, const double* vmax, const double* u,
                              const double* g, double omega, double tolerance, int32_t max_sweeps, double* sums,
                              double* grad_vmax, double* grad_x) {
    const int64_t nodes = static_cast<int64_t>(nx) * ny * nz;
    const double inv_dx = 1.0 / dx, inv_vol = inv_dx * inv_dx * inv_dx, h = dx * dx / diffusion;
    auto cell_corner = [&](int c, int& i0, int& j0, int& k0, double& fx, double& fy, double& fz) {
        const double ux = (pos[3 * c] - origin[0]) * inv_dx, uy = (pos[3 * c + 1] - origin[1]) * inv_dx,
                     uz = (pos[3 * c + 2] - origin[2]) * inv_dx;
        i0 = static_cast<int>(std::floor(ux));
        j0 = static_cast<int>(std::floor(uy));
        k0 = static_cast<int>(std::floor(uz));
        if (i0 < 0 || j0 < 0 || k0 < 0 || i0 + 1 >= nx || j0 + 1 >= ny || k0 + 1 >= nz) return false;
        fx = ux - i0;
        fy = uy - j0;
        fz = uz - k0;
        return true;
    };
    std::vector<double> U(nodes, 0.0), kappa(nodes, -1.0), mu(nodes, 0.0), phi(nodes, 0.0);
    for (int c = 0; c < n; ++c) {
        int i0, j0, k0;
        double fx, fy, fz;
        if (!cell_corner(c, i0, j0, k0, fx, fy, fz)) continue;
        for (int di = 0; di < 2; ++di)
            for (int dj = 0; dj < 2; ++dj)
                for (int dk = 0; dk < 2; ++dk)
                    U[(static_cast<int64_t>(i0 + di) * ny + (j0 + dj)) * nz + (k0 + dk)] +=
                        (di ? fx : 1.0 - fx) * (dj ? fy : 1.0 - fy) * (dk ? fz : 1.0 - fz) * vmax[c] * inv_vol;
    }
    auto interior = [&](int i, int j, int k) { return i > 0 && j > 0 && k > 0 && i < nx - 1 && j < ny - 1 && k < nz - 1; };
    for (int i = 1; i < nx - 1; ++i)
        for (int j = 1; j < ny - 1; ++j)
            for (int k = 1; k < nz - 1; ++k) {
                const int64_t a = (static_cast<int64_t>(i) * ny + j) * nz + k;
                if (u[a] > 0.0) kappa[a] = U[a] * michaelis_k / ((michaelis_k + u[a]) * (michaelis_k + u[a]));
            }
    const int64_t sx = static_cast<int64_t>(ny) * nz;
    int32_t sweeps = 0;
    while (sweeps < max_sweeps) {
        for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static)
            for (int i = 1; i < nx - 1; ++i)
                for (int j = 1; j < ny - 1; ++j)
                    for (int k = 1 + ((colour + i + j + 1) & 1); k < nz - 1; k += 2) {
                        const int64_t a = (static_cast<int64_t>(i) * ny + j) * nz + k;
                        if (!(kappa[a] >= 0.0)) continue;
                        const double nb = mu[a - sx] + mu[a + sx] + mu[a - nz] + mu[a + nz] + mu[a - 1] + mu[a + 1];
                        mu[a] = (1.0 - omega) * mu[a] + omega * (nb + g[a]) / (6.0 + h * kappa[a]);
                    }
        }
        ++sweeps;
        if (sweeps % 20 != 0) continue;
        double res = 0.0, scale = 0.0;
#pragma omp parallel for reduction(max : res, scale) schedule(static)
        for (int i = 1; i < nx - 1; ++i)
            for (int j = 1; j < ny - 1; ++j)
                for (int k = 1; k < nz - 1; ++k) {
                    const int64_t a = (static_cast<int64_t>(i) * ny + j) * nz + k;
                    if (!(kappa[a] >= 0.0)) continue;
                    const double nb = mu[a - sx] + mu[a + sx] + mu[a - nz] + mu[a + nz] + mu[a - 1] + mu[a + 1];
                    res = std::max(res, std::fabs(nb + g[a] - (6.0 + h * kappa[a]) * mu[a]));
                    scale = std::max(scale, std::max(6.0 * std::fabs(mu[a]), std::fabs(g[a])));
                }
        if (res <= tolerance * scale) break;
    }
    double s_k = 0.0, s_d = 0.0, s_b = 0.0;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const int64_t a = (static_cast<int64_t>(i) * ny + j) * nz + k;
                if (!interior(i, j, k)) {
                    s_b += g[a];
                    continue;
                }
                if (!(kappa[a] >= 0.0)) continue;
                const double ua = u[a], m = mu[a], sk = michaelis_k + ua;
                phi[a] = m * ua / sk;
                s_k += m * h * U[a] * ua / (sk * sk);
                s_d += m * h * U[a] * ua / (sk * diffusion);
                const int faces = (i == 1) + (i == nx - 2) + (j == 1) + (j == ny - 2) + (k == 1) + (k == nz - 2);
                s_b += m * faces;
            }
    sums[0] = s_k;
    sums[1] = s_d;
    sums[2] = s_b;
    const double coef = -h * inv_vol;
    for (int c = 0; c < n; ++c) {
        int i0, j0, k0;
        double fx, fy, fz;
        if (!cell_corner(c, i0, j0, k0, fx, fy, fz)) {
            grad_vmax[c] = 0.0;
            continue;
        }
        double sv = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
        for (int di = 0; di < 2; ++di)
            for (int dj = 0; dj < 2; ++dj)
                for (int dk = 0; dk < 2; ++dk) {
                    const double wx = di ? fx : 1.0 - fx, wy = dj ? fy : 1.0 - fy, wz = dk ? fz : 1.0 - fz;
                    const double dwx = di ? 1.0 : -1.0, dwy = dj ? 1.0 : -1.0, dwz = dk ? 1.0 : -1.0;
                    const double ph = phi[(static_cast<int64_t>(i0 + di) * ny + (j0 + dj)) * nz + (k0 + dk)];
                    sv += wx * wy * wz * ph;
                    gx += dwx * wy * wz * ph;
                    gy += wx * dwy * wz * ph;
                    gz += wx * wy * dwz * ph;
                }
        grad_vmax[c] = coef * sv;
        const double f = coef * vmax[c] * inv_dx;
        grad_x[3 * c] += f * gx;
        grad_x[3 * c + 1] += f * gy;
        grad_x[3 * c + 2] += f * gz;
    }
    return sweeps;
}

}  // extern "C"
