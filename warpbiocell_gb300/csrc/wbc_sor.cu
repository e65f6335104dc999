// Red-black SOR solve to convergence in one persistent, cooperative launch with the field held
// in shared memory (kernels/field_kernels.py:185-243 iterated as fields/diffusion.py:79-123).
//
// Decomposition: the (i, j) plane is cut into tx x ty tiles of ti x tj columns; each CTA (one
// per SM) owns one tile with the full z extent. Shared memory holds the tile plus a one-column
// halo ring, split by k parity (E[col][m] = f(k = 2m), O[col][m] = f(k = 2m + 1)): within a
// column all nodes of one colour share a k parity, so a warp that owns a column updates its
// colour with 32 consecutive words per access and no bank conflicts, and the k-neighbours of
// node m are entries m - 1 + kp and m + kp of the other parity (clamped at the ends, which is
// exactly the reference's mirror rule). At the start each CTA writes the uptake coefficients
// density * uptake_max of its columns, split the same way, to an L2-resident scratch copy (a
// negative value marks the nodes that are never updated: Dirichlet faces and pinned nodes).
//
// One colour half-sweep = every warp updates its columns' nodes of that colour from shared
// memory; the tile-edge columns' updated colour is published to a parity-split exchange buffer
// in global memory (L2, bypassing L1); a grid barrier; then the halo ring's updated colour is
// pulled back into shared memory. Every `check_every` sweeps the max-norm residual is reduced
// (warp shuffles, one atomicMax per CTA) and all CTAs stop together once it is below the
// tolerance: the reference's sweep count, residual and stopping rule, with no host round trip.
// Each node's update is the reference kernel's float expression in the same order, so the field
// after n sweeps is bit-identical to the oracle's and to the streaming kernels'.
//
// Grid barrier: every CTA stores the barrier's epoch to its own flag (release), then its threads
// poll all CTAs' flags in parallel (acquire); no two CTAs update the same word. The polls are
// bounded (about a second); on timeout the CTA raises an abort flag, every CTA leaves, and the
// host gets WBC_ERR_TIMEOUT.
#include <algorithm>
#include <mutex>

#include "wbc_common.cuh"

namespace wbc {

struct __align__(128) SorControl {
    unsigned int abort;
    unsigned int res_bits[2];
    int sweeps;
    float residual;
    int converged;
    int status;
    int pad[25];
};
static_assert(sizeof(SorControl) == 128, "SorControl is one 128-byte line");
constexpr int kMaxCtas = 1024;  // barrier flags that follow the control block

struct SorTiling {
    int tx, ty;  // CTAs along i and j
    int ti, tj;  // tile extent (columns) along i and j
    int M;       // (nz + 1) / 2 entries per parity per column
    int threads;
    size_t smem;
};

struct SorArgs {
    wbc_sor_params p;
    SorTiling t;
    const int32_t* fixed;
    const float* density;
    const float* production;
    const float* source;
    float* field;
    float* xchg;   // [2][nx][ny][M] halo exchange
    float* coeff;  // [2][nx][ny][M] density * uptake_max, -1 where not updated
    SorControl* ctl;
    unsigned int* flags;  // [gridDim.x] barrier epochs
    int check_every;
    int max_sweeps;
    double tolerance;  // compared in double, as the reference compares float(residual) < tolerance
};

constexpr unsigned kBarrierPolls = 1u << 21;  // L2 round trips: about a second
constexpr int kMaxLanesPerColumn = 8;         // M <= 256 (nz <= 511)

__device__ __forceinline__ unsigned int load_acquire(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void store_release(unsigned int* p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int mirror(int i, int n) { return i < 0 ? 1 : (i > n - 1 ? n - 2 : i); }

// Signals this CTA's arrival at the next epoch, then waits for the CTAs listed in `wait_for`
// (n_wait of them) or, with n_wait < 0, for every CTA. Returns false when aborted (timeout here or
// elsewhere). A halo exchange only needs the four neighbouring tiles; the residual needs all.
__device__ __forceinline__ bool grid_barrier(SorControl* ctl, unsigned int* flags, unsigned int& epoch,
                                             const int* wait_for = nullptr, int n_wait = -1) {
    epoch += 1;
    __syncthreads();  // the CTA's writes happen before thread 0's release (bar.sync is cumulative)
    if (threadIdx.x == 0) store_release(flags + blockIdx.x, epoch);
    int aborted = 0;
    const unsigned n = n_wait < 0 ? gridDim.x : static_cast<unsigned>(n_wait);
    for (unsigned t = threadIdx.x; t < n; t += blockDim.x) {
        const unsigned who = n_wait < 0 ? t : static_cast<unsigned>(wait_for[t]);
        unsigned polls = 0;
        while (static_cast<int>(load_acquire(flags + who) - epoch) < 0) {
            if ((++polls & 255u) == 0u) {
                if (load_acquire(&ctl->abort) != 0u) {
                    aborted = 1;
                    break;
                }
                if (polls > kBarrierPolls) {
                    atomicExch(&ctl->abort, 1u);
                    aborted = 1;
                    break;
                }
            }
        }
    }
    return __syncthreads_or(aborted) == 0;
}

struct TileGeom {
    int i0, j0, ai, aj;  // tile origin and actual extent
    int stride_i;        // columns per smem row (tj + 2)
    int ncm;             // (ti + 2) * (tj + 2) * M: floats per parity plane in shared memory
};

__device__ __forceinline__ float prod_term(const SorArgs& a, int64_t idx) {
    const float prod = a.production ? a.production[idx] : 0.0f;
    if (!a.p.has_source) return prod * 1.0f;
    const float v = a.source[idx];
    return prod * (v / (a.p.source_k + v));
}

// Column r of the halo ring (pull) as tile coordinates.
__device__ __forceinline__ void ring_column(const TileGeom& g, int r, int& li, int& lj) {
    if (r < g.aj) {
        li = -1;
        lj = r;
    } else if (r < 2 * g.aj) {
        li = g.ai;
        lj = r - g.aj;
    } else if (r < 2 * g.aj + g.ai) {
        li = r - 2 * g.aj;
        lj = -1;
    } else {
        li = r - 2 * g.aj - g.ai;
        lj = g.aj;
    }
}

// Column r of the published set: rows[0..nrow) x all lj, then cols[0..ncol) x all li.
__device__ __forceinline__ bool publish_column(const TileGeom& g, const int* rows, int nrow, const int* cols, int r,
                                               int& li, int& lj) {
    if (r < nrow * g.aj) {
        const int q = r / g.aj;
        li = rows[q];
        lj = r - q * g.aj;
    } else {
        const int rr = r - nrow * g.aj;
        const int q = rr / g.ai;
        lj = cols[q];
        li = rr - q * g.ai;
    }
    return li >= 0 && li < g.ai && lj >= 0 && lj < g.aj;
}

template <bool HAS_PROD, int LANES>
__global__ void __launch_bounds__(1024, 1) k_sor_resident(SorArgs a) {
    extern __shared__ float s[];
    __shared__ unsigned int s_red[32];
    const int M = a.t.M, nz = a.p.nz, nx = a.p.nx, ny = a.p.ny;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    TileGeom g;
    int neighbours[4], n_neighbours = 0;  // tiles whose edge columns form this tile's halo
    {
        const int bx = blockIdx.x / a.t.ty;
        const int by = blockIdx.x - bx * a.t.ty;
        g.i0 = bx * a.t.ti;
        g.j0 = by * a.t.tj;
        g.ai = min(a.t.ti, nx - g.i0);
        g.aj = min(a.t.tj, ny - g.j0);
        g.stride_i = a.t.tj + 2;
        g.ncm = (a.t.ti + 2) * (a.t.tj + 2) * M;
        if (bx > 0) neighbours[n_neighbours++] = blockIdx.x - a.t.ty;
        if (bx + 1 < a.t.tx) neighbours[n_neighbours++] = blockIdx.x + a.t.ty;
        if (by > 0) neighbours[n_neighbours++] = blockIdx.x - 1;
        if (by + 1 < a.t.ty) neighbours[n_neighbours++] = blockIdx.x + 1;
    }
    // Per (column, colour) table after the two parity planes: shared-memory offsets of the own
    // and other parity column, the coefficient row, and the entry count / last other entry / parity.
    int4* tab = reinterpret_cast<int4*>(s + ((2 * g.ncm + 3) & ~3));
    const int64_t sx = static_cast<int64_t>(ny) * nz;
    const int si = g.stride_i * M;
    // Columns other tiles read: the edge rows / columns, plus the second one on a Neumann face
    // (its mirror image is the halo of this very tile).
    int rows[4], cols[4], nrow = 0, ncol = 0;
    rows[nrow++] = 0;
    if (g.ai > 1) rows[nrow++] = g.ai - 1;
    if (a.p.bc_x == 1 && g.i0 == 0 && g.ai > 1) rows[nrow++] = 1;
    if (a.p.bc_x == 1 && g.i0 + g.ai == nx && g.ai > 2) rows[nrow++] = g.ai - 2;
    cols[ncol++] = 0;
    if (g.aj > 1) cols[ncol++] = g.aj - 1;
    if (a.p.bc_y == 1 && g.j0 == 0 && g.aj > 1) cols[ncol++] = 1;
    if (a.p.bc_y == 1 && g.j0 + g.aj == ny && g.aj > 2) cols[ncol++] = g.aj - 2;
    const int n_publish = nrow * g.aj + ncol * g.ai;
    const int n_ring = 2 * (g.ai + g.aj);
    const int ncolumns = g.ai * g.aj;

    // Tile + halo ring (mirrored at the domain faces) into shared memory; the owned columns'
    // coefficients into the parity-split scratch copy; the column table.
    {
        const int span = g.aj + 2;
        const int cols_all = (g.ai + 2) * span;
        for (int col = warp; col < cols_all; col += nwarps) {
            const int lrow = col / span;
            const int li = lrow - 1, lj = col - lrow * span - 1;
            const int gi = mirror(g.i0 + li, nx), gj = mirror(g.j0 + lj, ny);
            const int c2 = (li + 1) * g.stride_i + (lj + 1);
            const bool owned = li >= 0 && li < g.ai && lj >= 0 && lj < g.aj;
            const int64_t base = gi * sx + static_cast<int64_t>(gj) * nz;
            for (int k = lane; k < nz; k += 32) {
                const int64_t idx = base + k;
                s[(k & 1) * g.ncm + c2 * M + (k >> 1)] = a.field[idx];
                if (owned) {
                    const wbc_sor_params& p = a.p;
                    const bool face = (p.bc_x == 0 && (gi == 0 || gi == nx - 1)) ||
                                      (p.bc_y == 0 && (gj == 0 || gj == ny - 1)) ||
                                      (p.bc_z == 0 && (k == 0 || k == nz - 1));
                    float v = -1.0f;
                    if (!face && !(a.fixed && a.fixed[idx] != 0)) v = a.density[idx] * p.uptake_max;
                    a.coeff[((static_cast<int64_t>(k & 1) * nx + gi) * ny + gj) * M + (k >> 1)] = v;
                }
            }
        }
        for (int e = threadIdx.x; e < 2 * ncolumns; e += blockDim.x) {
            const int col = e >> 1, colour = e & 1;
            const int li = col / g.aj, lj = col - (col / g.aj) * g.aj;
            const int gi = g.i0 + li, gj = g.j0 + lj;
            const int kp = (colour + gi + gj) & 1;
            const int c2 = (li + 1) * g.stride_i + (lj + 1);
            const int cnt = kp ? nz / 2 : (nz + 1) / 2;
            const int last = (kp ? (nz + 1) / 2 : nz / 2) - 1;
            tab[e] = make_int4(kp * g.ncm + c2 * M, (kp ^ 1) * g.ncm + c2 * M,
                               static_cast<int>(((static_cast<int64_t>(kp) * nx + gi) * ny + gj) * M),
                               cnt | (last << 9) | (kp << 18));
        }
    }
    __syncthreads();

    const float omega = a.p.omega;
    const float one_minus_omega = 1.0f - omega;
    const float h = a.p.dx2_over_D;
    const float K = a.p.michaelis_k;
    const float* __restrict__ coeff = a.coeff;
    unsigned int epoch = 0;
    int sweeps = 0;
    float residual = __int_as_float(0x7f800000);
    bool converged = false;
    bool ok = true;
    int chunk_index = 0;
    while (sweeps < a.max_sweeps) {
        const int chunk = min(a.check_every, a.max_sweeps - sweeps);
        for (int sweep = 0; sweep < chunk && ok; ++sweep) {
            for (int colour = 0; colour < 2 && ok; ++colour) {
                for (int col = warp; col < ncolumns; col += nwarps) {
                    const int4 e = tab[2 * col + colour];
                    const int cnt = e.w & 511, last = (e.w >> 9) & 511, kp = e.w >> 18;
                    float du[LANES];
#pragma unroll
                    for (int r = 0; r < LANES; ++r) {
                        const int m = lane + 32 * r;
                        du[r] = m < cnt ? coeff[e.z + m] : -1.0f;
                    }
#pragma unroll
                    for (int r = 0; r < LANES; ++r) {
                        if (!(du[r] >= 0.0f)) continue;
                        const int m = lane + 32 * r;
                        const int io = e.x + m;
                        const float o = s[io];
                        const float c = du[r] / (K + o);
                        float prod = 0.0f;
                        if (HAS_PROD) {
                            const int li = col / g.aj, lj = col - (col / g.aj) * g.aj;
                            prod = prod_term(a, (g.i0 + li) * sx + static_cast<int64_t>(g.j0 + lj) * nz + 2 * m + kp);
                        }
                        const float nb = s[io - si] + s[io + si] + s[io - M] + s[io + M] + s[e.y + max(m + kp - 1, 0)] +
                                         s[e.y + min(m + kp, last)];
                        const float gs = (nb + h * prod) / (6.0f + h * c);
                        s[io] = fmaxf(one_minus_omega * o + omega * gs, 0.0f);
                    }
                }
                __syncthreads();
                // publish the updated colour of the columns other tiles read
                for (int r = warp; r < n_publish; r += nwarps) {
                    int li, lj;
                    if (!publish_column(g, rows, nrow, cols, r, li, lj)) continue;
                    const int gi = g.i0 + li, gj = g.j0 + lj;
                    const int kpar = (colour + gi + gj) & 1;
                    const int cnt = kpar ? nz / 2 : (nz + 1) / 2;
                    float* x = a.xchg + ((static_cast<int64_t>(kpar) * nx + gi) * ny + gj) * M;
                    const float* sm = s + kpar * g.ncm + ((li + 1) * g.stride_i + (lj + 1)) * M;
                    for (int m = lane; m < cnt; m += 32) __stcg(x + m, sm[m]);
                }
                // A neighbour overwrites these entries only after this tile has signalled the next
                // epoch, i.e. after the pull below: waiting for the four neighbours suffices.
                ok = grid_barrier(a.ctl, a.flags, epoch, neighbours, n_neighbours);
                if (!ok) break;
                // pull the halo ring's updated colour (mirroring moves i, j by 2: parity kept)
                for (int r = warp; r < n_ring; r += nwarps) {
                    int li, lj;
                    ring_column(g, r, li, lj);
                    const int gi_u = g.i0 + li, gj_u = g.j0 + lj;
                    const int kpar = (colour + gi_u + gj_u) & 1;
                    const int cnt = kpar ? nz / 2 : (nz + 1) / 2;
                    const int gi = mirror(gi_u, nx), gj = mirror(gj_u, ny);
                    const float* x = a.xchg + ((static_cast<int64_t>(kpar) * nx + gi) * ny + gj) * M;
                    float* sm = s + kpar * g.ncm + ((li + 1) * g.stride_i + (lj + 1)) * M;
                    for (int m = lane; m < cnt; m += 32) sm[m] = __ldcg(x + m);
                }
                __syncthreads();
            }
        }
        if (!ok) break;
        sweeps += chunk;
        // Max-norm residual of the current field over every updated node (both colours).
        unsigned int bits = 0u;
        for (int e2 = warp; e2 < 2 * ncolumns; e2 += nwarps) {
            const int4 e = tab[e2];
            const int col = e2 >> 1;
            const int cnt = e.w & 511, last = (e.w >> 9) & 511, kp = e.w >> 18;
            for (int m = lane; m < cnt; m += 32) {
                const float du = coeff[e.z + m];
                if (!(du >= 0.0f)) continue;
                const int io = e.x + m;
                const float o = s[io];
                const float c = du / (K + o);
                float prod = 0.0f;
                if (HAS_PROD) {
                    const int li = col / g.aj, lj = col - (col / g.aj) * g.aj;
                    prod = prod_term(a, (g.i0 + li) * sx + static_cast<int64_t>(g.j0 + lj) * nz + 2 * m + kp);
                }
                const float nb = s[io - si] + s[io + si] + s[io - M] + s[io + M] + s[e.y + max(m + kp - 1, 0)] +
                                 s[e.y + min(m + kp, last)];
                const float r = nb + h * prod - (6.0f + h * c) * o;
                const float val = fabsf(r) / fmaxf(6.0f * o, a.p.reference);
                bits = max(bits, __float_as_uint(val));
            }
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, d));
        if (lane == 0) s_red[warp] = bits;
        __syncthreads();
        const int slot = chunk_index & 1;
        if (warp == 0) {
            bits = lane < nwarps ? s_red[lane] : 0u;
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, d));
            if (lane == 0) atomicMax(&a.ctl->res_bits[slot], bits);
        }
        ok = grid_barrier(a.ctl, a.flags, epoch);
        if (!ok) break;
        residual = __uint_as_float(load_acquire(&a.ctl->res_bits[slot]));
        // The next chunk's slot was last read before this chunk's first barrier: safe to clear.
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(&a.ctl->res_bits[slot ^ 1], 0u);
        ++chunk_index;
        if (static_cast<double>(residual) < a.tolerance) {
            converged = true;
            break;
        }
    }
    if (!ok) {
        if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl->status = 1;
        return;
    }
    // Owned columns back to the field.
    for (int col = warp; col < ncolumns; col += nwarps) {
        const int li = col / g.aj;
        const int lj = col - li * g.aj;
        const int c2 = (li + 1) * g.stride_i + (lj + 1);
        float* out = a.field + (g.i0 + li) * sx + static_cast<int64_t>(g.j0 + lj) * nz;
        for (int k = lane; k < nz; k += 32) out[k] = s[(k & 1) * g.ncm + c2 * M + (k >> 1)];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ctl->sweeps = sweeps;
        a.ctl->residual = residual;
        a.ctl->converged = converged ? 1 : 0;
        a.ctl->status = 0;
    }
}

// ---- host side -------------------------------------------------------------------------------------------
using KernelFn = void (*)(SorArgs);

template <bool P>
static KernelFn kernel_for_lanes(int lanes) {
    switch (lanes) {
        case 1: return k_sor_resident<P, 1>;
        case 2: return k_sor_resident<P, 2>;
        case 3: return k_sor_resident<P, 3>;
        case 4: return k_sor_resident<P, 4>;
        case 5: return k_sor_resident<P, 5>;
        case 6: return k_sor_resident<P, 6>;
        case 7: return k_sor_resident<P, 7>;
        default: return k_sor_resident<P, 8>;
    }
}

static KernelFn kernel_for(bool has_prod, int lanes) {
    return has_prod ? kernel_for_lanes<true>(lanes) : kernel_for_lanes<false>(lanes);
}

struct DeviceInfo {
    int sms = 0;
    int smem_optin = 0;
};

static DeviceInfo device_info() {
    static std::mutex mu;
    static DeviceInfo cache[64];
    static bool have[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 0 && dev < 64 && have[dev]) return cache[dev];
    DeviceInfo d;
    cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (dev >= 0 && dev < 64) {
        cache[dev] = d;
        have[dev] = true;
    }
    return d;
}

// tx x ty tiles, at most one CTA per SM, minimising the columns of the largest tile (then the
// halo perimeter); the tile plus halo must fit in shared memory.
static bool choose_tiling(const wbc_sor_params& p, int sms, size_t smem_limit, SorTiling* out) {
    const int M = (p.nz + 1) / 2;
    if (M > 32 * kMaxLanesPerColumn) return false;
    bool found = false;
    SorTiling best{};
    long best_score = 0;
    const int max_ctas = std::min(sms, kMaxCtas);
    for (int tx = 1; tx <= std::min(p.nx, max_ctas); ++tx) {
        const int ty_max = std::min(p.ny, max_ctas / tx);
        for (int ty = 1; ty <= ty_max; ++ty) {
            const int ti = (p.nx + tx - 1) / tx, tj = (p.ny + ty - 1) / ty;
            if (ti < 2 || tj < 2) continue;
            const int ex = (p.nx + ti - 1) / ti, ey = (p.ny + tj - 1) / tj;
            const size_t planes = (2ull * (ti + 2) * (tj + 2) * M + 3) & ~3ull;
            const size_t smem = planes * sizeof(float) + 2ull * ti * tj * sizeof(int4);
            if (smem > smem_limit) continue;
            const long score = static_cast<long>(ti) * tj * 1000 + (ti + tj);
            if (!found || score < best_score) {
                found = true;
                best_score = score;
                const int warps = std::min(32, ti * tj);
                best = SorTiling{ex, ey, ti, tj, M, 32 * warps, smem};
            }
        }
    }
    if (found) *out = best;
    return found;
}

static size_t plane_bytes(const wbc_sor_params& p) {
    return 2ull * p.nx * p.ny * ((p.nz + 1) / 2) * sizeof(float);
}

static size_t header_bytes() { return sizeof(SorControl) + kMaxCtas * sizeof(unsigned int); }

size_t sor_workspace_bytes(const wbc_sor_params& p) { return header_bytes() + 2 * plane_bytes(p) + 256; }

int sor_solve_resident(const wbc_sor_params& p, int check_every, int max_sweeps, double tolerance,
                       const int32_t* fixed, const float* density, const float* production, const float* source,
                       float* field, wbc_sor_report* report, void* workspace, cudaStream_t stream, bool* feasible) {
    const DeviceInfo dev = device_info();
    SorTiling t{};
    const size_t reserve = 1024;  // static shared memory of the kernel
    *feasible = dev.sms > 0 && choose_tiling(p, dev.sms, static_cast<size_t>(dev.smem_optin) - reserve, &t);
    if (!*feasible) return WBC_OK;
    const bool has_prod = production != nullptr || p.has_source;
    KernelFn fn = kernel_for(has_prod, (t.M + 31) / 32);
    cudaError_t err = cudaFuncSetAttribute(reinterpret_cast<const void*>(fn),
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(t.smem));
    if (err != cudaSuccess) {
        set_error("wbc_sor_solve: cudaFuncSetAttribute", err);
        return WBC_ERR_CUDA;
    }
    int per_sm = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, t.threads, t.smem);
    if (err != cudaSuccess || per_sm < 1 || t.tx * t.ty > per_sm * dev.sms) {
        cudaGetLastError();
        *feasible = false;
        return WBC_OK;
    }
    char* base = reinterpret_cast<char*>(workspace);
    auto* ctl = reinterpret_cast<SorControl*>(base);
    auto* flags = reinterpret_cast<unsigned int*>(base + sizeof(SorControl));
    float* xchg = reinterpret_cast<float*>(base + header_bytes());
    float* coeff = reinterpret_cast<float*>(base + header_bytes() + plane_bytes(p));
    err = cudaMemsetAsync(base, 0, header_bytes(), stream);
    if (err != cudaSuccess) {
        set_error("wbc_sor_solve: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    SorArgs args{p,     t,    fixed,       density,    production, source,   field,
                 xchg,  coeff, ctl,        flags,      check_every, max_sweeps, tolerance};
    void* params[] = {&args};
    err = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(fn), dim3(t.tx * t.ty), dim3(t.threads), params,
                                      t.smem, stream);
    if (err != cudaSuccess) {
        set_error("wbc_sor_solve: cudaLaunchCooperativeKernel", err);
        return WBC_ERR_CUDA;
    }
    int rc = check_launch("wbc_sor_solve", 1);
    if (rc != WBC_OK) return rc;
    SorControl host{};
    err = cudaMemcpyAsync(&host, ctl, sizeof(SorControl), cudaMemcpyDeviceToHost, stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
    if (err != cudaSuccess) {
        set_error("wbc_sor_solve: reading the report", err);
        return WBC_ERR_CUDA;
    }
    if (host.status != 0) {
        set_error_msg("wbc_sor_solve: grid barrier timed out");
        return WBC_ERR_TIMEOUT;
    }
    report->sweeps = host.sweeps;
    report->residual = host.residual;
    report->converged = host.converged;
    report->path = 2;
    report->tiles = t.tx * t.ty;
    return WBC_OK;
}

}  // namespace wbc

using namespace wbc;

extern "C" {

size_t wbc_sor_solve_workspace_bytes(const wbc_sor_params* p) {
    if (!p) return 0;
    return sor_workspace_bytes(*p);
}

int wbc_sor_solve(const wbc_sor_params* p, int32_t check_every, int32_t max_sweeps, double tolerance,
                  const int32_t* fixed, const float* density, const float* production, const float* source,
                  float* field, wbc_sor_report* report, void* workspace, size_t workspace_bytes, int32_t path,
                  void* stream) {
    if (!p || p->nx < 3 || p->ny < 3 || p->nz < 3 || check_every < 1 || max_sweeps < 1 || !density || !field ||
        !report || !workspace || (p->has_source && !source) || path < 0 || path > 2)
        return WBC_ERR_INVALID;
    if (workspace_bytes < sor_workspace_bytes(*p)) return WBC_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    bool feasible = false;
    if (path != 1) {
        int rc = sor_solve_resident(*p, check_every, max_sweeps, tolerance, fixed, density, production, source, field,
                                    report, workspace, s, &feasible);
        if (rc != WBC_OK || feasible) return rc;
        if (path == 2) {
            set_error_msg("wbc_sor_solve: the grid does not fit the shared-memory resident solver");
            return WBC_ERR_INVALID;
        }
    }
    // Streaming path: colour launches with a host check of the residual every check_every sweeps.
    float* residual_dev = reinterpret_cast<float*>(reinterpret_cast<char*>(workspace) + header_bytes());
    int sweeps = 0;
    float residual = __builtin_inff();
    while (sweeps < max_sweeps) {
        const int chunk = std::min(check_every, max_sweeps - sweeps);
        int rc = wbc_sor_sweeps(p, chunk, fixed, density, production, source, field, residual_dev, stream);
        if (rc != WBC_OK) return rc;
        sweeps += chunk;
        cudaError_t err = cudaMemcpyAsync(&residual, residual_dev, sizeof(float), cudaMemcpyDeviceToHost, s);
        if (err == cudaSuccess) err = cudaStreamSynchronize(s);
        if (err != cudaSuccess) {
            set_error("wbc_sor_solve: reading the residual", err);
            return WBC_ERR_CUDA;
        }
        if (static_cast<double>(residual) < tolerance) break;
    }
    report->sweeps = sweeps;
    report->residual = residual;
    report->converged = static_cast<double>(residual) < tolerance ? 1 : 0;
    report->path = 1;
    report->tiles = 0;
    return WBC_OK;
}

}  // extern "C"
