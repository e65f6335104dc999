// Red-black SOR solve to convergence in one persistent, cooperative launch with the field held
// in shared memory (kernels/field_kernels.py:185-243 iterated as fields/diffusion.py:79-123).
//
// Decomposition: the (i, j) plane is cut into tx x ty tiles of ti x tj columns; each CTA (one
// per SM) owns one tile with the full z extent. Shared memory holds the tile plus a one-column
// halo ring, split by k parity (E[col][m] = f(k = 2m), O[col][m] = f(k = 2m + 1)): within a
// column all nodes of one colour share a k parity, so a warp that owns a column updates its
// colour with 32 consecutive words per access and no bank conflicts. At the start each CTA
// writes the uptake coefficients density * uptake_max of its columns, split the same way, to an
// L2-resident scratch copy (a negative value marks the nodes that are never updated: Dirichlet
// faces and pinned nodes); a colour reads only its own coefficients, contiguously.
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
// The grid barrier polls a bounded number of times (about a second); on timeout the CTA raises
// an abort flag, every CTA leaves, and the host gets WBC_ERR_TIMEOUT.
#include <algorithm>
#include <mutex>

#include "wbc_common.cuh"

namespace wbc {

struct SorControl {
    unsigned int bar_count;
    unsigned int bar_gen;
    unsigned int abort;
    unsigned int res_bits[2];
    int sweeps;
    float residual;
    int converged;
    int status;
    int pad[7];
};
static_assert(sizeof(SorControl) == 64, "SorControl is one 64-byte block");

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
    int check_every;
    int max_sweeps;
    double tolerance;  // compared in double, as the reference compares float(residual) < tolerance
};

constexpr unsigned kBarrierPolls = 1u << 24;  // x ~64 ns sleep: about a second
constexpr int kMaxLanesPerColumn = 8;         // M <= 256 (nz <= 511)

__device__ __forceinline__ int mirror(int i, int n) { return i < 0 ? 1 : (i > n - 1 ? n - 2 : i); }

// Returns false when the barrier was aborted (timeout here or elsewhere).
__device__ __forceinline__ bool grid_barrier(SorControl* ctl, unsigned nblocks, unsigned& gen, int* s_abort) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned arrived = atomicAdd(&ctl->bar_count, 1u);
        if (arrived == nblocks - 1) {
            atomicExch(&ctl->bar_count, 0u);
            __threadfence();
            atomicAdd(&ctl->bar_gen, 1u);
        } else {
            unsigned polls = 0;
            while (atomicAdd(&ctl->bar_gen, 0u) == gen) {
                if (atomicAdd(&ctl->abort, 0u) != 0u) break;
                if (++polls > kBarrierPolls) {
                    atomicExch(&ctl->abort, 1u);
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        *s_abort = atomicAdd(&ctl->abort, 0u) != 0u;
    }
    gen += 1;
    __syncthreads();
    return *s_abort == 0;
}

struct TileGeom {
    int i0, j0, ai, aj;  // tile origin and actual extent
    int stride_i;        // columns per smem row (tj + 2)
    int ncm;             // (ti + 2) * (tj + 2) * M: floats per parity plane in shared memory
};

// Sum of the six neighbours (im, ip, jm, jp, km, kp in the reference's order), mirrored in k.
__device__ __forceinline__ float neighbour_sum(const float* s, int ncm, int M, int nz, int stride_i, int c2, int k) {
    const int par = (k & 1) * ncm;
    const int km = k - 1 < 0 ? 1 : k - 1;
    const int kp = k + 1 > nz - 1 ? nz - 2 : k + 1;
    const int mk = k >> 1;
    return s[par + (c2 - stride_i) * M + mk] + s[par + (c2 + stride_i) * M + mk] + s[par + (c2 - 1) * M + mk] +
           s[par + (c2 + 1) * M + mk] + s[(km & 1) * ncm + c2 * M + (km >> 1)] +
           s[(kp & 1) * ncm + c2 * M + (kp >> 1)];
}

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

// Column r of the published set: rows rows[0..nrow) x all lj, then cols[0..ncol) x all li.
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

template <bool HAS_PROD>
__global__ void __launch_bounds__(1024, 1) k_sor_resident(SorArgs a) {
    extern __shared__ float s[];
    __shared__ unsigned int s_red[32];
    __shared__ int s_abort;
    const int M = a.t.M, nz = a.p.nz, nx = a.p.nx, ny = a.p.ny;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    TileGeom g;
    {
        const int bx = blockIdx.x / a.t.ty;
        const int by = blockIdx.x - bx * a.t.ty;
        g.i0 = bx * a.t.ti;
        g.j0 = by * a.t.tj;
        g.ai = min(a.t.ti, nx - g.i0);
        g.aj = min(a.t.tj, ny - g.j0);
        g.stride_i = a.t.tj + 2;
        g.ncm = (a.t.ti + 2) * (a.t.tj + 2) * M;
    }
    const int64_t sx = static_cast<int64_t>(ny) * nz;
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
    const int lanes_m = (M + 31) >> 5;

    // Tile + halo ring (mirrored at the domain faces) into shared memory; the owned columns'
    // coefficients into the parity-split scratch copy.
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
    }
    __syncthreads();

    const float omega = a.p.omega;
    const float one_minus_omega = 1.0f - omega;
    const float h = a.p.dx2_over_D;
    const float K = a.p.michaelis_k;
    unsigned gen = 0;
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
                    const int li = col / g.aj, lj = col - (col / g.aj) * g.aj;
                    const int gi = g.i0 + li, gj = g.j0 + lj;
                    const int kp = (colour + gi + gj) & 1;
                    const int c2 = (li + 1) * g.stride_i + (lj + 1);
                    const float* crow = a.coeff + ((static_cast<int64_t>(kp) * nx + gi) * ny + gj) * M;
                    float du[kMaxLanesPerColumn];
#pragma unroll
                    for (int r = 0; r < kMaxLanesPerColumn; ++r) {
                        const int m = lane + 32 * r;
                        du[r] = (r < lanes_m && m < M) ? crow[m] : -1.0f;
                    }
#pragma unroll
                    for (int r = 0; r < kMaxLanesPerColumn; ++r) {
                        if (r >= lanes_m) break;
                        const int m = lane + 32 * r;
                        const int k = 2 * m + kp;
                        if (!(du[r] >= 0.0f) || k >= nz) continue;
                        float* own = s + kp * g.ncm + c2 * M + m;
                        const float o = *own;
                        const float c = du[r] / (K + o);
                        float prod = 0.0f;
                        if (HAS_PROD) prod = prod_term(a, gi * sx + static_cast<int64_t>(gj) * nz + k);
                        const float gs =
                            (neighbour_sum(s, g.ncm, M, nz, g.stride_i, c2, k) + h * prod) / (6.0f + h * c);
                        *own = fmaxf(one_minus_omega * o + omega * gs, 0.0f);
                    }
                }
                __syncthreads();
                // publish the updated colour of the columns other tiles read
                for (int r = warp; r < n_publish; r += nwarps) {
                    int li, lj;
                    if (!publish_column(g, rows, nrow, cols, r, li, lj)) continue;
                    const int gi = g.i0 + li, gj = g.j0 + lj;
                    const int kpar = (colour + gi + gj) & 1;
                    const int c2 = (li + 1) * g.stride_i + (lj + 1);
                    float* x = a.xchg + ((static_cast<int64_t>(kpar) * nx + gi) * ny + gj) * M;
                    const float* sm = s + kpar * g.ncm + c2 * M;
                    for (int m = lane; m < M; m += 32)
                        if (2 * m + kpar < nz) __stcg(x + m, sm[m]);
                }
                ok = grid_barrier(a.ctl, gridDim.x, gen, &s_abort);
                if (!ok) break;
                // pull the halo ring's updated colour (mirroring moves i, j by 2: parity kept)
                for (int r = warp; r < n_ring; r += nwarps) {
                    int li, lj;
                    ring_column(g, r, li, lj);
                    const int gi_u = g.i0 + li, gj_u = g.j0 + lj;
                    const int kpar = (colour + gi_u + gj_u) & 1;
                    const int gi = mirror(gi_u, nx), gj = mirror(gj_u, ny);
                    const int c2 = (li + 1) * g.stride_i + (lj + 1);
                    const float* x = a.xchg + ((static_cast<int64_t>(kpar) * nx + gi) * ny + gj) * M;
                    float* sm = s + kpar * g.ncm + c2 * M;
                    for (int m = lane; m < M; m += 32)
                        if (2 * m + kpar < nz) sm[m] = __ldcg(x + m);
                }
                __syncthreads();
            }
        }
        if (!ok) break;
        sweeps += chunk;
        // Max-norm residual of the current field over every updated node.
        unsigned int bits = 0u;
        for (int col = warp; col < ncolumns; col += nwarps) {
            const int li = col / g.aj, lj = col - (col / g.aj) * g.aj;
            const int gi = g.i0 + li, gj = g.j0 + lj;
            const int c2 = (li + 1) * g.stride_i + (lj + 1);
            for (int kp = 0; kp < 2; ++kp) {
                const float* crow = a.coeff + ((static_cast<int64_t>(kp) * nx + gi) * ny + gj) * M;
                for (int m = lane; m < M; m += 32) {
                    const int k = 2 * m + kp;
                    if (k >= nz) continue;
                    const float du = crow[m];
                    if (!(du >= 0.0f)) continue;
                    const float o = s[kp * g.ncm + c2 * M + m];
                    const float c = du / (K + o);
                    float prod = 0.0f;
                    if (HAS_PROD) prod = prod_term(a, gi * sx + static_cast<int64_t>(gj) * nz + k);
                    const float r = neighbour_sum(s, g.ncm, M, nz, g.stride_i, c2, k) + h * prod - (6.0f + h * c) * o;
                    const float v = fabsf(r) / fmaxf(6.0f * o, a.p.reference);
                    bits = max(bits, __float_as_uint(v));
                }
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
        ok = grid_barrier(a.ctl, gridDim.x, gen, &s_abort);
        if (!ok) break;
        residual = __uint_as_float(atomicAdd(&a.ctl->res_bits[slot], 0u));
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
        const int li = col / g.aj, lj = col - (col / g.aj) * g.aj;
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
    for (int tx = 1; tx <= std::min(p.nx, sms); ++tx) {
        const int ty_max = std::min(p.ny, sms / tx);
        for (int ty = 1; ty <= ty_max; ++ty) {
            const int ti = (p.nx + tx - 1) / tx, tj = (p.ny + ty - 1) / ty;
            if (ti < 2 || tj < 2) continue;
            const int ex = (p.nx + ti - 1) / ti, ey = (p.ny + tj - 1) / tj;
            const size_t smem = 2ull * (ti + 2) * (tj + 2) * M * sizeof(float);
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

size_t sor_workspace_bytes(const wbc_sor_params& p) { return sizeof(SorControl) + 2 * plane_bytes(p) + 256; }

int sor_solve_resident(const wbc_sor_params& p, int check_every, int max_sweeps, double tolerance,
                       const int32_t* fixed, const float* density, const float* production, const float* source,
                       float* field, wbc_sor_report* report, void* workspace, cudaStream_t stream, bool* feasible) {
    const DeviceInfo dev = device_info();
    SorTiling t{};
    const size_t reserve = 1024;  // static shared memory of the kernel
    *feasible = dev.sms > 0 && choose_tiling(p, dev.sms, static_cast<size_t>(dev.smem_optin) - reserve, &t);
    if (!*feasible) return WBC_OK;
    const bool has_prod = production != nullptr || p.has_source;
    KernelFn fn = has_prod ? k_sor_resident<true> : k_sor_resident<false>;
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
    float* xchg = reinterpret_cast<float*>(base + sizeof(SorControl));
    float* coeff = reinterpret_cast<float*>(base + sizeof(SorControl) + plane_bytes(p));
    err = cudaMemsetAsync(ctl, 0, sizeof(SorControl), stream);
    if (err != cudaSuccess) {
        set_error("wbc_sor_solve: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    SorArgs args{p, t, fixed, density, production, source, field, xchg, coeff, ctl, check_every, max_sweeps, tolerance};
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
    float* residual_dev = reinterpret_cast<float*>(reinterpret_cast<char*>(workspace) + sizeof(SorControl));
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
