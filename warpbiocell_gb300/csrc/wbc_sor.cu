// Red-black SOR solve to convergence in one persistent, cooperative launch with the field held
// in shared memory (kernels/field_kernels.py:185-243 iterated as fields/diffusion.py:79-123).
//
// Decomposition: the (i, j) plane is cut into tx x ty tiles of ti x tj columns; each CTA (one
// per SM) owns one tile with the full z extent. Shared memory holds the tile plus a one-column
// halo ring, split by k parity (E[col][m] = f(k = 2m), O[col][m] = f(k = 2m + 1)) so a warp
// updating consecutive nodes of one colour reads consecutive words. At the start each CTA
// writes the uptake coefficients density * uptake_max of its columns, split the same way, to an
// L2-resident scratch copy (a negative value marks the nodes that are never updated: Dirichlet
// faces and pinned nodes), so a colour reads only its own coefficients, contiguously.
//
// One colour half-sweep = update the owned nodes of that colour from shared memory, publish the
// updated colour of the columns within one column of the tile edge to a parity-split exchange
// buffer in global memory (L2 resident, bypassing L1), a grid barrier, then pull the halo
// ring's updated colour back into shared memory. Every `check_every` sweeps the max-norm
// residual is reduced (warp shuffles, one atomicMax per CTA) and all CTAs stop together once it
// is below the tolerance: the reference's sweep count, residual and stopping rule, with no host
// round trip. Each node's update is the reference kernel's float expression in the same order,
// so the field after n sweeps is bit-identical to the oracle's and to the streaming kernels'.
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
    float* xchg;    // [2][nx][ny][M] halo exchange
    float* coeff;   // [2][nx][ny][M] density * uptake_max, -1 where not updated
    SorControl* ctl;
    int check_every;
    int max_sweeps;
    double tolerance;  // compared in double, as the reference compares float(residual) < tolerance
};

constexpr unsigned kBarrierPolls = 1u << 24;  // x ~64 ns sleep: about a second

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
                __nanosleep(64);
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

// Slot walker: the thread's slots are linear indices t, t + T, ... over (li, lj, m) in
// [0,ai) x [0,aj) x [0,M), advanced incrementally (no division inside the sweep loops).
struct Walker {
    int li, lj, m;
    int dli, dlj, dm;
    __device__ __forceinline__ void step(int M, int aj) {
        m += dm;
        lj += dlj;
        li += dli;
        if (m >= M) {
            m -= M;
            lj += 1;
        }
        if (lj >= aj) {
            lj -= aj;
            li += 1;
        }
    }
};

__device__ __forceinline__ Walker make_walker(int M, int aj) {
    Walker w;
    const int t = threadIdx.x, T = blockDim.x;
    const int lc = t / M;
    w.m = t - lc * M;
    w.li = lc / aj;
    w.lj = lc - w.li * aj;
    const int dlc = T / M;
    w.dm = T - dlc * M;
    w.dli = dlc / aj;
    w.dlj = dlc - w.dli * aj;
    return w;
}

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

// Publish the updated colour of the columns within one column of the tile edge (pull = false),
// or pull the halo ring's updated colour from the exchange buffer (pull = true).
__device__ __forceinline__ void exchange(float* s, const SorArgs& a, const TileGeom& g, int colour, bool pull) {
    const int M = a.t.M, nz = a.p.nz, nx = a.p.nx, ny = a.p.ny;
    const int perim = pull ? 2 * (g.ai + g.aj) : 4 * (g.ai + g.aj);
    const int total = perim * M;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int r = e / M;
        const int m = e - r * M;
        int li, lj;
        if (pull) {
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
        } else {
            // rows li in {0, 1, ai-2, ai-1} x all lj, then columns lj in {0, 1, aj-2, aj-1} x all li
            if (r < 4 * g.aj) {
                const int which = r / g.aj;
                lj = r - which * g.aj;
                li = which < 2 ? which : g.ai - 4 + which;
            } else {
                const int q = r - 4 * g.aj;
                const int which = q / g.ai;
                li = q - which * g.ai;
                lj = which < 2 ? which : g.aj - 4 + which;
            }
            if (li < 0 || li >= g.ai || lj < 0 || lj >= g.aj) continue;
        }
        const int gi_u = g.i0 + li, gj_u = g.j0 + lj;
        const int kpar = (colour + gi_u + gj_u) & 1;  // mirroring moves i, j by 2: parity kept
        if (2 * m + kpar >= nz) continue;
        const int c2 = (li + 1) * g.stride_i + (lj + 1);
        const int gi = mirror(gi_u, nx), gj = mirror(gj_u, ny);
        float* x = a.xchg + ((static_cast<int64_t>(kpar) * nx + gi) * ny + gj) * M + m;
        float* sm = s + kpar * g.ncm + c2 * M + m;
        if (pull)
            *sm = __ldcg(x);
        else
            __stcg(x, *sm);
    }
}

template <bool HAS_PROD>
__global__ void __launch_bounds__(1024, 1) k_sor_resident(SorArgs a) {
    extern __shared__ float s[];
    __shared__ unsigned int s_red[32];
    __shared__ int s_abort;
    const int M = a.t.M, nz = a.p.nz, nx = a.p.nx, ny = a.p.ny;
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

    // Tile + halo ring (mirrored at the domain faces) into shared memory; the owned columns'
    // coefficients into the parity-split scratch copy.
    {
        const int cols = (g.ai + 2) * (g.aj + 2);
        for (int e = threadIdx.x; e < cols * nz; e += blockDim.x) {
            const int col = e / nz;
            const int k = e - col * nz;
            const int lrow = col / (g.aj + 2);
            const int li = lrow - 1, lj = col - lrow * (g.aj + 2) - 1;
            const int gi_u = g.i0 + li, gj_u = g.j0 + lj;
            const int gi = mirror(gi_u, nx), gj = mirror(gj_u, ny);
            const int c2 = (li + 1) * g.stride_i + (lj + 1);
            const int64_t idx = gi * sx + static_cast<int64_t>(gj) * nz + k;
            s[(k & 1) * g.ncm + c2 * M + (k >> 1)] = a.field[idx];
            if (li >= 0 && li < g.ai && lj >= 0 && lj < g.aj) {
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
    __syncthreads();

    const float omega = a.p.omega;
    const float one_minus_omega = 1.0f - omega;
    const float h = a.p.dx2_over_D;
    const float K = a.p.michaelis_k;
    const int slots = g.ai * g.aj * M;
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
                Walker w = make_walker(M, g.aj);
                for (int L = threadIdx.x; L < slots; L += blockDim.x, w.step(M, g.aj)) {
                    const int gi = g.i0 + w.li, gj = g.j0 + w.lj;
                    const int kp = (colour + gi + gj) & 1;
                    const int k = 2 * w.m + kp;
                    if (k >= nz) continue;
                    const float du = a.coeff[((static_cast<int64_t>(kp) * nx + gi) * ny + gj) * M + w.m];
                    if (!(du >= 0.0f)) continue;
                    const int c2 = (w.li + 1) * g.stride_i + (w.lj + 1);
                    float* own = s + kp * g.ncm + c2 * M + w.m;
                    const float o = *own;
                    const float c = du / (K + o);
                    float prod = 0.0f;
                    if (HAS_PROD) prod = prod_term(a, gi * sx + static_cast<int64_t>(gj) * nz + k);
                    const float gs = (neighbour_sum(s, g.ncm, M, nz, g.stride_i, c2, k) + h * prod) / (6.0f + h * c);
                    *own = fmaxf(one_minus_omega * o + omega * gs, 0.0f);
                }
                __syncthreads();
                exchange(s, a, g, colour, false);
                ok = grid_barrier(a.ctl, gridDim.x, gen, &s_abort);
                if (!ok) break;
                exchange(s, a, g, colour, true);
                __syncthreads();
            }
        }
        if (!ok) break;
        sweeps += chunk;
        // Max-norm residual of the current field over every updated node.
        unsigned int bits = 0u;
        {
            Walker w = make_walker(M, g.aj);
            for (int L = threadIdx.x; L < slots; L += blockDim.x, w.step(M, g.aj)) {
                const int gi = g.i0 + w.li, gj = g.j0 + w.lj;
                const int c2 = (w.li + 1) * g.stride_i + (w.lj + 1);
#pragma unroll
                for (int kp = 0; kp < 2; ++kp) {
                    const int k = 2 * w.m + kp;
                    if (k >= nz) continue;
                    const float du = a.coeff[((static_cast<int64_t>(kp) * nx + gi) * ny + gj) * M + w.m];
                    if (!(du >= 0.0f)) continue;
                    const float o = s[kp * g.ncm + c2 * M + w.m];
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
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = bits;
        __syncthreads();
        const int slot = chunk_index & 1;
        if (threadIdx.x < 32) {
            bits = threadIdx.x < (blockDim.x >> 5) ? s_red[threadIdx.x] : 0u;
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, d));
            if (threadIdx.x == 0) atomicMax(&a.ctl->res_bits[slot], bits);
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
    {
        const int cols = g.ai * g.aj;
        for (int e = threadIdx.x; e < cols * nz; e += blockDim.x) {
            const int col = e / nz;
            const int k = e - col * nz;
            const int li = col / g.aj, lj = col - (col / g.aj) * g.aj;
            const int c2 = (li + 1) * g.stride_i + (lj + 1);
            a.field[(g.i0 + li) * sx + static_cast<int64_t>(g.j0 + lj) * nz + k] = s[(k & 1) * g.ncm + c2 * M + (k >> 1)];
        }
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
                const long cells = static_cast<long>(ti) * tj * M;
                const int threads = cells >= 1024 ? 1024 : static_cast<int>(((cells + 31) / 32) * 32);
                best = SorTiling{ex, ey, ti, tj, M, threads, smem};
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
