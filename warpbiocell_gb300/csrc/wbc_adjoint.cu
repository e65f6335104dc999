// Hand-written adjoint of the coupled steady state: K contact steps, a deposit of per-cell uptake
// capacities, and the quasi-steady Michaelis-Menten oxygen field.
//
// Forward model (per cell i: position x_i, radius r_i, uptake capacity Vmax_i; grid nodes a):
//   x_{t+1} = x_t + dt v(x_t),  v_i = sum_j rate ((r_i + r_j) / d_ij - 1) (x_i - x_j)   (overlapping pairs)
//   U_a     = inv_vol sum_i w_a(x_i) Vmax_i                      (trilinear weights at the final x)
//   G_a(u)  = sum_nb u_nb - (6 + h U_a / (K + u_a)) u_a = 0    (h = dx^2 / D, Dirichlet faces = O_b)
// Reverse mode, for a loss L(u, x_K):
//   field:     (6 + h kappa_a) mu_a - sum_nb mu_nb = dL/du_a,  kappa_a = U_a K / (K + u_a)^2, mu = 0 on
//              Dirichlet faces and on nodes held at zero by the clamp (a red-black SOR solve of the
//              transposed linearised operator, which is symmetric here)
//              dL/dVmax_i = -h inv_vol sum_a w_a(x_i) phi_a,  phi_a = mu_a u_a / (K + u_a)
//              dL/dK = sum_a mu_a h U_a u_a / (K + u_a)^2,  dL/dD = sum_a mu_a h U_a u_a / ((K + u_a) D)
//              dL/dO_b = sum_a mu_a (Dirichlet neighbours of a) + sum_{faces} dL/du
//              dL/dx_i += -h inv_vol Vmax_i grad_x (sum_a w_a(x) phi_a) at x_i
//   mechanics: lambda_t = lambda_{t+1} + dt J(x_t)^T lambda_{t+1},
//              (J^T lambda)_i = sum_j A_ij (lambda_i - lambda_j),
//              A_ij = rate ((R/d - 1) I - R e e^T / d^3), e = x_i - x_j, R = r_i + r_j;
//              dL/drate = sum_t dt sum_i lambda_{t+1,i} . v_i(x_t) / rate.
// The reference has no adjoint; the forward pieces are its contact law
// (kernels/mechanics_kernels.py:26-67), deposit (field_kernels.py:78-116) and SOR update
// (field_kernels.py:185-212) with a per-cell uptake.
#include <algorithm>
#include <cstring>

#include "wbc_bodies.cuh"

namespace wbc {

// ---- forward: per-cell uptake deposit --------------------------------------------------------------
// acc[node] += int64(w * weight_i * 2^24 + 0.5) for the 8 corners (weight_i = Vmax_i / scale).
__global__ void k_deposit_weighted(wbc_grid_geometry g, int32_t n, const float* __restrict__ position,
                                   const float* __restrict__ weight, unsigned long long* __restrict__ acc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
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
    const float wc = weight[c];
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
                const long long q = static_cast<long long>(w * wc * kFixedOne + 0.5f);
                const int64_t node = (static_cast<int64_t>(i0 + di) * g.ny + (j0 + dj)) * g.nz + (k0 + dk);
                atomicAdd(acc + node, static_cast<unsigned long long>(q));
            }
        }
    }
}

__global__ void k_weighted_convert(int64_t nodes, long long* __restrict__ acc, float factor, float* __restrict__ out,
                                   int clear) {
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (a >= nodes) return;
    out[a] = static_cast<float>(acc[a]) / kFixedOne * factor;
    if (clear) acc[a] = 0;
}

// ---- reverse: one contact step -----------------------------------------------------------------------
// Sorted slot t (cell i) of the grid built at x_t: lambda_out_i = lambda_in_i + dt (J^T lambda_in)_i
// and vdot_i = lambda_in_i . v_i(x_t) / rate (adjoint_contact_slot in wbc_bodies.cuh).
__global__ void __launch_bounds__(256) k_adjoint_contact(BucketMap map, int32_t n, const int32_t* __restrict__ bucket_start,
                                                         const int32_t* __restrict__ bucket_count,
                                                         const int32_t* __restrict__ sorted_id,
                                                         const float4* __restrict__ sorted_xyzr, float query_radius,
                                                         float rate, float dt, const float* __restrict__ lambda_in,
                                                         float* __restrict__ lambda_out, float* __restrict__ vdot) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i;
    const float v = adjoint_contact_slot(map, t, bucket_start, bucket_count, sorted_id, sorted_xyzr, query_radius,
                                         rate, dt, lambda_in, lambda_out, &i);
    vdot[i] = v;
}

// ---- reverse: the field ---------------------------------------------------------------------------------
__device__ __forceinline__ bool is_dirichlet(const wbc_sor_params& p, int i, int j, int k) {
    return (p.bc_x == 0 && (i == 0 || i == p.nx - 1)) || (p.bc_y == 0 && (j == 0 || j == p.ny - 1)) ||
           (p.bc_z == 0 && (k == 0 || k == p.nz - 1));
}

// kappa_a (or -1 where mu_a = 0: Dirichlet faces, nodes at the clamp), the right-hand side dL/du.
__global__ void k_adjoint_prepare(wbc_sor_params p, const float* __restrict__ u, const float* __restrict__ U,
                                  float* __restrict__ kappa) {
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t nodes = static_cast<int64_t>(p.nx) * p.ny * p.nz;
    if (a >= nodes) return;
    const int k = static_cast<int>(a % p.nz);
    const int64_t ij = a / p.nz;
    const int j = static_cast<int>(ij % p.ny);
    const int i = static_cast<int>(ij / p.ny);
    const float ua = u[a];
    if (is_dirichlet(p, i, j, k) || !(ua > 0.0f)) {
        kappa[a] = -1.0f;
        return;
    }
    const float s = p.michaelis_k + ua;
    kappa[a] = U[a] * p.michaelis_k / (s * s);
}

__device__ __forceinline__ float mu_at(const float* __restrict__ mu, const wbc_sor_params& p, int i, int j, int k) {
    // Neighbours across a Neumann face are the mirror images; Dirichlet faces hold mu = 0.
    const int ii = i < 0 ? 1 : (i > p.nx - 1 ? p.nx - 2 : i);
    const int jj = j < 0 ? 1 : (j > p.ny - 1 ? p.ny - 2 : j);
    const int kk = k < 0 ? 1 : (k > p.nz - 1 ? p.nz - 2 : k);
    return mu[(static_cast<int64_t>(ii) * p.ny + jj) * p.nz + kk];
}

// One colour of mu_a <- (1 - omega) mu_a + omega (sum_nb mu + g_a) / (6 + h kappa_a).
__global__ void k_adjoint_colour(wbc_sor_params p, int colour, const float* __restrict__ kappa,
                                 const float* __restrict__ g, float* __restrict__ mu) {
    // Thread t: column ij = t / ceil(nz / 2), the slot-th node of this colour in it (k stride 2).
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int slots = (p.nz + 1) / 2;
    const int64_t ij = t / slots;
    if (ij >= static_cast<int64_t>(p.nx) * p.ny) return;
    int kk = 2 * static_cast<int>(t - ij * slots);
    const int j = static_cast<int>(ij % p.ny);
    const int i = static_cast<int>(ij / p.ny);
    kk += (colour + i + j) & 1;
    if (kk >= p.nz) return;
    const int64_t a = ij * p.nz + kk;
    const float ka = kappa[a];
    if (!(ka >= 0.0f)) return;
    const float nb = mu_at(mu, p, i - 1, j, kk) + mu_at(mu, p, i + 1, j, kk) + mu_at(mu, p, i, j - 1, kk) +
                     mu_at(mu, p, i, j + 1, kk) + mu_at(mu, p, i, j, kk - 1) + mu_at(mu, p, i, j, kk + 1);
    const float gs = (nb + g[a]) / (6.0f + p.dx2_over_D * ka);
    mu[a] = (1.0f - p.omega) * mu[a] + p.omega * gs;
}

// out[0] = max_a |sum_nb mu + g_a - (6 + h kappa_a) mu_a|, out[1] = max_a max(6 |mu_a|, |g_a|), as
// float bits (non-negative: integer max works).
__global__ void k_adjoint_residual(wbc_sor_params p, const float* __restrict__ kappa, const float* __restrict__ g,
                                   const float* __restrict__ mu, unsigned int* __restrict__ out) {
    const int64_t nodes = static_cast<int64_t>(p.nx) * p.ny * p.nz;
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned int bits = 0u, scale = 0u;
    if (a < nodes) {
        const float ka = kappa[a];
        if (ka >= 0.0f) {
            const int k = static_cast<int>(a % p.nz);
            const int64_t ij = a / p.nz;
            const int j = static_cast<int>(ij % p.ny);
            const int i = static_cast<int>(ij / p.ny);
            const float nb = mu_at(mu, p, i - 1, j, k) + mu_at(mu, p, i + 1, j, k) + mu_at(mu, p, i, j - 1, k) +
                             mu_at(mu, p, i, j + 1, k) + mu_at(mu, p, i, j, k - 1) + mu_at(mu, p, i, j, k + 1);
            bits = __float_as_uint(fabsf(nb + g[a] - (6.0f + p.dx2_over_D * ka) * mu[a]));
            scale = __float_as_uint(fmaxf(6.0f * fabsf(mu[a]), fabsf(g[a])));
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, d));
        scale = max(scale, __shfl_xor_sync(0xffffffffu, scale, d));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, bits);
        atomicMax(out + 1, scale);
    }
}

// phi_a = mu_a u_a / (K + u_a) and the scalar sums: [0] dL/dK, [1] D dL/dD, [2] dL/dO_b.
__global__ void k_adjoint_field_grads(wbc_sor_params p, const float* __restrict__ u, const float* __restrict__ U,
                                      const float* __restrict__ mu, const float* __restrict__ kappa,
                                      const float* __restrict__ g, float* __restrict__ phi,
                                      double* __restrict__ sums) {
    const int64_t nodes = static_cast<int64_t>(p.nx) * p.ny * p.nz;
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    double s_k = 0.0, s_d = 0.0, s_b = 0.0;
    if (a < nodes) {
        const int k = static_cast<int>(a % p.nz);
        const int64_t ij = a / p.nz;
        const int j = static_cast<int>(ij % p.ny);
        const int i = static_cast<int>(ij / p.ny);
        float ph = 0.0f;
        if (is_dirichlet(p, i, j, k)) {
            s_b = g[a];
        } else if (kappa[a] >= 0.0f) {
            const float ua = u[a], m = mu[a];
            const float s = p.michaelis_k + ua;
            ph = m * ua / s;
            const double hU = static_cast<double>(p.dx2_over_D) * U[a];
            s_k = static_cast<double>(m) * hU * ua / (static_cast<double>(s) * s);
            s_d = static_cast<double>(m) * hU * ua / s;
            int faces = 0;
            faces += (p.bc_x == 0 && i == 1) + (p.bc_x == 0 && i == p.nx - 2);
            faces += (p.bc_y == 0 && j == 1) + (p.bc_y == 0 && j == p.ny - 2);
            faces += (p.bc_z == 0 && k == 1) + (p.bc_z == 0 && k == p.nz - 2);
            s_b = static_cast<double>(m) * faces;
        }
        phi[a] = ph;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        s_k += __shfl_xor_sync(0xffffffffu, s_k, d);
        s_d += __shfl_xor_sync(0xffffffffu, s_d, d);
        s_b += __shfl_xor_sync(0xffffffffu, s_b, d);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(sums, s_k);
        atomicAdd(sums + 1, s_d);
        atomicAdd(sums + 2, s_b);
    }
}

// Per cell: dL/dVmax_i = coef sum_a w_a(x_i) phi_a and dL/dx_i += coef Vmax_i grad_x sum_a w_a phi_a,
// coef = -h inv_vol; cells outside the deposit support get zero.
__global__ void k_adjoint_cells(wbc_grid_geometry g, int32_t n, const float* __restrict__ position,
                                const float* __restrict__ vmax, const float* __restrict__ phi, float coef,
                                float* __restrict__ grad_vmax, float* __restrict__ grad_x) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const float* p = position + 3 * static_cast<int64_t>(c);
    const float ux = (p[0] - g.origin_x) * g.inv_dx;
    const float uy = (p[1] - g.origin_y) * g.inv_dx;
    const float uz = (p[2] - g.origin_z) * g.inv_dx;
    const int i0 = static_cast<int>(floorf(ux));
    const int j0 = static_cast<int>(floorf(uy));
    const int k0 = static_cast<int>(floorf(uz));
    if (i0 < 0 || j0 < 0 || k0 < 0 || i0 + 1 >= g.nx || j0 + 1 >= g.ny || k0 + 1 >= g.nz) {
        grad_vmax[c] = 0.0f;
        return;
    }
    const float fx = ux - static_cast<float>(i0);
    const float fy = uy - static_cast<float>(j0);
    const float fz = uz - static_cast<float>(k0);
    float s = 0.0f, sx = 0.0f, sy = 0.0f, sz = 0.0f;
#pragma unroll
    for (int di = 0; di < 2; ++di) {
        const float wx = di == 0 ? 1.0f - fx : fx, dwx = di == 0 ? -1.0f : 1.0f;
#pragma unroll
        for (int dj = 0; dj < 2; ++dj) {
            const float wy = dj == 0 ? 1.0f - fy : fy, dwy = dj == 0 ? -1.0f : 1.0f;
#pragma unroll
            for (int dk = 0; dk < 2; ++dk) {
                const float wz = dk == 0 ? 1.0f - fz : fz, dwz = dk == 0 ? -1.0f : 1.0f;
                const float ph =
                    phi[(static_cast<int64_t>(i0 + di) * g.ny + (j0 + dj)) * g.nz + (k0 + dk)];
                s += wx * wy * wz * ph;
                sx += dwx * wy * wz * ph;
                sy += wx * dwy * wz * ph;
                sz += wx * wy * dwz * ph;
            }
        }
    }
    grad_vmax[c] = coef * s;
    const float f = coef * vmax[c] * g.inv_dx;
    const int64_t o = 3 * static_cast<int64_t>(c);
    grad_x[o] += f * sx;
    grad_x[o + 1] += f * sy;
    grad_x[o + 2] += f * sz;
}

// ---- mixed-precision refinement of the field and of its adjoint ----------------------------------------
// The fp32 solves stop near their rounding floor (a relative residual of about 1e-6), which leaves
// errors of order 1e-5 in the field and in the adjoint, and so in the gradients. One Newton
// correction of the field and one refinement step of the adjoint, with residuals formed in FP64
// and the corrections solved by the same fp32 SOR, bring both to their FP64 values.

template <typename T>
__device__ __forceinline__ double value_at(const T* __restrict__ u, const wbc_sor_params& p, int i, int j, int k) {
    // Neumann faces mirror; Dirichlet face nodes hold their own values in u.
    const int ii = i < 0 ? 1 : (i > p.nx - 1 ? p.nx - 2 : i);
    const int jj = j < 0 ? 1 : (j > p.ny - 1 ? p.ny - 2 : j);
    const int kk = k < 0 ? 1 : (k > p.nz - 1 ? p.nz - 2 : k);
    return static_cast<double>(u[(static_cast<int64_t>(ii) * p.ny + jj) * p.nz + kk]);
}

// Newton step of the steady field G(u) = sum_nb u - (6 + h U / (K + u)) u = 0 at the current u
// (FP64): diag = 6 + h U K / (K + u)^2 (the negated Jacobian's diagonal) and rhs = G(u), so that
// diag d - sum_nb d = rhs gives the correction d. A node is free where u > 0 or G(u) > 0 (a node at
// the zero clamp with G <= 0 stays there); faces and held nodes get diag = -1, rhs = 0.
__global__ void k_newton_prepare(wbc_sor_params p, const double* __restrict__ u, const float* __restrict__ U,
                                 float* __restrict__ diag, float* __restrict__ rhs) {
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t nodes = static_cast<int64_t>(p.nx) * p.ny * p.nz;
    if (a >= nodes) return;
    const int k = static_cast<int>(a % p.nz);
    const int64_t ij = a / p.nz;
    const int j = static_cast<int>(ij % p.ny);
    const int i = static_cast<int>(ij / p.ny);
    if (is_dirichlet(p, i, j, k)) {
        diag[a] = -1.0f;
        rhs[a] = 0.0f;
        return;
    }
    const double ua = u[a], K = p.michaelis_k, h = p.dx2_over_D, Ua = U[a];
    const double nb = value_at(u, p, i - 1, j, k) + value_at(u, p, i + 1, j, k) + value_at(u, p, i, j - 1, k) +
                      value_at(u, p, i, j + 1, k) + value_at(u, p, i, j, k - 1) + value_at(u, p, i, j, k + 1);
    const double g = nb - (6.0 + h * Ua / (K + ua)) * ua;
    if (!(ua > 0.0) && !(g > 0.0)) {
        diag[a] = -1.0f;
        rhs[a] = 0.0f;
        return;
    }
    const double s = K + ua;
    diag[a] = static_cast<float>(6.0 + h * Ua * K / (s * s));
    rhs[a] = static_cast<float>(g);
}

// u += d, clamped at zero (FP64).
__global__ void k_newton_apply(int64_t n, const float* __restrict__ d, double* __restrict__ u) {
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (a < n) u[a] = fmax(u[a] + static_cast<double>(d[a]), 0.0);
}

__global__ void k_widen(int64_t n, const float* __restrict__ in, double* __restrict__ out) {
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (a < n) out[a] = static_cast<double>(in[a]);
}

__global__ void k_narrow(int64_t n, const double* __restrict__ in, float* __restrict__ out) {
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (a < n) out[a] = static_cast<float>(in[a]);
}

__global__ void k_fill(int64_t n, float value, float* __restrict__ out) {
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (a < n) out[a] = value;
}

__global__ void k_divide(int64_t n, const float* __restrict__ in, float divisor, float* __restrict__ out) {
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (a < n) out[a] = in[a] / divisor;
}

// x64 = hi + lo in FP64 (exact for the compensated pairs, whose lo is below half an ulp of hi) and
// pos = x64 rounded to float.
__global__ void k_compensated_sum(int64_t n, const float* __restrict__ hi, const float* __restrict__ lo,
                                  double* __restrict__ x64, float* __restrict__ pos) {
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const double x = static_cast<double>(hi[a]) + static_cast<double>(lo[a]);
    x64[a] = x;
    pos[a] = static_cast<float>(x);
}

// The mean of n floats in FP64 in a fixed order: block b sums elements b, b + B, b + 2B, ... per
// thread in order and combines its threads by a fixed tree into partial[b + 1]; one block then
// combines the B partials the same way into partial[0]. Nothing depends on scheduling.
constexpr int kMeanThreads = 256;
constexpr int kMeanBlocks = 256;  // partials; WBC_MEAN_SCRATCH = kMeanBlocks + 1 doubles
__device__ __forceinline__ double block_sum(double v, double* part) {
    part[threadIdx.x] = v;
    __syncthreads();
    for (int width = kMeanThreads / 2; width > 0; width >>= 1) {
        if (static_cast<int>(threadIdx.x) < width) part[threadIdx.x] += part[threadIdx.x + width];
        __syncthreads();
    }
    return part[0];
}

__global__ void __launch_bounds__(kMeanThreads) k_mean_partial(int64_t n, const float* __restrict__ x,
                                                               double* __restrict__ partial) {
    __shared__ double part[kMeanThreads];
    double sum = 0.0;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * kMeanThreads;
    for (int64_t a = static_cast<int64_t>(blockIdx.x) * kMeanThreads + threadIdx.x; a < n; a += stride)
        sum += static_cast<double>(x[a]);
    const double total = block_sum(sum, part);
    if (threadIdx.x == 0) partial[blockIdx.x + 1] = total;
}

__global__ void __launch_bounds__(kMeanThreads) k_mean_final(int64_t n, int blocks, double* __restrict__ partial) {
    __shared__ double part[kMeanThreads];
    const double total = block_sum(static_cast<int>(threadIdx.x) < blocks ? partial[threadIdx.x + 1] : 0.0, part);
    if (threadIdx.x == 0) partial[0] = n > 0 ? total / static_cast<double>(n) : 0.0;
}

// r = b - (diag x - sum_nb x) in FP64 at the free nodes (diag > 0), 0 elsewhere.
__global__ void k_linear_residual(wbc_sor_params p, const float* __restrict__ diag, const float* __restrict__ b,
                                  const float* __restrict__ x, float* __restrict__ r) {
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t nodes = static_cast<int64_t>(p.nx) * p.ny * p.nz;
    if (a >= nodes) return;
    const float da = diag[a];
    if (!(da > 0.0f)) {
        r[a] = 0.0f;
        return;
    }
    const int k = static_cast<int>(a % p.nz);
    const int64_t ij = a / p.nz;
    const int j = static_cast<int>(ij % p.ny);
    const int i = static_cast<int>(ij / p.ny);
    const double nb = value_at(x, p, i - 1, j, k) + value_at(x, p, i + 1, j, k) + value_at(x, p, i, j - 1, k) +
                      value_at(x, p, i, j + 1, k) + value_at(x, p, i, j, k - 1) + value_at(x, p, i, j, k + 1);
    r[a] = static_cast<float>(static_cast<double>(b[a]) - (static_cast<double>(da) * x[a] - nb));
}

// The field's gradient sums from the refined field u (FP64) and adjoint mu = mu0 + dmu (FP64):
// phi_a = mu_a u_a / (K + u_a) and [0] dL/dK, [1] D dL/dD, [2] dL/dO_b, as k_adjoint_field_grads.
__global__ void k_adjoint_field_grads_refined(wbc_sor_params p, const double* __restrict__ u,
                                              const float* __restrict__ U, const float* __restrict__ mu0,
                                              const float* __restrict__ dmu, const float* __restrict__ diag,
                                              const float* __restrict__ g, float* __restrict__ phi,
                                              double* __restrict__ sums) {
    const int64_t nodes = static_cast<int64_t>(p.nx) * p.ny * p.nz;
    const int64_t a = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    double s_k = 0.0, s_d = 0.0, s_b = 0.0;
    if (a < nodes) {
        const int k = static_cast<int>(a % p.nz);
        const int64_t ij = a / p.nz;
        const int j = static_cast<int>(ij % p.ny);
        const int i = static_cast<int>(ij / p.ny);
        double ph = 0.0;
        if (is_dirichlet(p, i, j, k)) {
            s_b = g[a];
        } else if (diag[a] > 0.0f) {
            const double ua = u[a], m = static_cast<double>(mu0[a]) + static_cast<double>(dmu[a]);
            const double s = p.michaelis_k + ua;
            ph = m * ua / s;
            const double hU = static_cast<double>(p.dx2_over_D) * U[a];
            s_k = m * hU * ua / (s * s);
            s_d = m * hU * ua / s;
            int faces = 0;
            faces += (p.bc_x == 0 && i == 1) + (p.bc_x == 0 && i == p.nx - 2);
            faces += (p.bc_y == 0 && j == 1) + (p.bc_y == 0 && j == p.ny - 2);
            faces += (p.bc_z == 0 && k == 1) + (p.bc_z == 0 && k == p.nz - 2);
            s_b = m * faces;
        }
        phi[a] = static_cast<float>(ph);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        s_k += __shfl_xor_sync(0xffffffffu, s_k, d);
        s_d += __shfl_xor_sync(0xffffffffu, s_d, d);
        s_b += __shfl_xor_sync(0xffffffffu, s_b, d);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(sums, s_k);
        atomicAdd(sums + 1, s_d);
        atomicAdd(sums + 2, s_b);
    }
}

static BucketMap bucket_map(const wbc_neighbor_grid* g) {
    BucketMap m;
    m.inv_edge = 1.0f / (g->cell_size * 1.0009765625f);
    m.dim = g->dim;
    return m;
}

}  // namespace wbc

using namespace wbc;

extern "C" {

int wbc_deposit_weighted(const wbc_grid_geometry* geom, int32_t n, const float* position, const float* weight,
                         int64_t* accumulator, void* stream) {
    if (!geom || n < 0 || !accumulator || (n > 0 && (!position || !weight))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_deposit_weighted<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(
        *geom, n, position, weight, reinterpret_cast<unsigned long long*>(accumulator));
    return check_launch("wbc_deposit_weighted");
}

int wbc_weighted_convert(int64_t nodes, int64_t* accumulator, float factor, float* out, int32_t clear,
                         void* stream) {
    if (nodes < 0 || (nodes > 0 && (!accumulator || !out))) return WBC_ERR_INVALID;
    if (nodes == 0) return WBC_OK;
    k_weighted_convert<<<grid_for(nodes), kThreads, 0, as_stream(stream)>>>(
        nodes, reinterpret_cast<long long*>(accumulator), factor, out, clear);
    return check_launch("wbc_weighted_convert");
}

int wbc_adjoint_contact(const wbc_neighbor_grid* grid, int32_t n, float query_radius, float rate, float dt,
                        const float* lambda_in, float* lambda_out, float* vdot, void* stream) {
    if (!grid || n < 0 || (n > 0 && (!lambda_in || !lambda_out || !vdot)) || lambda_in == lambda_out)
        return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_adjoint_contact<<<grid_for(n), 256, 0, as_stream(stream)>>>(
        bucket_map(grid), n, grid->bucket_start, grid->bucket_count, grid->sorted_id,
        reinterpret_cast<const float4*>(grid->sorted_xyzr), query_radius, rate, dt, lambda_in, lambda_out, vdot);
    return check_launch("wbc_adjoint_contact");
}

int wbc_adjoint_field_solve(const wbc_sor_params* p, const float* u, const float* U, const float* grad_u, float* mu,
                            float* kappa, int32_t check_every, int32_t max_sweeps, float tolerance, float* phi,
                            double* sums, uint32_t* residual_bits, wbc_sor_report* report, void* stream) {
    if (!p || !u || !U || !grad_u || !mu || !kappa || !phi || !sums || !residual_bits || !report || check_every < 1 ||
        max_sweeps < 1 || p->nx < 3 || p->ny < 3 || p->nz < 3)
        return WBC_ERR_INVALID;
    if (p->bc_x != 0 || p->bc_y != 0 || p->bc_z != 0) {
        // With Dirichlet faces the linearised operator is symmetric, so its transpose is itself.
        set_error_msg("wbc_adjoint_field_solve: the adjoint needs Dirichlet faces on all sides");
        return WBC_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    const int64_t nodes = static_cast<int64_t>(p->nx) * p->ny * p->nz;
    const int64_t half = (static_cast<int64_t>(p->nx) * p->ny * ((p->nz + 1) / 2));
    k_adjoint_prepare<<<grid_for(nodes), kThreads, 0, s>>>(*p, u, U, kappa);
    int launches = 1;
    int sweeps = 0;
    float residual = __builtin_inff();
    while (sweeps < max_sweeps) {
        const int chunk = std::min(check_every, max_sweeps - sweeps);
        for (int k = 0; k < chunk; ++k) {
            k_adjoint_colour<<<grid_for(half), kThreads, 0, s>>>(*p, 0, kappa, grad_u, mu);
            k_adjoint_colour<<<grid_for(half), kThreads, 0, s>>>(*p, 1, kappa, grad_u, mu);
        }
        cudaError_t err = cudaMemsetAsync(residual_bits, 0, 2 * sizeof(uint32_t), s);
        k_adjoint_residual<<<grid_for(nodes), kThreads, 0, s>>>(*p, kappa, grad_u, mu, residual_bits);
        launches += 2 * chunk + 1;
        uint32_t bits[2] = {0, 0};
        if (err == cudaSuccess) err = cudaMemcpyAsync(bits, residual_bits, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        if (err == cudaSuccess) err = cudaStreamSynchronize(s);
        if (err != cudaSuccess) {
            set_error("wbc_adjoint_field_solve: reading the residual", err);
            return WBC_ERR_CUDA;
        }
        sweeps += chunk;
        float r_abs, r_scale;
        std::memcpy(&r_abs, &bits[0], sizeof(float));
        std::memcpy(&r_scale, &bits[1], sizeof(float));
        residual = r_scale > 0.0f ? r_abs / r_scale : 0.0f;
        if (residual < tolerance) break;
    }
    cudaError_t err = cudaMemsetAsync(sums, 0, 3 * sizeof(double), s);
    if (err != cudaSuccess) {
        set_error("wbc_adjoint_field_solve: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    k_adjoint_field_grads<<<grid_for(nodes), kThreads, 0, s>>>(*p, u, U, mu, kappa, grad_u, phi, sums);
    report->sweeps = sweeps;
    report->residual = residual;
    report->converged = residual < tolerance ? 1 : 0;
    report->path = 1;
    report->tiles = 0;
    report->strips = 0;
    return check_launch("wbc_adjoint_field_solve", launches + 1);
}

int wbc_adjoint_cells(const wbc_grid_geometry* geom, int32_t n, const float* position, const float* vmax,
                      const float* phi, float coef, float* grad_vmax, float* grad_x, void* stream) {
    if (!geom || n < 0 || (n > 0 && (!position || !vmax || !phi || !grad_vmax || !grad_x))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_adjoint_cells<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(*geom, n, position, vmax, phi, coef, grad_vmax,
                                                                    grad_x);
    return check_launch("wbc_adjoint_cells");
}


int wbc_adjoint_newton_prepare(const wbc_sor_params* p, const double* u, const float* U, float* diag, float* rhs,
                               void* stream) {
    if (!p || !u || !U || !diag || !rhs || p->nx < 3 || p->ny < 3 || p->nz < 3) return WBC_ERR_INVALID;
    const int64_t nodes = static_cast<int64_t>(p->nx) * p->ny * p->nz;
    k_newton_prepare<<<grid_for(nodes), kThreads, 0, as_stream(stream)>>>(*p, u, U, diag, rhs);
    return check_launch("wbc_adjoint_newton_prepare");
}

int wbc_adjoint_newton_apply(int64_t nodes, const float* delta, double* u, void* stream) {
    if (nodes < 0 || (nodes > 0 && (!delta || !u))) return WBC_ERR_INVALID;
    if (nodes == 0) return WBC_OK;
    k_newton_apply<<<grid_for(nodes), kThreads, 0, as_stream(stream)>>>(nodes, delta, u);
    return check_launch("wbc_adjoint_newton_apply");
}

int wbc_widen(int64_t n, const float* in, double* out, void* stream) {
    if (n < 0 || (n > 0 && (!in || !out))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_widen<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, in, out);
    return check_launch("wbc_widen");
}

int wbc_narrow(int64_t n, const double* in, float* out, void* stream) {
    if (n < 0 || (n > 0 && (!in || !out))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_narrow<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, in, out);
    return check_launch("wbc_narrow");
}

int wbc_fill(int64_t n, float value, float* out, void* stream) {
    if (n < 0 || (n > 0 && !out)) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_fill<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, value, out);
    return check_launch("wbc_fill");
}

int wbc_zero(void* ptr, size_t bytes, void* stream) {
    if (bytes > 0 && !ptr) return WBC_ERR_INVALID;
    if (bytes == 0) return WBC_OK;
    const cudaError_t err = cudaMemsetAsync(ptr, 0, bytes, as_stream(stream));
    if (err != cudaSuccess) {
        set_error("wbc_zero: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    return WBC_OK;
}

int wbc_divide(int64_t n, const float* in, float divisor, float* out, void* stream) {
    if (n < 0 || (n > 0 && (!in || !out))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_divide<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, in, divisor, out);
    return check_launch("wbc_divide");
}

int wbc_compensated_sum(int64_t n, const float* hi, const float* lo, double* x64, float* pos, void* stream) {
    if (n < 0 || (n > 0 && (!hi || !lo || !x64 || !pos))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_compensated_sum<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, hi, lo, x64, pos);
    return check_launch("wbc_compensated_sum");
}

int wbc_mean(int64_t n, const float* x, double* scratch, void* stream) {
    if (n < 0 || !scratch || (n > 0 && !x)) return WBC_ERR_INVALID;
    static_assert(kMeanBlocks <= kMeanThreads, "the final block combines every partial");
    const int blocks = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(kMeanBlocks, (n + 4095) / 4096)));
    cudaStream_t s = as_stream(stream);
    k_mean_partial<<<blocks, kMeanThreads, 0, s>>>(n, x, scratch);
    k_mean_final<<<1, kMeanThreads, 0, s>>>(n, blocks, scratch);
    return check_launch("wbc_mean", 2);
}

int wbc_adjoint_linear_residual(const wbc_sor_params* p, const float* diag, const float* b, const float* x, float* r,
                                void* stream) {
    if (!p || !diag || !b || !x || !r || p->nx < 3 || p->ny < 3 || p->nz < 3) return WBC_ERR_INVALID;
    const int64_t nodes = static_cast<int64_t>(p->nx) * p->ny * p->nz;
    k_linear_residual<<<grid_for(nodes), kThreads, 0, as_stream(stream)>>>(*p, diag, b, x, r);
    return check_launch("wbc_adjoint_linear_residual");
}

int wbc_adjoint_field_grads(const wbc_sor_params* p, const double* u, const float* U, const float* mu0,
                            const float* dmu, const float* diag, const float* grad_u, float* phi, double* sums,
                            void* stream) {
    if (!p || !u || !U || !mu0 || !dmu || !diag || !grad_u || !phi || !sums || p->nx < 3 || p->ny < 3 || p->nz < 3)
        return WBC_ERR_INVALID;
    const int64_t nodes = static_cast<int64_t>(p->nx) * p->ny * p->nz;
    cudaStream_t s = as_stream(stream);
    cudaError_t err = cudaMemsetAsync(sums, 0, 3 * sizeof(double), s);
    if (err != cudaSuccess) {
        set_error("wbc_adjoint_field_grads: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    k_adjoint_field_grads_refined<<<grid_for(nodes), kThreads, 0, s>>>(*p, u, U, mu0, dmu, diag, grad_u, phi, sums);
    return check_launch("wbc_adjoint_field_grads");
}

}  // extern "C"
