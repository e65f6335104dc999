// Red-black SOR solve to convergence in one persistent, cooperative launch with the field held
// in shared memory (kernels/field_kernels.py:185-243 iterated as fields/diffusion.py:79-123).
//
// Decomposition: the (i, j) plane of columns is cut into `strips` strips along j, and each strip's
// columns, taken row by row, into consecutive runs of equal length: one run per CTA (one CTA per
// SM), so every CTA owns the same number of columns to within one. A tile is thus a block of
// strip rows whose first and last rows may be partial (a staircase). Shared memory holds the
// tile's bounding box plus a one-column halo, split by colour: plane c holds the nodes with
// (i + j + k) % 2 == c, entry m of a column being its node k = 2m + ((c + i + j) & 1). All six
// neighbours of a node of colour c lie in plane 1 - c: the lateral ones at the same entry of the
// neighbouring columns, the k-neighbours at entries m - 1 + kp and m + kp (kp = the k parity of
// the node), clamped at the column ends when the z faces are Neumann (the reference's mirror
// rule). Dirichlet faces, pinned nodes and the padding entry of odd-length colour columns carry
// no uptake coefficient and are never written.
//
// Work: the tile's columns form runs of consecutive columns in a box row, and within one colour
// plane the entries of a run are contiguous; each run is cut into groups of 96 entries (three
// lane-chunks of 32) that may span several columns, and a warp relaxes one group at a time with one
// descriptor for its three lane-chunks, so no lane idles except at the end of a run (at 161 z
// levels a column holds 81 entries per colour: 32-entry slots per column would leave 16% of the
// lanes idle). At the start each CTA builds its group lists, loads its box, and writes the uptake
// coefficients density * uptake_max of its columns, split the same way, to an L2-resident copy
// (-1 marks nodes that are never updated), together with the production term when there is one.
//
// Halo exchange: the tile's edge columns (those with an in-domain neighbour owned by another
// tile) are relaxed first, and each new value is stored to an exchange buffer in L2 as one
// 64-bit word {value, half-sweep tag} with a relaxed store; the inner columns follow; then the
// halo columns are read from their owners' tagged words, re-reading any word whose tag is not yet
// this half-sweep's. No flag, fence or barrier is needed between neighbouring tiles: a neighbour
// rewrites a word two half-sweeps later, which needs this tile's words of the half-sweep in
// between, written after this read. Every `check_every` sweeps the max-norm residual is reduced
// (warp shuffles, one atomicMax per CTA, the only global barrier) and all CTAs stop together once
// it is below the tolerance: the reference's sweep count, residual and stopping rule, with no host
// round trip. The field after n sweeps is bit-identical to the oracle's and to the streaming
// kernels'.
//
// Every wait is bounded in time (kWaitLimitNs of the GPU's global timer, 2 s); on timeout the CTA
// raises an abort flag, every CTA leaves, and the host gets WBC_ERR_TIMEOUT.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "wbc_common.cuh"

namespace wbc {

struct __align__(128) SorControl {
    unsigned int abort;
    unsigned int res_bits[2];
    int sweeps;
    float residual;
    int converged;
    int status;
    unsigned int scale_bits[2];  // linear solves: the residual's scale, max(6 |x|, |b|)
    int pad[23];
};
static_assert(sizeof(SorControl) == 128, "SorControl is one 128-byte line");
constexpr int kMaxCtas = 1024;     // barrier flags that follow the control block
constexpr int kSorThreads = 1024;  // threads per CTA of the resident solver
constexpr int kMaxEntries = 1023;  // entries per colour column (nz <= 2045): 10 bits of a chunk word
constexpr int kPlaneSlack = 128;   // floats past the largest box: lanes beyond a group's end read there

// Shared-memory layout of one tile, sized for the largest tile of the solve.
struct SorTiling {
    int tiles, strips;  // CTAs; strips along j
    int M;              // entries per colour column: (nz + 1) / 2
    int max_box;        // columns of the largest bounding box (halo included)
    int relax_cap, pull_cap, mirror_cap, run_cap;
    size_t plane_floats;  // floats per colour plane
    size_t relax_off, masks_off, pull_off, mirror_off, run_off, kind_off, smem;
};

struct SorArgs {
    wbc_sor_params p;
    SorTiling t;
    const int32_t* fixed;
    const float* density;
    const float* production;
    const float* source;
    float* field;
    unsigned long long* xchg;  // [2 colours][nx][ny][M] tagged halo words
    float* coeff;              // [2][nx][ny][M] density * uptake_max, -1 where not updated
    float* pcopy;              // [2][nx][ny][M] production term of every updated node
    SorControl* ctl;
    unsigned int* flags;  // [tiles] barrier epochs
    float* residual_out;  // optional device float: the final residual
    int check_every;
    int max_sweeps;
    double tolerance;  // compared in double, as the reference compares float(residual) < tolerance
};

// Every device wait gives up after kWaitLimitNs nanoseconds of the GPU's global timer without
// progress. The timer is read every 256 polls, so a wait ends within a few microseconds of the limit.
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned int load_acquire(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void store_release(unsigned int* p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The clock of one bounded wait. `claims` (batched solves only) is the work list's claim counter:
// while fewer than `claims_needed` tiles have been claimed, some tile of this solve has no CTA yet
// and is waiting behind earlier work, so the wait has not really started and its clock is held.
struct WaitClock {
    unsigned long long start = 0;
    const unsigned int* claims = nullptr;
    unsigned int claims_needed = 0;
    // true once the wait has lasted longer than kWaitLimitNs
    __device__ __forceinline__ bool expired() {
        const unsigned long long now = global_ns();
        if (start == 0 || (claims && load_acquire(claims) < claims_needed)) {
            start = now;
            return false;
        }
        return now - start > kWaitLimitNs;
    }
};

// ---- halo exchange with tagged words --------------------------------------------------------------
// Each exchanged entry is one 64-bit word {value bits, tag} written with a single relaxed store, so a
// reader that sees the tag of the half-sweep it needs also sees that half-sweep's value.
__device__ __forceinline__ void store_tagged(unsigned long long* p, float v, unsigned int tag) {
    const unsigned long long word = (static_cast<unsigned long long>(tag) << 32) | __float_as_uint(v);
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(word) : "memory");
}

__device__ __forceinline__ unsigned long long load_tagged(const unsigned long long* p) {
    unsigned long long word;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(word) : "l"(p) : "memory");
    return word;
}

__host__ __device__ __forceinline__ int mirror(int i, int n) { return i < 0 ? 1 : (i > n - 1 ? n - 2 : i); }

// Signals this CTA's arrival at the next epoch, then waits for every CTA of the solve. Returns
// false when aborted (timeout here or elsewhere). `me` is this CTA's tile among `ntiles`.
__device__ __forceinline__ bool grid_barrier(SorControl* ctl, unsigned int* flags, unsigned int& epoch, int me,
                                             int ntiles, const unsigned int* claims = nullptr,
                                             unsigned int claims_needed = 0) {
    epoch += 1;
    __syncthreads();  // the CTA's writes happen before thread 0's release (bar.sync is cumulative)
    if (threadIdx.x == 0) store_release(flags + me, epoch);
    int aborted = 0;
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
        unsigned polls = 0;
        WaitClock clock{0ull, claims, claims_needed};
        while (static_cast<int>(load_acquire(flags + t) - epoch) < 0) {
            if ((++polls & 255u) == 0u) {
                if (load_acquire(&ctl->abort) != 0u) {
                    aborted = 1;
                    break;
                }
                if (clock.expired()) {
                    atomicExch(&ctl->abort, 1u);
                    aborted = 1;
                    break;
                }
            }
        }
    }
    return __syncthreads_or(aborted) == 0;
}

__device__ __forceinline__ float prod_term(const SorArgs& a, int64_t idx) {
    const float prod = a.production ? a.production[idx] : 0.0f;
    if (!a.p.has_source) return prod * 1.0f;
    const float v = a.source[idx];
    return prod * div_rn(v, a.p.source_k + v);
}

// ---- the partition ------------------------------------------------------------------------------------
// Strip s covers columns j in [strip_start(s), strip_start(s + 1)); its tiles are the runs
// tiles_before(s) ... tiles_before(s + 1) - 1 of its columns in (i, j) order, cut evenly.
struct TileRect {
    int ia, ib;  // first and last row
    int ja, jb;  // the first row starts at column ja, the last row ends before column jb
    int j0, j1;  // the strip's columns
};

__host__ __device__ __forceinline__ int strip_start(int s, int strips, int ny) {
    return static_cast<int>(static_cast<int64_t>(s) * ny / strips);
}

__host__ __device__ __forceinline__ int tiles_before(int s, int strips, int ny, int tiles) {
    const int64_t j = strip_start(s, strips, ny);
    return static_cast<int>((2 * static_cast<int64_t>(tiles) * j + ny) / (2 * static_cast<int64_t>(ny)));
}

__host__ __device__ __forceinline__ TileRect tile_rect(int t, int tiles, int strips, int nx, int ny) {
    int s = 0;
    while (s + 1 < strips && tiles_before(s + 1, strips, ny, tiles) <= t) ++s;
    TileRect r;
    r.j0 = strip_start(s, strips, ny);
    r.j1 = strip_start(s + 1, strips, ny);
    const int w = r.j1 - r.j0;
    const int t0 = tiles_before(s, strips, ny, tiles);
    const int tn = tiles_before(s + 1, strips, ny, tiles) - t0;
    const int64_t cols = static_cast<int64_t>(nx) * w;
    const int64_t q0 = (t - t0) * cols / tn, q1 = (t - t0 + 1) * cols / tn;
    r.ia = static_cast<int>(q0 / w);
    r.ja = r.j0 + static_cast<int>(q0 % w);
    r.ib = static_cast<int>((q1 - 1) / w);
    r.jb = r.j0 + static_cast<int>((q1 - 1) % w) + 1;
    return r;
}

__host__ __device__ __forceinline__ bool owns(const TileRect& r, int i, int j) {
    if (i < r.ia || i > r.ib || j < r.j0 || j >= r.j1) return false;
    if (i == r.ia && j < r.ja) return false;
    if (i == r.ib && j >= r.jb) return false;
    return true;
}

// Column kinds of the bounding box.
enum : unsigned char { kNone = 0, kInner = 1, kEdge = 2, kPull = 3, kMirror = 4 };

// Operand ranges of the update's two divisions, cu = u / (K + o) and gs = a2 / (6 + h cu), for the
// fast correctly rounded quotient (div_fast_range: both operands within [2^-60, 2^60], numerator
// possibly zero). Split into a part fixed for the whole solve and a per-node part:
//  * fixed: K in [2^-60, 2^57], h in [2^-60, 2^60], and every coefficient u of the tile either
//    marks a node that is not updated (u < 0), is +-0, or lies in [2^-60, 2^60] with
//    h u / K <= 2^57;
//  * per node: the old value o in [+0, 2^58] (as unsigned bits: no negative, -0 or NaN), and the
//    numerator a2 = +0 or within [2^-60, 2^60].
// Then K + o lies in [K, 2^59], h cu <= 2^58 (cu <= u / K up to two roundings) so 6 + h cu lies
// in [6, 2^59], and both quotients are within the normal range. A +-0 coefficient gives cu = +-0
// and 6 + h cu = 6 either way.
__device__ __forceinline__ bool solve_constants_in_range(float K, float h) {
    return K >= 0x1p-60f && K <= 0x1p57f && h >= 0x1p-60f && h <= 0x1p60f;
}

__device__ __forceinline__ bool coefficient_in_range(float u, float K, float h) {
    if (!(u >= 0.0f) || u == 0.0f) return true;
    return u >= 0x1p-60f && u <= 0x1p60f &&
           static_cast<double>(h) * static_cast<double>(u) <= 0x1p57 * static_cast<double>(K);
}

__device__ __forceinline__ bool old_value_in_range(float o) { return __float_as_uint(o) <= 0x5c800000u; }  // 2^58

__device__ __forceinline__ bool numerator_in_range(float a2) {
    const unsigned int b = __float_as_uint(a2);
    return b == 0u || b - 0x21800000u <= 0x5d800000u - 0x21800000u;  // +0 or [2^-60, 2^60]
}

// The update's quotient with IEEE divisions, for operands outside the fast quotient's range. Out
// of line, so the rarely taken branch to it stays a branch instead of predicated code in every
// node's path.
__device__ __noinline__ float gs_exact(float u, float b1, float nb, float prod, float h) {
    const float cc = __fdiv_rn(u, b1);
    const float b2 = 6.0f + h * cc;
    return __fdiv_rn(nb + h * prod, b2);
}

// The relative residual of one node with IEEE divisions (out of line, as gs_exact).
__device__ __noinline__ float residual_exact(float u, float b1, float nb, float prod, float h, float o, float den) {
    const float cc = __fdiv_rn(u, b1);
    const float res = nb + h * prod - (6.0f + h * cc) * o;
    return __fdiv_rn(fabsf(res), den);
}

// Loop invariants of the solve on one tile.
struct Sweep {
    float* s;  // plane 0; plane 1 follows `plane` floats later
    const int4* relax;  // groups
    const uint4* masks;
    const int4* pull;
    const int2* mir;
    int n_relax, n_pull, n_mir;
    int64_t plane;   // floats per shared-memory plane
    int64_t gplane;  // entries per colour plane of the global copies: nx * ny * M
    int M, si;       // entries per colour column; box row stride in floats
    float K, h, omega, one_minus_omega;
    bool fast;  // K, h and every coefficient of this tile pass the fixed range tests above
};

// Relaxed entries are listed in groups of up to kGroup consecutive entries of one run (one
// descriptor per group, so the per-group bookkeeping is shared by its kGroup / 32 lane-chunks).
// A group (int4): x = its first entry in a shared-memory plane, y = its first entry in colour
// plane 0 of the global copies, z = edge | (m of its first entry) << 8, w = valid entries; beside
// it a uint4 of lane masks, bit l of word r: (i + j) & 1 of the column of entry 32 r + l.
// A pull chunk (int4): x, y as above for 32 entries, z = valid lanes.
constexpr int kGroup = 96;
constexpr int kSub = kGroup / 32;
static_assert(kGroup % 32 == 0 && kSub <= 4, "a group's lane masks fit one uint4");
__device__ __forceinline__ bool group_edge(const int4& d) { return d.z & 1; }

// With Neumann z faces: the entry m of lane `lane` and the last entry of the other colour's
// column (which holds k parity 1 - kp: (nz + 1) / 2 entries for even k, nz / 2 for odd k).
__device__ __forceinline__ void lane_entry(const Sweep& w, const int4& d, int entry, int kp, int nz, int& m,
                                           int& last) {
    m = ((d.z >> 8) + entry) % w.M;
    last = (kp ? (nz + 1) / 2 : nz / 2) - 1;
}

// The six neighbours in the other colour's plane; pv points at the node's own entry there.
template <bool ZCLAMP>
__device__ __forceinline__ float neighbour_sum(const Sweep& w, const float* pv, int kp, int m, int last) {
    float vlo, vhi;
    if (ZCLAMP) {
        vlo = pv[max(m + kp - 1, 0) - m];
        vhi = pv[min(m + kp, last) - m];
    } else {
        vlo = pv[kp - 1];
        vhi = pv[kp];
    }
    return pv[-w.si] + pv[w.si] + pv[-w.M] + pv[w.M] + vlo + vhi;
}

// |r| / max(6 u, reference) of an updated node as float bits, r = nb + h prod - (6 + h c) u with
// c = du / (K + u) at its current value u (field_kernels.py:215-243); the residual pass and the
// last half-sweep of a chunk (for the colour it updates) share this expression.
template <bool HAS_PROD>
__device__ __forceinline__ unsigned int residual_bits(const SorArgs& a, const Sweep& w, float du, float nb, float prod,
                                                      float o) {
    const float pr = HAS_PROD ? prod : 0.0f;
    const float b1 = w.K + o;
    const float cc = div_rn_fast(du, b1);
    const float res = nb + w.h * pr - (6.0f + w.h * cc) * o;
    const float den = fmaxf(6.0f * o, a.p.reference);
    float val = div_rn_fast(fabsf(res), den);
    if (!(div_fast_range(du, b1) && div_fast_range(fabsf(res), den))) val = residual_exact(du, b1, nb, pr, w.h, o, den);
    return __float_as_uint(val);
}

// One lane-chunk (32 entries from `off` of group d) of colour `colour`: the reference's update
// (field_kernels.py:185-212) with the Michaelis-Menten uptake linearised at the old value,
// over-relaxed and clamped at zero. `own` and `oth` point at this lane's entry 0 of the two
// colour planes. Every lane computes; only nodes with a coefficient are written, and the IEEE
// division replaces the fast one only where the range tests above do not hold. An edge group also
// stores every valid entry (unchanged ones too) to the exchange buffer with this half-sweep's tag.
template <bool HAS_PROD, bool ZCLAMP, bool LINEAR, bool RESID>
__device__ __forceinline__ void relax_lanes(const SorArgs& a, const Sweep& w, float* po, const float* pv,
                                            unsigned long long* xp, const int4& d, int off, unsigned mask, float du,
                                            float prod, int colour, int lane, unsigned int tag, unsigned int& rbits) {
    const int kp = ((mask >> lane) & 1) ^ colour;
    int m = 0, last = 0;
    if (ZCLAMP) lane_entry(w, d, off + lane, kp, a.p.nz, m, last);
    const bool active = du >= 0.0f;
    const float o = *po;
    if (LINEAR) {
        // d x - sum_nb x = b: du holds 1 / d, prod holds b; no clamp.
        const float nb = neighbour_sum<ZCLAMP>(w, pv, kp, m, last);
        const float v = w.one_minus_omega * o + w.omega * ((nb + prod) * du);
        if (active) *po = v;
        if (group_edge(d) && off + lane < d.w) store_tagged(xp, active ? v : o, tag);
        return;
    }
    const float b1 = w.K + o;
    const float cc = div_rn_fast_nonneg_zero(du, b1);
    const float nb = neighbour_sum<ZCLAMP>(w, pv, kp, m, last);
    // Without production h * 0 = +0 and nb + 0 = nb except for nb = -0, which the range test
    // sends to the exact branch below.
    const float a2 = HAS_PROD ? nb + w.h * prod : nb;
    const float b2 = 6.0f + w.h * cc;
    float gs = div_rn_fast_nonneg_zero(a2, b2);
    if (active && !(w.fast && old_value_in_range(o) && numerator_in_range(a2))) gs = gs_exact(du, b1, nb, prod, w.h);
    const float v = fmaxf(w.one_minus_omega * o + w.omega * gs, 0.0f);
    if (active) *po = v;
    if (group_edge(d) && off + lane < d.w) store_tagged(xp, active ? v : o, tag);
    if (RESID && active) rbits = max(rbits, residual_bits<HAS_PROD>(a, w, du, nb, prod, v));
}

// The groups of one colour, a warp per group, edge groups first; the next group's coefficients
// (and production terms), which live in L2, are loaded before the current group is relaxed.
template <bool HAS_PROD, bool ZCLAMP, bool LINEAR, bool BRANCH_FREE, bool RESID = false>
__device__ __forceinline__ unsigned int relax_colour(const SorArgs& a, const Sweep& w, int colour, int warp,
                                                     int nwarps, int lane, unsigned int tag) {
    unsigned int rbits = 0u;
    int q = warp;
    if (q >= w.n_relax) return rbits;
    const float* coeff = a.coeff + colour * w.gplane + lane;
    const float* pc = HAS_PROD ? a.pcopy + colour * w.gplane + lane : nullptr;
    float* own = w.s + colour * w.plane + lane;
    const float* oth = w.s + (colour ^ 1) * w.plane + lane;
    unsigned long long* xrow = a.xchg + colour * w.gplane + lane;
    int4 d = w.relax[q];
    float du[kSub], pr[kSub];
#pragma unroll
    for (int r = 0; r < kSub; ++r) {
        du[r] = lane + 32 * r < d.w ? coeff[d.y + 32 * r] : -1.0f;
        pr[r] = HAS_PROD && du[r] >= 0.0f ? pc[d.y + 32 * r] : 0.0f;
    }
    while (true) {
        const int qn = q + nwarps;
        const bool more = qn < w.n_relax;
        int4 dn = d;
        float dun[kSub], prn[kSub];
        if (more) dn = w.relax[qn];
#pragma unroll
        for (int r = 0; r < kSub; ++r) {
            dun[r] = more && lane + 32 * r < dn.w ? coeff[dn.y + 32 * r] : -1.0f;
            prn[r] = HAS_PROD && dun[r] >= 0.0f ? pc[dn.y + 32 * r] : 0.0f;
        }
        const uint4 mk = w.masks[q];
        const unsigned mw[4] = {mk.x, mk.y, mk.z, mk.w};
        float* po = own + d.x;
        const float* pv = oth + d.x;
        unsigned long long* xp = xrow + d.y;
        // BRANCH_FREE: every chunk of the group, without branches between them, so that their
        // dependency chains interleave (lanes past the group's end compute on in-bounds slack and
        // store nothing); otherwise only the chunks with entries (the batched solves of small grids,
        // whose short runs end in many partial groups, run faster that way).
#pragma unroll
        for (int r = 0; r < kSub; ++r)
            if (BRANCH_FREE || r == 0 || d.w > 32 * r)
                relax_lanes<HAS_PROD, ZCLAMP, LINEAR, RESID>(a, w, po + 32 * r, pv + 32 * r, xp + 32 * r, d, 32 * r,
                                                             mw[r], du[r], pr[r], colour, lane, tag, rbits);
        if (!more) break;
        d = dn;
#pragma unroll
        for (int r = 0; r < kSub; ++r) {
            du[r] = dun[r];
            pr[r] = prn[r];
        }
        q = qn;
    }
    return rbits;
}

// Max-norm residual |r| / max(6 u, reference) of the group's nodes of colour `colour`, with
// r = nb + h prod - (6 + h c) u (field_kernels.py:215-243), as float bits (all values are >= 0).
template <bool HAS_PROD, bool ZCLAMP>
__device__ __forceinline__ unsigned int residual_group(const SorArgs& a, const Sweep& w, int q, int colour,
                                                       int lane) {
    const int4 d = w.relax[q];
    const uint4 mk = w.masks[q];
    const unsigned mw[4] = {mk.x, mk.y, mk.z, mk.w};
    unsigned int bits = 0u;
#pragma unroll
    for (int r = 0; r < kSub; ++r) {
        const int off = 32 * r;
        if (off >= d.w) break;
        const float du = off + lane < d.w ? a.coeff[colour * w.gplane + d.y + off + lane] : -1.0f;
        const bool active = du >= 0.0f;
        const float prod = HAS_PROD && active ? a.pcopy[colour * w.gplane + d.y + off + lane] : 0.0f;
        const int kp = ((mw[r] >> lane) & 1) ^ colour;
        const float* po = w.s + colour * w.plane + d.x + off + lane;
        const float* pv = w.s + (colour ^ 1) * w.plane + d.x + off + lane;
        int m = 0, last = 0;
        if (ZCLAMP) lane_entry(w, d, off + lane, kp, a.p.nz, m, last);
        const float o = *po;
        const float nb = neighbour_sum<ZCLAMP>(w, pv, kp, m, last);
        if (active) bits = max(bits, residual_bits<HAS_PROD>(a, w, du, nb, prod, o));
    }
    return bits;
}

// Linear solves: max |b + sum_nb x - d x| and max(6 |x|, |b|) over the group's nodes of colour
// `colour`, as float bits, into *res and *scale.
template <bool ZCLAMP>
__device__ __forceinline__ void residual_group_linear(const SorArgs& a, const Sweep& w, int q, int colour, int lane,
                                                      unsigned int& res, unsigned int& scale) {
    const int4 d = w.relax[q];
    const uint4 mk = w.masks[q];
    const unsigned mw[4] = {mk.x, mk.y, mk.z, mk.w};
#pragma unroll
    for (int r = 0; r < kSub; ++r) {
        const int off = 32 * r;
        if (off >= d.w) break;
        const float du = off + lane < d.w ? a.coeff[colour * w.gplane + d.y + off + lane] : -1.0f;
        if (!(du >= 0.0f)) continue;
        const float b = a.pcopy[colour * w.gplane + d.y + off + lane];
        const int kp = ((mw[r] >> lane) & 1) ^ colour;
        const float* po = w.s + colour * w.plane + d.x + off + lane;
        const float* pv = w.s + (colour ^ 1) * w.plane + d.x + off + lane;
        int m = 0, last = 0;
        if (ZCLAMP) lane_entry(w, d, off + lane, kp, a.p.nz, m, last);
        const float o = *po;
        const float nb = neighbour_sum<ZCLAMP>(w, pv, kp, m, last);
        const float rr = fabsf(b + nb - __frcp_rn(du) * o);
        res = max(res, __float_as_uint(rr));
        scale = max(scale, __float_as_uint(fmaxf(6.0f * fabsf(o), fabsf(b))));
    }
}

// Reads colour `colour` of the halo columns once every entry carries `tag` and stores the values
// in shared memory; each warp has the words of up to kBatch chunks in flight before it checks
// any (their descriptors are re-read from shared memory, so only the words occupy registers).
// Returns false when a wait timed out or another CTA aborted.
__device__ __forceinline__ bool pull_halo(const SorArgs& a, const Sweep& w, int colour, unsigned int tag, int warp,
                                          int nwarps, int lane) {
    constexpr int kBatch = 5;
    const unsigned long long* src = a.xchg + colour * w.gplane + lane;
    float* dst = w.s + colour * w.plane + lane;
    bool fine = true;
    for (int q0 = warp; q0 < w.n_pull; q0 += kBatch * nwarps) {
        unsigned long long v[kBatch];
#pragma unroll
        for (int b = 0; b < kBatch; ++b) {
            const int q = q0 + b * nwarps;
            v[b] = 0ull;
            if (q < w.n_pull) {
                const int4 d = w.pull[q];
                if (lane < d.z) v[b] = load_tagged(src + d.y);
            }
        }
#pragma unroll
        for (int b = 0; b < kBatch; ++b) {
            const int q = q0 + b * nwarps;
            if (q >= w.n_pull) break;
            const int4 d = w.pull[q];
            if (lane < d.z) {
                unsigned polls = 0;
                WaitClock clock;
                while (static_cast<unsigned int>(v[b] >> 32) != tag) {
                    if ((++polls & 255u) == 0u && (load_acquire(&a.ctl->abort) != 0u || clock.expired())) {
                        fine = false;
                        break;
                    }
                    v[b] = load_tagged(src + d.y);
                }
                dst[d.x] = __uint_as_float(static_cast<unsigned int>(v[b]));
            }
        }
    }
    return fine;
}

// Refreshes colour `colour` of the ghost columns outside a Neumann face from their mirror columns.
__device__ __forceinline__ void mirror_columns(const Sweep& w, int colour, int warp, int nwarps, int lane) {
    for (int q = warp; q < w.n_mir; q += nwarps) {
        const int2 c = w.mir[q];
        float* dst = w.s + colour * w.plane + static_cast<int64_t>(c.x) * w.M;
        const float* src = w.s + colour * w.plane + static_cast<int64_t>(c.y) * w.M;
        for (int m = lane; m < w.M; m += 32) dst[m] = src[m];
    }
}

// Builds the tile's column kinds, runs and chunk lists in shared memory and fills the list fields
// of `w`.
__device__ __forceinline__ void build_lists(const SorArgs& a, const TileRect& r, Sweep& w, int warp, int nwarps,
                                            int lane) {
    const int nx = a.p.nx, ny = a.p.ny, M = a.t.M;
    const int bw = r.j1 - r.j0 + 2;
    const int rows = r.ib - r.ia + 3;
    const int nbox = rows * bw;
    char* base = reinterpret_cast<char*>(w.s);
    unsigned char* kind = reinterpret_cast<unsigned char*>(base + a.t.kind_off);
    int4* runs = reinterpret_cast<int4*>(base + a.t.run_off);
    int4* relax = reinterpret_cast<int4*>(base + a.t.relax_off);
    uint4* masks = reinterpret_cast<uint4*>(base + a.t.masks_off);
    int4* pull = reinterpret_cast<int4*>(base + a.t.pull_off);
    int2* mir = reinterpret_cast<int2*>(base + a.t.mirror_off);
    __shared__ int s_counts[5];  // runs, edge groups, inner groups, pull chunks, mirror columns
    // pass 1: the kind of every box column
    for (int e = threadIdx.x; e < nbox; e += blockDim.x) {
        const int i = r.ia - 1 + e / bw, j = r.j0 - 1 + e % bw;
        unsigned char k = kNone;
        if (owns(r, i, j)) {
            k = kInner;
            const int ni[4] = {i - 1, i + 1, i, i};
            const int nj[4] = {j, j, j - 1, j + 1};
            for (int q = 0; q < 4; ++q)
                if (ni[q] >= 0 && ni[q] < nx && nj[q] >= 0 && nj[q] < ny && !owns(r, ni[q], nj[q])) k = kEdge;
        } else if (owns(r, i - 1, j) || owns(r, i + 1, j) || owns(r, i, j - 1) || owns(r, i, j + 1)) {
            const bool out_i = i < 0 || i >= nx, out_j = j < 0 || j >= ny;
            if (!out_i && !out_j) {
                k = kPull;
            } else if (out_i != out_j && (out_i ? a.p.bc_x != 0 : a.p.bc_y != 0)) {
                // Only the columns just outside a Neumann face are read (by the face column); across
                // a Dirichlet face nothing reads them.
                k = kMirror;
            }
        }
        kind[e] = k;
    }
    __syncthreads();
    // pass 2 (one thread): runs of one kind along each box row with their first group (pull chunk);
    // edge groups are numbered first, inner groups after every edge group.
    if (threadIdx.x == 0) {
        int n_runs = 0, n_edge = 0, n_inner = 0, n_pull = 0, n_mir = 0;
        for (int pass = 0; pass < 2; ++pass) {
            for (int row = 0; row < rows; ++row) {
                int c = 0;
                while (c < bw) {
                    const unsigned char k = kind[row * bw + c];
                    if (k == kMirror) {
                        if (pass == 0) {
                            const int i = r.ia - 1 + row, j = r.j0 - 1 + c;
                            const int mi = mirror(i, nx) - (r.ia - 1), mj = mirror(j, ny) - (r.j0 - 1);
                            mir[n_mir++] = make_int2(row * bw + c, mi * bw + mj);
                        }
                        c += 1;
                        continue;
                    }
                    int len = 1;
                    while (c + len < bw && kind[row * bw + c + len] == k) ++len;
                    const int chunks = k == kPull ? (len * M + 31) / 32 : (len * M + kGroup - 1) / kGroup;
                    if (pass == 0 ? (k == kEdge || k == kPull) : k == kInner) {
                        int first;
                        if (k == kEdge) {
                            first = n_edge;
                            n_edge += chunks;
                        } else if (k == kInner) {
                            first = n_edge + n_inner;
                            n_inner += chunks;
                        } else {
                            first = n_pull;
                            n_pull += chunks;
                        }
                        runs[n_runs++] = make_int4(row * bw + c, k | (len << 4), first, row);
                    }
                    c += len;
                }
            }
        }
        s_counts[0] = n_runs;
        s_counts[1] = n_edge;
        s_counts[2] = n_inner;
        s_counts[3] = n_pull;
        s_counts[4] = n_mir;
    }
    __syncthreads();
    const int n_runs = s_counts[0];
    // pass 3a: the pull chunks of each halo run, a warp per run
    for (int q = warp; q < n_runs; q += nwarps) {
        const int4 run = runs[q];
        if ((run.y & 15) != kPull) continue;
        const int len = run.y >> 4, box = run.x, row = run.w;
        const int i = r.ia - 1 + row, j = r.j0 - 1 + box % bw;
        const int total = len * M;
        for (int c = lane; 32 * c < total; c += 32)
            pull[run.z + c] = make_int4(box * M + 32 * c, (i * ny + j) * M + 32 * c, min(32, total - 32 * c), 0);
    }
    // pass 3b: the groups of each owned run, a warp per run
    for (int q = warp; q < n_runs; q += nwarps) {
        const int4 run = runs[q];
        const int k = run.y & 15;
        if (k != kEdge && k != kInner) continue;
        const int len = run.y >> 4, box = run.x, row = run.w;
        const int i = r.ia - 1 + row, j = r.j0 - 1 + box % bw;
        const int total = len * M;
        for (int c = 0; kGroup * c < total; ++c) {
            const int first = kGroup * c, end = min(first + kGroup, total);
            unsigned mw[4] = {0u, 0u, 0u, 0u};
#pragma unroll
            for (int rr = 0; rr < kSub; ++rr) {
                const int f = first + 32 * rr + lane;
                mw[rr] = __ballot_sync(0xffffffffu, f < end && ((i + j + f / M) & 1));
            }
            if (lane == 0) {
                relax[run.z + c] = make_int4(box * M + first, (i * ny + j) * M + first,
                                             (k == kEdge ? 1 : 0) | ((first % M) << 8), end - first);
                masks[run.z + c] = make_uint4(mw[0], mw[1], mw[2], mw[3]);
            }
        }
    }
    __syncthreads();
    w.relax = relax;
    w.masks = masks;
    w.pull = pull;
    w.mir = mir;
    w.n_relax = s_counts[1] + s_counts[2];
    w.n_pull = s_counts[3];
    w.n_mir = s_counts[4];
    w.si = bw * M;
}

// One tile (`tile` of `ntiles`) of one solve, for the whole solve. `claims` / `claims_needed`:
// see WaitClock (batched solves; null for a single solve). LINEAR: the linear system
// d x - sum_nb x = b (`density` holds d, d <= 0 holds x; `production` holds b).
template <bool HAS_PROD, bool ZCLAMP, bool LINEAR, bool BRANCH_FREE>
__device__ __forceinline__ void sor_tile(const SorArgs& a, int tile, int ntiles, const unsigned int* claims = nullptr,
                                         unsigned int claims_needed = 0) {
    extern __shared__ __align__(128) float s[];
    __shared__ unsigned int s_red[32];
    __shared__ unsigned int s_scale[32];
    __shared__ int s_outside_range;
    const int M = a.t.M, nz = a.p.nz, nx = a.p.nx, ny = a.p.ny;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const TileRect r = tile_rect(tile, ntiles, a.t.strips, nx, ny);
    Sweep w;
    w.s = s;
    w.plane = static_cast<int64_t>(a.t.plane_floats);
    w.gplane = static_cast<int64_t>(nx) * ny * M;
    w.M = M;
    w.K = a.p.michaelis_k;
    w.h = a.p.dx2_over_D;
    w.omega = a.p.omega;
    w.one_minus_omega = 1.0f - a.p.omega;
    if (threadIdx.x == 0) s_outside_range = solve_constants_in_range(w.K, w.h) ? 0 : 1;
    build_lists(a, r, w, warp, nwarps, lane);
    const int bw = r.j1 - r.j0 + 2;
    const int rows = r.ib - r.ia + 3;
    const unsigned char* kind = reinterpret_cast<const unsigned char*>(reinterpret_cast<char*>(s) + a.t.kind_off);
    const int64_t sx = static_cast<int64_t>(ny) * nz;

    // ---- box into shared memory; owned coefficients (and production terms) into the copies -----------
    for (int e = warp; e < rows * bw; e += nwarps) {
        const unsigned char k = kind[e];
        if (k == kNone) continue;
        const int i = r.ia - 1 + e / bw, j = r.j0 - 1 + e % bw;
        const int gi = mirror(i, nx), gj = mirror(j, ny);
        const int p = (i + j) & 1;  // a ghost column has the parity of its mirror column
        const int64_t base = gi * sx + static_cast<int64_t>(gj) * nz;
        for (int kk = lane; kk < 2 * M; kk += 32) {
            const int c = (p + kk) & 1;  // colour of node kk
            const float v = kk < nz ? a.field[base + kk] : 0.0f;
            s[c * w.plane + static_cast<int64_t>(e) * M + (kk >> 1)] = v;
            if (k == kInner || k == kEdge) {
                const wbc_sor_params& pp = a.p;
                float u = -1.0f;
                if (kk < nz) {
                    const int64_t idx = base + kk;
                    const bool face = (pp.bc_x == 0 && (gi == 0 || gi == nx - 1)) ||
                                      (pp.bc_y == 0 && (gj == 0 || gj == ny - 1)) ||
                                      (pp.bc_z == 0 && (kk == 0 || kk == nz - 1));
                    if (LINEAR) {
                        const float dd = a.density[idx];
                        if (!face && dd > 0.0f) u = 1.0f / dd;
                    } else {
                        if (!face && !(a.fixed && a.fixed[idx] != 0)) u = a.density[idx] * pp.uptake_max;
                        if (!coefficient_in_range(u, w.K, w.h)) s_outside_range = 1;
                    }
                }
                const int64_t at = c * w.gplane + (static_cast<int64_t>(gi) * ny + gj) * M + (kk >> 1);
                a.coeff[at] = u;
                // The production term is fixed for the solve: computed once here (only where a node
                // is updated, as the update itself would) instead of in every sweep.
                if (LINEAR)
                    a.pcopy[at] = u >= 0.0f ? a.production[base + kk] : 0.0f;
                else if (HAS_PROD)
                    a.pcopy[at] = u >= 0.0f ? prod_term(a, base + kk) : 0.0f;
                // The edge columns start with tag 0 (half-sweeps are tagged from 1), so words a
                // previous solve left in the buffer are never taken for this solve's.
                if (k == kEdge) store_tagged(a.xchg + at, v, 0u);
            }
        }
    }
    unsigned int epoch = 0;
    // The halo columns' coefficients and edge words are written by their owners: one barrier first.
    bool ok = grid_barrier(a.ctl, a.flags, epoch, tile, ntiles, claims, claims_needed);
    w.fast = s_outside_range == 0;  // read after the barrier's __syncthreads

    int sweeps = 0;
    float residual = __int_as_float(0x7f800000);
    bool converged = false;
    int chunk_index = 0;
    constexpr bool kFuseResidual = !LINEAR && !BRANCH_FREE;
    while (ok && sweeps < a.max_sweeps) {
        const int chunk = min(a.check_every, a.max_sweeps - sweeps);
        unsigned int fused_bits = 0u;
        for (int half = 0; half < 2 * chunk; ++half) {
            const int colour = half & 1;
            const unsigned int tag = static_cast<unsigned int>(2 * sweeps + half + 1);
            // In the batched kernel the chunk's last half-sweep (colour 1) also forms its nodes'
            // residuals: their neighbours (colour 0) are final for the chunk, so the residual pass
            // below needs only colour 0. (In the single-solve kernel a second copy of the
            // branch-free relaxation in the loop made every half-sweep 12% slower.)
            if (kFuseResidual && half == 2 * chunk - 1)
                fused_bits = relax_colour<HAS_PROD, ZCLAMP, false, BRANCH_FREE, true>(a, w, colour, warp, nwarps,
                                                                                     lane, tag);
            else
                relax_colour<HAS_PROD || LINEAR, ZCLAMP, LINEAR, BRANCH_FREE>(a, w, colour, warp, nwarps, lane, tag);
            const bool fine = pull_halo(a, w, colour, tag, warp, nwarps, lane);
            if (__syncthreads_or(!fine)) {
                if (threadIdx.x == 0) atomicExch(&a.ctl->abort, 1u);
                ok = false;
                break;
            }
            if (w.n_mir > 0) {
                mirror_columns(w, colour, warp, nwarps, lane);
                __syncthreads();
            }
        }
        if (!ok) break;
        sweeps += chunk;
        // Max-norm residual of the current field over every updated node (both colours); for a
        // linear solve also the scale it is compared against.
        unsigned int bits = fused_bits, sbits = 0u;
        for (int q = warp; q < w.n_relax; q += nwarps) {
            if (LINEAR) {
                residual_group_linear<ZCLAMP>(a, w, q, 0, lane, bits, sbits);
                residual_group_linear<ZCLAMP>(a, w, q, 1, lane, bits, sbits);
            } else {
                bits = max(bits, residual_group<HAS_PROD, ZCLAMP>(a, w, q, 0, lane));
                if (!kFuseResidual) bits = max(bits, residual_group<HAS_PROD, ZCLAMP>(a, w, q, 1, lane));
            }
        }
#pragma unroll
        for (int dd = 16; dd > 0; dd >>= 1) {
            bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, dd));
            if (LINEAR) sbits = max(sbits, __shfl_xor_sync(0xffffffffu, sbits, dd));
        }
        if (lane == 0) {
            s_red[warp] = bits;
            if (LINEAR) s_scale[warp] = sbits;
        }
        __syncthreads();
        const int slot = chunk_index & 1;
        if (warp == 0) {
            bits = lane < nwarps ? s_red[lane] : 0u;
            sbits = LINEAR && lane < nwarps ? s_scale[lane] : 0u;
#pragma unroll
            for (int dd = 16; dd > 0; dd >>= 1) {
                bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, dd));
                if (LINEAR) sbits = max(sbits, __shfl_xor_sync(0xffffffffu, sbits, dd));
            }
            if (lane == 0) {
                atomicMax(&a.ctl->res_bits[slot], bits);
                if (LINEAR) atomicMax(&a.ctl->scale_bits[slot], sbits);
            }
        }
        ok = grid_barrier(a.ctl, a.flags, epoch, tile, ntiles, claims, claims_needed);
        if (!ok) break;
        residual = __uint_as_float(load_acquire(&a.ctl->res_bits[slot]));
        float scale = 1.0f;
        if (LINEAR) scale = __uint_as_float(load_acquire(&a.ctl->scale_bits[slot]));
        // The next chunk's slot was last read before this chunk's first barrier: safe to clear.
        if (tile == 0 && threadIdx.x == 0) {
            atomicExch(&a.ctl->res_bits[slot ^ 1], 0u);
            if (LINEAR) atomicExch(&a.ctl->scale_bits[slot ^ 1], 0u);
        }
        ++chunk_index;
        if (LINEAR) {
            residual = scale > 0.0f ? residual / scale : 0.0f;  // relative to max(6 |x|, |b|)
            if (static_cast<double>(residual) < a.tolerance || scale == 0.0f) {
                converged = true;
                break;
            }
        } else if (static_cast<double>(residual) < a.tolerance) {
            converged = true;
            break;
        }
    }
    if (!ok) {
        if (tile == 0 && threadIdx.x == 0) a.ctl->status = 1;
        return;
    }
    // Owned columns back to the field.
    for (int e = warp; e < rows * bw; e += nwarps) {
        const unsigned char k = kind[e];
        if (k != kInner && k != kEdge) continue;
        const int i = r.ia - 1 + e / bw, j = r.j0 - 1 + e % bw;
        const int p = (i + j) & 1;
        float* out = a.field + i * sx + static_cast<int64_t>(j) * nz;
        for (int kk = lane; kk < nz; kk += 32)
            out[kk] = s[((p + kk) & 1) * w.plane + static_cast<int64_t>(e) * M + (kk >> 1)];
    }
    if (tile == 0 && threadIdx.x == 0) {
        a.ctl->sweeps = sweeps;
        a.ctl->residual = residual;
        a.ctl->converged = converged ? 1 : 0;
        a.ctl->status = 0;
        if (a.residual_out) *a.residual_out = residual;
    }
}

template <bool HAS_PROD, bool ZCLAMP, bool LINEAR>
__global__ void __launch_bounds__(kSorThreads, 1) k_sor_resident(SorArgs a) {
    sor_tile<HAS_PROD, ZCLAMP, LINEAR, true>(a, static_cast<int>(blockIdx.x), static_cast<int>(gridDim.x));
}

// The solver's grid barrier alone, for the self-test of the bounded waits: `ntiles` tiles are
// expected, gridDim.x of them run. With gridDim.x < ntiles the missing tiles never arrive, every
// launched CTA gives up after its bounded wait, and the control block's status says so.
__global__ void k_barrier_selftest(SorControl* ctl, unsigned int* flags, int ntiles, int rounds) {
    unsigned int epoch = 0;
    for (int r = 0; r < rounds; ++r) {
        if (!grid_barrier(ctl, flags, epoch, static_cast<int>(blockIdx.x), ntiles)) {
            if (threadIdx.x == 0) atomicExch(&ctl->status, 1);
            return;
        }
    }
}

// ---- batched solves ----------------------------------------------------------------------------------
// One persistent launch solves many grids. A CTA claims the next tile of the work list (the tiles
// of item 0, then of item 1, ...) and runs it until that item's solve ends, then claims again.
// An item's tiles wait for one another in its first barrier, so its tiles are all resident
// before it starts; since claims are handed out in order and no item has more tiles than there
// are CTAs, the tiles of every item eventually get CTAs.
__device__ __forceinline__ int find_batch_item(const int32_t* first, int n, int x) {
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

template <bool HAS_PROD, bool ZCLAMP>
__global__ void __launch_bounds__(kSorThreads, 1)
    k_sor_batched(const SorArgs* __restrict__ args, const int32_t* __restrict__ tile_first, int n,
                  unsigned int* __restrict__ next_tile) {
    __shared__ int s_tile;
    const int total = tile_first[n];
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) s_tile = static_cast<int>(atomicAdd(next_tile, 1u));
        __syncthreads();
        const int t = s_tile;
        if (t >= total) return;
        const int b = find_batch_item(tile_first, n, t);
        sor_tile<HAS_PROD, ZCLAMP, false, false>(args[b], t - tile_first[b], tile_first[b + 1] - tile_first[b], next_tile,
                                          static_cast<unsigned int>(tile_first[b + 1]));
    }
}

// Zeroes every item's control line and barrier flags, and the claim counter.
__global__ void k_sor_batch_reset(const SorArgs* __restrict__ args, const int32_t* __restrict__ tile_first, int n,
                                  unsigned int* __restrict__ next_tile) {
    for (int b = blockIdx.x; b < n; b += gridDim.x) {
        const SorArgs& a = args[b];
        unsigned int* ctl = reinterpret_cast<unsigned int*>(a.ctl);
        for (int k = threadIdx.x; k < static_cast<int>(sizeof(SorControl) / 4); k += blockDim.x) ctl[k] = 0u;
        const int tiles = tile_first[b + 1] - tile_first[b];
        for (int k = threadIdx.x; k < tiles; k += blockDim.x) a.flags[k] = 0u;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *next_tile = 0u;
}

// ---- host side -------------------------------------------------------------------------------------------
using KernelFn = void (*)(SorArgs);

static KernelFn kernel_for(bool has_prod, bool zclamp, bool linear) {
    if (linear) return zclamp ? k_sor_resident<true, true, true> : k_sor_resident<true, false, true>;
    if (has_prod) return zclamp ? k_sor_resident<true, true, false> : k_sor_resident<true, false, false>;
    return zclamp ? k_sor_resident<false, true, false> : k_sor_resident<false, false, false>;
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

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// The shared-memory layout for `tiles` tiles cut from `strips` strips; false if that partition is
// not valid for the grid (an empty strip or tile) or the largest tile does not fit in smem_limit.
// `score` (may be NULL): the largest tile's columns, then its bounding box, for choosing among
// partitions.
// Time model of one sweep of a tile in the batched solver, in ns (a fit to per-item run times
// traced in batched solves of 55^3-119^3 grids on 5-76 tiles each, on the GB300, within 5% rms):
// the relaxation of the tile's owned nodes, its halo (the bounding box's perimeter columns, whose
// pulls and mirrors scale with it) and a fixed cost per sweep (the halo exchanges' round trips and
// the closing barriers). An item's tiles advance together, so its largest tile sets the pace.
constexpr double kNsPerNode = 0.393, kNsPerHaloNode = 0.235, kNsPerSweep = 3140.0;
__host__ __device__ inline double tile_sweep_ns(int owned_columns, int perimeter_columns, int nz) {
    return kNsPerNode * owned_columns * nz + kNsPerHaloNode * perimeter_columns * nz + kNsPerSweep;
}

static bool tiling_for(const wbc_sor_params& p, int tiles, int strips, size_t smem_limit, SorTiling* out,
                       long* score = nullptr, double* sweep_ns = nullptr) {
    if (tiles < 1 || tiles > kMaxCtas || strips < 1 || strips > p.ny || strips > tiles) return false;
    const int M = (p.nz + 1) / 2;
    if (M > kMaxEntries || p.nx > 32767 || p.ny > 32767) return false;
    if (static_cast<int64_t>(p.nx) * p.ny * M >= (1ll << 31) - 64) return false;  // 32-bit chunk offsets
    for (int s = 0; s < strips; ++s) {
        const int w = strip_start(s + 1, strips, p.ny) - strip_start(s, strips, p.ny);
        const int tn = tiles_before(s + 1, strips, p.ny, tiles) - tiles_before(s, strips, p.ny, tiles);
        if (w < 1 || tn < 1 || static_cast<int64_t>(tn) > static_cast<int64_t>(p.nx) * w) return false;
    }
    int max_box = 0, max_rows = 0, max_owned = 0, max_perimeter = 0;
    for (int t = 0; t < tiles; ++t) {
        const TileRect r = tile_rect(t, tiles, strips, p.nx, p.ny);
        const int rows = r.ib - r.ia + 3, bw = r.j1 - r.j0 + 2;
        const int owned = (r.ib - r.ia + 1) * (r.j1 - r.j0) - (r.ja - r.j0) - (r.j1 - r.jb);
        max_box = std::max(max_box, rows * bw);
        max_rows = std::max(max_rows, rows);
        max_owned = std::max(max_owned, owned);
        max_perimeter = std::max(max_perimeter, 2 * (rows + bw));
    }
    SorTiling t{};
    t.tiles = tiles;
    t.strips = strips;
    t.M = M;
    t.max_box = max_box;
    // Groups: a run of len owned columns has ceil(len M / kGroup); every row of a tile has at most
    // five runs of owned columns (edge / inner / edge, and the staircase). Pull chunks: the halo
    // columns lie on the bounding box's perimeter, ceil(len M / 32) per run.
    t.relax_cap = (max_owned * M + kGroup - 1) / kGroup + 6 * max_rows + 8;
    t.pull_cap = (max_perimeter * M + 31) / 32 + max_perimeter + 8;
    t.mirror_cap = max_perimeter + 8;
    t.run_cap = max_box + 8;
    t.plane_floats = align_up(static_cast<size_t>(max_box) * M + kPlaneSlack, 32);
    t.relax_off = align_up(2 * t.plane_floats * sizeof(float), 16);
    t.masks_off = align_up(t.relax_off + static_cast<size_t>(t.relax_cap) * sizeof(int4), 16);
    t.pull_off = align_up(t.masks_off + static_cast<size_t>(t.relax_cap) * sizeof(uint4), 16);
    t.run_off = align_up(t.pull_off + static_cast<size_t>(t.pull_cap) * sizeof(int4), 16);
    t.mirror_off = align_up(t.run_off + static_cast<size_t>(t.run_cap) * sizeof(int4), 16);
    t.kind_off = align_up(t.mirror_off + static_cast<size_t>(t.mirror_cap) * sizeof(int2), 16);
    t.smem = align_up(t.kind_off + static_cast<size_t>(max_box), 16);
    if (t.smem > smem_limit) return false;
    *out = t;
    if (score) *score = static_cast<long>(max_owned) * 100000 + max_box;
    if (sweep_ns) *sweep_ns = tile_sweep_ns(max_owned, max_perimeter, p.nz);
    return true;
}

// `tiles` tiles (at most one CTA per SM and within the barrier flags); the strip count with the
// smallest largest tile, then the smallest bounding box, unless `want_strips` fixes it.
static bool choose_tiling(const wbc_sor_params& p, int tiles, size_t smem_limit, int want_strips, SorTiling* out) {
    tiles = std::min({tiles, kMaxCtas, p.nx * p.ny});
    if (tiles < 1) return false;
    if (want_strips > 0) return tiling_for(p, tiles, want_strips, smem_limit, out);
    bool found = false;
    long best = 0;
    for (int strips = 1; strips <= std::min(p.ny, tiles); ++strips) {
        SorTiling t{};
        long score = 0;
        if (!tiling_for(p, tiles, strips, smem_limit, &t, &score)) continue;
        if (!found || score < best) {
            found = true;
            best = score;
            *out = t;
        }
    }
    return found;
}

// The tiling of `tiles` tiles with the smallest modelled sweep time, over strip counts around the
// square shape (long thin tiles have long halos: at 101^3 on 34 tiles, 17 strips ran a sweep in
// 20.7 us against 15.8 us modelled for 4 strips); false if none fits in shared memory.
static bool compact_tiling(const wbc_sor_params& p, int tiles, size_t smem_limit, SorTiling* out, double* sweep_ns) {
    tiles = std::min({tiles, kMaxCtas, p.nx * p.ny});
    if (tiles < 1) return false;
    const double square = std::sqrt(static_cast<double>(tiles) * p.ny / p.nx);
    const int lo = std::max(1, static_cast<int>(square / 2.0));
    const int hi = std::min({p.ny, tiles, static_cast<int>(2.0 * square) + 2});
    bool found = false;
    for (int strips = lo; strips <= hi; ++strips) {
        SorTiling t{};
        double ns = 0.0;
        if (!tiling_for(p, tiles, strips, smem_limit, &t, nullptr, &ns)) continue;
        if (!found || ns < *sweep_ns) {
            found = true;
            *sweep_ns = ns;
            *out = t;
        }
    }
    return found;
}

static size_t plane_bytes(const wbc_sor_params& p, size_t element) {
    return 2ull * p.nx * p.ny * ((p.nz + 1) / 2) * element;
}

static size_t header_bytes() { return align_up(sizeof(SorControl) + kMaxCtas * sizeof(unsigned int), 256); }

// [control block + barrier flags][tagged exchange words][coefficient copy][production copy]
size_t sor_workspace_bytes(const wbc_sor_params& p) {
    return header_bytes() + align_up(plane_bytes(p, 8), 256) + 2 * align_up(plane_bytes(p, 4), 256) + 256;
}

static void place_workspace(const wbc_sor_params& p, void* workspace, SorArgs* a) {
    char* base = static_cast<char*>(workspace);
    a->ctl = reinterpret_cast<SorControl*>(base);
    a->flags = reinterpret_cast<unsigned int*>(base + sizeof(SorControl));
    size_t off = header_bytes();
    a->xchg = reinterpret_cast<unsigned long long*>(base + off);
    off += align_up(plane_bytes(p, 8), 256);
    a->coeff = reinterpret_cast<float*>(base + off);
    off += align_up(plane_bytes(p, 4), 256);
    a->pcopy = reinterpret_cast<float*>(base + off);
}

// Host record of a deferred solve's report (wbc_sor_solve_deferred): the solver's control line,
// copied by the solve's stream, and what the host knew at launch. `ready` = 1 when `report` is
// already final (a solve on the streaming path, which reads its residual on the host anyway).
struct SorReportRecord {
    SorControl ctl;
    int32_t ready, path, tiles, strips;
    wbc_sor_report report;
};

int sor_solve_resident(const wbc_sor_params& p, int check_every, int max_sweeps, double tolerance,
                       const int32_t* fixed, const float* density, const float* production, const float* source,
                       float* field, float* residual_out, wbc_sor_report* report, void* workspace,
                       const wbc_sor_tuning* tuning, cudaStream_t stream, bool* feasible, bool linear = false,
                       SorReportRecord* deferred = nullptr) {
    const DeviceInfo dev = device_info();
    const size_t limit = static_cast<size_t>(dev.smem_optin) - 1024;  // static shared memory of the kernel
    SorTiling t{};
    const int want_tiles = tuning && tuning->tiles > 0 ? tuning->tiles : dev.sms;
    const int want_strips = tuning ? tuning->strips : 0;
    *feasible = dev.sms > 0 && want_tiles <= dev.sms && choose_tiling(p, want_tiles, limit, want_strips, &t);
    if (!*feasible) return WBC_OK;
    const bool has_prod = production != nullptr || p.has_source;
    KernelFn fn = kernel_for(has_prod, p.bc_z != 0, linear);
    cudaError_t err = cudaFuncSetAttribute(reinterpret_cast<const void*>(fn),
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(t.smem));
    if (err != cudaSuccess) {
        set_error("wbc_sor_solve: cudaFuncSetAttribute", err);
        return WBC_ERR_CUDA;
    }
    int per_sm = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSorThreads, t.smem);
    if (err != cudaSuccess || per_sm < 1 || t.tiles > per_sm * dev.sms) {
        cudaGetLastError();
        *feasible = false;
        return WBC_OK;
    }
    SorArgs args{};
    args.p = p;
    args.t = t;
    args.fixed = fixed;
    args.density = density;
    args.production = production;
    args.source = source;
    args.field = field;
    args.residual_out = residual_out;
    args.check_every = check_every;
    args.max_sweeps = max_sweeps;
    args.tolerance = tolerance;
    place_workspace(p, workspace, &args);
    err = cudaMemsetAsync(workspace, 0, header_bytes(), stream);
    if (err != cudaSuccess) {
        set_error("wbc_sor_solve: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    void* params[] = {&args};
    err = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(fn), dim3(t.tiles), dim3(kSorThreads), params,
                                      t.smem, stream);
    if (err != cudaSuccess) {
        set_error("wbc_sor_solve: cudaLaunchCooperativeKernel", err);
        return WBC_ERR_CUDA;
    }
    int rc = check_launch("wbc_sor_solve", 1);
    if (rc != WBC_OK) return rc;
    if (deferred) {
        // the control line reaches the record when the stream gets there; nothing waits here
        deferred->ready = 0;
        deferred->path = 2;
        deferred->tiles = t.tiles;
        deferred->strips = t.strips;
        err = cudaMemcpyAsync(&deferred->ctl, args.ctl, sizeof(SorControl), cudaMemcpyDeviceToHost, stream);
        if (err != cudaSuccess) {
            set_error("wbc_sor_solve_deferred: copying the report", err);
            return WBC_ERR_CUDA;
        }
        return WBC_OK;
    }
    SorControl host{};
    err = cudaMemcpyAsync(&host, args.ctl, sizeof(SorControl), cudaMemcpyDeviceToHost, stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
    if (err != cudaSuccess) {
        set_error("wbc_sor_solve: reading the report", err);
        return WBC_ERR_CUDA;
    }
    if (host.status != 0) {
        set_error_msg("wbc_sor_solve: a device wait timed out");
        return WBC_ERR_TIMEOUT;
    }
    report->sweeps = host.sweeps;
    report->residual = host.residual;
    report->converged = host.converged;
    report->path = 2;
    report->tiles = t.tiles;
    report->strips = t.strips;
    return WBC_OK;
}

// Candidate tunings for the autotuner: every SM, and the strip counts around the one with the
// smallest largest tile and bounding box.
static std::vector<wbc_sor_tuning> tuning_candidates(const wbc_sor_params& p, int sms, size_t limit) {
    std::vector<wbc_sor_tuning> out;
    SorTiling best{};
    if (!choose_tiling(p, sms, limit, 0, &best)) return out;
    for (int strips : {best.strips, best.strips - 1, best.strips + 1, best.strips - 2, best.strips + 2}) {
        SorTiling t{};
        if (strips >= 1 && tiling_for(p, best.tiles, strips, limit, &t))
            out.push_back(wbc_sor_tuning{t.tiles, t.strips});
    }
    return out;
}

// ---- batched solves: host side -------------------------------------------------------------------------
using BatchedFn = void (*)(const SorArgs*, const int32_t*, int, unsigned int*);

static BatchedFn batched_for(bool has_prod, bool zclamp) {
    if (has_prod) return zclamp ? k_sor_batched<true, true> : k_sor_batched<true, false>;
    return zclamp ? k_sor_batched<false, true> : k_sor_batched<false, false>;
}

struct SorBatchLayout {
    size_t next, args, first, item, bytes;
};

// [claim counter | SorArgs per work-list position | tile offsets | item index per position]
static SorBatchLayout sor_batch_layout(int n) {
    SorBatchLayout L{};
    L.next = 0;
    L.args = 256;
    L.first = L.args + ((n * sizeof(SorArgs) + 255) / 256) * 256;
    L.item = L.first + (n + 1) * sizeof(int32_t);
    L.bytes = L.item + n * sizeof(int32_t);
    return L;
}

}  // namespace wbc

using namespace wbc;

// The batched solve's plan: the order of the items in the work list and each item's tiling, on G
// CTAs with `limit` bytes of shared memory each; false if some grid does not fit. `work` is the
// expected work per item (nodes x sweeps when `weighted`, else nodes).
//
// Waves: groups of items that run at the same time, each item on its own tiles, the next wave's
// tiles claimed as CTAs free up. The items are taken in order of sweep count (work / nodes; 1
// without weights), most first, and cut into contiguous waves by dynamic programming over the cut
// points, minimising the sum of the waves' durations under the time model of tile_sweep_ns (an
// item's duration: its sweeps x the modelled sweep time of its tiling). Within a wave the tile
// counts give every item the same duration, each with at least the fewest tiles that fit in shared
// memory, and CTAs left over go to the slowest items. Grouping items of similar sweep counts
// matters: a tile pays a fixed cost every sweep besides the relaxation of its nodes, so CTAs in
// proportion to work alone leave the items with more sweeps ending last while the wave's other
// CTAs wait in the next wave's first barrier. Every tiling is the compact one for its tile count.
static bool plan_batch(const std::vector<wbc_sor_params>& params, const std::vector<double>& work, bool weighted,
                       int G, size_t limit, std::vector<int32_t>& order, std::vector<SorTiling>& tiling,
                       std::vector<int32_t>* wave_of = nullptr, std::vector<double>* sweep_ns = nullptr) {
    const int n = static_cast<int>(params.size());
    // per distinct grid: the tile counts along which the modelled sweep time falls (the Pareto
    // front of count against time, from the fewest tiles that fit), with their tilings
    struct Front {
        int nx, ny, nz;
        std::vector<int> tiles;
        std::vector<double> ns;
        std::vector<SorTiling> tiling;
    };
    std::vector<Front> fronts;
    std::vector<int> front_of(n);
    std::vector<double> sweeps(n);
    for (int b = 0; b < n; ++b) {
        const wbc_sor_params& p = params[b];
        sweeps[b] = weighted ? work[b] / (static_cast<double>(p.nx) * p.ny * p.nz) : 1.0;
        int f = 0;
        while (f < static_cast<int>(fronts.size()) &&
               !(fronts[f].nx == p.nx && fronts[f].ny == p.ny && fronts[f].nz == p.nz))
            ++f;
        if (f == static_cast<int>(fronts.size())) {
            Front fr{p.nx, p.ny, p.nz, {}, {}, {}};
            for (int T = 1; T <= G; ++T) {
                SorTiling t{};
                double ns = 0.0;
                if (!compact_tiling(p, T, limit, &t, &ns)) continue;
                if (t.tiles != T) break;  // fewer columns than tiles
                if (fr.ns.empty() || ns < fr.ns.back()) {
                    fr.tiles.push_back(T);
                    fr.ns.push_back(ns);
                    fr.tiling.push_back(t);
                }
            }
            if (fr.tiles.empty()) return false;
            fronts.push_back(fr);
        }
        front_of[b] = f;
    }
    order.resize(n);
    for (int b = 0; b < n; ++b) order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        if (sweeps[x] != sweeps[y]) return sweeps[x] > sweeps[y];
        return work[x] > work[y];
    });
    // an item's choice is an index into its front; duration falls with the index
    auto duration = [&](int b, int k) { return sweeps[b] * fronts[front_of[b]].ns[k]; };
    auto count = [&](int b, int k) { return fronts[front_of[b]].tiles[k]; };
    auto last = [&](int b) { return static_cast<int>(fronts[front_of[b]].tiles.size()) - 1; };
    // the first index with duration <= D, or -1
    auto within = [&](int b, double D) {
        int lo = 0, hi = last(b);
        if (duration(b, hi) > D) return -1;
        while (lo < hi) {
            const int mid = (lo + hi) / 2;
            if (duration(b, mid) <= D)
                hi = mid;
            else
                lo = mid + 1;
        }
        return lo;
    };
    // equal-duration choices for the items order[lo, hi) on G CTAs; their duration, or -1
    auto wave_plan = [&](int lo, int hi, std::vector<int>* pick) {
        int need = 0;
        double D_hi = 0.0, D_lo = 0.0;
        for (int k = lo; k < hi; ++k) {
            need += count(order[k], 0);
            D_hi = std::max(D_hi, duration(order[k], 0));
        }
        if (need > G) return -1.0;
        for (int it = 0; it < 40; ++it) {
            const double D = 0.5 * (D_lo + D_hi);
            int total = 0;
            for (int k = lo; k < hi && total <= G; ++k) {
                const int q = within(order[k], D);
                total += q < 0 ? G + 1 : count(order[k], q);
            }
            (total <= G ? D_hi : D_lo) = D;
        }
        std::vector<int> K(hi - lo);
        int total = 0;
        for (int k = lo; k < hi; ++k) total += count(order[k], K[k - lo] = within(order[k], D_hi));
        while (true) {  // spare CTAs: the slowest item's next choice, while it fits
            int slow = 0;
            for (int q = 1; q < hi - lo; ++q)
                if (duration(order[lo + q], K[q]) > duration(order[lo + slow], K[slow])) slow = q;
            const int b = order[lo + slow];
            if (K[slow] == last(b) || total + count(b, K[slow] + 1) - count(b, K[slow]) > G) break;
            total += count(b, K[slow] + 1) - count(b, K[slow]);
            ++K[slow];
        }
        double D = 0.0;
        for (int q = 0; q < hi - lo; ++q) D = std::max(D, duration(order[lo + q], K[q]));
        if (pick) *pick = K;
        return D;
    };
    constexpr int kMaxWave = 48;  // items per wave (bounds the planning time of large batches)
    std::vector<double> best(n + 1, -1.0);
    std::vector<int> cut(n + 1, 0);
    best[0] = 0.0;
    for (int hi = 1; hi <= n; ++hi) {
        for (int lo = hi - 1; lo >= std::max(0, hi - kMaxWave); --lo) {
            const double D = wave_plan(lo, hi, nullptr);
            if (D < 0.0) break;  // a longer wave does not fit either
            if (best[lo] >= 0.0 && (best[hi] < 0.0 || best[lo] + D < best[hi])) {
                best[hi] = best[lo] + D;
                cut[hi] = lo;
            }
        }
    }
    if (best[n] < 0.0) return false;
    tiling.assign(n, SorTiling{});
    if (wave_of) wave_of->assign(n, 0);
    if (sweep_ns) sweep_ns->assign(n, 0.0);
    int waves = 0;
    for (int hi = n; hi > 0; hi = cut[hi]) ++waves;
    for (int hi = n; hi > 0; hi = cut[hi]) {
        std::vector<int> K;
        wave_plan(cut[hi], hi, &K);
        --waves;
        for (int k = cut[hi]; k < hi; ++k) {
            const Front& fr = fronts[front_of[order[k]]];
            tiling[k] = fr.tiling[K[k - cut[hi]]];
            if (wave_of) (*wave_of)[k] = waves;
            if (sweep_ns) (*sweep_ns)[k] = fr.ns[K[k - cut[hi]]];
        }
    }
    return true;
}

extern "C" {

size_t wbc_sor_batch_plan_bytes(int32_t n) { return n > 0 ? sor_batch_layout(n).bytes : 0; }

int wbc_sor_batch_plan_host(int32_t n, const wbc_sor_params* params, const float* weights, int32_t ctas,
                            int64_t smem_bytes, int32_t* order, int32_t* tiles, int32_t* strips, int32_t* wave,
                            double* sweep_ns) {
    if (n <= 0 || !params || ctas < 1 || ctas > kMaxCtas || smem_bytes <= 0 || !order || !tiles || !strips)
        return WBC_ERR_INVALID;
    std::vector<wbc_sor_params> p(params, params + n);
    std::vector<double> work(n);
    for (int b = 0; b < n; ++b) {
        if (p[b].nx < 3 || p[b].ny < 3 || p[b].nz < 3 || (weights && !(weights[b] > 0.0f))) {
            set_error_msg("wbc_sor_batch_plan_host: invalid item");
            return WBC_ERR_INVALID;
        }
        work[b] = weights ? static_cast<double>(weights[b]) : static_cast<double>(p[b].nx) * p[b].ny * p[b].nz;
    }
    std::vector<int32_t> ord, wv;
    std::vector<SorTiling> til;
    std::vector<double> ns;
    if (!plan_batch(p, work, weights != nullptr, ctas, static_cast<size_t>(smem_bytes), ord, til, &wv, &ns)) {
        set_error_msg("wbc_sor_batch_plan_host: a grid does not fit the shared-memory resident solver");
        return WBC_ERR_INVALID;
    }
    for (int k = 0; k < n; ++k) {
        order[k] = ord[k];
        tiles[k] = til[k].tiles;
        strips[k] = til[k].strips;
        if (wave) wave[k] = wv[k];
        if (sweep_ns) sweep_ns[k] = ns[k];
    }
    return WBC_OK;
}

int wbc_sor_batch_prepare(int32_t n, const wbc_sor_batch_item* items, const float* weights, int32_t check_every,
                          int32_t max_sweeps, double tolerance, void* plan, size_t plan_bytes, wbc_sor_batch* out,
                          void* stream) {
    if (n <= 0 || !items || !plan || !out || check_every < 1 || max_sweeps < 1) return WBC_ERR_INVALID;
    const SorBatchLayout L = sor_batch_layout(n);
    if (plan_bytes < L.bytes) return WBC_ERR_WORKSPACE;
    const DeviceInfo dev = device_info();
    if (dev.sms <= 0) {
        set_error_msg("wbc_sor_batch_prepare: no device");
        return WBC_ERR_CUDA;
    }
    const int G = std::min(dev.sms, kMaxCtas);
    const size_t limit = static_cast<size_t>(dev.smem_optin) - 1024;
    // Expected work per item: the caller's weight (e.g. nodes x sweeps of the previous solve), or
    // its node count.
    std::vector<double> work(n);
    for (int b = 0; b < n; ++b) {
        const wbc_sor_params& p = items[b].params;
        if (p.nx < 3 || p.ny < 3 || p.nz < 3 || !items[b].density || !items[b].field || !items[b].workspace ||
            (p.has_source && !items[b].source) || reinterpret_cast<uintptr_t>(items[b].workspace) % 16 != 0 ||
            (weights && !(weights[b] > 0.0f))) {
            set_error_msg("wbc_sor_batch_prepare: invalid item");
            return WBC_ERR_INVALID;
        }
        work[b] = weights ? static_cast<double>(weights[b]) : static_cast<double>(p.nx) * p.ny * p.nz;
    }
    std::vector<int32_t> order;
    std::vector<SorTiling> tiling;
    std::vector<wbc_sor_params> params(n);
    for (int b = 0; b < n; ++b) params[b] = items[b].params;
    if (!plan_batch(params, work, weights != nullptr, G, limit, order, tiling)) {
        set_error_msg("wbc_sor_batch_prepare: a grid does not fit the shared-memory resident solver");
        return WBC_ERR_INVALID;
    }
    std::vector<SorArgs> args(n);
    std::vector<int32_t> first(n + 1, 0);
    bool has_prod = false, zclamp = false;
    size_t smem = 0;
    for (int k = 0; k < n; ++k) {
        const int b = order[k];
        const wbc_sor_batch_item& it = items[b];
        const wbc_sor_params& p = it.params;
        const SorTiling& t = tiling[k];
        SorArgs& a = args[k];
        a.p = p;
        a.t = t;
        a.fixed = it.fixed;
        a.density = it.density;
        a.production = it.production;
        a.source = it.source;
        a.field = it.field;
        a.residual_out = nullptr;
        a.check_every = check_every;
        a.max_sweeps = max_sweeps;
        a.tolerance = tolerance;
        place_workspace(p, it.workspace, &a);
        first[k + 1] = first[k] + t.tiles;
        smem = std::max(smem, t.smem);
        has_prod = has_prod || it.production != nullptr || p.has_source;
        zclamp = zclamp || p.bc_z != 0;
    }
    BatchedFn fn = batched_for(has_prod, zclamp);
    cudaError_t err = cudaFuncSetAttribute(reinterpret_cast<const void*>(fn),
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    int per_sm = 0;
    if (err == cudaSuccess) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSorThreads, smem);
    if (err != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        set_error_msg("wbc_sor_batch_prepare: the batched solver does not fit on an SM");
        return WBC_ERR_INVALID;
    }
    const int ctas = std::min(G, first[n]);
    std::vector<char> host(L.bytes, 0);
    std::memcpy(host.data() + L.args, args.data(), n * sizeof(SorArgs));
    std::memcpy(host.data() + L.first, first.data(), (n + 1) * sizeof(int32_t));
    std::memcpy(host.data() + L.item, order.data(), n * sizeof(int32_t));
    cudaStream_t s = as_stream(stream);
    err = cudaMemcpyAsync(plan, host.data(), L.bytes, cudaMemcpyHostToDevice, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);  // `host` goes out of scope
    if (err != cudaSuccess) {
        set_error("wbc_sor_batch_prepare: copying the plan", err);
        return WBC_ERR_CUDA;
    }
    out->items = n;
    out->total_tiles = first[n];
    out->ctas = ctas;
    out->threads = kSorThreads;
    out->zclamp = zclamp ? 1 : 0;
    out->has_prod = has_prod ? 1 : 0;
    out->smem_bytes = static_cast<int64_t>(smem);
    out->device_plan = plan;
    return WBC_OK;
}

int wbc_sor_batch_solve(const wbc_sor_batch* b, void* stream) {
    if (!b || b->items <= 0 || !b->device_plan || b->ctas < 1) return WBC_ERR_INVALID;
    const SorBatchLayout L = sor_batch_layout(b->items);
    char* base = static_cast<char*>(b->device_plan);
    const SorArgs* args = reinterpret_cast<const SorArgs*>(base + L.args);
    const int32_t* first = reinterpret_cast<const int32_t*>(base + L.first);
    unsigned int* next = reinterpret_cast<unsigned int*>(base + L.next);
    cudaStream_t s = as_stream(stream);
    k_sor_batch_reset<<<std::min(b->items, 1024), 128, 0, s>>>(args, first, b->items, next);
    BatchedFn fn = batched_for(b->has_prod != 0, b->zclamp != 0);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b->ctas);
    cfg.blockDim = dim3(kSorThreads);
    cfg.dynamicSmemBytes = static_cast<size_t>(b->smem_bytes);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int items = b->items;
    cudaError_t err = cudaLaunchKernelEx(&cfg, fn, args, first, items, next);
    if (err != cudaSuccess) {
        set_error("wbc_sor_batch_solve: cudaLaunchKernelEx", err);
        return WBC_ERR_CUDA;
    }
    return check_launch("wbc_sor_batch_solve", 2);
}

int wbc_sor_batch_reports(const wbc_sor_batch* b, wbc_sor_report* reports, void* stream) {
    if (!b || b->items <= 0 || !b->device_plan || !reports) return WBC_ERR_INVALID;
    const SorBatchLayout L = sor_batch_layout(b->items);
    std::vector<SorArgs> args(b->items);
    std::vector<int32_t> first(b->items + 1), order(b->items);
    cudaStream_t s = as_stream(stream);
    char* base = static_cast<char*>(b->device_plan);
    cudaError_t err = cudaMemcpyAsync(args.data(), base + L.args, b->items * sizeof(SorArgs), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(first.data(), base + L.first, (b->items + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(order.data(), base + L.item, b->items * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    std::vector<SorControl> ctl(b->items);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    for (int i = 0; i < b->items && err == cudaSuccess; ++i)
        err = cudaMemcpyAsync(&ctl[i], args[i].ctl, sizeof(SorControl), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) {
        set_error("wbc_sor_batch_reports: reading the reports", err);
        return WBC_ERR_CUDA;
    }
    int rc = WBC_OK;
    for (int k = 0; k < b->items; ++k) {
        wbc_sor_report& r = reports[order[k]];
        r.sweeps = ctl[k].sweeps;
        r.residual = ctl[k].residual;
        r.converged = ctl[k].converged;
        r.path = 2;
        r.tiles = first[k + 1] - first[k];
        r.strips = args[k].t.strips;
        if (ctl[k].status != 0) rc = WBC_ERR_TIMEOUT;
    }
    if (rc != WBC_OK) set_error_msg("wbc_sor_batch_reports: a solve timed out");
    return rc;
}

size_t wbc_sor_solve_workspace_bytes(const wbc_sor_params* p) {
    if (!p) return 0;
    return sor_workspace_bytes(*p);
}

int wbc_sor_autotune(const wbc_sor_params* p, int32_t check_every, const int32_t* fixed, const float* density,
                     const float* production, const float* source, const float* field, float* scratch_field,
                     void* workspace, size_t workspace_bytes, wbc_sor_tuning* best, float* best_us_per_sweep,
                     void* stream) {
    if (!p || p->nx < 3 || p->ny < 3 || p->nz < 3 || check_every < 1 || !density || !field || !scratch_field ||
        !workspace || !best || (p->has_source && !source))
        return WBC_ERR_INVALID;
    if (workspace_bytes < sor_workspace_bytes(*p)) return WBC_ERR_WORKSPACE;
    if (reinterpret_cast<uintptr_t>(workspace) % 16 != 0) {
        set_error_msg("wbc_sor_autotune: the workspace must be 16-byte aligned");
        return WBC_ERR_INVALID;
    }
    *best = wbc_sor_tuning{0, 0};
    if (best_us_per_sweep) *best_us_per_sweep = 0.0f;
    const DeviceInfo dev = device_info();
    if (dev.sms <= 0) return WBC_OK;
    const size_t limit = static_cast<size_t>(dev.smem_optin) - 1024;
    const std::vector<wbc_sor_tuning> cands = tuning_candidates(*p, dev.sms, limit);
    if (cands.empty()) return WBC_OK;
    cudaStream_t s = as_stream(stream);
    const size_t field_bytes = static_cast<size_t>(p->nx) * p->ny * p->nz * sizeof(float);
    const int sweeps = 2 * check_every;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    if (err != cudaSuccess) {
        set_error("wbc_sor_autotune: cudaEventCreate", err);
        if (e0) cudaEventDestroy(e0);
        return WBC_ERR_CUDA;
    }
    std::vector<float> best_ms(cands.size(), -1.0f);
    int rc = WBC_OK;
    for (int rep = 0; rep < 2 && rc == WBC_OK; ++rep) {
        for (size_t c = 0; c < cands.size() && rc == WBC_OK; ++c) {
            err = cudaMemcpyAsync(scratch_field, field, field_bytes, cudaMemcpyDeviceToDevice, s);
            if (err == cudaSuccess) err = cudaEventRecord(e0, s);
            if (err != cudaSuccess) {
                set_error("wbc_sor_autotune: copying the field", err);
                rc = WBC_ERR_CUDA;
                break;
            }
            wbc_sor_report r{};
            bool feasible = false;
            // A negative tolerance never converges: every candidate runs the same sweeps.
            rc = sor_solve_resident(*p, check_every, sweeps, -1.0, fixed, density, production, source, scratch_field,
                                    nullptr, &r, workspace, &cands[c], s, &feasible);
            if (rc != WBC_OK) break;
            err = cudaEventRecord(e1, s);
            if (err == cudaSuccess) err = cudaEventSynchronize(e1);
            float ms = 0.0f;
            if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
            if (err != cudaSuccess) {
                set_error("wbc_sor_autotune: timing", err);
                rc = WBC_ERR_CUDA;
                break;
            }
            if (feasible && (best_ms[c] < 0.0f || ms < best_ms[c])) best_ms[c] = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != WBC_OK) return rc;
    int pick = -1;
    for (size_t c = 0; c < cands.size(); ++c)
        if (best_ms[c] >= 0.0f && (pick < 0 || best_ms[c] < best_ms[pick])) pick = static_cast<int>(c);
    if (pick >= 0) {
        *best = cands[pick];
        if (best_us_per_sweep) *best_us_per_sweep = best_ms[pick] * 1000.0f / sweeps;
    }
    return WBC_OK;
}

int wbc_sor_linear_solve(const wbc_sor_params* p, int32_t check_every, int32_t max_sweeps, double tolerance,
                         const float* diag, const float* rhs, float* x, wbc_sor_report* report, void* workspace,
                         size_t workspace_bytes, void* stream) {
    if (!p || p->nx < 3 || p->ny < 3 || p->nz < 3 || check_every < 1 || max_sweeps < 1 || !diag || !rhs || !x ||
        !report || !workspace || !(p->omega > 0.0f && p->omega < 2.0f))
        return WBC_ERR_INVALID;
    if (workspace_bytes < sor_workspace_bytes(*p)) return WBC_ERR_WORKSPACE;
    if (reinterpret_cast<uintptr_t>(workspace) % 16 != 0) {
        set_error_msg("wbc_sor_linear_solve: the workspace must be 16-byte aligned");
        return WBC_ERR_INVALID;
    }
    bool feasible = false;
    wbc_sor_params q = *p;
    q.has_source = 0;
    const int rc = sor_solve_resident(q, check_every, max_sweeps, tolerance, nullptr, diag, rhs, nullptr, x, nullptr,
                                      report, workspace, nullptr, as_stream(stream), &feasible, true);
    if (rc == WBC_OK && !feasible) {
        set_error_msg("wbc_sor_linear_solve: the grid does not fit the shared-memory resident solver");
        return WBC_ERR_INVALID;
    }
    return rc;
}

int wbc_sor_wait_selftest(int32_t ctas, int32_t missing, int32_t rounds, void* workspace, size_t workspace_bytes,
                          void* stream) {
    if (ctas < 1 || ctas > kMaxCtas || missing < 0 || missing >= ctas || rounds < 1 || !workspace)
        return WBC_ERR_INVALID;
    if (workspace_bytes < header_bytes() || reinterpret_cast<uintptr_t>(workspace) % 16 != 0) return WBC_ERR_WORKSPACE;
    const DeviceInfo dev = device_info();
    if (ctas > dev.sms) {
        set_error_msg("wbc_sor_wait_selftest: more CTAs than SMs");
        return WBC_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    char* base = static_cast<char*>(workspace);
    SorControl* ctl = reinterpret_cast<SorControl*>(base);
    unsigned int* flags = reinterpret_cast<unsigned int*>(base + sizeof(SorControl));
    cudaError_t err = cudaMemsetAsync(base, 0, header_bytes(), s);
    int launched = ctas - missing;
    void* params[] = {&ctl, &flags, &ctas, &rounds};
    if (err == cudaSuccess)
        err = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_barrier_selftest), dim3(launched), dim3(64),
                                          params, 0, s);
    SorControl host{};
    if (err == cudaSuccess) err = cudaMemcpyAsync(&host, ctl, sizeof(SorControl), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) {
        set_error("wbc_sor_wait_selftest", err);
        return WBC_ERR_CUDA;
    }
    if (host.status != 0) {
        set_error_msg("wbc_sor_wait_selftest: a grid barrier timed out");
        return WBC_ERR_TIMEOUT;
    }
    return WBC_OK;
}

int wbc_sor_solve(const wbc_sor_params* p, int32_t check_every, int32_t max_sweeps, double tolerance,
                  const int32_t* fixed, const float* density, const float* production, const float* source,
                  float* field, float* residual_out, wbc_sor_report* report, void* workspace,
                  size_t workspace_bytes, int32_t path, const wbc_sor_tuning* tuning, void* stream) {
    if (!p || p->nx < 3 || p->ny < 3 || p->nz < 3 || check_every < 1 || max_sweeps < 1 || !density || !field ||
        !report || !workspace || (p->has_source && !source) || path < 0 || path > 2)
        return WBC_ERR_INVALID;
    if (workspace_bytes < sor_workspace_bytes(*p)) return WBC_ERR_WORKSPACE;
    if (reinterpret_cast<uintptr_t>(workspace) % 16 != 0) {
        set_error_msg("wbc_sor_solve: the workspace must be 16-byte aligned");
        return WBC_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    bool feasible = false;
    if (path != 1) {
        int rc = sor_solve_resident(*p, check_every, max_sweeps, tolerance, fixed, density, production, source, field,
                                    residual_out, report, workspace, tuning, s, &feasible);
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
    if (residual_out) {
        cudaError_t err = cudaMemcpyAsync(residual_out, residual_dev, sizeof(float), cudaMemcpyDeviceToDevice, s);
        if (err != cudaSuccess) {
            set_error("wbc_sor_solve: writing the residual", err);
            return WBC_ERR_CUDA;
        }
    }
    report->sweeps = sweeps;
    report->residual = residual;
    report->converged = static_cast<double>(residual) < tolerance ? 1 : 0;
    report->path = 1;
    report->tiles = 0;
    report->strips = 0;
    return WBC_OK;
}

size_t wbc_sor_report_record_bytes(void) { return sizeof(SorReportRecord); }

int wbc_sor_solve_deferred(const wbc_sor_params* p, int32_t check_every, int32_t max_sweeps, double tolerance,
                           const int32_t* fixed, const float* density, const float* production, const float* source,
                           float* field, float* residual_out, void* record, void* workspace, size_t workspace_bytes,
                           int32_t path, const wbc_sor_tuning* tuning, void* stream) {
    if (!p || p->nx < 3 || p->ny < 3 || p->nz < 3 || check_every < 1 || max_sweeps < 1 || !density || !field ||
        !record || !workspace || (p->has_source && !source) || path < 0 || path > 2)
        return WBC_ERR_INVALID;
    if (workspace_bytes < sor_workspace_bytes(*p)) return WBC_ERR_WORKSPACE;
    if (reinterpret_cast<uintptr_t>(workspace) % 16 != 0) {
        set_error_msg("wbc_sor_solve_deferred: the workspace must be 16-byte aligned");
        return WBC_ERR_INVALID;
    }
    SorReportRecord* rec = static_cast<SorReportRecord*>(record);
    cudaStream_t s = as_stream(stream);
    if (path != 1) {
        bool feasible = false;
        wbc_sor_report unused{};
        int rc = sor_solve_resident(*p, check_every, max_sweeps, tolerance, fixed, density, production, source, field,
                                    residual_out, &unused, workspace, tuning, s, &feasible, false, rec);
        if (rc != WBC_OK || feasible) return rc;
    }
    // not resident: the synchronous solve (its report is final at once)
    wbc_sor_report report{};
    int rc = wbc_sor_solve(p, check_every, max_sweeps, tolerance, fixed, density, production, source, field,
                           residual_out, &report, workspace, workspace_bytes, path, tuning, stream);
    if (rc != WBC_OK) return rc;
    rec->ready = 1;
    rec->report = report;
    return WBC_OK;
}

int wbc_sor_report_decode(const void* record, wbc_sor_report* report) {
    if (!record || !report) return WBC_ERR_INVALID;
    const SorReportRecord* rec = static_cast<const SorReportRecord*>(record);
    if (rec->ready) {
        *report = rec->report;
        return WBC_OK;
    }
    if (rec->ctl.status != 0) {
        set_error_msg("wbc_sor_solve_deferred: a device wait timed out");
        return WBC_ERR_TIMEOUT;
    }
    report->sweeps = rec->ctl.sweeps;
    report->residual = rec->ctl.residual;
    report->converged = rec->ctl.converged;
    report->path = rec->path;
    report->tiles = rec->tiles;
    report->strips = rec->strips;
    return WBC_OK;
}

}  // extern "C"
