// Red-black SOR solve to convergence in one persistent, cooperative launch with the field held
// in shared memory (kernels/field_kernels.py:185-243 iterated as fields/diffusion.py:79-123).
//
// Decomposition: the (i, j) plane is cut into tx x ty tiles of ti x tj columns; each CTA (one
// per SM) owns one tile with the full z extent. Shared memory holds the tile plus a halo of all
// columns within L1 distance H of it, split by k parity (E[col][m] = f(k = 2m),
// O[col][m] = f(k = 2m + 1)): within a column all nodes of one colour share a k parity, so a warp
// that owns a column updates its colour with 32 consecutive words per access and no bank
// conflicts, and the k-neighbours of entry m are entries m - 1 + kp and m + kp of the other
// parity (clamped at the ends, which is exactly the reference's mirror rule). At the start each
// CTA writes the uptake coefficients density * uptake_max of its columns, split the same way, to
// an L2-resident scratch copy (a negative value marks the nodes that are never updated:
// Dirichlet faces and pinned nodes).
//
// Temporal blocking: between two halo exchanges a tile performs H colour half-sweeps; the p-th
// updates the columns within distance H - 1 - p of the tile (the ring columns redundantly, with
// the same inputs and the same float expression as their owner, hence the same bits), so each
// half-sweep still reads only values that are current. Columns outside the domain (on a Neumann
// face) are refreshed by copying their mirror column after every half-sweep. After the H
// half-sweeps the columns within H of the tile edge are published to a double-buffered,
// parity-split exchange buffer in L2, the tile waits for its neighbouring tiles' epoch flags
// (release / acquire; 4 neighbours for H = 1, 8 for H > 1), and pulls its halo. Every
// `check_every` sweeps the max-norm residual is reduced (warp shuffles, one atomicMax per CTA,
// the only global barrier) and all CTAs stop together once it is below the tolerance: the
// reference's sweep count, residual and stopping rule, with no host round trip. The field after
// n sweeps is bit-identical to the oracle's and to the streaming kernels'.
//
// Every wait is bounded in time (kWaitLimitNs of the GPU's global timer, 2 s); on timeout the CTA
// raises an abort flag, every CTA leaves, and the host gets WBC_ERR_TIMEOUT.
#include <algorithm>
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
    int pad[25];
};
static_assert(sizeof(SorControl) == 128, "SorControl is one 128-byte line");
constexpr int kMaxCtas = 1024;  // barrier flags that follow the control block

struct SorTiling {
    int tx, ty;  // CTAs along i and j
    int ti, tj;  // tile extent (columns) along i and j
    int M;       // column stride per parity: (nz + 1) / 2 entries rounded up to 4 (16-byte rows)
    int lanes;   // 32-entry chunks per parity column
    int threads;
    int H;       // halo depth = half-sweeps between exchanges
    int nbox;    // columns of the bounding box (ti + 2H) * (tj + 2H)
    size_t planes_bytes;
    size_t table_offset;  // byte offset of the column table (2 int4 per box column)
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
    float* xchg;   // [2 buffers][2 parities][nx][ny][M] halo exchange
    float* coeff;  // [2][nx][ny][M] density * uptake_max, -1 where not updated
    SorControl* ctl;
    unsigned int* flags;  // [tiles] barrier epochs
    int check_every;
    int max_sweeps;
    double tolerance;  // compared in double, as the reference compares float(residual) < tolerance
    float* pcopy;      // [2][nx][ny][M] production term of every updated node (production, source)
};

// Every device wait gives up after kWaitLimitNs nanoseconds of the GPU's global timer without
// progress. The timer is read every 256 polls, so a wait ends within a few microseconds of the limit.
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s
constexpr int kMaxLanesPerColumn = 8;         // M <= 256 (nz <= 511)

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

// ---- halo exchange with tagged words (H = 1) ------------------------------------------------------------
// Each exchanged entry is one 64-bit word {value bits, tag} written with a single relaxed store, so a
// reader that sees the tag of the half-sweep it needs also sees that half-sweep's value: no flag,
// fence or barrier between neighbouring tiles. The buffer has the layout of the coefficient copy
// ([parity][nx][ny][M]) in 8-byte words.
__device__ __forceinline__ void store_tagged(unsigned long long* p, float v, unsigned int tag) {
    const unsigned long long word = (static_cast<unsigned long long>(tag) << 32) | __float_as_uint(v);
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(word) : "memory");
}

__device__ __forceinline__ unsigned long long load_tagged(const unsigned long long* p) {
    unsigned long long word;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(word) : "l"(p) : "memory");
    return word;
}

__device__ __forceinline__ int mirror(int i, int n) { return i < 0 ? 1 : (i > n - 1 ? n - 2 : i); }

// Signals this CTA's arrival at the next epoch, then waits for the CTAs listed in `wait_for`
// (n_wait of them) or, with n_wait < 0, for every CTA. Returns false when aborted (timeout here or
// elsewhere). A halo exchange only needs the neighbouring tiles; the residual needs all.
// `me` is this CTA's tile among the `ntiles` tiles of its solve.
__device__ __forceinline__ bool grid_barrier(SorControl* ctl, unsigned int* flags, unsigned int& epoch, int me,
                                             int ntiles, const int* wait_for = nullptr, int n_wait = -1,
                                             const unsigned int* claims = nullptr, unsigned int claims_needed = 0) {
    epoch += 1;
    __syncthreads();  // the CTA's writes happen before thread 0's release (bar.sync is cumulative)
    if (threadIdx.x == 0) store_release(flags + me, epoch);
    int aborted = 0;
    const unsigned n = n_wait < 0 ? static_cast<unsigned>(ntiles) : static_cast<unsigned>(n_wait);
    for (unsigned t = threadIdx.x; t < n; t += blockDim.x) {
        const unsigned who = n_wait < 0 ? t : static_cast<unsigned>(wait_for[t]);
        unsigned polls = 0;
        WaitClock clock{0ull, claims, claims_needed};
        while (static_cast<int>(load_acquire(flags + who) - epoch) < 0) {
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

// Column lists in shared memory, after the two parity planes. A column is an int2:
// x = index in the bounding box, y = (gi << 16) | gj with gi, gj its (mirrored) global position.
struct Lists {
    int2* upd;       // in-domain columns within distance H - 1, by distance (owned first)
    int* upd_end;    // upd_end[d]: columns within distance d (d = 0 .. H - 1)
    int2* pull;      // in-domain columns at distance 1 .. H
    int2* publish;   // owned columns within H of the tile edge
    int2* inner;     // owned columns farther than H from the tile edge
    int2* mir;       // outside the domain: x = box index, y = box index of the mirror column
    int n_pull, n_publish, n_inner, n_mir;
};

// Loop invariants of a colour half-sweep.
struct Sweep {
    float* s;
    const int4* tab;
    const float* coeff;
    float* xchg;  // exchange buffer, laid out like the coefficient scratch copy
    int ncm, M, si, nx, ny, nz, cnt_even, cnt_odd;
    int64_t sx;
    float K, h, omega, one_minus_omega;
    bool zclamp;  // Neumann z faces: the k-neighbours of the end nodes are mirrored
    bool fast;    // K, h and every coefficient of this tile pass the fixed range tests below
};

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

// Per (box column, colour) entry of the column table in shared memory:
// x = offset of entry 0 of the parity the colour updates, y = the same for the other parity,
// z = offset of the column's coefficient row (that parity) in the scratch copy,
// w = kp | cnt << 1 | last << 11 (kp: the parity updated, cnt: its entries, last: the other
// parity's last entry).
__device__ __forceinline__ int4 column_entry(const Sweep& w, int box, int gi, int gj, int colour) {
    const int kp = (colour + gi + gj) & 1;
    const int cnt = kp ? w.cnt_odd : w.cnt_even;
    const int last = (kp ? w.cnt_even : w.cnt_odd) - 1;
    return make_int4(kp * w.ncm + box * w.M, (kp ^ 1) * w.ncm + box * w.M, ((kp * w.nx + gi) * w.ny + gj) * w.M,
                     kp | (cnt << 1) | (last << 11));
}

template <int LANES>
__device__ __forceinline__ void load_column(const Sweep& w, const int2* list, int q, int colour, int lane, int2& c,
                                            int4& e, float (&du)[LANES]) {
    c = list[q];
    e = w.tab[2 * c.x + colour];
    const int cnt = (e.w >> 1) & 1023;
    const float* crow = w.coeff + e.z + lane;
#pragma unroll
    for (int r = 0; r < LANES; ++r) du[r] = lane + 32 * r < cnt ? crow[32 * r] : -1.0f;
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

// Entries m = lane + 32 r of one parity column: `po` points at entry `lane`, the four lateral
// neighbours are po -+ si (i) and po -+ M (j). The k-neighbours of entry m are entries m + kp - 1
// and m + kp of the other parity: with Dirichlet z faces every updated node has both inside the
// column (pv points at entry lane + kp - 1), with Neumann z faces they are clamped to the column
// ends (the mirror rule k = -1 -> 1, k = nz -> nz - 2). Every lane computes; only nodes with a
// coefficient (not a Dirichlet face, a pinned node or past the column end) are written, and the
// IEEE division replaces the fast one only where the range tests above do not hold.
template <bool HAS_PROD, bool ZCLAMP, int LANES>
__device__ __forceinline__ void relax_nodes(const SorArgs& a, const Sweep& w, float* po, const float* pv, int lane,
                                            int kp, int last, const float* prow, unsigned long long* xrow, int cnt,
                                            unsigned int tag, const float (&du)[LANES]) {
    const float* pim = po - w.si;
    const float* pip = po + w.si;
    const float* pjm = po - w.M;
    const float* pjp = po + w.M;
#pragma unroll
    for (int r = 0; r < LANES; ++r) {
        const int off = 32 * r;
        const bool active = du[r] >= 0.0f;
        const float o = po[off];
        const float b1 = w.K + o;
        float cc = div_rn_fast_nonneg_zero(du[r], b1);
        float prod = 0.0f;
        if (HAS_PROD) {
            if (active) prod = prow[off];
        }
        float vlo, vhi;
        if (ZCLAMP) {
            const int m = lane + off;
            vlo = pv[max(m + kp - 1, 0)];
            vhi = pv[min(m + kp, last)];
        } else {
            vlo = pv[off];
            vhi = pv[off + 1];
        }
        const float nb = pim[off] + pip[off] + pjm[off] + pjp[off] + vlo + vhi;
        // Without production h * 0 = +0 and nb + 0 = nb except for nb = -0, which the range test
        // sends to the exact branch below.
        float a2 = HAS_PROD ? nb + w.h * prod : nb;
        float b2 = 6.0f + w.h * cc;
        float gs = div_rn_fast_nonneg_zero(a2, b2);
        if (active && !(w.fast && old_value_in_range(o) && numerator_in_range(a2))) gs = gs_exact(du[r], b1, nb, prod, w.h);
        const float v = fmaxf(w.one_minus_omega * o + w.omega * gs, 0.0f);
        if (active) po[off] = v;
        // An edge column publishes every entry (unchanged ones too) with this half-sweep's tag.
        if (xrow && lane + off < cnt) store_tagged(xrow + off, active ? v : o, tag);
    }
}

// One colour of one column: the reference's update (field_kernels.py:185-212) with the
// Michaelis-Menten uptake linearised at the old value, over-relaxed and clamped at zero.
template <bool HAS_PROD, int LANES>
__device__ __forceinline__ void relax_column(const SorArgs& a, const Sweep& w, int2 c, int4 e, int lane,
                                             unsigned int tag, const float (&du)[LANES]) {
    const int kp = e.w & 1;
    const int last = e.w >> 11;
    float* po = w.s + e.x + lane;
    const float* oth = w.s + e.y;
    const float* prow = HAS_PROD ? a.pcopy + e.z + lane : nullptr;
    unsigned long long* xrow = tag ? reinterpret_cast<unsigned long long*>(w.xchg) + e.z + lane : nullptr;
    const int cnt = (e.w >> 1) & 1023;
    if (w.zclamp)
        relax_nodes<HAS_PROD, true, LANES>(a, w, po, oth, lane, kp, last, prow, xrow, cnt, tag, du);
    else
        relax_nodes<HAS_PROD, false, LANES>(a, w, po, oth + kp - 1 + lane, lane, kp, last, prow, xrow, cnt, tag,
                                            du);
}

// The columns list[0 .. end) for one colour, a warp per column; the next column's table entry and
// coefficients are loaded before the current column is relaxed. A nonzero `tag` also publishes
// the columns to the exchange buffer.
template <bool HAS_PROD, int LANES>
__device__ __forceinline__ void relax_columns(const SorArgs& a, const Sweep& w, const int2* list, int end, int colour,
                                              int warp, int nwarps, int lane, unsigned int tag = 0u) {
    int q = warp;
    if (q >= end) return;
    int2 c;
    int4 e;
    float du[LANES];
    load_column<LANES>(w, list, q, colour, lane, c, e, du);
    while (true) {
        const int qn = q + nwarps;
        const bool more = qn < end;
        int2 cn = c;
        int4 en = e;
        float dn[LANES];
        if (more) load_column<LANES>(w, list, qn, colour, lane, cn, en, dn);
        relax_column<HAS_PROD, LANES>(a, w, c, e, lane, tag, du);
        if (!more) break;
        c = cn;
        e = en;
#pragma unroll
        for (int r = 0; r < LANES; ++r) du[r] = dn[r];
        q = qn;
    }
}

// Max-norm residual |r| / max(6 u, reference) of the nodes relax_nodes would update, with
// r = nb + h prod - (6 + h c) u (field_kernels.py:215-243), as float bits (all values are >= 0).
template <bool HAS_PROD, bool ZCLAMP, int LANES>
__device__ __forceinline__ unsigned int residual_nodes(const SorArgs& a, const Sweep& w, const float* po,
                                                       const float* pv, int lane, int kp, int last, const float* prow,
                                                       const float (&du)[LANES]) {
    const float* pim = po - w.si;
    const float* pip = po + w.si;
    const float* pjm = po - w.M;
    const float* pjp = po + w.M;
    unsigned int bits = 0u;
#pragma unroll
    for (int r = 0; r < LANES; ++r) {
        const int off = 32 * r;
        const bool active = du[r] >= 0.0f;
        const float o = po[off];
        const float b1 = w.K + o;
        float cc = div_rn_fast(du[r], b1);
        float prod = 0.0f;
        if (HAS_PROD) {
            if (active) prod = prow[off];
        }
        float vlo, vhi;
        if (ZCLAMP) {
            const int m = lane + off;
            vlo = pv[max(m + kp - 1, 0)];
            vhi = pv[min(m + kp, last)];
        } else {
            vlo = pv[off];
            vhi = pv[off + 1];
        }
        const float nb = pim[off] + pip[off] + pjm[off] + pjp[off] + vlo + vhi;
        float res = nb + w.h * prod - (6.0f + w.h * cc) * o;
        const float den = fmaxf(6.0f * o, a.p.reference);
        float val = div_rn_fast(fabsf(res), den);
        if (active && !(div_fast_range(du[r], b1) && div_fast_range(fabsf(res), den)))
            val = residual_exact(du[r], b1, nb, prod, w.h, o, den);
        if (active) bits = max(bits, __float_as_uint(val));
    }
    return bits;
}

// Residual bits of one column's `colour` nodes.
template <bool HAS_PROD, int LANES>
__device__ __forceinline__ unsigned int residual_column(const SorArgs& a, const Sweep& w, const int2* list, int q,
                                                        int colour, int lane) {
    int2 c;
    int4 e;
    float du[LANES];
    load_column<LANES>(w, list, q, colour, lane, c, e, du);
    const int kp = e.w & 1;
    const int last = e.w >> 11;
    const float* po = w.s + e.x + lane;
    const float* oth = w.s + e.y;
    const float* prow = HAS_PROD ? a.pcopy + e.z + lane : nullptr;
    if (w.zclamp) return residual_nodes<HAS_PROD, true, LANES>(a, w, po, oth, lane, kp, last, prow, du);
    return residual_nodes<HAS_PROD, false, LANES>(a, w, po, oth + kp - 1 + lane, lane, kp, last, prow, du);
}

// Reads the parity `colour` updated in each listed halo column once every entry carries `tag`
// (two columns per warp at a time, all of their words in flight before any is checked) and stores
// the values in shared memory. Returns false when a wait timed out or another CTA aborted.
template <int LANES>
__device__ __forceinline__ bool pull_tagged(const Sweep& w, const int2* list, int n, int colour, unsigned int tag,
                                            const SorControl* ctl, int warp, int nwarps, int lane) {
    const unsigned long long* ll = reinterpret_cast<const unsigned long long*>(w.xchg);
    bool fine = true;
    for (int q0 = warp; q0 < n; q0 += 2 * nwarps) {
        const unsigned long long* src[2];
        float* dst[2];
        int cnt[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int q = q0 + u * nwarps;
            cnt[u] = 0;
            src[u] = nullptr;
            dst[u] = nullptr;
            if (q < n) {
                const int2 c = list[q];
                const int gi = c.y >> 16, gj = c.y & 0xffff;
                const int par = (colour + gi + gj) & 1;
                cnt[u] = par ? w.cnt_odd : w.cnt_even;
                src[u] = ll + ((static_cast<int64_t>(par) * w.nx + gi) * w.ny + gj) * w.M + lane;
                dst[u] = w.s + par * w.ncm + c.x * w.M + lane;
            }
        }
        unsigned long long v[2][LANES];
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int r = 0; r < LANES; ++r)
                if (lane + 32 * r < cnt[u]) v[u][r] = load_tagged(src[u] + 32 * r);
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int r = 0; r < LANES; ++r)
                if (lane + 32 * r < cnt[u]) {
                    unsigned polls = 0;
                    WaitClock clock;
                    while (static_cast<unsigned int>(v[u][r] >> 32) != tag) {
                        if ((++polls & 255u) == 0u && (load_acquire(&ctl->abort) != 0u || clock.expired())) {
                            fine = false;
                            break;
                        }
                        v[u][r] = load_tagged(src[u] + 32 * r);
                    }
                    dst[u][32 * r] = __uint_as_float(static_cast<unsigned int>(v[u][r]));
                }
    }
    return fine;
}

// Copies one parity (the one colour `colour` updates in each column) or both parities of the
// listed columns between the exchange buffer and shared memory. A warp moves two column parities
// at a time and loads all of their entries before storing any, so two whole columns are in flight.
template <int LANES>
__device__ __forceinline__ void copy_columns(const Sweep& w, const int2* list, int n, float* xb, int colour,
                                             bool both, bool to_xchg, int warp, int nwarps, int lane) {
    const int per = both ? 2 : 1;
    const int items = n * per;
    for (int t0 = warp; t0 < items; t0 += 2 * nwarps) {
        float* src[2];
        float* dst[2];
        int cnt[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int t = t0 + u * nwarps;
            cnt[u] = 0;
            src[u] = dst[u] = nullptr;
            if (t < items) {
                const int2 c = list[both ? (t >> 1) : t];
                const int gi = c.y >> 16, gj = c.y & 0xffff;
                const int par = both ? (t & 1) : ((colour + gi + gj) & 1);
                cnt[u] = par ? w.cnt_odd : w.cnt_even;
                float* x = xb + ((static_cast<int64_t>(par) * w.nx + gi) * w.ny + gj) * w.M + lane;
                float* sm = w.s + par * w.ncm + c.x * w.M + lane;
                src[u] = to_xchg ? sm : x;
                dst[u] = to_xchg ? x : sm;
            }
        }
        float v[2][LANES];
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int r = 0; r < LANES; ++r)
                if (lane + 32 * r < cnt[u]) v[u][r] = to_xchg ? src[u][32 * r] : __ldcg(src[u] + 32 * r);
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int r = 0; r < LANES; ++r)
                if (lane + 32 * r < cnt[u]) {
                    if (to_xchg)
                        __stcg(dst[u] + 32 * r, v[u][r]);
                    else
                        dst[u][32 * r] = v[u][r];
                }
    }
}

// Refreshes the outside-the-domain columns from their mirror images: the parity that colour
// `colour` updates in the mirror column, or both.
__device__ __forceinline__ void mirror_columns(const Sweep& w, const int2* list, int n, int bw, int gi0, int gj0,
                                               int colour, bool both, int warp, int nwarps, int lane) {
    for (int q = warp; q < n; q += nwarps) {
        const int2 c = list[q];
        const int mi = c.y / bw, mj = c.y - (c.y / bw) * bw;
        const int kp_colour = (colour + gi0 + mi + gj0 + mj) & 1;
        for (int par = 0; par < 2; ++par) {
            if (!both && par != kp_colour) continue;
            const int cnt = par ? w.cnt_odd : w.cnt_even;
            float* dst = w.s + par * w.ncm + c.x * w.M;
            const float* src = w.s + par * w.ncm + c.y * w.M;
            for (int m = lane; m < cnt; m += 32) dst[m] = src[m];
        }
    }
}

// Columns longer than 3 x 32 entries per parity run 16 warps per CTA (128 registers a thread).
constexpr int max_threads_for_lanes(int lanes) { return lanes > 3 ? 512 : 1024; }

// One tile (`tile` of `ntiles`) of one solve, for the whole solve.
// `claims` / `claims_needed`: see WaitClock (batched solves; null for a single solve).
template <bool HAS_PROD, int LANES, int H>
__device__ __forceinline__ void sor_tile(const SorArgs& a, int tile, int ntiles, const unsigned int* claims = nullptr,
                                         unsigned int claims_needed = 0) {
    extern __shared__ __align__(128) float s[];
    __shared__ unsigned int s_red[32];
    __shared__ int s_counts[8 + 4];  // per distance class, then pull / publish / inner / mirror counters
    const int M = a.t.M, nz = a.p.nz, nx = a.p.nx, ny = a.p.ny;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int bx = tile / a.t.ty;
    const int by = tile - bx * a.t.ty;
    const int i0 = bx * a.t.ti, j0 = by * a.t.tj;
    const int ai = min(a.t.ti, nx - i0), aj = min(a.t.tj, ny - j0);
    const int bw = a.t.tj + 2 * H;  // bounding-box row length
    const int nbox = a.t.nbox;
    Sweep w;
    w.s = s;
    w.coeff = a.coeff;
    w.M = M;
    w.ncm = nbox * M;  // floats per parity plane
    w.si = bw * M;
    w.nx = nx;
    w.ny = ny;
    w.nz = nz;
    w.cnt_even = (nz + 1) / 2;
    w.cnt_odd = nz / 2;
    w.sx = static_cast<int64_t>(ny) * nz;
    w.K = a.p.michaelis_k;
    w.h = a.p.dx2_over_D;
    w.omega = a.p.omega;
    w.one_minus_omega = 1.0f - a.p.omega;
    w.zclamp = a.p.bc_z != 0;
    w.tab = reinterpret_cast<const int4*>(reinterpret_cast<char*>(s) + a.t.table_offset);
    w.xchg = a.xchg;
    __shared__ int s_neighbours[8];
    __shared__ int s_n_neighbours;
    if (threadIdx.x == 0) {
        int n = 0;
        for (int di = -1; di <= 1; ++di)
            for (int dj = -1; dj <= 1; ++dj) {
                if ((di == 0 && dj == 0) || (H == 1 && di != 0 && dj != 0)) continue;
                const int nbx = bx + di, nby = by + dj;
                if (nbx >= 0 && nbx < a.t.tx && nby >= 0 && nby < a.t.ty) s_neighbours[n++] = nbx * a.t.ty + nby;
            }
        s_n_neighbours = n;
    }

    // ---- column lists ---------------------------------------------------------------------------------
    Lists L;
    {
        int2* base = reinterpret_cast<int2*>(reinterpret_cast<char*>(s) + a.t.planes_bytes);
        L.upd = base;
        L.pull = base + nbox;
        L.publish = base + 2 * nbox;
        L.inner = base + 3 * nbox;
        L.mir = base + 4 * nbox;
        L.upd_end = reinterpret_cast<int*>(base + 5 * nbox);
    }
    __shared__ int s_outside_range;
    if (threadIdx.x < 12) s_counts[threadIdx.x] = 0;
    if (threadIdx.x == 0) s_outside_range = solve_constants_in_range(w.K, w.h) ? 0 : 1;
    __syncthreads();
    const int box_rows = ai + 2 * H, box_cols = aj + 2 * H;
    auto dist_of = [&](int li, int lj) {
        const int di = li < 0 ? -li : (li >= ai ? li - ai + 1 : 0);
        const int dj = lj < 0 ? -lj : (lj >= aj ? lj - aj + 1 : 0);
        return di + dj;
    };
    // pass 1: count in-domain columns per distance class
    for (int e = threadIdx.x; e < box_rows * box_cols; e += blockDim.x) {
        const int li = e / box_cols - H, lj = e - (e / box_cols) * box_cols - H;
        const int d = dist_of(li, lj);
        const int gi = i0 + li, gj = j0 + lj;
        if (d < H && gi >= 0 && gi < nx && gj >= 0 && gj < ny) atomicAdd(&s_counts[d], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int d = 0; d < H; ++d) {
            const int c = s_counts[d];
            s_counts[d] = run;  // start of class d
            run += c;
            L.upd_end[d] = run;
        }
    }
    __syncthreads();
    // pass 2: fill the lists
    for (int e = threadIdx.x; e < box_rows * box_cols; e += blockDim.x) {
        const int li = e / box_cols - H, lj = e - (e / box_cols) * box_cols - H;
        const int d = dist_of(li, lj);
        if (d > H) continue;
        const int gi = i0 + li, gj = j0 + lj;
        const int box = (li + H) * bw + (lj + H);
        const bool inside = gi >= 0 && gi < nx && gj >= 0 && gj < ny;
        if (inside) {
            const int2 c = make_int2(box, (gi << 16) | gj);
            if (d < H) {
                L.upd[atomicAdd(&s_counts[d], 1)] = c;
                int4* tab = const_cast<int4*>(w.tab);
                tab[2 * box] = column_entry(w, box, gi, gj, 0);
                tab[2 * box + 1] = column_entry(w, box, gi, gj, 1);
            }
            if (d >= 1) L.pull[atomicAdd(&s_counts[8], 1)] = c;
            if (d == 0) {
                if (li < H || li >= ai - H || lj < H || lj >= aj - H)
                    L.publish[atomicAdd(&s_counts[9], 1)] = c;
                else
                    L.inner[atomicAdd(&s_counts[10], 1)] = c;
            }
        } else {
            // Only the columns just outside a Neumann face are read (by the face column, which is
            // updated); across a Dirichlet face, at a corner or farther out nothing reads them.
            const bool out_i = gi < 0 || gi >= nx, out_j = gj < 0 || gj >= ny;
            const bool read = out_i != out_j && (out_i ? (a.p.bc_x != 0 && (gi == -1 || gi == nx))
                                                       : (a.p.bc_y != 0 && (gj == -1 || gj == ny)));
            if (read) {
                const int mi = mirror(gi, nx) - i0 + H, mj = mirror(gj, ny) - j0 + H;
                L.mir[atomicAdd(&s_counts[11], 1)] = make_int2(box, mi * bw + mj);
            }
        }
    }
    __syncthreads();
    L.n_pull = s_counts[8];
    L.n_publish = s_counts[9];
    L.n_inner = s_counts[10];
    L.n_mir = s_counts[11];
    const int n_neighbours = s_n_neighbours;
    const int gi0 = i0 - H, gj0 = j0 - H;  // global position of box row / column 0

    // ---- tile + halo into shared memory; owned coefficients into the scratch copy -------------------
    for (int e = warp; e < box_rows * box_cols; e += nwarps) {
        const int li = e / box_cols - H, lj = e - (e / box_cols) * box_cols - H;
        if (dist_of(li, lj) > H) continue;
        const int gi = mirror(i0 + li, nx), gj = mirror(j0 + lj, ny);
        const int box = (li + H) * bw + (lj + H);
        const bool owned = li >= 0 && li < ai && lj >= 0 && lj < aj;
        const int64_t base = gi * w.sx + static_cast<int64_t>(gj) * nz;
        for (int k = lane; k < nz; k += 32) {
            const int64_t idx = base + k;
            s[(k & 1) * w.ncm + box * M + (k >> 1)] = a.field[idx];
            if (owned) {
                const wbc_sor_params& p = a.p;
                const bool face = (p.bc_x == 0 && (gi == 0 || gi == nx - 1)) ||
                                  (p.bc_y == 0 && (gj == 0 || gj == ny - 1)) ||
                                  (p.bc_z == 0 && (k == 0 || k == nz - 1));
                float v = -1.0f;
                if (!face && !(a.fixed && a.fixed[idx] != 0)) v = a.density[idx] * p.uptake_max;
                const int64_t at = ((static_cast<int64_t>(k & 1) * nx + gi) * ny + gj) * M + (k >> 1);
                a.coeff[at] = v;
                // The production term is fixed for the solve: computed once here (only where a node
                // is updated, as the update itself would) instead of in every sweep.
                if (HAS_PROD) a.pcopy[at] = v >= 0.0f ? prod_term(a, idx) : 0.0f;
                if (!coefficient_in_range(v, w.K, w.h)) s_outside_range = 1;
            }
        }
    }
    unsigned int epoch = 0;
    if (H == 1) {
        // The edge rows start with tag 0 (half-sweeps are tagged from 1), so words a previous solve
        // left in the buffer are never taken for this solve's.
        __syncthreads();
        unsigned long long* ll = reinterpret_cast<unsigned long long*>(a.xchg);
        for (int q = warp; q < L.n_publish; q += nwarps) {
            const int2 c = L.publish[q];
            const int gi = c.y >> 16, gj = c.y & 0xffff;
            for (int par = 0; par < 2; ++par) {
                const int cnt = par ? w.cnt_odd : w.cnt_even;
                for (int m = lane; m < cnt; m += 32)
                    store_tagged(ll + ((static_cast<int64_t>(par) * nx + gi) * ny + gj) * M + m,
                                 s[par * w.ncm + c.x * M + m], 0u);
            }
        }
    }
    // The ring columns' coefficients (and edge rows) are written by their owners: one global
    // barrier first.
    bool ok = grid_barrier(a.ctl, a.flags, epoch, tile, ntiles, nullptr, -1, claims, claims_needed);
    w.fast = s_outside_range == 0;  // read after the barrier's __syncthreads

    int sweeps = 0;
    float residual = __int_as_float(0x7f800000);
    bool converged = false;
    int chunk_index = 0;
    unsigned int interval = 0;
    while (ok && sweeps < a.max_sweeps) {
        const int chunk = min(a.check_every, a.max_sweeps - sweeps);
        int half_left = 2 * chunk;
        int colour = 0;
        while (ok && half_left > 0) {
            if constexpr (H == 1) {
                // Edge columns first, each new value also stored to the exchange buffer tagged
                // with this half-sweep; then the inner columns; then the halo is read from the
                // neighbours' tagged words. A neighbour rewrites a word two half-sweeps later, which
                // needs this tile's words of the half-sweep in between, written after this pull.
                const unsigned int tag = static_cast<unsigned int>(2 * sweeps + (2 * chunk - half_left) + 1);
                relax_columns<HAS_PROD, LANES>(a, w, L.publish, L.n_publish, colour, warp, nwarps, lane, tag);
                relax_columns<HAS_PROD, LANES>(a, w, L.inner, L.n_inner, colour, warp, nwarps, lane);
                const bool fine = pull_tagged<LANES>(w, L.pull, L.n_pull, colour, tag, a.ctl, warp, nwarps, lane);
                if (__syncthreads_or(!fine)) {
                    if (threadIdx.x == 0) atomicExch(&a.ctl->abort, 1u);
                    ok = false;
                    break;
                }
                if (L.n_mir > 0) {
                    mirror_columns(w, L.mir, L.n_mir, bw, gi0, gj0, colour, false, warp, nwarps, lane);
                    __syncthreads();
                }
                colour ^= 1;
                half_left -= 1;
            } else {
                // H half-sweeps over shrinking regions (the halo columns relaxed redundantly), then
                // one exchange of both parities through a double buffer.
                const int nph = min(H, half_left);
                for (int ph = 0; ph < nph; ++ph) {
                    relax_columns<HAS_PROD, LANES>(a, w, L.upd, L.upd_end[nph - 1 - ph], colour, warp, nwarps, lane);
                    __syncthreads();
                    if (L.n_mir > 0) {
                        mirror_columns(w, L.mir, L.n_mir, bw, gi0, gj0, colour, false, warp, nwarps, lane);
                        __syncthreads();
                    }
                    colour ^= 1;
                }
                half_left -= nph;
                float* xb = a.xchg + static_cast<int64_t>(interval & 1u) * 2 * nx * ny * M;
                copy_columns<LANES>(w, L.publish, L.n_publish, xb, 0, true, true, warp, nwarps, lane);
                // A neighbour overwrites this buffer two exchanges later, i.e. only after this tile
                // has signalled the next epoch, which comes after the pull below.
                ok = grid_barrier(a.ctl, a.flags, epoch, tile, ntiles, s_neighbours, n_neighbours, claims,
                                  claims_needed);
                if (!ok) break;
                copy_columns<LANES>(w, L.pull, L.n_pull, xb, 0, true, false, warp, nwarps, lane);
                __syncthreads();
                if (L.n_mir > 0) {
                    mirror_columns(w, L.mir, L.n_mir, bw, gi0, gj0, 0, true, warp, nwarps, lane);
                    __syncthreads();
                }
                ++interval;
            }
        }
        if (!ok) break;
        sweeps += chunk;
        __syncthreads();  // the halo warp may be ahead of the relaxing warps
        // Max-norm residual of the current field over every updated node (both colours).
        unsigned int bits = 0u;
        const int n_owned = L.upd_end[0];
        for (int q = warp; q < n_owned; q += nwarps) {
            bits = max(bits, residual_column<HAS_PROD, LANES>(a, w, L.upd, q, 0, lane));
            bits = max(bits, residual_column<HAS_PROD, LANES>(a, w, L.upd, q, 1, lane));
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
        ok = grid_barrier(a.ctl, a.flags, epoch, tile, ntiles, nullptr, -1, claims, claims_needed);
        if (!ok) break;
        residual = __uint_as_float(load_acquire(&a.ctl->res_bits[slot]));
        // The next chunk's slot was last read before this chunk's first barrier: safe to clear.
        if (tile == 0 && threadIdx.x == 0) atomicExch(&a.ctl->res_bits[slot ^ 1], 0u);
        ++chunk_index;
        if (static_cast<double>(residual) < a.tolerance) {
            converged = true;
            break;
        }
    }
    if (!ok) {
        if (tile == 0 && threadIdx.x == 0) a.ctl->status = 1;
        return;
    }
    // Owned columns back to the field.
    const int n_owned = L.upd_end[0];
    for (int q = warp; q < n_owned; q += nwarps) {
        const int2 c = L.upd[q];
        const int gi = c.y >> 16, gj = c.y & 0xffff;
        float* out = a.field + gi * w.sx + static_cast<int64_t>(gj) * nz;
        for (int k = lane; k < nz; k += 32) out[k] = s[(k & 1) * w.ncm + c.x * M + (k >> 1)];
    }
    if (tile == 0 && threadIdx.x == 0) {
        a.ctl->sweeps = sweeps;
        a.ctl->residual = residual;
        a.ctl->converged = converged ? 1 : 0;
        a.ctl->status = 0;
    }
}

template <bool HAS_PROD, int LANES, int H>
__global__ void __launch_bounds__(max_threads_for_lanes(LANES), 1) k_sor_resident(SorArgs a) {
    sor_tile<HAS_PROD, LANES, H>(a, static_cast<int>(blockIdx.x), static_cast<int>(gridDim.x));
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

template <bool HAS_PROD, int LANES>
__global__ void __launch_bounds__(max_threads_for_lanes(LANES), 1)
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
        sor_tile<HAS_PROD, LANES, 1>(args[b], t - tile_first[b], tile_first[b + 1] - tile_first[b], next_tile,
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

template <bool P, int Hd>
static KernelFn kernel_for_lanes(int lanes) {
    switch (lanes) {
        case 1: return k_sor_resident<P, 1, Hd>;
        case 2: return k_sor_resident<P, 2, Hd>;
        case 3: return k_sor_resident<P, 3, Hd>;
        case 4: return k_sor_resident<P, 4, Hd>;
        case 5: return k_sor_resident<P, 5, Hd>;
        case 6: return k_sor_resident<P, 6, Hd>;
        case 7: return k_sor_resident<P, 7, Hd>;
        default: return k_sor_resident<P, 8, Hd>;
    }
}

static KernelFn kernel_for(bool has_prod, int lanes, int H) {
    if (has_prod) {
        if (H == 1) return kernel_for_lanes<true, 1>(lanes);
        if (H == 2) return kernel_for_lanes<true, 2>(lanes);
        return kernel_for_lanes<true, 4>(lanes);
    }
    if (H == 1) return kernel_for_lanes<false, 1>(lanes);
    if (H == 2) return kernel_for_lanes<false, 2>(lanes);
    return kernel_for_lanes<false, 4>(lanes);
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

static bool tiling_for(const wbc_sor_params& p, int tx, int ty, int H, size_t smem_limit, SorTiling* out) {
    const int entries = (p.nz + 1) / 2;
    const int M = (entries + 3) & ~3;
    const int lanes = (entries + 31) / 32;
    const int ti = (p.nx + tx - 1) / tx, tj = (p.ny + ty - 1) / ty;
    if (ti < H || tj < H || ti < 2 || tj < 2) return false;
    const int ex = (p.nx + ti - 1) / ti, ey = (p.ny + tj - 1) / tj;
    const int nbox = (ti + 2 * H) * (tj + 2 * H);
    const size_t planes = ((2ull * nbox * M * sizeof(float)) + 15) & ~15ull;
    const size_t lists = 5ull * nbox * sizeof(int2) + 16 * sizeof(int);
    const size_t table = (planes + lists + 15) & ~15ull;
    const size_t smem = table + 2ull * nbox * sizeof(int4);
    if (smem > smem_limit) return false;
    if (2ll * p.nx * p.ny * M >= (1ll << 31)) return false;  // coefficient offsets are 32-bit
    const int warps = std::min(max_threads_for_lanes(lanes) / 32, std::max(1, ti * tj));
    *out = SorTiling{ex, ey, ti, tj, M, lanes, 32 * warps, H, nbox, planes, table, smem};
    return true;
}

// tx x ty tiles, at most one CTA per SM (and within the barrier flags), minimising the columns of
// the largest tile, then the halo perimeter.
static bool choose_tiling(const wbc_sor_params& p, int sms, size_t smem_limit, int H, int want_tx, int want_ty,
                          SorTiling* out) {
    const int entries = (p.nz + 1) / 2;
    if (entries > 32 * kMaxLanesPerColumn || p.nx > 32767 || p.ny > 32767) return false;
    const int max_ctas = std::min(sms, kMaxCtas);
    if (want_tx > 0 && want_ty > 0) return want_tx * want_ty <= max_ctas && tiling_for(p, want_tx, want_ty, H, smem_limit, out);
    bool found = false;
    long best_score = 0;
    for (int tx = 1; tx <= std::min(p.nx, max_ctas); ++tx) {
        const int ty_max = std::min(p.ny, max_ctas / tx);
        for (int ty = 1; ty <= ty_max; ++ty) {
            SorTiling t{};
            if (!tiling_for(p, tx, ty, H, smem_limit, &t)) continue;
            const long score = static_cast<long>(t.ti) * t.tj * 1000 + (t.ti + t.tj);
            if (!found || score < best_score) {
                found = true;
                best_score = score;
                *out = t;
            }
        }
    }
    return found;
}

static size_t plane_bytes(const wbc_sor_params& p) {
    return 2ull * p.nx * p.ny * ((((p.nz + 1) / 2) + 3) & ~3) * sizeof(float);
}

static size_t header_bytes() { return sizeof(SorControl) + kMaxCtas * sizeof(unsigned int); }

// [control block + barrier flags][exchange: 2 planes][coefficient copy][production copy]
size_t sor_workspace_bytes(const wbc_sor_params& p) { return header_bytes() + 4 * plane_bytes(p) + 256; }

int sor_solve_resident(const wbc_sor_params& p, int check_every, int max_sweeps, double tolerance,
                       const int32_t* fixed, const float* density, const float* production, const float* source,
                       float* field, wbc_sor_report* report, void* workspace, const wbc_sor_tuning* tuning,
                       cudaStream_t stream, bool* feasible) {
    const DeviceInfo dev = device_info();
    const size_t reserve = 1024;  // static shared memory of the kernel
    const size_t limit = static_cast<size_t>(dev.smem_optin) - reserve;
    SorTiling t{};
    int H = tuning && tuning->halo_depth > 0 ? tuning->halo_depth : 0;
    const int want_tx = tuning ? tuning->tiles_i : 0, want_ty = tuning ? tuning->tiles_j : 0;
    if (H != 0 && H != 1 && H != 2 && H != 4) {
        set_error_msg("wbc_sor_solve: halo_depth must be 1, 2 or 4");
        return WBC_ERR_INVALID;
    }
    *feasible = false;
    if (dev.sms > 0) {
        if (H != 0) {
            *feasible = choose_tiling(p, dev.sms, limit, H, want_tx, want_ty, &t);
        } else {
            // Default: a one-column halo, exchanged while the inner columns are relaxed, when
            // the tiles have inner columns to hide it behind; otherwise the deepest halo that fits
            // (fewer exchanges for small grids, where the exchange latency dominates).
            SorTiling t1{};
            const bool f1 = choose_tiling(p, dev.sms, limit, 1, want_tx, want_ty, &t1);
            if (f1 && std::min(t1.ti, t1.tj) >= 4) {
                t = t1;
                *feasible = true;
            } else {
                for (int depth : {4, 2}) {
                    if (choose_tiling(p, dev.sms, limit, depth, want_tx, want_ty, &t)) {
                        *feasible = true;
                        break;
                    }
                }
                if (!*feasible && f1) {
                    t = t1;
                    *feasible = true;
                }
            }
        }
    }
    if (!*feasible) return WBC_OK;
    const bool has_prod = production != nullptr || p.has_source;
    KernelFn fn = kernel_for(has_prod, t.lanes, t.H);
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
    float* coeff = reinterpret_cast<float*>(base + header_bytes() + 2 * plane_bytes(p));
    err = cudaMemsetAsync(base, 0, header_bytes(), stream);
    if (err != cudaSuccess) {
        set_error("wbc_sor_solve: cudaMemsetAsync", err);
        return WBC_ERR_CUDA;
    }
    SorArgs args{p,    t,     fixed, density, production, source,      field,
                 xchg, coeff, ctl,   flags,   check_every, max_sweeps, tolerance};
    args.pcopy = reinterpret_cast<float*>(base + header_bytes() + 3 * plane_bytes(p));
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
    report->halo_depth = t.H;
    report->tiles_i = t.tx;
    report->tiles_j = t.ty;
    return WBC_OK;
}

// Candidate tunings for the autotuner: per halo depth, the tile grid with the fewest columns per
// tile, its transpose, and the squarest grid within the SM count.
static std::vector<wbc_sor_tuning> tuning_candidates(const wbc_sor_params& p, int sms, size_t limit) {
    std::vector<wbc_sor_tuning> out;
    auto add = [&](int H, int want_tx, int want_ty) {
        SorTiling t{};
        if (!choose_tiling(p, sms, limit, H, want_tx, want_ty, &t)) return;
        for (const wbc_sor_tuning& c : out)
            if (c.halo_depth == H && c.tiles_i == t.tx && c.tiles_j == t.ty) return;
        out.push_back(wbc_sor_tuning{H, t.tx, t.ty});
    };
    int q = 1;
    while ((q + 1) * (q + 1) <= std::min(sms, kMaxCtas)) ++q;
    for (int H : {1, 2, 4}) {
        SorTiling t{};
        if (!choose_tiling(p, sms, limit, H, 0, 0, &t)) continue;
        add(H, t.tx, t.ty);
        add(H, t.ty, t.tx);
        add(H, q, q);
    }
    return out;
}

}  // namespace wbc

using namespace wbc;

// ---- batched solves: host side -------------------------------------------------------------------------
namespace wbc {

using BatchedFn = void (*)(const SorArgs*, const int32_t*, int, unsigned int*);

template <bool P>
static BatchedFn batched_for_lanes(int lanes) {
    switch (lanes) {
        case 1: return k_sor_batched<P, 1>;
        case 2: return k_sor_batched<P, 2>;
        case 3: return k_sor_batched<P, 3>;
        case 4: return k_sor_batched<P, 4>;
        case 5: return k_sor_batched<P, 5>;
        case 6: return k_sor_batched<P, 6>;
        case 7: return k_sor_batched<P, 7>;
        default: return k_sor_batched<P, 8>;
    }
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

extern "C" {

size_t wbc_sor_batch_plan_bytes(int32_t n) { return n > 0 ? sor_batch_layout(n).bytes : 0; }

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
    // its node count. Items go on the work list heaviest first, each with CTAs in proportion to
    // its work (three times its share of the GPU: the grids rarely all fit in shared memory at
    // once, and smaller tiles shorten the heaviest solves, which bound the launch), raised until
    // its tiles fit in shared memory.
    std::vector<double> work(n);
    double total_work = 0.0;
    for (int b = 0; b < n; ++b) {
        const wbc_sor_params& p = items[b].params;
        if (p.nx < 3 || p.ny < 3 || p.nz < 3 || !items[b].density || !items[b].field || !items[b].workspace ||
            (p.has_source && !items[b].source) || reinterpret_cast<uintptr_t>(items[b].workspace) % 16 != 0 ||
            (weights && !(weights[b] > 0.0f))) {
            set_error_msg("wbc_sor_batch_prepare: invalid item");
            return WBC_ERR_INVALID;
        }
        work[b] = weights ? static_cast<double>(weights[b]) : static_cast<double>(p.nx) * p.ny * p.nz;
        total_work += work[b];
    }
    std::vector<int32_t> order(n);
    for (int b = 0; b < n; ++b) order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return work[x] > work[y]; });
    // First choice: waves. Heaviest first, items join the current wave while every item of the wave
    // can be tiled with floor(G x its share of the wave's work) CTAs in shared memory and the
    // wave's tiles fit on the GPU at once; then a new wave starts. A wave's items start together
    // and, their CTAs being proportional to their work, end together, so the next wave's tiles are
    // claimed when a whole wave of CTAs frees up. If some item cannot be tiled that way, the
    // proportional plan below is used instead.
    std::vector<SorTiling> tiling(n);
    bool waves = true;
    {
        auto plan_wave = [&](int lo, int hi, bool commit) {
            double w = 0.0;
            for (int k = lo; k < hi; ++k) w += work[order[k]];
            int tiles = 0;
            for (int k = lo; k < hi; ++k) {
                const int b = order[k];
                const int share = std::max(1, static_cast<int>(G * work[b] / w));
                SorTiling t{};
                if (!choose_tiling(items[b].params, share, limit, 1, 0, 0, &t)) return false;
                tiles += t.tx * t.ty;
                if (commit) tiling[k] = t;
            }
            return tiles <= G;
        };
        int lo = 0;
        while (lo < n && waves) {
            int hi = lo + 1;
            if (!plan_wave(lo, hi, false)) {
                waves = false;
                break;
            }
            while (hi < n && plan_wave(lo, hi + 1, false)) ++hi;
            plan_wave(lo, hi, true);
            lo = hi;
        }
    }
    std::vector<SorArgs> args(n);
    std::vector<int32_t> first(n + 1, 0);
    int lanes = 1, threads = 32;
    bool has_prod = false;
    size_t smem = 0;
    for (int k = 0; k < n; ++k) {
        const int b = order[k];
        const wbc_sor_batch_item& it = items[b];
        const wbc_sor_params& p = it.params;
        SorTiling t = tiling[k];
        if (!waves) {
            int share = std::min(G, std::max(1, static_cast<int>(3.0 * G * work[b] / total_work + 0.5)));
            bool fits = false;
            for (; share <= G && !fits; ++share) fits = choose_tiling(p, share, limit, 1, 0, 0, &t);
            if (!fits) {
                set_error_msg("wbc_sor_batch_prepare: a grid does not fit the shared-memory resident solver");
                return WBC_ERR_INVALID;
            }
        }
        char* base = static_cast<char*>(it.workspace);
        SorArgs& a = args[k];
        a.p = p;
        a.t = t;
        a.fixed = it.fixed;
        a.density = it.density;
        a.production = it.production;
        a.source = it.source;
        a.field = it.field;
        a.xchg = reinterpret_cast<float*>(base + header_bytes());
        a.coeff = reinterpret_cast<float*>(base + header_bytes() + 2 * plane_bytes(p));
        a.pcopy = reinterpret_cast<float*>(base + header_bytes() + 3 * plane_bytes(p));
        a.ctl = reinterpret_cast<SorControl*>(base);
        a.flags = reinterpret_cast<unsigned int*>(base + sizeof(SorControl));
        a.check_every = check_every;
        a.max_sweeps = max_sweeps;
        a.tolerance = tolerance;
        first[k + 1] = first[k] + t.tx * t.ty;
        lanes = std::max(lanes, t.lanes);
        threads = std::max(threads, t.threads);
        smem = std::max(smem, t.smem);
        has_prod = has_prod || it.production != nullptr || p.has_source;
    }
    threads = std::min(threads, max_threads_for_lanes(lanes));
    BatchedFn fn = has_prod ? batched_for_lanes<true>(lanes) : batched_for_lanes<false>(lanes);
    cudaError_t err = cudaFuncSetAttribute(reinterpret_cast<const void*>(fn),
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    int per_sm = 0;
    if (err == cudaSuccess) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
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
    out->threads = threads;
    out->lanes = lanes;
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
    BatchedFn fn = b->has_prod ? batched_for_lanes<true>(b->lanes) : batched_for_lanes<false>(b->lanes);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b->ctas);
    cfg.blockDim = dim3(b->threads);
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
        r.halo_depth = 1;
        r.tiles_i = args[k].t.tx;
        r.tiles_j = args[k].t.ty;
        if (ctl[k].status != 0) rc = WBC_ERR_TIMEOUT;
    }
    if (rc != WBC_OK) set_error_msg("wbc_sor_batch_reports: a solve timed out");
    return rc;
}

}  // extern "C"

extern "C" {

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
    *best = wbc_sor_tuning{0, 0, 0};
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
                                    &r, workspace, &cands[c], s, &feasible);
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
                  float* field, wbc_sor_report* report, void* workspace, size_t workspace_bytes, int32_t path,
                  const wbc_sor_tuning* tuning, void* stream) {
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
                                    report, workspace, tuning, s, &feasible);
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
    report->halo_depth = 0;
    report->tiles_i = 0;
    report->tiles_j = 0;
    return WBC_OK;
}

}  // extern "C"
