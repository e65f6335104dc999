// One Boolean network per cell, bit-packed: node i at word i/64, bit i%64 of uint64[n_words].
//
// The state words of a cell stay in registers for the whole launch (all update sweeps), and the
// postfix programs (ops/args/start/length, shared by every cell) are staged once per block in
// shared memory; every lane of a warp walks the same program, so the interpreter never
// diverges. A node whose program reads at most 6 distinct nodes is evaluated from its truth table
// instead (when the caller passes tables): its input bits form an index into a 64-bit table, a
// handful of operations against one interpreter step per postfix op (the random 2-4 input
// networks compile to DNF programs of tens of ops per node). Evaluation follows kernels/network_kernels.py:50-78: a boolean stack in one uint64,
// top = bit 0. Update semantics: synchronous (:157-175, every updatable node from the old state),
// asynchronous (:135-154, uniform random single-node picks from the cell's stream) and MaBoSS
// Gillespie (:178-245, with the project's log for the waiting times).
#include "wbc_common.cuh"

namespace wbc {

constexpr int kMaxProgram = 8192;  // ops staged in shared memory; longer programs read global memory
constexpr int kMaxNodes = 256;

// log(x) for x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s), s = (m-1)/(m+1),
// from the odd series 2(s + s^3/3 + ... + s^11/11) (|s| <= 0.1716, truncation < 1e-10), plus
// e ln2 with ln2 split in head and tail. Correctly rounded float steps only, so the oracle
// reproduces it exactly. Used for the Gillespie waiting times.
__device__ __forceinline__ float wbc_logf(float x) {
    if (!(x > 0.0f)) return x == 0.0f ? -__int_as_float(0x7f800000) : __int_as_float(0x7fc00000);
    if (x == __int_as_float(0x7f800000)) return x;
    int e = 0;
    if (x < 1.17549435e-38f) {  // subnormal: scale into the normal range first
        x = x * 16777216.0f;
        e = -24;
    }
    uint32_t bits = __float_as_uint(x);
    e += static_cast<int>((bits >> 23) & 0xff) - 127;
    float m = __uint_as_float((bits & 0x007fffffu) | 0x3f800000u);  // [1, 2)
    if (m > 1.41421353816986083984375f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 9.09090909090909090909e-2f;  // 1/11
    p = p * s2 + 1.11111111111111111111e-1f;  // 1/9
    p = p * s2 + 1.42857142857142857143e-1f;  // 1/7
    p = p * s2 + 2.0e-1f;                    // 1/5
    p = p * s2 + 3.33333333333333333333e-1f;  // 1/3
    p = p * s2 + 1.0f;
    const float log_m = 2.0f * s * p;
    const float ef = static_cast<float>(e);
    return (ef * 0.693145751953125f + log_m) + ef * 1.42860682030941723212e-06f;
}

template <int W>
struct Words {
    uint64_t w[W];
    __device__ __forceinline__ uint64_t get(int idx) const {
        const int k = idx >> 6;
        uint64_t v = w[0];
#pragma unroll
        for (int q = 1; q < W; ++q)
            if (k == q) v = w[q];
        return (v >> (idx & 63)) & 1ull;
    }
    __device__ __forceinline__ void set(int idx, uint64_t value) {
        const int k = idx >> 6;
        const uint64_t mask = 1ull << (idx & 63);
#pragma unroll
        for (int q = 0; q < W; ++q)
            if (k == q) w[q] = value ? (w[q] | mask) : (w[q] & ~mask);
    }
    __device__ __forceinline__ void load(const uint64_t* s, int64_t c) {
#pragma unroll
        for (int q = 0; q < W; ++q) w[q] = s[c * W + q];
    }
    __device__ __forceinline__ void store(uint64_t* s, int64_t c) const {
#pragma unroll
        for (int q = 0; q < W; ++q) s[c * W + q] = w[q];
    }
};

struct Program {
    const int32_t* ops;    // shared or global
    const int32_t* args;
    const int32_t* tarity;   // shared: per node, table inputs (0..6) or -1; null = no tables
    const int32_t* tinputs;  // shared: 6 per node
    const int32_t* tbits;    // shared: per node, the 64-bit table as two 32-bit halves (low first)
    const int32_t* start;  // global
    const int32_t* length;
    const int32_t* updatable;
    int n_updatable;
};

template <int W>
__device__ __forceinline__ uint64_t eval_program(const Program& p, int node, const Words<W>& s) {
    const int b = __ldg(p.start + node);
    const int len = __ldg(p.length + node);
    uint64_t stack = 0;
    for (int k = 0; k < len; ++k) {
        const int op = p.ops[b + k];
        const int a = p.args[b + k];
        if (op == 0) {
            stack = (stack << 1) | s.get(a);
        } else if (op == 4) {
            stack = (stack << 1) | static_cast<uint64_t>(static_cast<int64_t>(a));
        } else if (op == 1) {
            stack = stack ^ 1ull;
        } else if (op == 2) {
            const uint64_t top = stack & 1ull;
            stack = stack >> 1;
            stack = (stack & ~1ull) | ((stack & 1ull) & top);
        } else if (op == 3) {
            const uint64_t top = stack & 1ull;
            stack = stack >> 1;
            stack = (stack & ~1ull) | ((stack & 1ull) | top);
        }
    }
    return stack & 1ull;
}

// A node's logic value: from its truth table when it has one, else by running its program.
template <int W>
__device__ __forceinline__ uint64_t eval_node(const Program& p, int node, const Words<W>& s) {
    if (p.tarity) {
        const int arity = p.tarity[node];
        if (arity >= 0) {
            const int32_t* in = p.tinputs + 6 * node;
            unsigned int idx = 0u;
            for (int j = 0; j < arity; ++j) idx |= static_cast<unsigned int>(s.get(in[j])) << j;
            const unsigned int half = static_cast<unsigned int>(p.tbits[2 * node + (idx >> 5)]);
            return (half >> (idx & 31u)) & 1u;
        }
    }
    return eval_program<W>(p, node, s);
}

// Stage the truth tables (when present) and ops/args (when they fit) in shared memory; returns the
// program view for this block. Layout: arity [n_nodes], inputs [6 n_nodes], table halves
// [2 n_nodes], then ops [n_ops] and args [n_ops].
__device__ __forceinline__ Program stage_program(const wbc_network_program& g, int32_t* smem, bool use_smem) {
    Program p;
    int32_t* base = smem;
    p.tarity = p.tinputs = p.tbits = nullptr;
    const bool tables = g.table_arity != nullptr;
    if (tables) {
        const int nn = g.n_nodes;
        for (int t = threadIdx.x; t < nn; t += blockDim.x) {
            base[t] = g.table_arity[t];
            const uint64_t b = g.table_bits[t];
            base[7 * nn + 2 * t] = static_cast<int32_t>(static_cast<uint32_t>(b));
            base[7 * nn + 2 * t + 1] = static_cast<int32_t>(static_cast<uint32_t>(b >> 32));
        }
        for (int t = threadIdx.x; t < 6 * nn; t += blockDim.x) base[nn + t] = g.table_inputs[t];
        p.tarity = base;
        p.tinputs = base + nn;
        p.tbits = base + 7 * nn;
        base += 9 * nn;
    }
    if (use_smem) {
        for (int t = threadIdx.x; t < g.n_ops; t += blockDim.x) {
            base[t] = g.ops[t];
            base[g.n_ops + t] = g.args[t];
        }
        p.ops = base;
        p.args = base + g.n_ops;
    } else {
        p.ops = g.ops;
        p.args = g.args;
    }
    if (tables || use_smem) __syncthreads();
    p.start = g.start;
    p.length = g.length;
    p.updatable = g.updatable;
    p.n_updatable = g.n_updatable;
    return p;
}

template <int W>
__global__ void k_update_sync(wbc_network_program g, int32_t n, int32_t sweeps, uint64_t* __restrict__ states,
                              bool use_smem) {
    extern __shared__ int32_t smem[];
    const Program p = stage_program(g, smem, use_smem);
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    Words<W> cur;
    cur.load(states, c);
    for (int s = 0; s < sweeps; ++s) {
        Words<W> next = cur;
        for (int k = 0; k < p.n_updatable; ++k) {
            const int node = __ldg(p.updatable + k);
            next.set(node, eval_node<W>(p, node, cur));
        }
        cur = next;
    }
    cur.store(states, c);
}

template <int W>
__global__ void k_update_async(wbc_network_program g, int32_t n, int32_t n_updates, uint32_t* __restrict__ rng_state,
                               uint64_t* __restrict__ states, bool use_smem) {
    extern __shared__ int32_t smem[];
    const Program p = stage_program(g, smem, use_smem);
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    Words<W> cur;
    cur.load(states, c);
    uint32_t rng = rng_state[c];
    const uint32_t inc = rng_increment(static_cast<uint32_t>(c));
    const int m = p.n_updatable;
    for (int k = 0; k < n_updates; ++k) {
        const int pick = min(static_cast<int>(randf(rng, inc) * static_cast<float>(m)), m - 1);
        const int node = __ldg(p.updatable + pick);
        cur.set(node, eval_node<W>(p, node, cur));
    }
    rng_state[c] = rng;
    cur.store(states, c);
}

__device__ __forceinline__ float node_rate(uint64_t on, uint64_t logic, int node, const float* up_t, const float* up_f,
                                           const float* down_t, const float* down_f) {
    if (on == 0ull) return logic ? __ldg(up_t + node) : __ldg(up_f + node);
    return logic ? __ldg(down_t + node) : __ldg(down_f + node);
}

template <int W>
__global__ void k_update_maboss(wbc_network_program g, int32_t n, float duration, int32_t max_events,
                                const float* __restrict__ up_t, const float* __restrict__ up_f,
                                const float* __restrict__ down_t, const float* __restrict__ down_f,
                                uint32_t* __restrict__ rng_state, uint64_t* __restrict__ states, bool use_smem) {
    extern __shared__ int32_t smem[];
    const Program p = stage_program(g, smem, use_smem);
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    Words<W> cur;
    cur.load(states, c);
    uint32_t rng = rng_state[c];
    const uint32_t inc = rng_increment(static_cast<uint32_t>(c));
    const int m = p.n_updatable;
    float t = 0.0f;
    for (int event = 0; event < max_events; ++event) {
        // Logic values of every updatable node for the current state (k-th bit = k-th updatable).
        Words<4> logic;
#pragma unroll
        for (int q = 0; q < 4; ++q) logic.w[q] = 0ull;
        float total = 0.0f;
        for (int k = 0; k < m; ++k) {
            const int node = __ldg(p.updatable + k);
            const uint64_t l = eval_node<W>(p, node, cur);
            if (l) logic.set(k, 1ull);
            total += node_rate(cur.get(node), l, node, up_t, up_f, down_t, down_f);
        }
        if (total <= 0.0f) break;
        const float u1 = fmaxf(randf(rng, inc), 1.0e-12f);
        const float tau = -wbc_logf(u1) / total;
        if (t + tau > duration) break;
        t += tau;
        const float target = randf(rng, inc) * total;
        float acc = 0.0f;
        int chosen = -1;
        for (int k = 0; k < m && chosen < 0; ++k) {
            const int node = __ldg(p.updatable + k);
            const float r = node_rate(cur.get(node), logic.get(k), node, up_t, up_f, down_t, down_f);
            acc += r;
            if (acc >= target && r > 0.0f) chosen = node;
        }
        if (chosen < 0) chosen = __ldg(p.updatable + m - 1);
        cur.set(chosen, 1ull - cur.get(chosen));
    }
    rng_state[c] = rng;
    cur.store(states, c);
}

__global__ void k_initialize(int32_t n, int32_t n_nodes, int32_t n_words, const float* __restrict__ p_on,
                             uint32_t* __restrict__ rng_state, uint64_t* __restrict__ states) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    uint32_t rng = rng_state[c];
    const uint32_t inc = rng_increment(static_cast<uint32_t>(c));
    uint64_t w[4] = {0ull, 0ull, 0ull, 0ull};
    for (int i = 0; i < n_nodes; ++i)
        if (randf(rng, inc) < __ldg(p_on + i)) w[i >> 6] |= 1ull << (i & 63);
    for (int q = 0; q < n_words; ++q) states[static_cast<int64_t>(c) * n_words + q] = w[q];
    rng_state[c] = rng;
}

__global__ void k_clamp(int32_t n, int32_t n_words, int32_t n_clamps, const int32_t* __restrict__ node,
                        const int32_t* __restrict__ source, const float* __restrict__ threshold,
                        const int32_t* __restrict__ above, const float* __restrict__ oxygen,
                        const float* __restrict__ glucose, const float* __restrict__ extra_a,
                        const float* __restrict__ extra_b, uint64_t* __restrict__ states) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    uint64_t* w = states + static_cast<int64_t>(c) * n_words;
    for (int k = 0; k < n_clamps; ++k) {
        const int src = __ldg(source + k);
        float value = 0.0f;
        if (src == 0)
            value = oxygen[c];
        else if (src == 1)
            value = glucose[c];
        else if (src == 2)
            value = extra_a[c];
        else if (src == 3)
            value = extra_b[c];
        const float thr = __ldg(threshold + k);
        bool on;
        if (src == 4)
            on = thr > 0.0f;
        else if (__ldg(above + k) != 0)
            on = value > thr;
        else
            on = value < thr;
        const int idx = __ldg(node + k);
        const uint64_t mask = 1ull << (idx & 63);
        w[idx >> 6] = on ? (w[idx >> 6] | mask) : (w[idx >> 6] & ~mask);
    }
}

__global__ void k_read_fates(int32_t n, int32_t n_words, int32_t np, int32_t na, int32_t ng, int32_t nn,
                             const uint64_t* __restrict__ states, int32_t* __restrict__ fate_flags) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const uint64_t* w = states + static_cast<int64_t>(c) * n_words;
    auto bit = [&](int idx) { return (w[idx >> 6] >> (idx & 63)) & 1ull; };
    int flags = 0;
    if (np >= 0 && bit(np)) flags |= WBC_FATE_PROLIFERATION;
    if (na >= 0 && bit(na)) flags |= WBC_FATE_APOPTOSIS;
    if (ng >= 0 && bit(ng)) flags |= WBC_FATE_GROWTH_ARREST;
    if (nn >= 0 && bit(nn)) flags |= WBC_FATE_NECROSIS;
    fate_flags[c] = flags;
}

__global__ void k_inherit(int32_t count_before, int32_t n_words, const int32_t* __restrict__ divide_flag,
                          const int32_t* __restrict__ division_offset, uint64_t* __restrict__ states) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count_before || divide_flag[i] == 0) return;
    const int j = count_before + division_offset[i] - 1;
    for (int q = 0; q < n_words; ++q)
        states[static_cast<int64_t>(j) * n_words + q] = states[static_cast<int64_t>(i) * n_words + q];
}

__global__ void k_count_on(int32_t n, int32_t n_words, int32_t n_query, const int32_t* __restrict__ nodes,
                           int32_t living_only, const int32_t* __restrict__ cell_state,
                           const uint64_t* __restrict__ states, int32_t* __restrict__ counts) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    if (living_only != 0 && cell_state[c] == WBC_STATE_DEAD) return;
    const uint64_t* w = states + static_cast<int64_t>(c) * n_words;
    for (int k = 0; k < n_query; ++k) {
        const int node = __ldg(nodes + k);
        if (node >= 0 && ((w[node >> 6] >> (node & 63)) & 1ull)) atomicAdd(counts + k, 1);
    }
}

static bool program_ok(const wbc_network_program* g) {
    if (!g || g->n_nodes < 1 || g->n_nodes > kMaxNodes || g->n_words != (g->n_nodes + 63) / 64 || g->n_ops < 1 ||
        g->n_updatable < 0 || g->n_updatable > g->n_nodes || !g->ops || !g->args || !g->start || !g->length ||
        (g->n_updatable > 0 && !g->updatable))
        return false;
    const int tables = (g->table_arity != nullptr) + (g->table_inputs != nullptr) + (g->table_bits != nullptr);
    return tables == 0 || tables == 3;
}

static size_t program_smem(const wbc_network_program* g, bool* use) {
    *use = g->n_ops <= kMaxProgram;
    const size_t tables = g->table_arity ? 9 * sizeof(int32_t) * static_cast<size_t>(g->n_nodes) : 0;
    return tables + (*use ? 2 * sizeof(int32_t) * static_cast<size_t>(g->n_ops) : 0);
}

}  // namespace wbc

using namespace wbc;

#define WBC_DISPATCH_WORDS(W, ...) \
    switch (W) {                    \
        case 1: {                   \
            constexpr int kW = 1;   \
            __VA_ARGS__;            \
        } break;                    \
        case 2: {                   \
            constexpr int kW = 2;   \
            __VA_ARGS__;            \
        } break;                    \
        case 3: {                   \
            constexpr int kW = 3;   \
            __VA_ARGS__;            \
        } break;                    \
        default: {                  \
            constexpr int kW = 4;   \
            __VA_ARGS__;            \
        } break;                    \
    }

extern "C" {

int wbc_network_initialize(const wbc_network_program* prog, int32_t n, const float* p_on, uint32_t* rng_state,
                           uint64_t* states, void* stream) {
    if (!program_ok(prog) || n < 0 || (n > 0 && (!p_on || !rng_state || !states))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_initialize<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, prog->n_nodes, prog->n_words, p_on, rng_state,
                                                                  states);
    return check_launch("wbc_network_initialize");
}

int wbc_network_clamp_inputs(int32_t n, int32_t n_words, int32_t n_clamps, const int32_t* clamp_node,
                             const int32_t* clamp_source, const float* clamp_threshold, const int32_t* clamp_above,
                             const float* oxygen_local, const float* glucose_local, const float* extra_a,
                             const float* extra_b, uint64_t* states, void* stream) {
    if (n < 0 || n_words < 1 || n_words > 4 || n_clamps < 0) return WBC_ERR_INVALID;
    if (n == 0 || n_clamps == 0) return WBC_OK;
    if (!clamp_node || !clamp_source || !clamp_threshold || !clamp_above || !oxygen_local || !glucose_local ||
        !extra_a || !extra_b || !states)
        return WBC_ERR_INVALID;
    k_clamp<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, n_words, n_clamps, clamp_node, clamp_source,
                                                             clamp_threshold, clamp_above, oxygen_local,
                                                             glucose_local, extra_a, extra_b, states);
    return check_launch("wbc_network_clamp_inputs");
}

int wbc_network_update_sync(const wbc_network_program* prog, int32_t n, int32_t sweeps, uint64_t* states,
                            void* stream) {
    if (!program_ok(prog) || n < 0 || sweeps < 0 || (n > 0 && !states)) return WBC_ERR_INVALID;
    if (n == 0 || sweeps == 0 || prog->n_updatable == 0) return WBC_OK;
    bool use = false;
    const size_t smem = program_smem(prog, &use);
    cudaStream_t s = as_stream(stream);
    WBC_DISPATCH_WORDS(prog->n_words,
                       k_update_sync<kW><<<grid_for(n, 128), 128, smem, s>>>(*prog, n, sweeps, states, use));
    return check_launch("wbc_network_update_sync");
}

int wbc_network_update_async(const wbc_network_program* prog, int32_t n, int32_t n_updates, uint32_t* rng_state,
                             uint64_t* states, void* stream) {
    if (!program_ok(prog) || n < 0 || n_updates < 0 || (n > 0 && (!states || !rng_state))) return WBC_ERR_INVALID;
    if (n == 0 || n_updates == 0) return WBC_OK;
    if (prog->n_updatable == 0) return WBC_ERR_INVALID;
    bool use = false;
    const size_t smem = program_smem(prog, &use);
    cudaStream_t s = as_stream(stream);
    WBC_DISPATCH_WORDS(prog->n_words, k_update_async<kW><<<grid_for(n, 128), 128, smem, s>>>(
                                          *prog, n, n_updates, rng_state, states, use));
    return check_launch("wbc_network_update_async");
}

int wbc_network_update_maboss(const wbc_network_program* prog, int32_t n, float duration, int32_t max_events,
                              const float* rate_up_true, const float* rate_up_false, const float* rate_down_true,
                              const float* rate_down_false, uint32_t* rng_state, uint64_t* states, void* stream) {
    if (!program_ok(prog) || n < 0 || max_events < 0 ||
        (n > 0 && (!states || !rng_state || !rate_up_true || !rate_up_false || !rate_down_true || !rate_down_false)))
        return WBC_ERR_INVALID;
    if (n == 0 || max_events == 0 || prog->n_updatable == 0) return WBC_OK;
    bool use = false;
    const size_t smem = program_smem(prog, &use);
    cudaStream_t s = as_stream(stream);
    WBC_DISPATCH_WORDS(prog->n_words, k_update_maboss<kW><<<grid_for(n, 128), 128, smem, s>>>(
                                          *prog, n, duration, max_events, rate_up_true, rate_up_false,
                                          rate_down_true, rate_down_false, rng_state, states, use));
    return check_launch("wbc_network_update_maboss");
}

int wbc_network_read_fates(int32_t n, int32_t n_words, int32_t node_proliferation, int32_t node_apoptosis,
                           int32_t node_growth_arrest, int32_t node_necrosis, const uint64_t* states,
                           int32_t* fate_flags, void* stream) {
    if (n < 0 || n_words < 1 || n_words > 4 || (n > 0 && (!states || !fate_flags))) return WBC_ERR_INVALID;
    if (n == 0) return WBC_OK;
    k_read_fates<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, n_words, node_proliferation, node_apoptosis,
                                                                  node_growth_arrest, node_necrosis, states,
                                                                  fate_flags);
    return check_launch("wbc_network_read_fates");
}

int wbc_network_inherit(int32_t count_before, int32_t n_words, const int32_t* divide_flag,
                        const int32_t* division_offset, uint64_t* states, void* stream) {
    if (count_before < 0 || n_words < 1 || n_words > 4 ||
        (count_before > 0 && (!divide_flag || !division_offset || !states)))
        return WBC_ERR_INVALID;
    if (count_before == 0) return WBC_OK;
    k_inherit<<<grid_for(count_before), kThreads, 0, as_stream(stream)>>>(count_before, n_words, divide_flag,
                                                                          division_offset, states);
    return check_launch("wbc_network_inherit");
}

int wbc_network_count_on(int32_t n, int32_t n_words, int32_t n_query, const int32_t* nodes, int32_t living_only,
                         const int32_t* cell_state, const uint64_t* states, int32_t* counts, void* stream) {
    if (n < 0 || n_words < 1 || n_words > 4 || n_query < 0 || !counts ||
        (n > 0 && n_query > 0 && (!nodes || !cell_state || !states)))
        return WBC_ERR_INVALID;
    if (n == 0 || n_query == 0) return WBC_OK;
    k_count_on<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(n, n_words, n_query, nodes, living_only, cell_state,
                                                                states, counts);
    return check_launch("wbc_network_count_on");
}

}  // extern "C"
