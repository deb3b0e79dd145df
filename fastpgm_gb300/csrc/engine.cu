// GB300 PC-stable CI-testing engine: device kernels and the C ABI.
//
// Batched mode (the product path) keeps the whole skeleton on the device:
//   * the adjacency is an n x n bitset; each level snapshots it into sorted
//     per-node neighbour lists (PCStable.cpp:272, FindAdjacencies :500-515);
//   * every remaining edge x<y owns the ranked sequence of its candidate
//     conditioning sets: C(|adj(x)\y|, d) x-side sets, then C(|adj(y)\x|, d)
//     y-side sets, each in the lexicographic order of ChoiceGenerator
//     (CheckEdge :399-494, ChoiceGenerator.cpp:55-85);
//   * a level runs in waves; a wave gives each unresolved edge the next q
//     ranks (q grows geometrically), one persistent kernel drains all tests
//     of the wave from a work counter, and a reduction keeps, per edge, the
//     FIRST independent rank -- the reference's sepset (Testing :526-614);
//   * removals are applied to the bitset at the end of the level and the
//     FreeDegree stop rule (:620-626, :387) is evaluated on the device.
// Plain mode is the reference's control flow on the host with one kernel
// launch (whole GPU) per CI test; it is the comparison baseline.
#include <cuda_runtime.h>
#include <cub/cub.cuh>

#include <algorithm>
#include <chrono>
#include <mutex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ci_device.cuh"
#include "ci_kernels.cuh"
#include "fastpgm_gb300.h"
#include "engine_internal.h"

using namespace fpgm;

// ------------------------------------------------------------------ errors
namespace {
thread_local std::string g_last_error;
}

namespace fpgm {
int set_error(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}
}  // namespace fpgm

extern "C" const char *fpgm_last_error(void) { return g_last_error.c_str(); }

namespace {
std::mutex g_alloc_mu;
size_t g_alloc_bytes = 0;
}  // namespace

namespace fpgm {
int dev_alloc(void **p, size_t bytes) {
    *p = nullptr;
    static const size_t cap = [] {
        const char *c = getenv("FPGM_DEVICE_MEM_CAP");
        return c ? (size_t)strtoull(c, nullptr, 10) : (size_t)0;
    }();
    {
        std::lock_guard<std::mutex> lk(g_alloc_mu);
        if (cap && g_alloc_bytes + bytes > cap)
            return set_error(FPGM_ERR_OOM, "cudaMalloc(%zu) refused: %zu bytes held, cap %zu (FPGM_DEVICE_MEM_CAP)",
                             bytes, g_alloc_bytes, cap);
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return set_error(FPGM_ERR_OOM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    std::lock_guard<std::mutex> lk(g_alloc_mu);
    g_alloc_bytes += bytes;
    return FPGM_OK;
}

void dev_free(void *p, size_t bytes) {
    if (!p) return;
    cudaFree(p);
    std::lock_guard<std::mutex> lk(g_alloc_mu);
    g_alloc_bytes -= std::min(bytes, g_alloc_bytes);
}
}  // namespace fpgm

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return set_error(e_ == cudaErrorMemoryAllocation ? FPGM_ERR_OOM : FPGM_ERR_CUDA,       \
                             "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

#define RET(call)                    \
    do {                             \
        int r_ = (call);             \
        if (r_ != FPGM_OK) return r_; \
    } while (0)

// ------------------------------------------------------------------ device buffers
namespace {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    int ensure(size_t need, bool keep = false, cudaStream_t st = nullptr) {
        if (need <= bytes) return FPGM_OK;
        size_t nb = std::max(need, bytes + bytes / 2);
        void *q = nullptr;
        const int rc = dev_alloc(&q, nb);
        if (rc != FPGM_OK) return rc;
        if (keep && p && bytes) {
            cudaError_t e = cudaMemcpyAsync(q, p, bytes, cudaMemcpyDeviceToDevice, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) {
                dev_free(q, nb);
                return set_error(FPGM_ERR_CUDA, "buffer grow copy failed: %s", cudaGetErrorString(e));
            }
        }
        if (p) dev_free(p, bytes);
        p = q;
        bytes = nb;
        return FPGM_OK;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
    void release() {
        if (p) dev_free(p, bytes);
        p = nullptr;
        bytes = 0;
    }
};

constexpr int kStatusActive = 0, kStatusRemoved = 1, kStatusKept = 2;
constexpr int64_t kPlainInts = (int64_t)1 << 25;       // plain kernel's global table (128 MB)
constexpr int64_t kMaxItems = (int64_t)1 << 22;        // tests per wave

}  // namespace

struct fpgm_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0, ci_blocks = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    // data
    int n = 0;
    int64_t S = 0, S_pad = 0;  // one dataset: its samples and column pitch; several: the largest
    int n_jobs = 1;            // independent datasets sharing the engine (variables in job order)
    int64_t E = 0;             // level-0 pairs: within each dataset
    DevBuf cols, card, var_off, var_S, var_lo, var_hi;
    std::vector<uint8_t> h_card;
    std::vector<int64_t> h_var_off;         // byte offset of each variable's column
    std::vector<int32_t> h_var_S, h_var_lo, h_var_hi;  // its dataset's samples and variable range
    DevBuf btab;
    // level workspace
    DevBuf bits, deg, adjl, edges_x, edges_y, pxy, pyx, cntx, total, next, status, seprank, g, off, flag,
        counters, stats, scan_tmp, log_pair, log_vars, log_meta, node_cnt, node_off;
    DevBuf slots, plain_ws, tests_buf, detail_buf, item_vars, lists, band, phase_timers;
    DevBuf wide, wide_items;  // partition-parallel scoring: one WideTest per slot, kPartMax items each
    DevBuf wave_ctl;          // device-driven wave loop: q, wave count, per-group device time
    DevBuf res_adj_d, res_key, res_idx, res_removed_d, res_cnt, res_vars_d;  // result assembly
    bool graph_on = true;     // FPGM_GRAPH=0: the host drives every wave (as FPGM_WAVE_LOG does)
    DevBuf mle_counts, mle_pot, mle_meta;  // parameter learning: counts, potentials, per-node tables
    double band_alpha = -1.0;
    int n_slots = 0, hash_cap_global = 0;
    int part_max_log = kPartMaxLog;  // FPGM_PART_MAX_LOG (tests): fewer partitions before the global hash
    int64_t slot_bytes = 0, slot_S = 0;  // slot_S: the sample count the slots' layout was made for
    bool wave_log = false;               // FPGM_WAVE_LOG: one stderr line per wave (tier sizes, kernel times)
    bool warp_small = true;              // 8 KB warp-tier slices, 3 CTAs per SM (FPGM_WARP_SLICE=3072: 12 KB, 2)
    bool dense_rows = true;              // FPGM_DENSE_ROWS=0: lane groups score the dense strata table
    int warp_blocks_small = 0;
    // level 0 on the tensor cores (FPGM_GRAM=0 keeps it on the counting kernels)
    GramLevel0 *gram = nullptr;
    bool gram_on = true, gram_planned = false, gram_ok = false;
    int gram_score_ctas = 2;  // resident CTAs per SM of the level-0 scoring kernel for this dataset
    // partition-parallel scoring of the last partitioned tests of a wave (FPGM_WIDE=0 turns it off)
    bool wide_on = true;
    int wide_small_n2 = -1;    // tier-2 tests per wave at most for tests under 65,536 samples (-1: one per slot)
    int wide_min_log = 1;      // least partitions (log2) of a published test
    int wide_part_min = 1024;  // samples per partition at least when splitting for parallelism
    bool wide_direct = true;   // hand a small wave's tier-2 tests over before the compact kernel hashes them
    // tier-2 method: the autotuner's table (fastpgm_gb300/tune_table.txt, FPGM_TUNE_TABLE) or a
    // fixed sample-count cut-over (FPGM_PART_CUTOVER, default 65,536)
    int64_t part_min_samples = kPartMinSamples;
    DevBuf tune, tune_obs;  // a fixed table (FPGM_TUNE_TABLE) / the online autotuner's timings
    DevBuf ovf;             // per bucket: how often tier-2 tests overflowed the shared strata hash
    bool ovf_on = true;     // FPGM_OVF_SKIP=0: every tier-2 test tries the shared hash first
    int stage_rec = 0;      // FPGM_STAGE_REC=n (tests): at most n records per staged super-partition
    // contributing-sample bitmaps of the partition path (FPGM_LIVE=0: off), two pools used by
    // alternate levels: level d writes pool d & 1 and reads pool (d - 1) & 1
    bool live_on = true;
    int live_min_level = 3;             // FPGM_LIVE_MIN_LEVEL: first level that writes bitmaps
    DevBuf live_pool[2], live_tab[2], live_cnt;
    int64_t live_cap = 0;               // bitmaps per pool
    int32_t live_tab_cap = 0, live_words = 0;
    int live_level[2] = {-1, -1};       // the level whose bitmaps each pool holds
    bool live_write = false;            // this level writes (set per level)
    bool live_in_skeleton = false;      // bitmaps are used only by a batched skeleton's waves
    DevBuf live_stat;                   // samples in contributing strata, samples counted (partition path)
    unsigned long long live_prev[2] = {0ull, 0ull};
    bool live_next = false;             // the level just measured had few enough contributing samples
    double live_frac = 0.55;            // FPGM_LIVE_FRAC: write bitmaps below this contributing fraction
    bool tune_loaded = false, tune_online = true;
    std::string tune_source;
    // result
    bool has_result = false;
    std::vector<uint8_t> res_adj;
    std::vector<int32_t> res_removed, res_off, res_vars;
};

// ------------------------------------------------------------------ kernels
namespace {

// ---- data preparation
// First-appearance ids per column (Dataset.cpp:459-467) and observed cardinality.
__global__ void relabel_kernel(uint8_t *cols, const int64_t *var_off, const int32_t *var_S, uint8_t *card,
                               int relabel) {
    __shared__ unsigned first[256];
    __shared__ uint8_t map[256];
    __shared__ unsigned s_max;
    uint8_t *c = cols + var_off[blockIdx.x];
    const int64_t S = var_S[blockIdx.x];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) first[i] = 0xffffffffu;
    if (threadIdx.x == 0) s_max = 0;
    __syncthreads();
    if (relabel) {
        for (int64_t s = threadIdx.x; s < S; s += blockDim.x) {
            unsigned v = c[s];
            if ((unsigned)s < first[v]) atomicMin(&first[v], (unsigned)s);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int next = 0;
            // values sorted by first appearance: repeated min-selection over <= 256 values
            bool used[256];
            for (int i = 0; i < 256; ++i) used[i] = first[i] == 0xffffffffu;
            for (;;) {
                int best = -1;
                unsigned bp = 0xffffffffu;
                for (int i = 0; i < 256; ++i)
                    if (!used[i] && first[i] < bp) { bp = first[i]; best = i; }
                if (best < 0) break;
                used[best] = true;
                map[best] = (uint8_t)next++;
            }
            card[blockIdx.x] = (uint8_t)next;
        }
        __syncthreads();
        for (int64_t s = threadIdx.x; s < S; s += blockDim.x) c[s] = map[c[s]];
    } else {
        for (int64_t s = threadIdx.x; s < S; s += blockDim.x) atomicMax(&s_max, (unsigned)c[s]);
        __syncthreads();
        if (threadIdx.x == 0) card[blockIdx.x] = (uint8_t)(s_max + 1);
    }
}

// ---- level machinery
// complete graph within each dataset: v is adjacent to [var_lo[v], var_hi[v]) minus itself
__global__ void init_bits_kernel(uint32_t *bits, int n, int W, const int32_t *var_lo, const int32_t *var_hi) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)n * W) return;
    int v = (int)(i / W), w = (int)(i % W);
    const int lo = w * 32, a = max(var_lo[v], lo), b = min(var_hi[v], lo + 32);
    uint32_t m = 0u;
    if (b > a) m = (b - a >= 32 ? 0xffffffffu : ((1u << (b - a)) - 1u)) << (a - lo);
    if (v >= lo && v < lo + 32) m &= ~(1u << (v - lo));
    bits[i] = m;
}

// level-0 pairs of several datasets: v with each higher neighbour of the initial bitset, in
// (v, u) order like the complete graph's (Network.cpp:270-283), one test each
__global__ void level0_csr_edges_kernel(int n, const int32_t *adjl, int stride, const int32_t *deg,
                                        const int32_t *node_off, int32_t *ex, int32_t *ey, int32_t *pxy,
                                        int32_t *pyx, uint64_t *cntx, uint64_t *total, uint64_t *next,
                                        uint8_t *status) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int32_t *L = adjl + (int64_t)v * stride;
    int64_t e = node_off[v];
    for (int k = 0; k < deg[v]; ++k) {
        const int u = L[k];
        if (u <= v) continue;
        ex[e] = v;
        ey[e] = u;
        pxy[e] = 0;
        pyx[e] = 0;
        cntx[e] = 1;
        total[e] = 1;
        next[e] = 0;
        status[e] = kStatusActive;
        ++e;
    }
}

// all pairs i<j in complete-graph order (Network.cpp:270-283)
__global__ void level0_edges_kernel(int n, int32_t *ex, int32_t *ey, int32_t *pxy, int32_t *pyx, uint64_t *cntx,
                                    uint64_t *total, uint64_t *next, uint8_t *status) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t E = (int64_t)n * (n - 1) / 2;
    if (e >= E) return;
    // row i: first index base(i) = i*(2n-i-1)/2
    double nn = 2.0 * n - 1.0;
    int i = (int)floor((nn - sqrt(nn * nn - 8.0 * (double)e)) / 2.0);
    if (i < 0) i = 0;
    while (i > 0 && (int64_t)i * (2 * n - i - 1) / 2 > e) --i;
    while ((int64_t)(i + 1) * (2 * n - i - 2) / 2 <= e) ++i;
    int64_t base = (int64_t)i * (2 * n - i - 1) / 2;
    int j = (int)(e - base) + i + 1;
    ex[e] = i;
    ey[e] = j;
    pxy[e] = 0;
    pyx[e] = 0;
    cntx[e] = 1;
    total[e] = 1;
    next[e] = 0;
    status[e] = kStatusActive;
}

// sorted neighbour lists from the bitset (the level snapshot)
__global__ void csr_kernel(const uint32_t *bits, int n, int W, int32_t *adjl, int stride, int32_t *deg,
                           int32_t *node_cnt) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    int k = 0, higher = 0;
    const uint32_t *row = bits + (int64_t)v * W;
    int32_t *L = adjl + (int64_t)v * stride;
    for (int w = 0; w < W; ++w) {
        uint32_t m = row[w];
        while (m) {
            int b = __ffs(m) - 1;
            m &= m - 1;
            int u = w * 32 + b;
            L[k++] = u;
            higher += u > v;
        }
    }
    deg[v] = k;
    node_cnt[v] = higher;
}

__device__ inline int find_pos(const int32_t *L, int len, int u) {
    int lo = 0, hi = len;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (L[mid] < u) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ inline uint64_t sat_binom(const uint64_t *btab, int na, int d, unsigned long long *unsup) {
    if (na < d) return 0;
    if (na >= kBinomN) {
        atomicAdd(unsup, 1ull);
        return 0;
    }
    uint64_t c = btab[(int64_t)na * kBinomK + d];
    if (c == ~0ull) {
        atomicAdd(unsup, 1ull);
        return 0;
    }
    return c;
}

__global__ void level_edges_kernel(int n, int d, const int32_t *adjl, int stride, const int32_t *deg,
                                   const int32_t *node_off, const uint64_t *btab, int32_t *ex, int32_t *ey,
                                   int32_t *pxy, int32_t *pyx, uint64_t *cntx, uint64_t *total, uint64_t *next,
                                   uint8_t *status, unsigned long long *stats) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int32_t *L = adjl + (int64_t)v * stride;
    int dv = deg[v];
    int64_t o = node_off[v];
    int start = find_pos(L, dv, v + 1);
    for (int k = start; k < dv; ++k, ++o) {
        int u = L[k];
        const int32_t *Lu = adjl + (int64_t)u * stride;
        ex[o] = v;
        ey[o] = u;
        pxy[o] = k;
        pyx[o] = find_pos(Lu, deg[u], v);
        uint64_t cx = sat_binom(btab, dv - 1, d, &stats[ST_UNSUPPORTED]);
        uint64_t cy = sat_binom(btab, deg[u] - 1, d, &stats[ST_UNSUPPORTED]);
        cntx[o] = cx;
        total[o] = cx + cy;
        next[o] = 0;
        status[o] = (cx + cy) == 0 ? kStatusKept : kStatusActive;
    }
}

__global__ void wave_plan_kernel(int n_edges, const uint8_t *status, const uint64_t *total, const uint64_t *next,
                                 int q, int32_t *g) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e > n_edges) return;
    if (e == n_edges) {
        g[e] = 0;
        return;
    }
    int v = 0;
    if (status[e] == kStatusActive) {
        uint64_t rem = total[e] - next[e];
        v = rem < (uint64_t)q ? (int)rem : q;
    }
    g[e] = v;
}

__global__ void wave_reduce_kernel(int n_edges, const int32_t *off, const uint8_t *flag, uint8_t *status,
                                   uint64_t *next, const uint64_t *total, uint64_t *seprank,
                                   unsigned long long *stats) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long bad = 0, exec = 0, det = 0, unresolved = 0;
    if (e < n_edges) {
        const int o = off[e], g = off[e + 1] - o;
        if (g > 0) {
            int first = -1;
            for (int k = 0; k < g; ++k) {
                const uint8_t f = flag[o + k];
                if (f == 2) bad = 1;
                if (f == 1) {
                    first = k;
                    break;
                }
            }
            exec = (unsigned long long)g;
            if (first >= 0) {
                status[e] = kStatusRemoved;
                seprank[e] = next[e] + first;
                det = (unsigned long long)(first + 1);
            } else {
                const uint64_t nx = next[e] + g;
                next[e] = nx;
                det = (unsigned long long)g;
                if (nx == total[e]) status[e] = kStatusKept;
                else unresolved = 1;
            }
        }
    }
    // one atomic per warp and counter: the level-0 wave has one edge per thread
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        bad += __shfl_xor_sync(0xffffffffu, bad, s);
        exec += __shfl_xor_sync(0xffffffffu, exec, s);
        det += __shfl_xor_sync(0xffffffffu, det, s);
        unresolved += __shfl_xor_sync(0xffffffffu, unresolved, s);
    }
    if ((threadIdx.x & 31) == 0) {
        if (bad) atomicAdd(&stats[ST_UNSUPPORTED], bad);
        if (exec) atomicAdd(&stats[ST_EXEC], exec);
        if (det) atomicAdd(&stats[ST_DET], det);
        if (unresolved) atomicAdd(&stats[ST_UNRESOLVED], unresolved);
    }
}

// apply removals, log (pair, sepset) -- sepset rebuilt from its rank
__global__ void level_finalize_kernel(int n_edges, int d, int W, const int32_t *ex, const int32_t *ey,
                                      const int32_t *pxy, const int32_t *pyx, const uint64_t *cntx,
                                      const uint64_t *seprank, const uint8_t *status, const int32_t *adjl,
                                      int stride, const int32_t *deg, const uint64_t *btab, uint32_t *bits,
                                      int32_t *log_pair, int32_t *log_meta, int32_t *log_vars, int64_t log_base,
                                      int64_t var_base, unsigned long long *stats) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_edges) return;
    if (status[e] != kStatusRemoved) return;
    const int x = ex[e], y = ey[e];
    atomicAnd(&bits[(int64_t)x * W + (y >> 5)], ~(1u << (y & 31)));
    atomicAnd(&bits[(int64_t)y * W + (x >> 5)], ~(1u << (x & 31)));
    const int64_t slot = (int64_t)atomicAdd(&stats[ST_REMOVED], 1ull);
    log_pair[2 * (log_base + slot)] = x;
    log_pair[2 * (log_base + slot) + 1] = y;
    log_meta[2 * (log_base + slot)] = d;
    log_meta[2 * (log_base + slot) + 1] = (int32_t)(var_base + slot * d);  // fits: checked by host
    if (d == 0) return;
    uint64_t rank = seprank[e];
    int side_node, skip;
    if (rank < cntx[e]) {
        side_node = x;
        skip = pxy[e];
    } else {
        rank -= cntx[e];
        side_node = y;
        skip = pyx[e];
    }
    int c[kMaxCond];
    unrank_lex(btab, deg[side_node] - 1, d, rank, c);
    const int32_t *L = adjl + (int64_t)side_node * stride;
    for (int k = 0; k < d; ++k) log_vars[var_base + slot * d + k] = L[c[k] < skip ? c[k] : c[k] + 1];
}

__global__ void degree_kernel(const uint32_t *bits, int n, int W, unsigned long long *stats) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    int dg = 0;
    for (int w = 0; w < W; ++w) dg += __popc(bits[(int64_t)v * W + w]);
    atomicMax(&stats[ST_MAXDEG], (unsigned long long)dg);
}

inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

// ---- result assembly: 0/1 adjacency, removal log sorted by pair
__global__ void expand_adj_kernel(const uint32_t *bits, int n, int W, uint8_t *adj) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)n * n) return;
    const int a = (int)(i / n), b = (int)(i - (int64_t)a * n);
    adj[i] = (uint8_t)((bits[(int64_t)a * W + (b >> 5)] >> (b & 31)) & 1u);
}

__global__ void log_keys_kernel(int R, int n, const int32_t *log_pair, uint32_t *key, int32_t *idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R) return;
    key[i] = (uint32_t)log_pair[2 * i] * (uint32_t)n + (uint32_t)log_pair[2 * i + 1];
    idx[i] = i;
}

// k-th record in pair order: its pair and its separating set's size (cnt[R] = 0 ends the scan)
__global__ void log_gather_kernel(int R, const int32_t *order, const int32_t *log_pair, const int32_t *log_meta,
                                  int32_t *removed, int32_t *cnt) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > R) return;
    if (k == R) {
        cnt[R] = 0;
        return;
    }
    const int i = order[k];
    removed[2 * k] = log_pair[2 * i];
    removed[2 * k + 1] = log_pair[2 * i + 1];
    cnt[k] = log_meta[2 * i];
}

__global__ void log_vars_kernel(int R, const int32_t *order, const int32_t *log_meta, const int32_t *log_vars,
                                const int32_t *off, int32_t *vars) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= R) return;
    const int i = order[k];
    const int dd = log_meta[2 * i], vo = log_meta[2 * i + 1];
    for (int t = 0; t < dd; ++t) vars[off[k] + t] = log_vars[vo + t];
}

// ---- device-driven wave loop (one CUDA graph per level: a WHILE conditional node whose body
// is one wave; the wave's tail kernel decides whether another wave runs)
struct WaveCtl {
    long long wave, q, n_waves;
    unsigned long long t_prev, count_ns, large_ns;
};
constexpr long long kMaxWaves = 1 << 20;  // bound on waves per level (each wave resolves >= 1 rank per edge)

// Start of a wave: q = ranks per unresolved edge this wave (the host loop's rule: doubling from
// 1, raised so the wave fills the GPU, capped by the item buffers), counters cleared.
__global__ void wave_prep_kernel(WaveCtl *c, unsigned long long *stats, int32_t *counters, long long n_active,
                                 long long ci_blocks, long long max_items) {
    if (threadIdx.x < 16) counters[threadIdx.x] = 0;
    if (threadIdx.x != 0) return;
    const long long unresolved = (long long)stats[ST_UNRESOLVED];
    stats[ST_UNRESOLVED] = 0;
    long long q = 1ll << (c->wave < 12 ? c->wave : 12);
    const long long target = ci_blocks * 64;
    if (unresolved > 0 && q * unresolved < target) {
        const long long r = (target + unresolved - 1) / unresolved;
        q = r < 4096 ? r : 4096;
    }
    const long long qmax = max_items / (n_active > 1 ? n_active : 1);
    q = q < qmax ? q : qmax;
    c->q = q > 1 ? q : 1;
}

__global__ void wave_plan_dev_kernel(int n_edges, const uint8_t *status, const uint64_t *total, const uint64_t *next,
                                     const WaveCtl *c, int32_t *g) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e > n_edges) return;
    if (e == n_edges) {
        g[e] = 0;
        return;
    }
    int v = 0;
    if (status[e] == kStatusActive) {
        const uint64_t q = (uint64_t)c->q, rem = total[e] - next[e];
        v = (int)(rem < q ? rem : q);
    }
    g[e] = v;
}

// Device clock between kernels of a wave: slot -1 marks the start of the counting kernels,
// 0 adds the shared-memory tiers' span, 1 the tier-2 kernels' span.
__global__ void wave_stamp_kernel(WaveCtl *c, int slot) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (slot == 0) c->count_ns += t - c->t_prev;
    if (slot == 1) c->large_ns += t - c->t_prev;
    c->t_prev = t;
}

__global__ void wave_tail_kernel(WaveCtl *c, const unsigned long long *stats, cudaGraphConditionalHandle h) {
    c->wave += 1;
    c->n_waves += 1;
    const bool more = stats[ST_UNRESOLVED] > 0 && stats[ST_UNSUPPORTED] == 0 && c->wave < kMaxWaves;
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

__global__ void wave_ctl_init_kernel(WaveCtl *c, unsigned long long *stats, long long n_active) {
    c->wave = c->q = c->n_waves = 0;
    c->t_prev = c->count_ns = c->large_ns = 0;
    stats[ST_UNRESOLVED] = (unsigned long long)n_active;
    stats[ST_BYTES_SHARED] = 0;
    stats[ST_BYTES_LARGE] = 0;
}

// Level 0 from the tensor-core Gram matrix (gram.cu): one warp per pair x < y (at level 0
// item e is edge e, one test each).  The pair's dx x dy block of G -- rows of x's states,
// columns of y's -- goes into the warp's shared slice, then the same scoring and decision
// as the counting tiers (score_dense, CellTable.cpp:430-455 / IndependenceTest.cpp:295-364).
__global__ void __launch_bounds__(kThreads) level0_gram_score_kernel(WaveArgs a, const int32_t *G, int ld,
                                                                     const int32_t *row_off, int n_items, int slice) {
    extern __shared__ int smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *tab = smem + warp * slice;  // slice: the largest pair table + marginals of this dataset
    const WarpGroup g{lane};
    for (int item = blockIdx.x * kWarps + warp; item < n_items; item += gridDim.x * kWarps) {
        const int x = a.ex[item], y = a.ey[item];
        const int dx = a.card[x], dy = a.card[y];
        const int cells = dx * dy;
        int *ni = tab + cells, *nj = ni + dx, *nk = nj + dy;
        const int32_t *src = G + (int64_t)row_off[x] * ld + row_off[y];
        // the block's rows: every lane's loads issued before any is stored
        for (int c0 = 0; c0 < cells; c0 += 128) {
            int v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int c = c0 + 32 * u + lane;
                const int i = c / dy, j = c - i * dy;
                v[u] = c < cells ? __ldg(src + (int64_t)i * ld + j) : 0;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (c0 + 32 * u + lane < cells) tab[c0 + 32 * u + lane] = v[u];
        }
        __syncwarp();
        const Verdict v = score_dense(g, tab, ni, nj, nk, dx, dy, 1, a.alpha, a.bt, a.detail != nullptr,
                                      a.want_hash != 0, nullptr);
        if (lane == 0) record(a, item, v, cells, a.want_hash ? table_hash(tab, cells) : 0, 0);
        __syncwarp();
    }
}

}  // namespace

// ------------------------------------------------------------------ engine setup
namespace {
// A fixed tier-2 method table in place of the online autotuner (FPGM_TUNE_TABLE=<file>, e.g.
// written by fastpgm_gb300/tune.py): lines "sb db cb method"; any entry not listed keeps the
// fixed cut-over.  FPGM_TUNE_TABLE=off keeps the fixed 65,536-sample cut-over alone.
int load_tune_table(fpgm_engine *e) {
    const char *env = getenv("FPGM_TUNE_TABLE");
    if (!env || !*env || strcmp(env, "off") == 0) {
        if (env && strcmp(env, "off") == 0) e->tune_online = false;  // the fixed cut-over alone
        return FPGM_OK;
    }
    const std::string path = env;
    FILE *f = fopen(path.c_str(), "r");
    if (!f) return set_error(FPGM_ERR_IO, "FPGM_TUNE_TABLE: cannot open %s", path.c_str());
    std::vector<int8_t> t((size_t)kTuneSB * kTuneDB * kTuneCB);
    for (int sb = 0; sb < kTuneSB; ++sb)
        for (int db = 0; db < kTuneDB; ++db)
            for (int cb = 0; cb < kTuneCB; ++cb) {
                const int64_t S_lo = sb == 0 ? 1 : (int64_t)12500 << (sb - 1);
                t[((size_t)sb * kTuneDB + db) * kTuneCB + cb] = S_lo >= e->part_min_samples ? 1 : 0;
            }
    char line[256];
    int entries = 0;
    while (fgets(line, sizeof line, f)) {
        if (line[0] == '#' || line[0] == '\n') continue;
        int sb, db, cb, m;
        if (sscanf(line, "%d %d %d %d", &sb, &db, &cb, &m) == 4 && sb >= 0 && sb < kTuneSB && db >= 0 &&
            db < kTuneDB && cb >= 0 && cb < kTuneCB && (m == 0 || m == 1)) {
            t[((size_t)sb * kTuneDB + db) * kTuneCB + cb] = (int8_t)m;
            ++entries;
        }
    }
    fclose(f);
    if (!entries) return FPGM_OK;
    RET(e->tune.ensure(t.size()));
    CK(cudaMemcpy(e->tune.p, t.data(), t.size(), cudaMemcpyHostToDevice));
    e->tune_loaded = true;
    e->tune_source = path;
    return FPGM_OK;
}
}  // namespace

extern "C" int fpgm_engine_create(int32_t device, fpgm_engine **out) {
    if (!out) return set_error(FPGM_ERR_INVALID, "fpgm_engine_create: out is NULL");
    *out = nullptr;
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev)
        return set_error(FPGM_ERR_INVALID, "fpgm_engine_create: device %d out of range (%d devices)", device, ndev);
    CK(cudaSetDevice(device));
    fpgm_engine *e = new fpgm_engine();
    e->device = device;
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, device));
    e->num_sms = prop.multiProcessorCount;
    CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&e->ev0));
    CK(cudaEventCreate(&e->ev1));
    CK(cudaEventCreate(&e->ev2));
    CK(cudaFuncSetAttribute(ci_warp_kernel<kWarpInts, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    CK(cudaFuncSetAttribute(ci_warp_kernel<kWarpIntsSmall, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            kWarps * kWarpIntsSmall * 4));
    CK(cudaFuncSetAttribute(ci_cta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    CK(cudaFuncSetAttribute(ci_compact_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    CK(cudaFuncSetAttribute(ci_compact_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    CK(cudaFuncSetAttribute(ci_part_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    CK(cudaFuncSetAttribute(ci_part_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    CK(cudaFuncSetAttribute(level0_gram_score_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    CK(cudaFuncSetAttribute(ci_plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    int occ = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ci_warp_kernel<kWarpInts, 2>, kThreads, kSmemBytes));
    e->ci_blocks = e->num_sms * std::max(1, occ);
    if (const char *w = getenv("FPGM_WARP_SLICE")) e->warp_small = atoi(w) != kWarpInts;
    if (const char *w = getenv("FPGM_DENSE_ROWS")) e->dense_rows = atoi(w) != 0;
    int occ_small = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_small, ci_warp_kernel<kWarpIntsSmall, 3>, kThreads,
                                                     kWarps * kWarpIntsSmall * 4));
    e->warp_blocks_small = e->num_sms * std::max(1, occ_small);
    // binomial table, saturating
    std::vector<uint64_t> bt((size_t)kBinomN * kBinomK, 0);
    for (int n = 0; n < kBinomN; ++n) {
        bt[(size_t)n * kBinomK] = 1;
        for (int k = 1; k < kBinomK; ++k) {
            if (n == 0) continue;
            uint64_t a = bt[(size_t)(n - 1) * kBinomK + k - 1], b = bt[(size_t)(n - 1) * kBinomK + k];
            uint64_t s = a + b;
            bt[(size_t)n * kBinomK + k] = (s < a || a == ~0ull || b == ~0ull) ? ~0ull : s;
        }
    }
    RET(e->btab.ensure(bt.size() * 8));
    CK(cudaMemcpy(e->btab.p, bt.data(), bt.size() * 8, cudaMemcpyHostToDevice));
    RET(e->counters.ensure(64));
    RET(e->stats.ensure(ST_COUNT * 8));
    e->wave_log = getenv("FPGM_WAVE_LOG") != nullptr;
    if (const char *pm = getenv("FPGM_PART_MAX_LOG")) e->part_max_log = std::min(kPartMaxLog, std::max(1, atoi(pm)));
    if (const char *w = getenv("FPGM_WIDE")) e->wide_on = atoi(w) != 0;
    if (const char *w = getenv("FPGM_GRAM")) e->gram_on = atoi(w) != 0;
    if (const char *w = getenv("FPGM_GRAPH")) e->graph_on = atoi(w) != 0;
    e->gram = gram_create();
    if (const char *w = getenv("FPGM_WIDE_N2")) e->wide_small_n2 = atoi(w);
    if (const char *w = getenv("FPGM_WIDE_MIN_LOG")) e->wide_min_log = std::min(kPartMaxLog, std::max(0, atoi(w)));
    if (const char *w = getenv("FPGM_WIDE_PART_MIN")) e->wide_part_min = std::max(64, atoi(w));
    if (const char *w = getenv("FPGM_WIDE_DIRECT")) e->wide_direct = atoi(w) != 0;
    if (const char *w = getenv("FPGM_PART_CUTOVER")) {
        e->part_min_samples = std::max<int64_t>(0, atoll(w));
        e->tune_online = false;
    }
    if (const char *w = getenv("FPGM_TUNE")) e->tune_online = e->tune_online && atoi(w) != 0;
    RET(load_tune_table(e));
    if (e->tune_online && !e->tune_loaded) {
        RET(e->tune_obs.ensure((size_t)kTuneBuckets * 8 * 8));
        CK(cudaMemset(e->tune_obs.p, 0, (size_t)kTuneBuckets * 8 * 8));
    }
    if (const char *w = getenv("FPGM_OVF_SKIP")) e->ovf_on = atoi(w) != 0;
    if (const char *w = getenv("FPGM_STAGE_REC")) e->stage_rec = std::max(0, atoi(w)) & ~7;
    if (const char *w = getenv("FPGM_LIVE")) e->live_on = atoi(w) != 0;
    if (const char *w = getenv("FPGM_LIVE_MIN_LEVEL")) e->live_min_level = std::max(1, atoi(w));
    if (const char *w = getenv("FPGM_LIVE_FRAC")) e->live_frac = atof(w);
    if (e->ovf_on) {
        RET(e->ovf.ensure((size_t)kTuneBuckets * 8 * 8));
        CK(cudaMemset(e->ovf.p, 0, (size_t)kTuneBuckets * 8 * 8));
    }
    if (getenv("FPGM_PHASE_TIMERS")) {
        RET(e->phase_timers.ensure(32 * 8));
        CK(cudaMemset(e->phase_timers.p, 0, 32 * 8));
    }
    *out = e;
    return FPGM_OK;
}

extern "C" int fpgm_engine_destroy(fpgm_engine *e) {
    if (!e) return FPGM_OK;
    cudaSetDevice(e->device);
    DevBuf *bufs[] = {&e->cols, &e->card, &e->btab, &e->bits, &e->deg, &e->adjl, &e->edges_x, &e->edges_y,
                      &e->pxy, &e->pyx, &e->cntx, &e->total, &e->next, &e->status, &e->seprank, &e->g,
                      &e->off, &e->flag, &e->counters, &e->stats, &e->scan_tmp, &e->log_pair,
                      &e->log_vars, &e->log_meta, &e->node_cnt, &e->node_off, &e->slots, &e->plain_ws,
                      &e->tests_buf, &e->detail_buf, &e->item_vars, &e->lists, &e->band,
                      &e->phase_timers, &e->var_off, &e->var_S, &e->var_lo, &e->var_hi, &e->mle_counts,
                      &e->mle_pot, &e->mle_meta, &e->wide, &e->wide_items, &e->tune, &e->wave_ctl,
                      &e->tune_obs, &e->ovf, &e->live_pool[0], &e->live_pool[1], &e->live_tab[0], &e->live_tab[1],
                      &e->live_cnt, &e->live_stat, &e->res_adj_d, &e->res_key, &e->res_idx, &e->res_removed_d, &e->res_cnt,
                      &e->res_vars_d};
    for (DevBuf *b : bufs) b->release();
    gram_destroy(e->gram);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->ev1) cudaEventDestroy(e->ev1);
    if (e->ev2) cudaEventDestroy(e->ev2);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return FPGM_OK;
}

namespace {
// Column layout of `jobs` datasets (variables in job order): offsets, samples, variable
// ranges on the host and the device, then the relabelling and the cardinality check.
// job_vars[j] variables of job_samples[j] samples each, column-major in cols[j].
int load_datasets(fpgm_engine *e, int32_t n_jobs, const int32_t *job_vars, const int64_t *job_samples,
                  const uint8_t *const *cols, int32_t relabel, uint8_t *out_card, const char *fn) {
    int64_t n = 0, bytes = 0, smax = 0, pairs = 0;
    for (int32_t j = 0; j < n_jobs; ++j) {
        if (!cols[j]) return set_error(FPGM_ERR_INVALID, "%s: NULL columns for dataset %d", fn, j);
        if (job_vars[j] < 2 || job_samples[j] < 1 || job_samples[j] > ((int64_t)1 << 31) - 16)
            return set_error(FPGM_ERR_INVALID, "%s: dataset %d has %d variables and %lld samples", fn, j, job_vars[j],
                             (long long)job_samples[j]);
        n += job_vars[j];
        bytes += (int64_t)job_vars[j] * ((job_samples[j] + 63) & ~(int64_t)63);
        smax = std::max<int64_t>(smax, job_samples[j]);
        pairs += (int64_t)job_vars[j] * (job_vars[j] - 1) / 2;
    }
    if (n > 65535) return set_error(FPGM_ERR_INVALID, "%s: %lld variables in all (at most 65535)", fn, (long long)n);
    CK(cudaSetDevice(e->device));
    e->n = 0;
    e->has_result = false;
    e->gram_planned = false;  // the one-hot layout follows the dataset
    e->n_jobs = n_jobs;
    e->S = smax;
    e->S_pad = (smax + 63) & ~(int64_t)63;
    e->E = pairs;
    e->h_var_off.resize(n);
    e->h_var_S.resize(n);
    e->h_var_lo.resize(n);
    e->h_var_hi.resize(n);
    RET(e->cols.ensure((size_t)bytes + 64));
    RET(e->card.ensure(std::max<size_t>(256, (size_t)n)));
    CK(cudaMemsetAsync(e->cols.p, 0, (size_t)bytes, e->stream));
    int64_t off = 0;
    int32_t v0 = 0;
    for (int32_t j = 0; j < n_jobs; ++j) {
        const int64_t Sj = job_samples[j], pitch = (Sj + 63) & ~(int64_t)63;
        CK(cudaMemcpy2DAsync(e->cols.as<uint8_t>() + off, (size_t)pitch, cols[j], (size_t)Sj, (size_t)Sj,
                             (size_t)job_vars[j], cudaMemcpyHostToDevice, e->stream));
        for (int32_t k = 0; k < job_vars[j]; ++k) {
            e->h_var_off[v0 + k] = off + k * pitch;
            e->h_var_S[v0 + k] = (int32_t)Sj;
            e->h_var_lo[v0 + k] = v0;
            e->h_var_hi[v0 + k] = v0 + job_vars[j];
        }
        off += job_vars[j] * pitch;
        v0 += job_vars[j];
    }
    RET(e->var_off.ensure((size_t)n * 8));
    RET(e->var_S.ensure((size_t)n * 4));
    RET(e->var_lo.ensure((size_t)n * 4));
    RET(e->var_hi.ensure((size_t)n * 4));
    CK(cudaMemcpyAsync(e->var_off.p, e->h_var_off.data(), (size_t)n * 8, cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync(e->var_S.p, e->h_var_S.data(), (size_t)n * 4, cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync(e->var_lo.p, e->h_var_lo.data(), (size_t)n * 4, cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync(e->var_hi.p, e->h_var_hi.data(), (size_t)n * 4, cudaMemcpyHostToDevice, e->stream));
    relabel_kernel<<<(int)n, 256, 0, e->stream>>>(e->cols.as<uint8_t>(), e->var_off.as<int64_t>(),
                                                  e->var_S.as<int32_t>(), e->card.as<uint8_t>(), relabel);
    CK(cudaGetLastError());
    e->h_card.resize(n);
    CK(cudaMemcpyAsync(e->h_card.data(), e->card.p, n, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    for (int64_t v = 0; v < n; ++v)
        if (e->h_card[v] == 0)  // 256 states wrap the uint8 cardinality to 0
            return set_error(FPGM_ERR_UNSUPPORTED, "%s: column %lld has 256 states; at most 255 are supported", fn,
                             (long long)v);
    e->n = (int)n;
    if (out_card) memcpy(out_card, e->h_card.data(), n);
    return FPGM_OK;
}
}  // namespace

extern "C" int fpgm_dataset_upload(fpgm_engine *e, const uint8_t *columns, int32_t n_vars, int64_t n_samples,
                                   int32_t relabel, uint8_t *out_card) {
    if (!e || !columns) return set_error(FPGM_ERR_INVALID, "fpgm_dataset_upload: NULL argument");
    if (n_vars < 2 || n_vars > 65535)
        return set_error(FPGM_ERR_INVALID, "fpgm_dataset_upload: n_vars %d outside [2, 65535]", n_vars);
    if (n_samples < 1 || n_samples > ((int64_t)1 << 31) - 16)
        return set_error(FPGM_ERR_INVALID, "fpgm_dataset_upload: n_samples %lld outside [1, 2^31-16]",
                         (long long)n_samples);
    return load_datasets(e, 1, &n_vars, &n_samples, &columns, relabel, out_card, "fpgm_dataset_upload");
}

extern "C" int fpgm_dataset_upload_jobs(fpgm_engine *e, int32_t n_jobs, const int32_t *job_vars,
                                        const int64_t *job_samples, const uint8_t *const *job_columns,
                                        int32_t relabel, uint8_t *out_card) {
    if (!e || !job_vars || !job_samples || !job_columns || n_jobs < 1)
        return set_error(FPGM_ERR_INVALID, "fpgm_dataset_upload_jobs: NULL argument or no dataset");
    return load_datasets(e, n_jobs, job_vars, job_samples, job_columns, relabel, out_card,
                         "fpgm_dataset_upload_jobs");
}

extern "C" int fpgm_dataset_download(fpgm_engine *e, uint8_t *columns) {
    if (!e || !columns) return set_error(FPGM_ERR_INVALID, "fpgm_dataset_download: NULL argument");
    if (!e->n) return set_error(FPGM_ERR_STATE, "fpgm_dataset_download: no dataset uploaded");
    if (e->n_jobs != 1)
        return set_error(FPGM_ERR_UNSUPPORTED, "fpgm_dataset_download: the engine holds %d datasets", e->n_jobs);
    CK(cudaSetDevice(e->device));
    CK(cudaMemcpy2DAsync(columns, (size_t)e->S, e->cols.p, (size_t)e->S_pad, (size_t)e->S, (size_t)e->n,
                         cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return FPGM_OK;
}

// ------------------------------------------------------------------ batched skeleton
namespace {

// Band-edge tables for alpha (cached per alpha).
int ensure_band(fpgm_engine *e, double alpha) {
    if (e->band_alpha == alpha && e->band.p) return FPGM_OK;
    RET(e->band.ensure((size_t)2 * (kBandDfMax + 1) * sizeof(double)));
    double *lo = e->band.as<double>(), *hi = lo + kBandDfMax + 1;
    band_table_kernel<<<blocks_for(kBandDfMax + 1, 128), 128, 0, e->stream>>>(alpha, lo, hi, kBandDfMax);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(e->stream));
    e->band_alpha = alpha;
    return FPGM_OK;
}

// Largest table + marginals a level-d test can need, from the largest cardinality m.
int64_t max_table_ints(const std::vector<uint8_t> &card, int d) {
    int64_t m = 1;
    for (uint8_t c : card) m = std::max<int64_t>(m, c);
    int64_t dz = 1;
    for (int k = 0; k < d; ++k) {
        dz *= m;
        if (dz > ((int64_t)1 << 36)) return (int64_t)1 << 40;
    }
    return dz * m * m + dz * (2 * m + 1);
}

// Global slots of the compact tier, allocated the first time a level can need them.
// The global strata hash must hold every sample's stratum at load <= 1/2, so it is
// resized whenever a dataset with more samples is uploaded.
int ensure_slots(fpgm_engine *e) {
    // The regions are laid out for slot_S samples and reused, as they are, for any dataset of
    // at most slot_S samples, so the regions kept zeroed between tests stay where they were.
    if (e->slots.p && e->S <= e->slot_S) return FPGM_OK;
    uint32_t cap = 4096;
    while ((int64_t)cap < 2 * e->S) cap <<= 1;
    e->slots.release();
    e->slot_S = e->S;
    e->hash_cap_global = (int)cap;
    e->n_slots = 2 * e->num_sms;
    e->slot_bytes = slot_layout(e->slot_S, cap).total;
    RET(e->slots.ensure((size_t)e->slot_bytes * e->n_slots));
    CK(cudaMemsetAsync(e->slots.p, 0, (size_t)e->slot_bytes * e->n_slots, e->stream));  // zeroed tables
    RET(e->wide.ensure((size_t)e->n_slots * sizeof(WideTest)));
    RET(e->wide_items.ensure((size_t)e->n_slots * kPartMax * 4));
    return FPGM_OK;
}

// Contributing-sample bitmaps for level d: the pools are made once (up to 32 GB or 30%
// of the free device memory; none when that fails), the pool of this level's parity gets an
// empty key table, and the other keeps the previous level's bitmaps for the readers.
int live_setup(fpgm_engine *e, int d) {
    e->live_write = false;
    if (!e->live_on || !e->live_next || d < e->live_min_level || max_table_ints(e->h_card, d) <= kCtaInts - 64)
        return FPGM_OK;
    if (e->live_cap > 0 && (e->S + 31) / 32 > e->live_words) {  // a larger dataset since: bigger bitmaps
        for (int q = 0; q < 2; ++q) {
            e->live_pool[q].release();
            e->live_tab[q].release();
        }
        e->live_cap = 0;
    }
    if (e->live_cap == 0) {
        const int64_t words = (e->S + 31) / 32;
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return FPGM_OK;
        const double budget = std::min(32.0e9, 0.3 * (double)free_b);
        int64_t cap = (int64_t)(budget / 2.0 / (double)(words * 4));
        cap = std::min<int64_t>(cap, (int64_t)1 << 21);
        if (cap < 1024) {
            e->live_on = false;
            return FPGM_OK;
        }
        int32_t tcap = 1024;
        while (tcap < 2 * cap) tcap <<= 1;
        for (int par = 0; par < 2; ++par) {
            if (e->live_pool[par].ensure((size_t)cap * words * 4) != FPGM_OK ||
                e->live_tab[par].ensure((size_t)tcap * sizeof(LiveKey)) != FPGM_OK) {
                for (int q = 0; q < 2; ++q) {
                    e->live_pool[q].release();
                    e->live_tab[q].release();
                }
                e->live_on = false;  // no room: every test counts all of its samples
                return FPGM_OK;
            }
        }
        RET(e->live_cnt.ensure(16));
        e->live_cap = cap;
        e->live_tab_cap = tcap;
        e->live_words = (int32_t)words;
    }
    const int par = d & 1;
    CK(cudaMemsetAsync(e->live_tab[par].p, 0, (size_t)e->live_tab_cap * sizeof(LiveKey), e->stream));
    CK(cudaMemsetAsync(e->live_cnt.as<int32_t>() + par, 0, 4, e->stream));
    e->live_level[par] = d;
    e->live_write = true;
    return FPGM_OK;
}

int wave_args_base(fpgm_engine *e, WaveArgs &a, double alpha, int d, int64_t items) {
    memset(&a, 0, sizeof a);
    a.cols = e->cols.as<uint8_t>();
    a.var_off = e->var_off.as<int64_t>();
    a.var_S = e->var_S.as<int32_t>();
    a.card = e->card.as<uint8_t>();
    a.d = d;
    a.btab = e->btab.as<uint64_t>();
    a.counters = e->counters.as<int32_t>();
    a.stats = e->stats.as<unsigned long long>();
    a.alpha = alpha;
    RET(ensure_band(e, alpha));
    a.bt.lo = e->band.as<double>();
    a.bt.hi = a.bt.lo + kBandDfMax + 1;
    a.bt.dfmax = kBandDfMax;
    RET(e->item_vars.ensure((size_t)std::max<int64_t>(items, 1) * (2 + d) * 2 + 16));
    RET(e->lists.ensure((size_t)6 * std::max<int64_t>(items, 1) * 4 + 16));
    RET(e->flag.ensure((size_t)std::max<int64_t>(items, 1) + 16));
    a.item_vars = e->item_vars.as<uint16_t>();
    a.lists = e->lists.as<int32_t>();
    a.list_cap = std::max<int64_t>(items, 1);
    a.flag = e->flag.as<uint8_t>();
    if (max_table_ints(e->h_card, d) > kCtaInts - 64) {
        RET(ensure_slots(e));
        a.slot_mem = e->slots.as<char>();
        a.slot_bytes = e->slot_bytes;
        a.slot_S = e->slot_S;
        a.hash_cap_global = e->hash_cap_global;
        if (e->wide_on) {
            a.wide = e->wide.as<WideTest>();
            a.wide_items = e->wide_items.as<int32_t>();
            a.wide_small_n2 = e->wide_small_n2 >= 0 ? e->wide_small_n2 : e->n_slots;
            a.wide_min_log = e->wide_min_log;
            a.wide_part_min = e->wide_part_min;
            a.wide_direct = e->wide_direct;
        }
        a.tune = e->tune_loaded ? e->tune.as<int8_t>() : nullptr;
        a.tune_obs = (e->tune_online && !e->tune_loaded) ? e->tune_obs.as<unsigned long long>() : nullptr;
        a.ovf = e->ovf_on ? e->ovf.as<unsigned long long>() : nullptr;
        a.part_min_samples = e->part_min_samples;
        if (e->live_on && e->live_in_skeleton && e->live_stat.p) a.live_stat = e->live_stat.as<unsigned long long>();
        if (e->live_on && e->live_in_skeleton && e->live_cap > 0 && d >= 1) {
            const int par = d & 1, prev = (d - 1) & 1;
            a.bm_words = e->live_words;
            if (e->live_write && e->live_level[par] == d) {
                a.bm_pool = e->live_pool[par].as<uint32_t>();
                a.bm_tab = e->live_tab[par].as<LiveKey>();
                a.bm_count = e->live_cnt.as<int32_t>() + par;
                a.bm_cap = (int32_t)e->live_cap;
                a.bm_tab_cap = e->live_tab_cap;
            }
            if (e->live_level[prev] == d - 1) {
                a.bm_prev_pool = e->live_pool[prev].as<uint32_t>();
                a.bm_prev_tab = e->live_tab[prev].as<LiveKey>();
                a.bm_prev_tab_cap = e->live_tab_cap;
            }
        }
    }
    a.part_max_log = e->part_max_log;
    a.warp_ints = e->warp_small ? kWarpIntsSmall : kWarpInts;
    a.dense_rows = e->dense_rows;
    a.stage_rec = e->stage_rec;
    return FPGM_OK;
}

// The warp tier (tier 0) with the engine's slice size.
void launch_warp_tier(fpgm_engine *e, const WaveArgs &a) {
    if (e->warp_small)
        ci_warp_kernel<kWarpIntsSmall, 3><<<e->warp_blocks_small, kThreads, kWarps * kWarpIntsSmall * 4, e->stream>>>(a);
    else
        ci_warp_kernel<kWarpInts, 2><<<e->ci_blocks, kThreads, kSmemBytes, e->stream>>>(a);
}

// Tier 2 on the current stream: the compact kernel, the partitioned kernel for the tests it
// hands over, and the compact kernel again for any the partitioned one hands back (each a
// persistent loop over its list; an empty list ends at once).  Returns launches issued.
int launch_compact(fpgm_engine *e, const WaveArgs &a, int grid) {
    ci_compact_kernel<false><<<grid, kThreads, kSmemBytes, e->stream>>>(a);
    ci_part_kernel<<<grid, kThreads, kSmemBytes, e->stream>>>(a);
    int n = 3;
    if (a.wide) {
        ci_part_wide_kernel<<<grid, kThreads, kSmemBytes, e->stream>>>(a);
        ++n;
    }
    ci_compact_kernel<true><<<grid, kThreads, kSmemBytes, e->stream>>>(a);
    return n;
}

// Classify + the three tiers on the current stream.  Returns launches issued.
template <int kSource>
int launch_tiers(fpgm_engine *e, const WaveArgs &a) {
    classify_kernel<kSource><<<e->ci_blocks, kThreads, 0, e->stream>>>(a);
    launch_warp_tier(e, a);
    ci_cta_kernel<<<e->ci_blocks, kThreads, kSmemBytes, e->stream>>>(a);
    int n = 3;
    if (a.slot_mem) n += launch_compact(e, a, e->n_slots);
    return n;
}

// One level's waves driven by the device: a CUDA graph whose WHILE conditional node runs the
// wave body (prep, plan, scan, classify, the counting tiers, reduce) until the tail kernel
// finds no unresolved edge.  The graph is captured and instantiated once per level (the
// level's edge count, |Z| and buffers are its parameters) and the host waits once per level.
int run_waves_graph(fpgm_engine *e, double alpha, int d, int64_t n_active, fpgm_pc_stats *st, int level_idx,
                    const WaveArgs &proto) {
    unsigned long long *dstat = e->stats.as<unsigned long long>();
    const int64_t cap = std::max<int64_t>(n_active, kMaxItems);  // items of one wave at most
    WaveArgs a = proto;
    RET(wave_args_base(e, a, alpha, d, cap));
    a.adjl = proto.adjl;
    a.adj_stride = proto.adj_stride;
    a.deg = proto.deg;
    a.ex = proto.ex;
    a.ey = proto.ey;
    a.pxy = proto.pxy;
    a.pyx = proto.pyx;
    a.cntx = proto.cntx;
    a.next = proto.next;
    a.off = e->off.as<int32_t>();
    a.n_edges = (int32_t)n_active;
    a.dbg = nullptr;
    size_t sb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, sb, e->g.as<int32_t>(), e->off.as<int32_t>(), (int)(n_active + 1),
                                  e->stream);
    RET(e->scan_tmp.ensure(sb + 16));
    sb = e->scan_tmp.bytes;
    RET(e->wave_ctl.ensure(sizeof(WaveCtl)));
    WaveCtl *ctl = e->wave_ctl.as<WaveCtl>();
    wave_ctl_init_kernel<<<1, 1, 0, e->stream>>>(ctl, dstat, (long long)n_active);
    CK(cudaGetLastError());
    const auto t0 = std::chrono::steady_clock::now();
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int per_wave = 0;
    auto build = [&]() -> int {
        CK(cudaGraphCreate(&graph, 0));
        cudaGraphConditionalHandle h;
        CK(cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault));
        alignas(cudaGraphNodeParams) unsigned char cp_raw[sizeof(cudaGraphNodeParams)] = {};
        cudaGraphNodeParams &cp = *reinterpret_cast<cudaGraphNodeParams *>(cp_raw);
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cn;
        CK(cudaGraphAddNode(&cn, graph, nullptr, nullptr, 0, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        CK(cudaStreamBeginCaptureToGraph(e->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
        wave_prep_kernel<<<1, 32, 0, e->stream>>>(ctl, dstat, e->counters.as<int32_t>(), (long long)n_active,
                                                  (long long)e->ci_blocks, (long long)kMaxItems);
        wave_plan_dev_kernel<<<blocks_for(n_active + 1, 256), 256, 0, e->stream>>>(
            (int)n_active, e->status.as<uint8_t>(), e->total.as<uint64_t>(), e->next.as<uint64_t>(), ctl,
            e->g.as<int32_t>());
        cub::DeviceScan::ExclusiveSum(e->scan_tmp.p, sb, e->g.as<int32_t>(), e->off.as<int32_t>(),
                                      (int)(n_active + 1), e->stream);
        wave_stamp_kernel<<<1, 1, 0, e->stream>>>(ctl, -1);
        classify_kernel<SRC_WAVE><<<e->ci_blocks, kThreads, 0, e->stream>>>(a);
        launch_warp_tier(e, a);
        ci_cta_kernel<<<e->ci_blocks, kThreads, kSmemBytes, e->stream>>>(a);
        wave_stamp_kernel<<<1, 1, 0, e->stream>>>(ctl, 0);
        per_wave = 9;  // prep, plan, 3 stamps, classify, warp tier, CTA tier, reduce, tail (+ tier 2)
        if (a.slot_mem) per_wave += launch_compact(e, a, e->n_slots);
        wave_stamp_kernel<<<1, 1, 0, e->stream>>>(ctl, 1);
        wave_reduce_kernel<<<blocks_for(n_active, 256), 256, 0, e->stream>>>(
            (int)n_active, e->off.as<int32_t>(), e->flag.as<uint8_t>(), e->status.as<uint8_t>(),
            e->next.as<uint64_t>(), e->total.as<uint64_t>(), e->seprank.as<uint64_t>(), dstat);
        wave_tail_kernel<<<1, 1, 0, e->stream>>>(ctl, dstat, h);
        const cudaError_t le = cudaGetLastError();
        const cudaError_t ce = cudaStreamEndCapture(e->stream, &body);
        if (le != cudaSuccess) return set_error(FPGM_ERR_CUDA, "level %d graph capture: %s", d, cudaGetErrorString(le));
        CK(ce);
        CK(cudaGraphInstantiate(&exec, graph, 0));
        return FPGM_OK;
    };
    int rc = build();
    st->graph_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (rc == FPGM_OK) {
        const cudaError_t le = cudaGraphLaunch(exec, e->stream);
        if (le != cudaSuccess) rc = set_error(FPGM_ERR_CUDA, "cudaGraphLaunch: %s", cudaGetErrorString(le));
    }
    WaveCtl hc;
    unsigned long long hs[ST_COUNT];
    if (rc == FPGM_OK) {
        cudaError_t ce = cudaMemcpyAsync(&hc, ctl, sizeof hc, cudaMemcpyDeviceToHost, e->stream);
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(hs, dstat, sizeof hs, cudaMemcpyDeviceToHost, e->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
        if (ce != cudaSuccess) rc = set_error(FPGM_ERR_CUDA, "level %d graph: %s", d, cudaGetErrorString(ce));
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (rc != FPGM_OK) return rc;
    if (hs[ST_UNSUPPORTED])
        return set_error(FPGM_ERR_UNSUPPORTED,
                         "level %d: %llu CI test(s) are outside the engine's limits (joint table beyond 2^62 "
                         "cells or a node degree >= %d)",
                         d, hs[ST_UNSUPPORTED], kBinomN);
    if (hs[ST_UNRESOLVED]) return set_error(FPGM_ERR_STATE, "level %d: wave limit reached with edges unresolved", d);
    st->waves[level_idx] = (int32_t)hc.n_waves;
    st->count_ms += hc.count_ns / 1e6;
    st->large_ms += hc.large_ns / 1e6;
    st->count_bytes += (double)hs[ST_BYTES_SHARED];
    st->large_bytes += (double)hs[ST_BYTES_LARGE];
    st->count_launches += hc.n_waves;
    st->kernel_launches += 1 + hc.n_waves * per_wave;  // + the control-block init
    return FPGM_OK;
}

int run_waves_and_count(fpgm_engine *e, double alpha, int d, int64_t n_active, fpgm_pc_stats *st, int level_idx,
                        const WaveArgs &proto, bool gram = false) {
    if (d >= 1 && e->graph_on && !e->wave_log && !e->phase_timers.p)
        return run_waves_graph(e, alpha, d, n_active, st, level_idx, proto);
    unsigned long long *dstat = e->stats.as<unsigned long long>();
    int wave = 0;
    int64_t unresolved = n_active;
    size_t scan_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, e->g.as<int32_t>(), e->off.as<int32_t>(),
                                  (int)(n_active + 1), e->stream);
    RET(e->scan_tmp.ensure(scan_bytes + 16));
    while (unresolved > 0) {
        int64_t q = (int64_t)1 << std::min(wave, 12);
        const int64_t target = (int64_t)e->ci_blocks * 64;
        if (q * unresolved < target) q = std::min<int64_t>(4096, (target + unresolved - 1) / unresolved);
        if (d == 0) q = 1;
        q = std::max<int64_t>(1, std::min<int64_t>(q, kMaxItems / std::max<int64_t>(1, n_active)));
        const int64_t items = std::max<int64_t>(q * n_active, 1);
        WaveArgs a = proto;
        RET(wave_args_base(e, a, alpha, d, items));
        a.adjl = proto.adjl;
        a.adj_stride = proto.adj_stride;
        a.deg = proto.deg;
        a.ex = proto.ex;
        a.ey = proto.ey;
        a.pxy = proto.pxy;
        a.pyx = proto.pyx;
        a.cntx = proto.cntx;
        a.next = proto.next;
        wave_plan_kernel<<<blocks_for(n_active + 1, 256), 256, 0, e->stream>>>(
            (int)n_active, e->status.as<uint8_t>(), e->total.as<uint64_t>(), e->next.as<uint64_t>(), (int)q,
            e->g.as<int32_t>());
        CK(cudaGetLastError());
        size_t sb = e->scan_tmp.bytes;
        CK(cub::DeviceScan::ExclusiveSum(e->scan_tmp.p, sb, e->g.as<int32_t>(), e->off.as<int32_t>(),
                                         (int)(n_active + 1), e->stream));
        CK(cudaMemsetAsync(e->counters.p, 0, 64, e->stream));
        CK(cudaMemsetAsync(dstat + ST_BYTES_SHARED, 0, 16, e->stream));  // this wave's bytes
        a.off = e->off.as<int32_t>();
        a.n_edges = (int32_t)n_active;
        CK(cudaEventRecord(e->ev0, e->stream));
        if (gram) {  // level 0: every pair's table from the tensor-core Gram matrix (one wave, one test per edge)
            int nl = 0;
            RET(gram_run(e->gram, e->stream, dstat + ST_TIMEOUT, &nl));
            const int slice = gram_slice_ints(e->gram);
            level0_gram_score_kernel<<<e->num_sms * e->gram_score_ctas, kThreads, kWarps * slice * 4, e->stream>>>(
                a, gram_counts(e->gram), gram_ld(e->gram), gram_row_off(e->gram), (int)n_active, slice);
            CK(cudaGetLastError());
            st->kernel_launches += nl + 3;  // plan, one-hot + GEMM, scoring, reduce
        } else {
            classify_kernel<SRC_WAVE><<<e->ci_blocks, kThreads, 0, e->stream>>>(a);
            launch_warp_tier(e, a);
            ci_cta_kernel<<<e->ci_blocks, kThreads, kSmemBytes, e->stream>>>(a);
            CK(cudaGetLastError());
            st->kernel_launches += 5;  // plan, classify, warp tier, CTA tier, reduce
        }
        CK(cudaEventRecord(e->ev1, e->stream));
        a.dbg = e->phase_timers.as<unsigned long long>();
        if (a.slot_mem && !gram) {
            st->kernel_launches += launch_compact(e, a, e->n_slots);
            CK(cudaGetLastError());
        }
        if (a.dbg) {  // FPGM_PHASE_TIMERS: per-wave breakdown of the compact tier on stderr
            unsigned long long h[32];
            CK(cudaMemcpyAsync(h, a.dbg, sizeof h, cudaMemcpyDeviceToHost, e->stream));

            CK(cudaMemsetAsync(a.dbg, 0, sizeof h, e->stream));
            CK(cudaStreamSynchronize(e->stream));
            if (h[23]) fprintf(stderr, "partition-parallel d=%d tests=%llu\n", d, h[23]);
            if (h[27])
                fprintf(stderr, "staged d=%llu records=%llu re-split=%llu big strata=%llu holding %llu samples\n",
                        (unsigned long long)d, h[27], h[24], h[25], h[26]);
            if (h[29])
                fprintf(stderr, "bitmaps d=%llu tests-with-parent=%llu writing=%llu samples=%llu kept=%llu (%.3f)\n",
                        (unsigned long long)d, h[28], h[31], h[29], h[30], (double)h[30] / (double)h[29]);
            if (h[13])
                fprintf(stderr,
                        "partitioned d=%d tests=%llu strata/test=%.0f partitions/test=%.1f us/test: records=%.1f "
                        "counted+scored=%.1f [clear=%.1f insert=%.1f scan=%.1f place=%.1f small=%.1f big=%.1f]\n",
                        d, h[13], (double)h[9] / h[13], (double)h[22] / h[13], h[14] / 1e3 / h[13],
                        h[15] / 1e3 / h[13], h[16] / 1e3 / h[13], h[17] / 1e3 / h[13], h[18] / 1e3 / h[13],
                        h[19] / 1e3 / h[13], h[20] / 1e3 / h[13], h[21] / 1e3 / h[13]);
            if (h[11])
                fprintf(stderr,
                        "compact d=%d tests=%llu strata/test=%.0f us/test: shared-hash=%.1f global-hash=%.1f "
                        "count=%.1f sort=%.1f small=%.1f big=%.1f | dense tests=%llu scatter=%.1f score=%.1f | "
                        "decide=%.1f\n",
                        d, h[11], (double)h[10] / h[11], h[0] / 1e3 / h[11], h[1] / 1e3 / h[11], h[2] / 1e3 / h[11],
                        h[3] / 1e3 / h[11], h[4] / 1e3 / h[11], h[5] / 1e3 / h[11], h[12], h[7] / 1e3 / h[11],
                        h[8] / 1e3 / h[11], h[6] / 1e3 / h[11]);
        }
        CK(cudaEventRecord(e->ev2, e->stream));
        CK(cudaMemsetAsync(dstat + ST_UNRESOLVED, 0, 8, e->stream));
        wave_reduce_kernel<<<blocks_for(n_active, 256), 256, 0, e->stream>>>(
            (int)n_active, e->off.as<int32_t>(), e->flag.as<uint8_t>(), e->status.as<uint8_t>(),
            e->next.as<uint64_t>(), e->total.as<uint64_t>(), e->seprank.as<uint64_t>(), dstat);
        CK(cudaGetLastError());
        unsigned long long hs[ST_COUNT];
        int32_t T = 0, tiers[C_COUNT];
        CK(cudaMemcpyAsync(hs, dstat, sizeof hs, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaMemcpyAsync(&T, e->off.as<int32_t>() + n_active, 4, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaMemcpyAsync(tiers, e->counters.p, sizeof tiers, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        float ms = 0.f, ms2 = 0.f;
        CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
        CK(cudaEventElapsedTime(&ms2, e->ev1, e->ev2));
        if (gram) {
            st->gram_ms += ms;
            st->gram_flops += gram_flops(e->gram);
            st->gram_tests += n_active;
        } else {
            st->count_ms += ms;
        }
        st->large_ms += ms2;
        // algorithmic bytes: (2 + d) columns of the test's samples per test, split by kernel
        st->count_bytes += (double)hs[ST_BYTES_SHARED];
        st->large_bytes += (double)hs[ST_BYTES_LARGE];
        if (!gram) st->count_launches += 1;
        if (hs[ST_TIMEOUT])
            return set_error(FPGM_ERR_TIMEOUT, "level %d: a bounded wait of the tensor-core level-0 kernel gave up", d);
        if (e->wave_log)
            fprintf(stderr,
                    "wave level=%d tests=%d tier0=%d tier1=%d tier2=%d (partitioned=%d parallel=%d retried=%d) "
                    "compact_launched=%d count_ms=%.4f compact_ms=%.4f count_bytes=%.0f compact_bytes=%.0f\n",
                    d, T, tiers[C_TIER0], tiers[C_TIER1], tiers[C_TIER2], tiers[C_PART], tiers[C_WIDET], tiers[C_RETRY],
                    a.slot_mem != nullptr, ms, ms2, (double)hs[ST_BYTES_SHARED], (double)hs[ST_BYTES_LARGE]);
        if (hs[ST_UNSUPPORTED])
            return set_error(FPGM_ERR_UNSUPPORTED,
                             "level %d: %llu CI test(s) are outside the engine's limits (joint table beyond 2^62 "
                             "cells or a node degree >= %d)",
                             d, hs[ST_UNSUPPORTED], kBinomN);
        unresolved = (int64_t)hs[ST_UNRESOLVED];
        ++wave;
    }
    st->waves[level_idx] = wave;
    return FPGM_OK;
}

int run_batched(fpgm_engine *e, double alpha, int depth, fpgm_pc_stats *st) {
    const int n = e->n;
    const int W = (n + 31) / 32;
    const int64_t E = e->E;  // level-0 pairs (within each dataset)
    unsigned long long *dstat = e->stats.as<unsigned long long>();
    CK(cudaMemsetAsync(dstat, 0, ST_COUNT * 8, e->stream));
    // bitmaps live only inside this skeleton: none carries over to a later call (the data may change)
    struct LiveScope {
        fpgm_engine *e;
        explicit LiveScope(fpgm_engine *x) : e(x) {
            e->live_level[0] = e->live_level[1] = -1;
            e->live_write = false;
            e->live_in_skeleton = true;
        }
        ~LiveScope() {
            e->live_level[0] = e->live_level[1] = -1;
            e->live_write = false;
            e->live_in_skeleton = false;
        }
    } live_scope(e);
    if (e->live_on) {  // contributing-sample counts, measured level by level
        RET(e->live_stat.ensure(16));
        CK(cudaMemsetAsync(e->live_stat.p, 0, 16, e->stream));
        e->live_prev[0] = e->live_prev[1] = 0ull;
        e->live_next = false;
    }
    RET(e->bits.ensure((size_t)n * W * 4));
    init_bits_kernel<<<blocks_for((int64_t)n * W, 256), 256, 0, e->stream>>>(
        e->bits.as<uint32_t>(), n, W, e->var_lo.as<int32_t>(), e->var_hi.as<int32_t>());
    CK(cudaGetLastError());
    st->kernel_launches += 1;
    RET(e->log_pair.ensure((size_t)E * 8 + 16));
    RET(e->log_meta.ensure((size_t)E * 8 + 16));
    RET(e->log_vars.ensure((size_t)1 << 20));
    RET(e->deg.ensure((size_t)n * 4 + 16));
    RET(e->node_cnt.ensure((size_t)(n + 1) * 4));
    RET(e->node_off.ensure((size_t)(n + 1) * 4));
    int64_t log_count = 0, var_count = 0;
    int max_deg = 0;  // largest dataset - 1
    for (int v = 0; v < n; ++v) max_deg = std::max(max_deg, e->h_var_hi[v] - e->h_var_lo[v] - 1);
    bool more = true;
    st->n_levels = 0;
    for (int d = 0; (d == 0 || d < depth) && d < 64; ++d) {  // level 0 always runs (PCStable.cpp:133-177)
        if (d >= 2 && !more) break;
        auto t0 = std::chrono::steady_clock::now();
        if (d > kMaxCond)
            return set_error(FPGM_ERR_UNSUPPORTED, "conditioning sets beyond %d variables are not supported",
                             kMaxCond);
        int64_t n_active;
        int stride = 1;
        if (d == 0 && e->n_jobs == 1) {
            n_active = E;
        } else {  // the level's snapshot (several datasets: also at level 0)
            stride = std::max(1, max_deg);
            RET(e->adjl.ensure((size_t)n * stride * 4));
            csr_kernel<<<blocks_for(n, 128), 128, 0, e->stream>>>(e->bits.as<uint32_t>(), n, W, e->adjl.as<int32_t>(),
                                                                 stride, e->deg.as<int32_t>(),
                                                                 e->node_cnt.as<int32_t>());
            CK(cudaGetLastError());
            st->kernel_launches += 1;
            CK(cudaMemsetAsync(e->node_cnt.as<int32_t>() + n, 0, 4, e->stream));
            size_t sb = 0;
            cub::DeviceScan::ExclusiveSum(nullptr, sb, e->node_cnt.as<int32_t>(), e->node_off.as<int32_t>(), n + 1,
                                          e->stream);
            RET(e->scan_tmp.ensure(sb + 16));
            sb = e->scan_tmp.bytes;
            CK(cub::DeviceScan::ExclusiveSum(e->scan_tmp.p, sb, e->node_cnt.as<int32_t>(), e->node_off.as<int32_t>(),
                                             n + 1, e->stream));
            int32_t na = 0;
            CK(cudaMemcpyAsync(&na, e->node_off.as<int32_t>() + n, 4, cudaMemcpyDeviceToHost, e->stream));
            CK(cudaStreamSynchronize(e->stream));
            n_active = na;
        }
        const size_t ne = (size_t)std::max<int64_t>(n_active, 1) + 1;
        RET(e->edges_x.ensure(ne * 4));
        RET(e->edges_y.ensure(ne * 4));
        RET(e->pxy.ensure(ne * 4));
        RET(e->pyx.ensure(ne * 4));
        RET(e->cntx.ensure(ne * 8));
        RET(e->total.ensure(ne * 8));
        RET(e->next.ensure(ne * 8));
        RET(e->seprank.ensure(ne * 8));
        RET(e->status.ensure(ne));
        RET(e->g.ensure(ne * 4));
        RET(e->off.ensure(ne * 4));
        if (n_active > 0) {
            if (d == 0 && e->n_jobs == 1) {
                level0_edges_kernel<<<blocks_for(E, 256), 256, 0, e->stream>>>(
                    n, e->edges_x.as<int32_t>(), e->edges_y.as<int32_t>(), e->pxy.as<int32_t>(),
                    e->pyx.as<int32_t>(), e->cntx.as<uint64_t>(), e->total.as<uint64_t>(), e->next.as<uint64_t>(),
                    e->status.as<uint8_t>());
            } else if (d == 0) {
                level0_csr_edges_kernel<<<blocks_for(n, 128), 128, 0, e->stream>>>(
                    n, e->adjl.as<int32_t>(), stride, e->deg.as<int32_t>(), e->node_off.as<int32_t>(),
                    e->edges_x.as<int32_t>(), e->edges_y.as<int32_t>(), e->pxy.as<int32_t>(), e->pyx.as<int32_t>(),
                    e->cntx.as<uint64_t>(), e->total.as<uint64_t>(), e->next.as<uint64_t>(),
                    e->status.as<uint8_t>());
            } else {
                level_edges_kernel<<<blocks_for(n, 128), 128, 0, e->stream>>>(
                    n, d, e->adjl.as<int32_t>(), stride, e->deg.as<int32_t>(), e->node_off.as<int32_t>(),
                    e->btab.as<uint64_t>(), e->edges_x.as<int32_t>(), e->edges_y.as<int32_t>(), e->pxy.as<int32_t>(),
                    e->pyx.as<int32_t>(), e->cntx.as<uint64_t>(), e->total.as<uint64_t>(), e->next.as<uint64_t>(),
                    e->status.as<uint8_t>(), dstat);
            }
            CK(cudaGetLastError());
            st->kernel_launches += 1;
            CK(cudaMemsetAsync(dstat + ST_DET, 0, 8 * 2, e->stream));
            WaveArgs a;
            memset(&a, 0, sizeof a);
            a.adjl = e->adjl.as<int32_t>();
            a.adj_stride = stride;
            a.deg = e->deg.as<int32_t>();
            a.ex = e->edges_x.as<int32_t>();
            a.ey = e->edges_y.as<int32_t>();
            a.pxy = e->pxy.as<int32_t>();
            a.pyx = e->pyx.as<int32_t>();
            a.cntx = e->cntx.as<uint64_t>();
            a.next = e->next.as<uint64_t>();
            bool gram = false;
            if (d == 0 && e->n_jobs == 1 && e->gram_on) {
                if (!e->gram_planned) {
                    RET(gram_plan(e->gram, n, e->h_card.data(), e->S, e->cols.as<uint8_t>(), e->var_off.as<int64_t>(),
                                  e->card.as<uint8_t>(), e->num_sms, e->stream, &e->gram_ok));
                    e->gram_planned = true;
                    if (e->gram_ok) {
                        int occ = 0;
                        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, level0_gram_score_kernel, kThreads,
                                                                         kWarps * gram_slice_ints(e->gram) * 4));
                        e->gram_score_ctas = std::max(1, occ);
                    }
                }
                gram = e->gram_ok;
            }
            if (!gram) RET(live_setup(e, d));
            RET(run_waves_and_count(e, alpha, d, n_active, st, st->n_levels, a, gram));
            if (e->live_on && e->live_stat.p) {
                // Bitmaps pay for themselves when the next level can leave enough samples out:
                // the next level writes them when this one's partition-path tests had fewer than
                // live_frac of their samples in contributing strata (the fraction falls with |Z|).
                unsigned long long ls[2];
                CK(cudaMemcpyAsync(ls, e->live_stat.p, 16, cudaMemcpyDeviceToHost, e->stream));
                CK(cudaStreamSynchronize(e->stream));
                const unsigned long long din = ls[0] - e->live_prev[0], dall = ls[1] - e->live_prev[1];
                e->live_prev[0] = ls[0];
                e->live_prev[1] = ls[1];
                e->live_next = dall > 0 && (double)din < e->live_frac * (double)dall;
                if (e->wave_log && dall > 0)
                    fprintf(stderr, "live level=%d contributing=%.3f wrote=%d next_writes=%d\n", d,
                            (double)din / (double)dall, (int)e->live_write, (int)e->live_next);
            }
        }
        // finalize: removals into the bitset and the removal log
        RET(e->log_vars.ensure((size_t)(var_count + std::max<int64_t>(n_active, 1) * std::max(d, 1)) * 4 + 16, true,
                               e->stream));
        if (var_count + n_active * (int64_t)d > INT32_MAX)
            return set_error(FPGM_ERR_UNSUPPORTED, "separating-set storage beyond 2^31 entries");
        CK(cudaMemsetAsync(dstat + ST_REMOVED, 0, 16, e->stream));
        if (n_active > 0) {
            level_finalize_kernel<<<blocks_for(n_active, 256), 256, 0, e->stream>>>(
                (int)n_active, d, W, e->edges_x.as<int32_t>(), e->edges_y.as<int32_t>(), e->pxy.as<int32_t>(),
                e->pyx.as<int32_t>(), e->cntx.as<uint64_t>(), e->seprank.as<uint64_t>(), e->status.as<uint8_t>(),
                e->adjl.as<int32_t>(), stride, e->deg.as<int32_t>(), e->btab.as<uint64_t>(), e->bits.as<uint32_t>(),
                e->log_pair.as<int32_t>(), e->log_meta.as<int32_t>(), e->log_vars.as<int32_t>(), log_count, var_count,
                dstat);
            CK(cudaGetLastError());
            st->kernel_launches += 1;
        }
        degree_kernel<<<blocks_for(n, 128), 128, 0, e->stream>>>(e->bits.as<uint32_t>(), n, W, dstat);
        CK(cudaGetLastError());
        st->kernel_launches += 1;
        unsigned long long hs[ST_COUNT];
        CK(cudaMemcpyAsync(hs, dstat, sizeof hs, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        const int64_t removed = (int64_t)hs[ST_REMOVED];
        log_count += removed;
        var_count += removed * d;
        max_deg = (int)hs[ST_MAXDEG];
        const int li = st->n_levels;
        st->tests[li] = n_active > 0 ? (int64_t)hs[ST_DET] : 0;
        st->tests_executed[li] = n_active > 0 ? (int64_t)hs[ST_EXEC] : 0;
        st->edges_after[li] = (int32_t)(n_active - removed);
        st->ms[li] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        st->n_levels++;
        more = (max_deg - 1) > d;  // PCStable.cpp:387 (evaluated after levels >= 1)
    }
    // global statistics
    unsigned long long hs[ST_COUNT];
    CK(cudaMemcpyAsync(hs, dstat, sizeof hs, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    st->rechecks = (int64_t)hs[ST_RECHECK];
    st->near_ties = (int64_t)hs[ST_NEARTIE];
    st->large_tests = (int64_t)hs[ST_LARGE];
    unsigned long long mdp = hs[ST_MAXDP];
    double dp;
    memcpy(&dp, &mdp, 8);
    st->max_abs_dp = dp;
    if (e->tune_online && e->tune_obs.p) {  // what the online autotuner has learnt so far
        std::vector<unsigned long long> o((size_t)kTuneBuckets * 8);
        CK(cudaMemcpyAsync(o.data(), e->tune_obs.p, o.size() * 8, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        for (int b = 0; b < kTuneBuckets; ++b) {
            const unsigned long long *q = &o[(size_t)8 * b];
            st->tune_timed += (int64_t)(q[0] + q[2]);
            if (q[0] && q[2]) {
                ++st->tune_buckets;
                if ((double)q[1] / q[0] <= (double)q[3] / q[2]) ++st->tune_partition;
            }
        }
    }
    // result, assembled on the device: the 0/1 adjacency expanded from the bitset, and the
    // removal log sorted by pair (a < b, ascending) with each separating set gathered in that
    // order; the host only copies it back
    RET(e->res_adj_d.ensure((size_t)n * n + 16));
    expand_adj_kernel<<<blocks_for((int64_t)n * n, 256), 256, 0, e->stream>>>(e->bits.as<uint32_t>(), n, W,
                                                                             e->res_adj_d.as<uint8_t>());
    CK(cudaGetLastError());
    st->kernel_launches += 1;
    const int R = (int)log_count;
    if (R > 0) {
        RET(e->res_key.ensure((size_t)R * 4 * 2 + 16));
        RET(e->res_idx.ensure((size_t)R * 4 * 2 + 16));
        RET(e->res_removed_d.ensure((size_t)R * 8 + 16));
        RET(e->res_cnt.ensure((size_t)(R + 1) * 4 * 2 + 16));
        RET(e->res_vars_d.ensure((size_t)var_count * 4 + 16));
        uint32_t *k0 = e->res_key.as<uint32_t>(), *k1 = k0 + R;
        int32_t *i0 = e->res_idx.as<int32_t>(), *i1 = i0 + R;
        int32_t *cnt = e->res_cnt.as<int32_t>(), *off = cnt + R + 1;
        log_keys_kernel<<<blocks_for(R, 256), 256, 0, e->stream>>>(R, n, e->log_pair.as<int32_t>(), k0, i0);
        CK(cudaGetLastError());
        int bits = 1;
        while (bits < 32 && ((uint64_t)1 << bits) < (uint64_t)n * n) ++bits;
        size_t sb = 0;
        CK(cub::DeviceRadixSort::SortPairs(nullptr, sb, k0, k1, i0, i1, R, 0, bits, e->stream));
        size_t sb2 = 0;
        CK(cub::DeviceScan::ExclusiveSum(nullptr, sb2, cnt, off, R + 1, e->stream));
        RET(e->scan_tmp.ensure(std::max(sb, sb2) + 16));
        sb = e->scan_tmp.bytes;
        CK(cub::DeviceRadixSort::SortPairs(e->scan_tmp.p, sb, k0, k1, i0, i1, R, 0, bits, e->stream));
        log_gather_kernel<<<blocks_for(R + 1, 256), 256, 0, e->stream>>>(R, i1, e->log_pair.as<int32_t>(),
                                                                     e->log_meta.as<int32_t>(),
                                                                     e->res_removed_d.as<int32_t>(), cnt);
        CK(cudaGetLastError());
        sb2 = e->scan_tmp.bytes;
        CK(cub::DeviceScan::ExclusiveSum(e->scan_tmp.p, sb2, cnt, off, R + 1, e->stream));
        if (var_count > 0) {
            log_vars_kernel<<<blocks_for(R, 256), 256, 0, e->stream>>>(R, i1, e->log_meta.as<int32_t>(),
                                                                       e->log_vars.as<int32_t>(), off,
                                                                       e->res_vars_d.as<int32_t>());
            CK(cudaGetLastError());
        }
        st->kernel_launches += 3;
    }
    e->res_adj.resize((size_t)n * n);
    e->res_removed.resize((size_t)R * 2);
    e->res_off.assign((size_t)R + 1, 0);
    e->res_vars.resize((size_t)var_count);
    CK(cudaMemcpyAsync(e->res_adj.data(), e->res_adj_d.p, (size_t)n * n, cudaMemcpyDeviceToHost, e->stream));
    if (R > 0) {
        CK(cudaMemcpyAsync(e->res_removed.data(), e->res_removed_d.p, (size_t)R * 8, cudaMemcpyDeviceToHost,
                           e->stream));
        CK(cudaMemcpyAsync(e->res_off.data(), e->res_cnt.as<int32_t>() + R + 1, (size_t)(R + 1) * 4,
                           cudaMemcpyDeviceToHost, e->stream));
        if (var_count)
            CK(cudaMemcpyAsync(e->res_vars.data(), e->res_vars_d.p, (size_t)var_count * 4, cudaMemcpyDeviceToHost,
                               e->stream));
    }
    CK(cudaStreamSynchronize(e->stream));
    return FPGM_OK;
}

// ------------------------------------------------------------------ plain path
int plain_grid(const fpgm_engine *e, int64_t S) {
    int64_t nvec = S >> 4;
    int64_t g = nvec / kThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, e->ci_blocks));
}

int plain_test(fpgm_engine *e, int x, int y, const int *z, int d, double alpha, int want_hash,
               fpgm_ci_result *out, fpgm_pc_stats *st = nullptr) {
    if (!e->plain_ws.p) {
        RET(e->plain_ws.ensure((size_t)kPlainInts * 4 + 64));
        CK(cudaMemsetAsync(e->plain_ws.p, 0, e->plain_ws.bytes, e->stream));
    }
    RET(e->detail_buf.ensure(sizeof(fpgm_ci_result) * 64));
    RET(ensure_band(e, alpha));
    // table size decides: dense grid-wide kernel, or the compact-strata kernel on one CTA
    double cells = (double)e->h_card[x] * e->h_card[y], dz = 1.0;
    for (int k = 0; k < d; ++k) dz *= e->h_card[z[k]];
    cells *= dz;
    const double need = cells + dz * (e->h_card[x] + e->h_card[y] + 1);
    if (need <= (double)kPlainInts) {
        PlainArgs p;
        memset(&p, 0, sizeof p);
        p.cols = e->cols.as<uint8_t>();
        p.S = e->h_var_S[x];
        p.card = e->card.as<uint8_t>();
        p.ncols = d + 2;
        for (int k = 0; k < d; ++k) p.vars[k] = z[k];
        p.vars[d] = x;
        p.vars[d + 1] = y;
        for (int k = 0; k < d + 2; ++k) p.col_off[k] = e->h_var_off[p.vars[k]];
        p.alpha = alpha;
        p.bt.lo = e->band.as<double>();
        p.bt.hi = p.bt.lo + kBandDfMax + 1;
        p.bt.dfmax = kBandDfMax;
        p.want_hash = want_hash;
        p.gtab = e->plain_ws.as<int32_t>();
        p.done = reinterpret_cast<int32_t *>(e->plain_ws.as<char>() + (size_t)kPlainInts * 4);
        p.out = e->detail_buf.as<fpgm_ci_result>();
        p.stats = e->stats.as<unsigned long long>();
        ci_plain_kernel<<<plain_grid(e, p.S), kThreads, kSmemBytes, e->stream>>>(p);
        CK(cudaGetLastError());
    } else {
        WaveArgs a;
        RET(wave_args_base(e, a, alpha, d, 1));
        RET(ensure_slots(e));
        a.slot_mem = e->slots.as<char>();
        a.slot_bytes = e->slot_bytes;
        a.slot_S = e->slot_S;
        a.hash_cap_global = e->hash_cap_global;
        a.wide = nullptr;  // the single test stays on its one CTA
        a.detail = e->detail_buf.as<fpgm_ci_result>();
        a.want_hash = want_hash;
        uint16_t iv[kMaxCols];
        for (int k = 0; k < d; ++k) iv[k] = (uint16_t)z[k];
        iv[d] = (uint16_t)x;
        iv[d + 1] = (uint16_t)y;
        int32_t ctr[C_COUNT] = {};
        ctr[C_TIER2] = 1;
        int32_t zero = 0;
        CK(cudaMemcpyAsync(a.item_vars, iv, (d + 2) * 2, cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemcpyAsync(a.lists + 2 * a.list_cap, &zero, 4, cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemcpyAsync(a.counters, ctr, sizeof ctr, cudaMemcpyHostToDevice, e->stream));
        const int n = launch_compact(e, a, 1);
        CK(cudaGetLastError());
        if (st) st->kernel_launches += n - 1;
    }
    if (st) st->kernel_launches += 1;
    CK(cudaMemcpyAsync(out, e->detail_buf.p, sizeof(fpgm_ci_result), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return FPGM_OK;
}

bool next_combination(std::vector<int> &c, int a, int b) {
    int i = b - 1;
    while (i >= 0 && c[i] == a - b + i) --i;
    if (i < 0) return false;
    c[i]++;
    for (int j = i + 1; j < b; ++j) c[j] = c[j - 1] + 1;
    return true;
}

int run_plain(fpgm_engine *e, double alpha, int depth, fpgm_pc_stats *st) {
    const int n = e->n;
    unsigned long long *dstat = e->stats.as<unsigned long long>();
    CK(cudaMemsetAsync(dstat, 0, ST_COUNT * 8, e->stream));
    std::vector<uint8_t> adj((size_t)n * n, 0);  // complete graph within each dataset
    for (int i = 0; i < n; ++i)
        for (int j = e->h_var_lo[i]; j < e->h_var_hi[i]; ++j) adj[(size_t)i * n + j] = i != j;
    struct Rem { int a, b; std::vector<int> z; };
    std::vector<Rem> rem;
    fpgm_ci_result r;
    auto t0 = std::chrono::steady_clock::now();
    int64_t tests = 0;
    std::vector<std::pair<int, int>> kill;
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < e->h_var_hi[i]; ++j) {
            RET(plain_test(e, i, j, nullptr, 0, alpha, 0, &r, st));
            ++tests;
            if (r.independent) {
                kill.push_back({i, j});
                rem.push_back({i, j, {}});
            }
        }
    for (auto &k : kill) adj[(size_t)k.first * n + k.second] = adj[(size_t)k.second * n + k.first] = 0;
    int64_t edges = e->E - (int64_t)kill.size();
    st->n_levels = 1;
    st->tests[0] = st->tests_executed[0] = tests;
    st->edges_after[0] = (int32_t)edges;
    st->ms[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    bool more = true;
    std::vector<uint8_t> snap;
    std::vector<int> cand, c, z;
    for (int d = 1; d < depth && d < 64 && more; ++d) {
        if (d > kMaxCond) return set_error(FPGM_ERR_UNSUPPORTED, "conditioning sets beyond %d variables", kMaxCond);
        t0 = std::chrono::steady_clock::now();
        snap = adj;
        kill.clear();
        tests = 0;
        for (int x = 0; x < n; ++x)
            for (int y = x + 1; y < n; ++y) {
                if (!snap[(size_t)x * n + y]) continue;
                bool found = false;
                for (int side = 0; side < 2 && !found; ++side) {
                    int a = side == 0 ? x : y, b = side == 0 ? y : x;
                    cand.clear();
                    for (int v = 0; v < n; ++v)
                        if (v != b && snap[(size_t)a * n + v]) cand.push_back(v);
                    if ((int)cand.size() < d) continue;
                    c.resize(d);
                    z.resize(d);
                    for (int k = 0; k < d; ++k) c[k] = k;
                    do {
                        for (int k = 0; k < d; ++k) z[k] = cand[c[k]];
                        RET(plain_test(e, x, y, z.data(), d, alpha, 0, &r, st));
                        ++tests;
                        if (r.independent) {
                            found = true;
                            kill.push_back({x, y});
                            rem.push_back({x, y, z});
                            break;
                        }
                    } while (next_combination(c, (int)cand.size(), d));
                }
            }
        for (auto &k : kill) adj[(size_t)k.first * n + k.second] = adj[(size_t)k.second * n + k.first] = 0;
        edges -= (int64_t)kill.size();
        int maxdeg = 0;
        for (int i = 0; i < n; ++i) {
            int dg = 0;
            for (int j = 0; j < n; ++j) dg += adj[(size_t)i * n + j];
            maxdeg = std::max(maxdeg, dg);
        }
        const int li = st->n_levels;
        st->tests[li] = st->tests_executed[li] = tests;
        st->edges_after[li] = (int32_t)edges;
        st->ms[li] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        st->n_levels++;
        more = (maxdeg - 1) > d;
    }
    unsigned long long hs[ST_COUNT];
    CK(cudaMemcpyAsync(hs, dstat, sizeof hs, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    st->rechecks = (int64_t)hs[ST_RECHECK];
    st->near_ties = (int64_t)hs[ST_NEARTIE];
    unsigned long long mdp = hs[ST_MAXDP];
    memcpy(&st->max_abs_dp, &mdp, 8);
    std::sort(rem.begin(), rem.end(), [](const Rem &p, const Rem &q) { return p.a != q.a ? p.a < q.a : p.b < q.b; });
    e->res_adj = adj;
    e->res_removed.clear();
    e->res_off.assign(1, 0);
    e->res_vars.clear();
    for (auto &q : rem) {
        e->res_removed.push_back(q.a);
        e->res_removed.push_back(q.b);
        for (int v : q.z) e->res_vars.push_back(v);
        e->res_off.push_back((int32_t)e->res_vars.size());
    }
    return FPGM_OK;
}

}  // namespace

// ------------------------------------------------------------------ parameter learning
// Maximum-likelihood tables with Laplace smoothing for a known DAG
// (ParameterLearning::LearnParamsKnowStructCompData, parameter_learning/ParameterLearning.cpp:22-86):
// node v's table is over (v, parents ascending), v slowest (PotentialTableBase.cpp:102-130).
namespace {
struct MleNode {
    int64_t off;    // table offset in the counts / potentials
    int32_t np;     // parents
    int32_t par0;   // first parent in the parent list
    int32_t cum0;   // parent configurations (table size / card[v])
    int32_t smem;   // 1: the table fits in shared memory
};

// One CTA per (node, slice of its samples): every sample's configuration code (Horner,
// node first) counted in a shared-memory copy of the table when it fits, else in global
// memory directly; 16 samples per thread step from 128-bit column loads.
__global__ void __launch_bounds__(kThreads) mle_count_kernel(const uint8_t *cols, const int64_t *var_off,
                                                             const int32_t *var_S, const uint8_t *card,
                                                             const MleNode *nodes, const int32_t *parents,
                                                             int32_t *counts) {
    extern __shared__ int smem[];
    __shared__ const uint8_t *s_col[kMaxCols];
    __shared__ uint32_t s_dim[kMaxCols];
    const int v = blockIdx.x;
    const MleNode nd = nodes[v];
    const int ncols = nd.np + 1;
    const int64_t S = var_S[v];
    if (threadIdx.x < ncols) {
        const int var = threadIdx.x == 0 ? v : parents[nd.par0 + threadIdx.x - 1];
        s_col[threadIdx.x] = cols + var_off[var];
        s_dim[threadIdx.x] = card[var];
    }
    const int64_t size = (int64_t)nd.cum0 * card[v];
    int32_t *tab = nd.smem ? smem : counts + nd.off;
    if (nd.smem)
        for (int64_t i = threadIdx.x; i < size; i += blockDim.x) smem[i] = 0;
    __syncthreads();
    const int64_t nvec = S >> 4;
    const int64_t per = (nvec + gridDim.y - 1) / gridDim.y;
    const int64_t v0 = min(nvec, per * blockIdx.y), v1 = min(nvec, v0 + per);
    for (int64_t q = v0 + threadIdx.x; q < v1; q += blockDim.x) {
        uint32_t code[16];
#pragma unroll
        for (int b = 0; b < 16; ++b) code[b] = 0;
        for (int j = 0; j < ncols; ++j) {
            const uint4 w = __ldg(reinterpret_cast<const uint4 *>(s_col[j]) + q);
            const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
            const uint32_t dm = s_dim[j];
#pragma unroll
            for (int b = 0; b < 16; ++b) code[b] = code[b] * dm + ((ww[b >> 2] >> (8 * (b & 3))) & 0xffu);
        }
#pragma unroll
        for (int b = 0; b < 16; ++b) atomicAdd(&tab[code[b]], 1);
    }
    if (blockIdx.y == gridDim.y - 1)  // the ragged tail
        for (int64_t s = (S & ~(int64_t)15) + threadIdx.x; s < S; s += blockDim.x) {
            uint32_t c = 0;
            for (int j = 0; j < ncols; ++j) c = c * s_dim[j] + s_col[j][s];
            atomicAdd(&tab[c], 1);
        }
    if (nd.smem) {
        __syncthreads();
        for (int64_t i = threadIdx.x; i < size; i += blockDim.x)
            if (smem[i]) atomicAdd(&counts[nd.off + i], smem[i]);
    }
}

// potential[j] = (N[j] + alpha) / (N(B of j) + alpha * card[v]), the reference's expression
// (ParameterLearning.cpp:73-83) in FP64; N(B) sums the node's states for j's parent configuration.
__global__ void mle_prob_kernel(const uint8_t *card, const MleNode *nodes, const int32_t *counts, int alpha,
                                double *pot) {
    const int v = blockIdx.x;
    const MleNode nd = nodes[v];
    const int dv = card[v];
    const int64_t size = (int64_t)nd.cum0 * dv;
    for (int64_t j = threadIdx.x; j < size; j += blockDim.x) {
        const int64_t b = j % nd.cum0;
        int num2 = 0;
        for (int a = 0; a < dv; ++a) num2 += counts[nd.off + (int64_t)a * nd.cum0 + b];
        const int num1 = counts[nd.off + j];
        pot[nd.off + j] = ((double)num1 + alpha) / ((double)num2 + alpha * dv);
    }
}
}  // namespace

extern "C" int fpgm_mle_cpts(fpgm_engine *e, const int32_t *parent_off, const int32_t *parents, int32_t alpha,
                             int64_t *table_off, double *potentials) {
    if (!e || !parent_off || !table_off) return set_error(FPGM_ERR_INVALID, "fpgm_mle_cpts: NULL argument");
    if (!e->n) return set_error(FPGM_ERR_STATE, "fpgm_mle_cpts: no dataset uploaded");
    if (alpha < 0) return set_error(FPGM_ERR_INVALID, "fpgm_mle_cpts: alpha %d < 0", alpha);
    const int n = e->n;
    if (parent_off[0] != 0) return set_error(FPGM_ERR_INVALID, "fpgm_mle_cpts: parent_off[0] must be 0");
    std::vector<MleNode> nodes(n);
    int64_t total = 0;
    table_off[0] = 0;
    for (int v = 0; v < n; ++v) {
        const int np = parent_off[v + 1] - parent_off[v];
        if (np < 0 || np > kMaxCols - 1 || (np > 0 && !parents))
            return set_error(FPGM_ERR_INVALID, "fpgm_mle_cpts: node %d has %d parents (at most %d)", v, np,
                             kMaxCols - 1);
        double cum0 = 1.0;
        for (int k = 0; k < np; ++k) {
            const int p = parents[parent_off[v] + k];
            if (p < 0 || p >= n || p == v || e->h_var_lo[p] != e->h_var_lo[v] ||
                (k > 0 && p <= parents[parent_off[v] + k - 1]))
                return set_error(FPGM_ERR_INVALID,
                                 "fpgm_mle_cpts: parents of node %d must be other variables of its dataset, ascending",
                                 v);
            cum0 *= e->h_card[p];
        }
        const double size = cum0 * e->h_card[v];
        if (size > (double)((int64_t)1 << 30))
            return set_error(FPGM_ERR_UNSUPPORTED, "fpgm_mle_cpts: node %d's table has %.0f entries (at most 2^30)", v,
                             size);
        nodes[v].off = total;
        nodes[v].np = np;
        nodes[v].par0 = parent_off[v];
        nodes[v].cum0 = (int32_t)cum0;
        nodes[v].smem = size <= (double)(kSmemBytes / 4);
        total += (int64_t)size;
        table_off[v + 1] = total;
    }
    if (!potentials) return FPGM_OK;
    CK(cudaSetDevice(e->device));
    const int64_t npar = std::max<int64_t>(parent_off[n], 1);
    RET(e->mle_meta.ensure(sizeof(MleNode) * n + npar * 4 + 64));
    RET(e->mle_counts.ensure((size_t)total * 4 + 16));
    RET(e->mle_pot.ensure((size_t)total * 8 + 16));
    MleNode *d_nodes = e->mle_meta.as<MleNode>();
    int32_t *d_par = reinterpret_cast<int32_t *>(e->mle_meta.as<char>() + (sizeof(MleNode) * n + 15) / 16 * 16);
    CK(cudaMemcpyAsync(d_nodes, nodes.data(), sizeof(MleNode) * n, cudaMemcpyHostToDevice, e->stream));
    if (parent_off[n] > 0)
        CK(cudaMemcpyAsync(d_par, parents, (size_t)parent_off[n] * 4, cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemsetAsync(e->mle_counts.p, 0, (size_t)total * 4, e->stream));
    // slices per node: enough CTAs to fill the GPU, at least 64 vectors each
    int64_t smax = 0;
    for (int v = 0; v < n; ++v) smax = std::max<int64_t>(smax, e->h_var_S[v]);
    const int want = std::max(1, (4 * e->num_sms + n - 1) / n);
    const int slices = (int)std::max<int64_t>(1, std::min<int64_t>(want, (smax >> 4) / 64));
    CK(cudaFuncSetAttribute(mle_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    mle_count_kernel<<<dim3(n, slices), kThreads, kSmemBytes, e->stream>>>(
        e->cols.as<uint8_t>(), e->var_off.as<int64_t>(), e->var_S.as<int32_t>(), e->card.as<uint8_t>(), d_nodes, d_par,
        e->mle_counts.as<int32_t>());
    CK(cudaGetLastError());
    mle_prob_kernel<<<n, kThreads, 0, e->stream>>>(e->card.as<uint8_t>(), d_nodes, e->mle_counts.as<int32_t>(), alpha,
                                                  e->mle_pot.as<double>());
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(potentials, e->mle_pot.p, (size_t)total * 8, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return FPGM_OK;
}

// ------------------------------------------------------------------ C ABI: tests and skeleton
extern "C" int fpgm_ci_test(fpgm_engine *e, int32_t x, int32_t y, const int32_t *z, int32_t nz, double alpha,
                            int32_t want_hash, fpgm_ci_result *out) {
    if (!e || !out || (nz > 0 && !z)) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test: NULL argument");
    if (!e->n) return set_error(FPGM_ERR_STATE, "fpgm_ci_test: no dataset uploaded");
    if (!(alpha >= 0.0 && alpha <= 1.0))
        return set_error(FPGM_ERR_INVALID, "Error with incorrect significance level alpha!");
    if (nz < 0 || nz > kMaxCond) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test: |Z| = %d outside [0, %d]", nz, kMaxCond);
    if (x < 0 || x >= e->n || y < 0 || y >= e->n) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test: variable out of range");
    for (int k = 0; k < nz; ++k)
        if (z[k] < 0 || z[k] >= e->n) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test: variable out of range");
    for (int k = 0; k < nz; ++k)
        if (e->h_var_lo[z[k]] != e->h_var_lo[x])
            return set_error(FPGM_ERR_INVALID, "fpgm_ci_test: the variables belong to different datasets");
    if (e->h_var_lo[y] != e->h_var_lo[x])
        return set_error(FPGM_ERR_INVALID, "fpgm_ci_test: the variables belong to different datasets");
    CK(cudaSetDevice(e->device));
    return plain_test(e, x, y, z, nz, alpha, want_hash, out);
}

extern "C" int fpgm_ci_test_batch(fpgm_engine *e, const int32_t *tests, int32_t n_tests, int32_t d, double alpha,
                                  int32_t want_hash, fpgm_ci_result *out) {
    if (!e || !out || (n_tests > 0 && !tests)) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_batch: NULL argument");
    if (!e->n) return set_error(FPGM_ERR_STATE, "fpgm_ci_test_batch: no dataset uploaded");
    if (!(alpha >= 0.0 && alpha <= 1.0))
        return set_error(FPGM_ERR_INVALID, "Error with incorrect significance level alpha!");
    if (d < 0 || d > kMaxCond) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_batch: d = %d outside [0, %d]", d, kMaxCond);
    if (n_tests < 0 || n_tests > (1 << 26)) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_batch: n_tests out of range");
    if (n_tests == 0) return FPGM_OK;
    for (int64_t i = 0; i < (int64_t)n_tests * (2 + d); ++i)
        if (tests[i] < 0 || tests[i] >= e->n) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_batch: variable out of range");
    for (int64_t t = 0; t < n_tests; ++t)
        for (int k = 1; k < 2 + d; ++k)
            if (e->h_var_lo[tests[t * (2 + d) + k]] != e->h_var_lo[tests[t * (2 + d)]])
                return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_batch: test %lld mixes datasets", (long long)t);
    CK(cudaSetDevice(e->device));
    RET(e->tests_buf.ensure((size_t)n_tests * (2 + d) * 4));
    RET(e->detail_buf.ensure((size_t)n_tests * sizeof(fpgm_ci_result)));
    CK(cudaMemcpyAsync(e->tests_buf.p, tests, (size_t)n_tests * (2 + d) * 4, cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemsetAsync(e->counters.p, 0, 64, e->stream));
    CK(cudaMemsetAsync(e->stats.p, 0, ST_COUNT * 8, e->stream));
    WaveArgs a;
    RET(wave_args_base(e, a, alpha, d, n_tests));
    a.tests = e->tests_buf.as<int32_t>();
    a.n_tests = n_tests;
    a.detail = e->detail_buf.as<fpgm_ci_result>();
    a.want_hash = want_hash;
    launch_tiers<SRC_EXPLICIT>(e, a);
    CK(cudaGetLastError());
    unsigned long long hs[ST_COUNT];
    CK(cudaMemcpyAsync(out, a.detail, (size_t)n_tests * sizeof(fpgm_ci_result), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaMemcpyAsync(hs, e->stats.p, sizeof hs, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    if (hs[ST_UNSUPPORTED])
        return set_error(FPGM_ERR_UNSUPPORTED, "%llu CI test(s) need a joint table beyond 2^62 cells",
                         hs[ST_UNSUPPORTED]);
    return FPGM_OK;
}

extern "C" int fpgm_pc_skeleton(fpgm_engine *e, double alpha, int32_t depth, int32_t mode, fpgm_pc_stats *stats) {
    if (!e) return set_error(FPGM_ERR_INVALID, "fpgm_pc_skeleton: NULL engine");
    if (!e->n) return set_error(FPGM_ERR_STATE, "fpgm_pc_skeleton: no dataset uploaded");
    if (!(alpha >= 0.0 && alpha <= 1.0))
        return set_error(FPGM_ERR_INVALID, "Error with incorrect significance level alpha!");
    if (mode != FPGM_MODE_BATCHED && mode != FPGM_MODE_PLAIN)
        return set_error(FPGM_ERR_INVALID, "fpgm_pc_skeleton: unknown mode %d", mode);
    if (e->n > 16384 && mode == FPGM_MODE_BATCHED)
        return set_error(FPGM_ERR_UNSUPPORTED, "fpgm_pc_skeleton: %d nodes exceed the 16384-node limit", e->n);
    CK(cudaSetDevice(e->device));
    fpgm_pc_stats local;
    fpgm_pc_stats *st = stats ? stats : &local;
    memset(st, 0, sizeof *st);
    e->has_result = false;
    cudaEvent_t span0, span1;
    CK(cudaEventCreate(&span0));
    CK(cudaEventCreate(&span1));
    CK(cudaStreamSynchronize(e->stream));
    auto t0 = std::chrono::steady_clock::now();
    CK(cudaEventRecord(span0, e->stream));
    int rc = mode == FPGM_MODE_BATCHED ? run_batched(e, alpha, depth, st) : run_plain(e, alpha, depth, st);
    if (rc == FPGM_OK) {
        CK(cudaEventRecord(span1, e->stream));
        CK(cudaEventSynchronize(span1));
        float sp = 0.f;
        CK(cudaEventElapsedTime(&sp, span0, span1));
        st->span_ms = sp;
    }
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    cudaEventDestroy(span0);
    cudaEventDestroy(span1);
    if (rc == FPGM_OK) e->has_result = true;
    return rc;
}

extern "C" int fpgm_pc_result_sizes(fpgm_engine *e, int32_t *n_nodes, int32_t *n_removed, int64_t *n_sep_vars) {
    if (!e) return set_error(FPGM_ERR_INVALID, "fpgm_pc_result_sizes: NULL engine");
    if (!e->has_result) return set_error(FPGM_ERR_STATE, "fpgm_pc_result_sizes: no skeleton result");
    if (n_nodes) *n_nodes = e->n;
    if (n_removed) *n_removed = (int32_t)(e->res_removed.size() / 2);
    if (n_sep_vars) *n_sep_vars = (int64_t)e->res_vars.size();
    return FPGM_OK;
}

extern "C" int fpgm_pc_result_fetch(fpgm_engine *e, uint8_t *adj, int32_t *removed, int32_t *sep_offsets,
                                    int32_t *sep_vars) {
    if (!e) return set_error(FPGM_ERR_INVALID, "fpgm_pc_result_fetch: NULL engine");
    if (!e->has_result) return set_error(FPGM_ERR_STATE, "fpgm_pc_result_fetch: no skeleton result");
    if (adj) memcpy(adj, e->res_adj.data(), e->res_adj.size());
    if (removed && !e->res_removed.empty()) memcpy(removed, e->res_removed.data(), e->res_removed.size() * 4);
    if (sep_offsets) memcpy(sep_offsets, e->res_off.data(), e->res_off.size() * 4);
    if (sep_vars && !e->res_vars.empty()) memcpy(sep_vars, e->res_vars.data(), e->res_vars.size() * 4);
    return FPGM_OK;
}

// ------------------------------------------------------------------ CI test without allocation
// For callers that cannot allocate device memory: a process whose device memory
// is owned by another allocator (a host framework's caching pool or a fixed
// arena), or code running where a cudaMalloc would synchronise the device or is
// not allowed.  Such a caller already holds its samples on the device and wants
// one G^2 test on them.  This entry point uses only the fixed scratch array
// below, which every GPU that loads the library holds until the process exits,
// and calls no cudaMalloc, cudaFree or allocating library routine.
namespace {

constexpr int64_t kNoAllocTableInts = (int64_t)1 << 20;  // table + marginals: 4 MB
constexpr int kNoAllocMaxVars = 65536;
// [table + marginals | done counter + pad | cardinality per variable | stats]
constexpr int64_t kNoAllocDoneOff = kNoAllocTableInts;                    // ints
constexpr int64_t kNoAllocCardOff = kNoAllocTableInts + 64;               // ints
constexpr int64_t kNoAllocStatsOff = kNoAllocCardOff + kNoAllocMaxVars / 4;  // ints (8-byte aligned)
constexpr int64_t kNoAllocInts = kNoAllocStatsOff + 2 * ST_COUNT + 64;

static __device__ __align__(256) int32_t g_noalloc_scratch[kNoAllocInts];

struct NoAllocDevice {
    bool ready = false;
    int32_t *scratch = nullptr;  // device address of g_noalloc_scratch on this device
    int num_sms = 0;
};
std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[64];

// Largest id + 1 of each listed column (the cardinality of dense ids).
__global__ void noalloc_card_kernel(const uint8_t *columns, int64_t pitch, int64_t S, PlainArgs p, uint8_t *card) {
    __shared__ unsigned s_max;
    const int var = p.vars[blockIdx.x];
    if (threadIdx.x == 0) s_max = 0;
    __syncthreads();
    const uint8_t *c = columns + (int64_t)var * pitch;
    unsigned m = 0;
    for (int64_t s = threadIdx.x; s < S; s += blockDim.x) m = max(m, (unsigned)c[s]);
    atomicMax(&s_max, m);
    __syncthreads();
    if (threadIdx.x == 0) card[var] = (uint8_t)(s_max + 1);
}

// Per device, with that device current: resolve the scratch array's device
// address (the host-side symbol is only a stand-in) and prepare the kernel.
int noalloc_setup(int dev, NoAllocDevice **out) {
    if (dev < 0 || dev >= 64) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (!d.ready) {
        void *p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        CK(cudaFuncSetAttribute(ci_plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
        CK(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev));
        d.scratch = static_cast<int32_t *>(p);
        d.ready = true;
    }
    *out = &d;
    return FPGM_OK;
}

}  // namespace

extern "C" int fpgm_ci_test_noalloc(const uint8_t *columns, int64_t pitch, int32_t n_vars, int64_t n_samples,
                                    int32_t x, int32_t y, const int32_t *z, int32_t nz, double alpha,
                                    int32_t want_hash, fpgm_ci_result *result, void *stream) {
    if (!columns || !result || (nz > 0 && !z)) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_noalloc: NULL argument");
    if (reinterpret_cast<uintptr_t>(result) % alignof(fpgm_ci_result) != 0)
        return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_noalloc: result must be %zu-byte aligned",
                         alignof(fpgm_ci_result));
    if (!(alpha >= 0.0 && alpha <= 1.0))
        return set_error(FPGM_ERR_INVALID, "Error with incorrect significance level alpha!");
    if (n_vars < 2 || n_vars > kNoAllocMaxVars || n_samples < 1 || n_samples > ((int64_t)1 << 31) - 16)
        return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_noalloc: n_vars %d / n_samples %lld out of range", n_vars,
                         (long long)n_samples);
    if (pitch < n_samples || pitch % 16 != 0 || reinterpret_cast<uintptr_t>(columns) % 16 != 0)
        return set_error(FPGM_ERR_INVALID,
                         "fpgm_ci_test_noalloc: columns must be 16-byte aligned with a pitch that is a multiple of 16 "
                         "and >= n_samples");
    if (nz < 0 || nz > kMaxCond) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_noalloc: |Z| = %d outside [0, %d]", nz, kMaxCond);
    if (x < 0 || x >= n_vars || y < 0 || y >= n_vars)
        return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_noalloc: variable out of range");
    for (int k = 0; k < nz; ++k)
        if (z[k] < 0 || z[k] >= n_vars) return set_error(FPGM_ERR_INVALID, "fpgm_ci_test_noalloc: variable out of range");
    int dev = 0;
    CK(cudaGetDevice(&dev));
    NoAllocDevice *nd = nullptr;
    RET(noalloc_setup(dev, &nd));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int32_t *scratch = nd->scratch;
    uint8_t *card = reinterpret_cast<uint8_t *>(scratch + kNoAllocCardOff);
    PlainArgs p;
    memset(&p, 0, sizeof p);
    p.ncols = nz + 2;
    for (int k = 0; k < nz; ++k) p.vars[k] = z[k];
    p.vars[nz] = x;
    p.vars[nz + 1] = y;
    // cardinalities of the involved columns, then the size check on the host
    noalloc_card_kernel<<<p.ncols, 256, 0, st>>>(columns, pitch, n_samples, p, card);
    CK(cudaGetLastError());
    uint8_t hc[kMaxCols];
    for (int k = 0; k < p.ncols; ++k)
        CK(cudaMemcpyAsync(&hc[k], card + p.vars[k], 1, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int k = 0; k < p.ncols; ++k)
        if (hc[k] == 0)
            return set_error(FPGM_ERR_UNSUPPORTED, "fpgm_ci_test_noalloc: variable %d has 256 states (at most 255)",
                             p.vars[k]);
    double dz = 1.0;
    for (int k = 0; k < nz; ++k) dz *= hc[k];
    const double need = dz * hc[nz] * hc[nz + 1] + dz * (hc[nz] + hc[nz + 1] + 1);
    if (need > (double)kNoAllocTableInts)
        return set_error(FPGM_ERR_UNSUPPORTED,
                         "fpgm_ci_test_noalloc: the test needs %.0f table ints, beyond the fixed scratch of %lld; use "
                         "fpgm_ci_test, which allocates",
                         need, (long long)kNoAllocTableInts);
    // the scratch keeps the previous call's contents: clear what must start at zero
    CK(cudaMemsetAsync(scratch, 0, (size_t)need * 4, st));
    CK(cudaMemsetAsync(scratch + kNoAllocDoneOff, 0, 4, st));
    CK(cudaMemsetAsync(scratch + kNoAllocStatsOff, 0, (size_t)ST_COUNT * 8, st));
    p.cols = columns;
    p.S = n_samples;
    for (int k = 0; k < p.ncols; ++k) p.col_off[k] = (int64_t)p.vars[k] * pitch;
    p.card = card;
    p.alpha = alpha;
    p.bt.lo = nullptr;  // no band tables: every df > 0 is decided by the FP64 recheck path
    p.bt.hi = nullptr;
    p.bt.dfmax = 0;
    p.want_hash = want_hash;
    p.gtab = scratch;
    p.done = scratch + kNoAllocDoneOff;
    p.out = result;
    p.stats = reinterpret_cast<unsigned long long *>(scratch + kNoAllocStatsOff);
    const int64_t nvec = n_samples >> 4;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(nvec / kThreads, 2 * nd->num_sms));
    ci_plain_kernel<<<grid, kThreads, kSmemBytes, st>>>(p);
    CK(cudaGetLastError());
    return FPGM_OK;
}
