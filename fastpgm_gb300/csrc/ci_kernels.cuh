// CI-test kernels of the engine.  Every test of a wave (or of an explicit
// batch) is first classified by the size of its joint table and sent to one
// of three persistent kernels:
//
//   tier 0  ci_warp_kernel     one warp per test, table + marginals in a 12 KB
//                              per-warp slice of shared memory (<= 3072 ints)
//   tier 1  ci_cta_kernel      one CTA per test, table in 96 KB of shared memory
//   tier 2  ci_compact_kernel  one CTA per test; the observed Z strata are hashed
//                              to compact ids, then either counted into a dense
//                              strata x (x,y) table (when it has at most 8 cells
//                              per sample and 32 per stratum) or counting-sorted
//                              by stratum and scored per stratum -- work
//                              O(samples + strata * dx * dy), never O(dz)
//
// Tiers 0/1 count with 128-bit column loads folded into packed 16-bit Horner
// codes (two samples per 32-bit multiply-add) and shared-memory atomics into R
// replicas of the table interleaved cell by cell (cell c of replica r at c*R + r):
// lane l adds into replica l mod R, so with R = 32 each lane owns one bank and a
// warp's increments never conflict, whichever cells they hit; the replicas are
// then summed into the dense table.
#pragma once
#include "ci_device.cuh"

namespace fpgm {

// counters[] slots (int32)
// C_PART / C_RETRY: tier-2 tests handed to the partitioned kernel, and from it back to the
// compact kernel's global hash (lists 3-4 and 5 of WaveArgs::lists)
// C_WIDET / C_WIDEQ / C_WIDEW: tests published for partition-parallel scoring, the
// (test, partition) items queued for it, and the items taken
enum { C_TIER0 = 0, C_TIER1, C_TIER2, C_WORK0, C_WORK1, C_WORK2, C_PART, C_WORKP, C_RETRY, C_WORKR, C_WIDET, C_WIDEQ,
       C_WIDEW, C_COUNT };
static_assert(C_COUNT <= 16, "counters are cleared as 64 bytes");
// stats[] slots (unsigned long long)
// ST_TIMEOUT: a bounded device wait gave up (the tensor-core level-0 kernel)
enum { ST_RECHECK = 0, ST_NEARTIE, ST_LARGE, ST_MAXDP, ST_UNSUPPORTED, ST_DET, ST_EXEC, ST_UNRESOLVED,
       ST_REMOVED, ST_MAXDEG, ST_TIER0, ST_TIER1, ST_TIER2, ST_BYTES_SHARED, ST_BYTES_LARGE, ST_TIMEOUT, ST_COUNT };

enum { SRC_WAVE = 0, SRC_EXPLICIT = 1 };

constexpr int kPartMaxLog = 8;  // at most 256 partitions per partitioned test
constexpr int kPartMax = 1 << kPartMaxLog;

// A partitioned test published for partition-parallel scoring: its records stay in the
// owner CTA's slot, every (test, partition) pair is a queue item that any CTA may take, the
// partial statistics are summed here, and the CTA that finishes the last partition decides.
struct WideTest {
    int32_t item, owner, lp, code32, dx, dy, n_items;
    int32_t done, over, n_obs;  // partitions finished; a partition overflowed; strata seen
    unsigned long long df;
    double g2, err, abs_g2;
    unsigned long long hash;
    int32_t pcnt[kPartMax];      // records per partition
    int32_t poff[kPartMax + 1];  // first record of each partition (runs padded to 8 records)
    int32_t sp[kPartMax + 1];    // super-partitions (queue items): partitions sp[i] .. sp[i + 1] - 1
    uint32_t *bmw;               // the test's contributing-sample bitmap being written (null: none)
    int32_t bm_slot, bm_bad;     // its pool slot; set when a partition could not write it
};

// Contributing-sample bitmaps.  A stratum adds a degree of freedom and a G^2 term only when
// its samples take at least two values of x and at least two of y; every other stratum adds
// exactly zero, and so does every stratum that refines it.  A test (x, y | Z) counted by the
// partition kernels records, one bit per sample, which samples lie in strata that do add
// something; at the next level the test (x, y | Z + v), whose strata refine those of Z (v
// past Z's last variable), counts only those samples.  An edge that reaches a level ran every
// test of the level before, so the parent exists whenever the edge is still tested; it has a
// bitmap when the partition kernels counted it in full (no partition from global memory).
// Tests are keyed by (min(x, y), max(x, y), Z ascending).
struct LiveKey {
    unsigned long long h;      // 0: empty; else the key's hash (never 0)
    int32_t slot;              // bitmap in the pool
    int32_t nz;                // |Z|
    uint16_t v[2 + kMaxCond];  // min(x, y), max(x, y), Z ascending
};
__device__ inline unsigned long long live_hash(const uint16_t *v, int n) {
    unsigned long long h = 0x9E3779B97F4A7C15ull ^ (unsigned long long)n;
    for (int i = 0; i < n; ++i) {
        h = (h ^ v[i]) * 0x100000001B3ull;
        h ^= h >> 29;
    }
    return h | 1ull;
}
// key of a test from its item variables (z1 .. zd ascending, x, y), its first nz Z variables
__device__ inline int live_key(const uint16_t *iv, int d, int nz, uint16_t *v) {
    const uint16_t x = iv[d], y = iv[d + 1];
    v[0] = x < y ? x : y;
    v[1] = x < y ? y : x;
    for (int k = 0; k < nz; ++k) v[2 + k] = iv[k];
    return nz + 2;
}
__device__ inline void live_insert(LiveKey *tab, int cap, const uint16_t *v, int n, int slot) {
    const unsigned long long h = live_hash(v, n);
    uint32_t i = (uint32_t)(h >> 7) & (uint32_t)(cap - 1);
    for (int p = 0; p < cap; ++p) {
        if (atomicCAS(&tab[i].h, 0ull, h) == 0ull) {
            tab[i].slot = slot;
            tab[i].nz = n - 2;
            for (int k = 0; k < n; ++k) tab[i].v[k] = v[k];
            return;
        }
        i = (i + 1) & (uint32_t)(cap - 1);
    }
}
__device__ inline int live_find(const LiveKey *tab, int cap, const uint16_t *v, int n) {
    const unsigned long long h = live_hash(v, n);
    uint32_t i = (uint32_t)(h >> 7) & (uint32_t)(cap - 1);
    for (int p = 0; p < cap; ++p) {
        const unsigned long long e = tab[i].h;
        if (e == 0ull) return -1;
        if (e == h && tab[i].nz == n - 2) {
            bool eq = true;
            for (int k = 0; k < n && eq; ++k) eq = tab[i].v[k] == v[k];
            if (eq) return tab[i].slot;
        }
        i = (i + 1) & (uint32_t)(cap - 1);
    }
    return -1;
}

struct WaveArgs {
    const uint8_t *cols;
    const int64_t *var_off;  // byte offset of each variable's column in cols
    const int32_t *var_S;    // samples of each variable's dataset (all variables of a test share it)
    const uint8_t *card;
    int d;
    // wave source
    const int32_t *adjl;
    int32_t adj_stride;
    const int32_t *deg;
    const int32_t *ex, *ey, *pxy, *pyx;
    const uint64_t *cntx, *next;
    const int32_t *off;
    int32_t n_edges;
    const uint64_t *btab;
    // explicit source
    const int32_t *tests;  // [n][2+d]: x, y, z...
    int32_t n_tests;
    // classified items
    uint16_t *item_vars;   // [T][2+d], Horner order: z1..zd, x, y
    int32_t *lists;        // 6 lists of list_cap entries: tiers 0-2, partitioned items + their
                           // strata estimates (float bits), items retried on the global hash
    int64_t list_cap;
    // outputs
    uint8_t *flag;         // 1 independent, 0 dependent, 2 unsupported
    fpgm_ci_result *detail;
    int32_t want_hash;
    int32_t *counters;
    unsigned long long *stats;
    double alpha;
    BandTables bt;
    // compact tier: per-CTA global slots
    char *slot_mem;
    int64_t slot_bytes;
    int64_t slot_S;           // sample count the slot layout was made for (>= S)
    int32_t hash_cap_global;  // power of two >= 2 * slot_S
    unsigned long long *dbg;  // compact-tier phase timers (FPGM_PHASE_TIMERS), else null
    int32_t part_max_log;     // partitioned kernel: at most 2^part_max_log partitions (<= kPartMaxLog)
    // partition-parallel scoring (null: every partitioned test stays on its own CTA)
    WideTest *wide;           // one per CTA of the partition kernel
    int32_t *wide_items;      // (test << 8) | partition, kPartMax per test
    int32_t wide_small_n2;    // tests of fewer than kPartMinSamples samples are partitioned too when
                              // the wave has at most this many tier-2 tests (0: never)
    int32_t wide_min_log;     // least partitions (log2) of a published test
    int32_t wide_part_min;    // published tests are split no finer than this many samples per partition
    int32_t wide_direct;      // in such a wave, hand every tier-2 test over before any hashing
    // Tier-2 method for a test whose strata overflow the shared hash: partition kernel or the
    // global strata hash.  tune: a fixed table (kTuneSB x kTuneDB x kTuneCB bytes, 1 =
    // partitions); else tune_obs: the online autotuner's per-bucket timings; else
    // part_min_samples decides (samples >= it: partitions).
    const int8_t *tune;
    unsigned long long *tune_obs;  // 8 per bucket: n_part, ns_part, n_hash, ns_hash, decisions
    // Shared-hash overflow record per autotuner bucket (8 each: tests that overflowed, tests
    // that fit, sum of strata / samples * 2^16 and its count, tests seen); null: every tier-2
    // test tries the shared hash first.
    unsigned long long *ovf;
    int32_t warp_ints;             // ints of the warp tier's per-warp slice (its table limit)
    int32_t dense_rows;            // compact kernel's dense strata table: a thread per stratum (else lane groups)
    int32_t stage_rec;             // records staged in shared memory at most (0: as many as fit; tests lower it)
    // contributing-sample bitmaps (null: off): written by this level's partition-path tests
    // into bm_pool (bm_cap bitmaps of bm_words words, keys in bm_tab), read from the previous
    // level's (bm_prev_*)
    uint32_t *bm_pool;
    LiveKey *bm_tab;
    int32_t *bm_count;
    int32_t bm_cap, bm_tab_cap, bm_words;
    const uint32_t *bm_prev_pool;
    const LiveKey *bm_prev_tab;
    int32_t bm_prev_tab_cap;
    unsigned long long *live_stat;  // [0] samples in contributing strata, [1] samples scored (partition path)
    int64_t part_min_samples;
};

// Autotuner table keys: sample count, |Z| and joint cardinality (cells = dz dx dy) relative
// to the sample count.
constexpr int kTuneSB = 6;   // samples: < 12.5k, < 25k, < 50k, < 100k, < 200k, more
constexpr int kTuneDB = 12;  // |Z| = 1 .. 11, 12 and more
constexpr int kTuneCB = 6;   // cells / samples: < 4, < 16, < 64, < 256, < 1024, more
constexpr int kTuneBuckets = kTuneSB * kTuneDB * kTuneCB;
constexpr unsigned long long kTuneExplore = 8;    // tests timed with each method before either is preferred
constexpr unsigned long long kTuneRefresh = 256;  // then one test in this many takes the other method ...
constexpr unsigned long long kTuneSettled = 32;   // ... until that method has this many timed tests
__host__ __device__ inline int tune_index(int64_t S, int d, double cells) {
    int sb = 0;
    for (int64_t lim = 12500; sb < kTuneSB - 1 && S >= lim; lim *= 2) ++sb;
    const int db = d < 1 ? 0 : (d > kTuneDB ? kTuneDB - 1 : d - 1);
    const double r = cells / (double)(S > 0 ? S : 1);
    int cb = 0;
    for (double lim = 4.0; cb < kTuneCB - 1 && r >= lim; lim *= 4.0) ++cb;
    return (sb * kTuneDB + db) * kTuneCB + cb;
}

// Online autotuner (one thread decides for its CTA): per (samples, |Z|, cells/samples)
// bucket, the device time of tests counted each way is summed as they finish; a bucket
// first alternates the two methods until each has kTuneExplore timed tests, then keeps the
// fixed rule's method unless the other is at least 10% faster on average, giving one test
// in kTuneRefresh to the other until it has kTuneSettled timed tests
// (measured at 1,041 variables x 100,000 samples: one in 32 cost 4% against the best fixed
// rule, as the slower method is 1.5-3x slower there).
// *bucket = the bucket whose hash-path time the caller must add (-1: none).
__device__ inline bool tier2_pick_partitions(const WaveArgs &a, int64_t S, int d, double cells, int *bucket) {
    *bucket = -1;
    if (a.tune) return a.tune[tune_index(S, d, cells)] != 0;
    if (!a.tune_obs) return S >= a.part_min_samples;
    const int b = tune_index(S, d, cells);
    unsigned long long *o = a.tune_obs + 8 * b;
    const unsigned long long np = *(volatile unsigned long long *)&o[0], nh = *(volatile unsigned long long *)&o[2];
    const unsigned long long k = atomicAdd(&o[4], 1ull);
    bool part;
    if (np < kTuneExplore || nh < kTuneExplore) {
        part = (k & 1ull) == 0;
    } else {
        // leave the fixed rule's method only for one at least 10% faster on average
        const double mp = (double)*(volatile unsigned long long *)&o[1] / (double)np;
        const double mh = (double)*(volatile unsigned long long *)&o[3] / (double)nh;
        part = S >= a.part_min_samples ? !(mh < 0.9 * mp) : mp < 0.9 * mh;
        if (k % kTuneRefresh == 0 && (part ? nh : np) < kTuneSettled) part = !part;
    }
    if (!part) *bucket = b;
    return part;
}

// A bucket whose tests have (almost) all overflowed the compact kernel's shared hash skips
// that attempt: est gets the strata expected from the bucket's observed strata per sample
// (raised by a third, so it errs high); one test in 64 still tries, to keep the record fresh.
constexpr unsigned long long kOvfMin = 16;  // overflowed tests before any is skipped
__device__ inline bool ovf_skip(const WaveArgs &a, int b, int64_t S, double *est) {
    if (!a.ovf || b < 0) return false;
    unsigned long long *o = a.ovf + 8 * b;
    const unsigned long long over = *(volatile unsigned long long *)&o[0], fit = *(volatile unsigned long long *)&o[1];
    const unsigned long long rs = *(volatile unsigned long long *)&o[2], rn = *(volatile unsigned long long *)&o[3];
    if (over < kOvfMin || over <= 8 * fit || rn < 4) return false;
    if ((atomicAdd(&o[4], 1ull) & 63ull) == 0) return false;
    *est = fmin((double)S, 1.34 * ((double)rs / 65536.0 / (double)rn) * (double)S);
    return true;
}
__device__ inline void ovf_strata(const WaveArgs &a, int b, int64_t S, int n_obs) {
    if (!a.ovf || b < 0 || S <= 0) return;
    atomicAdd(&a.ovf[8 * b + 2], (unsigned long long)(((double)n_obs * 65536.0) / (double)S));
    atomicAdd(&a.ovf[8 * b + 3], 1ull);
}

__device__ inline int upper_bound_i32(const int32_t *a, int n, int v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Item -> (x, y, Z) -> tier.  One thread per item, grid-stride.
template <int kSource>
__global__ void classify_kernel(WaveArgs a) {
    const int T = kSource == SRC_EXPLICIT ? a.n_tests : a.off[a.n_edges];
    const int d = a.d, ncols = d + 2;
    unsigned long long bytes_shared = 0, bytes_large = 0;  // algorithmic column bytes per tier group
    for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < T; item += gridDim.x * blockDim.x) {
        int x, y, z[kMaxCond];
        if (kSource == SRC_EXPLICIT) {
            const int32_t *tt = a.tests + (int64_t)item * ncols;
            x = tt[0];
            y = tt[1];
            for (int k = 0; k < d; ++k) z[k] = tt[2 + k];
        } else {
            const int e = upper_bound_i32(a.off, a.n_edges + 1, item) - 1;
            uint64_t rank = a.next[e] + (uint64_t)(item - a.off[e]);
            x = a.ex[e];
            y = a.ey[e];
            if (d > 0) {
                int side_node, skip;
                if (rank < a.cntx[e]) {
                    side_node = x;
                    skip = a.pxy[e];
                } else {
                    rank -= a.cntx[e];
                    side_node = y;
                    skip = a.pyx[e];
                }
                int c[kMaxCond];
                unrank_lex(a.btab, a.deg[side_node] - 1, d, rank, c);
                const int32_t *L = a.adjl + (int64_t)side_node * a.adj_stride;
                for (int k = 0; k < d; ++k) z[k] = L[c[k] < skip ? c[k] : c[k] + 1];
            }
        }
        uint16_t *iv = a.item_vars + (int64_t)item * ncols;
        double dzf = 1.0;
        int64_t dz = 1;
        for (int k = 0; k < d; ++k) {
            iv[k] = (uint16_t)z[k];
            const int dk = a.card[z[k]];
            dzf *= dk;
            dz *= dk;
        }
        iv[d] = (uint16_t)x;
        iv[d + 1] = (uint16_t)y;
        const int dx = a.card[x], dy = a.card[y];
        int tier;
        if (dzf * dx * dy > 4e18) {
            tier = 3;  // stratum codes would not fit 64 bits
        } else {
            const int64_t need = dz * dx * dy + dz * (dx + dy + 1);
            tier = need <= a.warp_ints - 32 ? 0 : (need <= kCtaInts - 64 ? 1 : 2);
            if (tier == 2 && a.slot_mem == nullptr) tier = 3;
        }
        if (tier == 3) {
            a.flag[item] = 2;
            atomicAdd(&a.stats[ST_UNSUPPORTED], 1ull);
            continue;
        }
        const int slot = atomicAdd(&a.counters[C_TIER0 + tier], 1);
        a.lists[tier * a.list_cap + slot] = item;
        const unsigned long long b = (unsigned long long)(2 + d) * (unsigned long long)a.var_S[x];
        if (tier < 2) bytes_shared += b; else bytes_large += b;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bytes_shared += __shfl_xor_sync(0xffffffffu, bytes_shared, o);
        bytes_large += __shfl_xor_sync(0xffffffffu, bytes_large, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (bytes_shared) atomicAdd(&a.stats[ST_BYTES_SHARED], bytes_shared);
        if (bytes_large) atomicAdd(&a.stats[ST_BYTES_LARGE], bytes_large);
    }
}

// Packed Horner codes of two 16-sample vectors (va, and vb when two) over ncols
// columns, with up to eight 128-bit column loads in flight before they are folded.
__device__ __forceinline__ void horner_pair(uint32_t (&ca)[8], uint32_t (&cb)[8], const uint8_t *const *col,
                                            const uint32_t *dim, int ncols, int64_t va, int64_t vb, bool two) {
#pragma unroll
    for (int q = 0; q < 8; ++q) ca[q] = cb[q] = 0;
    for (int j0 = 0; j0 < ncols; j0 += 4) {
        uint4 wa[4], wb[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            wa[t] = wb[t] = make_uint4(0, 0, 0, 0);
            if (j0 + t < ncols) {
                wa[t] = __ldg(reinterpret_cast<const uint4 *>(col[j0 + t]) + va);
                if (two) wb[t] = __ldg(reinterpret_cast<const uint4 *>(col[j0 + t]) + vb);
            }
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            if (j0 + t >= ncols) break;
            horner16(ca, wa[t], dim[j0 + t]);
            horner16(cb, wb[t], dim[j0 + t]);
        }
    }
}

__device__ inline void record(const WaveArgs &a, int item, const Verdict &v, int64_t cells, uint64_t fnv, int path) {
    a.flag[item] = (uint8_t)v.indep;
    if (v.rechecked) {
        atomicAdd(&a.stats[ST_RECHECK], 1ull);
        if (fabs(v.p - a.alpha) < 1e-12) atomicAdd(&a.stats[ST_NEARTIE], 1ull);
        atomicMax(&a.stats[ST_MAXDP], (unsigned long long)__double_as_longlong(v.dp));
    }
    if (a.detail) {
        fpgm_ci_result r;
        r.table_hash = fnv;
        r.cell_hash = v.hash;
        r.cells = cells;
        r.df = (int32_t)v.df;
        r.independent = v.indep;
        r.g2 = v.g2;
        r.p_value = v.p;
        r.rechecked = v.rechecked;
        r.path = path;
        a.detail[item] = r;
    }
}

// ---------------------------------------------------------------- tier 0: warp per test
// kSlice: ints of a warp's shared slice; kMinBlocks: resident CTAs per SM the launch bounds
// ask for (12 KB slices: 2 CTAs; 8 KB slices: 3 CTAs, more warps per SM for smaller tables).
template <int kSlice, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks) ci_warp_kernel(WaveArgs a) {
    constexpr int kWarpInts = kSlice;
    extern __shared__ int smem[];
    __shared__ const uint8_t *s_col[kWarps][kMaxCols];
    __shared__ uint32_t s_dim[kWarps][kMaxCols];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *wreg = smem + warp * kWarpInts;
    const int n0 = a.counters[C_TIER0];
    const int d = a.d, ncols = d + 2;
    const WarpGroup g{lane};
    for (;;) {
        int idx = 0;
        if (lane == 0) idx = atomicAdd(&a.counters[C_WORK0], 1);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= n0) break;
        const int item = a.lists[idx];
        const int64_t S = a.var_S[a.item_vars[(int64_t)item * ncols + d]];
        const int64_t nvec = S >> 4;
        uint32_t dim = 1;
        if (lane < ncols) {
            const int var = a.item_vars[(int64_t)item * ncols + lane];
            dim = a.card[var];
            s_col[warp][lane] = a.cols + a.var_off[var];
            s_dim[warp][lane] = dim;
        }
        uint32_t cells = dim;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cells *= __shfl_xor_sync(0xffffffffu, cells, o);
        const int dx = __shfl_sync(0xffffffffu, (int)dim, d), dy = __shfl_sync(0xffffffffu, (int)dim, d + 1);
        const int dz = (int)cells / (dx * dy);
        __syncwarp();
        const int marg = dz * (dx + dy + 1);
        int lgR = 0;  // replicas: 2^lgR interleaved copies of the table, then the reduced table
        for (int l = 5; l >= 1; --l)
            if (((int)cells << l) + (int)cells + marg <= kWarpInts) { lgR = l; break; }
        const int R = 1 << lgR;
        int *rep = wreg;                                  // cell c of replica r at rep[c * R + r]
        int *tab = R > 1 ? wreg + ((int)cells << lgR) : wreg;  // dense table in reference cell order
        int *ni = tab + cells, *nj = ni + dz * dx, *nk = nj + dz * dy;
        for (int i = lane; i < ((int)cells << lgR); i += 32) rep[i] = 0;
        __syncwarp();
        // lane l counts into replica l mod R: with 32 replicas every lane owns one bank, so a
        // warp's 32 increments never conflict whatever cells they hit
        int *myrep = rep + (lane & (R - 1));
        for (int64_t v = lane; v < nvec; v += 64) {
            const bool two = v + 32 < nvec;
            uint32_t ca[8], cb[8];
            horner_pair(ca, cb, s_col[warp], s_dim[warp], ncols, v, v + 32, two);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                atomicAdd(&myrep[(ca[q] & 0xffffu) << lgR], 1);
                atomicAdd(&myrep[(ca[q] >> 16) << lgR], 1);
            }
            if (two) {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    atomicAdd(&myrep[(cb[q] & 0xffffu) << lgR], 1);
                    atomicAdd(&myrep[(cb[q] >> 16) << lgR], 1);
                }
            }
        }
        for (int64_t s = (S & ~(int64_t)15) + lane; s < S; s += 32) {
            uint32_t c = 0;
            for (int j = 0; j < ncols; ++j) c = c * s_dim[warp][j] + s_col[warp][j][s];
            atomicAdd(&myrep[c << lgR], 1);
        }
        __syncwarp();
        if (R > 1) {
            for (int c = lane; c < (int)cells; c += 32) {
                int s = 0;
                for (int r = 0; r < R; ++r) s += rep[(c << lgR) + r];
                tab[c] = s;
            }
            __syncwarp();
        }
        const Verdict v = score_dense(g, tab, ni, nj, nk, dx, dy, dz, a.alpha, a.bt, a.detail != nullptr,
                                      a.want_hash != 0, nullptr);
        if (lane == 0) record(a, item, v, cells, a.want_hash ? table_hash(tab, cells) : 0, 0);
        __syncwarp();
    }
}

// ---------------------------------------------------------------- tier 1: CTA per test
__global__ void __launch_bounds__(kThreads, 2) ci_cta_kernel(WaveArgs a) {
    extern __shared__ int smem[];
    __shared__ const uint8_t *s_col[kMaxCols];
    __shared__ uint32_t s_dim[kMaxCols];
    __shared__ int s_idx;
    __shared__ Partial scratch[kWarps];
    const int tid = threadIdx.x, lane = tid & 31;
    const int n1 = a.counters[C_TIER1];
    const int d = a.d, ncols = d + 2;
    const CtaGroup g{tid};
    for (;;) {
        if (tid == 0) s_idx = atomicAdd(&a.counters[C_WORK1], 1);
        __syncthreads();
        const int idx = s_idx;
        if (idx >= n1) break;
        const int item = a.lists[a.list_cap + idx];
        const int64_t S = a.var_S[a.item_vars[(int64_t)item * ncols + d]];
        const int64_t nvec = S >> 4;
        if (tid < ncols) {
            const int var = a.item_vars[(int64_t)item * ncols + tid];
            s_dim[tid] = a.card[var];
            s_col[tid] = a.cols + a.var_off[var];
        }
        __syncthreads();
        int cells = 1;
        for (int j = 0; j < ncols; ++j) cells *= (int)s_dim[j];
        const int dx = s_dim[d], dy = s_dim[d + 1];
        const int dz = cells / (dx * dy);
        const int marg = dz * (dx + dy + 1);
        int lgR = 0;  // replicas interleaved cell by cell, as in the warp tier
        for (int l = 5; l >= 1; --l)
            if ((cells << l) + cells + marg <= kCtaInts) { lgR = l; break; }
        const int R = 1 << lgR;
        int *rep = smem;
        int *tab = R > 1 ? smem + (cells << lgR) : smem;
        int *ni = tab + cells, *nj = ni + dz * dx, *nk = nj + dz * dy;
        for (int i = tid; i < (cells << lgR); i += kThreads) rep[i] = 0;
        __syncthreads();
        int *myrep = rep + (lane & (R - 1));
        for (int64_t v = tid; v < nvec; v += 2 * kThreads) {
            const bool two = v + kThreads < nvec;
            uint32_t ca[8], cb[8];
            horner_pair(ca, cb, s_col, s_dim, ncols, v, v + kThreads, two);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                atomicAdd(&myrep[(ca[q] & 0xffffu) << lgR], 1);
                atomicAdd(&myrep[(ca[q] >> 16) << lgR], 1);
            }
            if (two) {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    atomicAdd(&myrep[(cb[q] & 0xffffu) << lgR], 1);
                    atomicAdd(&myrep[(cb[q] >> 16) << lgR], 1);
                }
            }
        }
        for (int64_t s = (S & ~(int64_t)15) + tid; s < S; s += kThreads) {
            uint32_t c = 0;
            for (int j = 0; j < ncols; ++j) c = c * s_dim[j] + s_col[j][s];
            atomicAdd(&myrep[c << lgR], 1);
        }
        __syncthreads();
        if (R > 1) {
            for (int c = tid; c < cells; c += kThreads) {
                int s = 0;
                for (int r = 0; r < R; ++r) s += rep[(c << lgR) + r];
                tab[c] = s;
            }
            __syncthreads();
        }
        const Verdict v = score_dense(g, tab, ni, nj, nk, dx, dy, dz, a.alpha, a.bt, a.detail != nullptr,
                                      a.want_hash != 0, scratch);
        if (tid == 0) record(a, item, v, cells, a.want_hash ? table_hash(tab, cells) : 0, 1);
        __syncthreads();
    }
}

// ---------------------------------------------------------------- tier 2: compact strata
// Shared-memory plan of the compact kernel (kSmemBytes), phase by phase:
//   phase 1  strata hash: keys u64[kZCap64] or u32[kZCap32] at 0 (32-bit when every stratum
//            code fits), 16-bit ids at kZIdsOff
//   phase 2  per-stratum counts cnt[] at 0 and cursors cur[] at kZCurOff (over the dead keys)
//   phase 3  per-warp x,y tables from kZTabOff (over the dead ids)
// Up to kZStrata strata stay in shared memory; beyond that the same arrays live in the
// CTA's global slot (hash sized >= 2 n_samples).
constexpr int kZCap64 = 8192;    // shared hash slots with 64-bit stratum codes
constexpr int kZCap32 = 16384;   // ... with 32-bit codes (same 64 KB)
constexpr int kZStrata = kZCap32 / 2;  // most strata kept in shared memory (load <= 1/2)
constexpr int kZIdsOff = kZCap64 * 8;
constexpr int kZCurOff = ((kZStrata + 1) * 4 + 15) / 16 * 16;
constexpr int kZTabOff = (kZCurOff + (kZStrata + 1) * 4 + 15) / 16 * 16;
static_assert(kZIdsOff + kZCap32 * 2 <= kSmemBytes, "shared hash ids");
static_assert(3 * 32 * kThreads * 4 <= kSmemBytes, "dense-table scoring columns");
constexpr int kSparseWarpTab = (kSmemBytes - kZTabOff) / 4 / kWarps;  // ints per warp
constexpr int kLaneStratum = 8;   // strata of up to this many samples: one lane each
constexpr int kRegStratum = 64;   // larger strata up to this size keep their codes in registers
constexpr int kDenseMul = 8;      // dense strata x cells table when it has at most this many cells per sample

// Fibonacci hashing: the top log2(cap) bits of z times 2^64/phi (cap a power of two).
// The top bits mix every bit of the mixed-radix stratum code; the middle bits used before
// left long probe runs (c4: 1.8x longer global-hash phase).
__device__ __forceinline__ uint32_t zhash(uint64_t z, uint32_t cap) {
    return (uint32_t)((z * 0x9E3779B97F4A7C15ull) >> (64 - __popc(cap - 1)));
}

// Inserts stratum code z; a new code takes the next id from *counter, written to ids[slot]
// (16- or 32-bit ids) and, when gzk is given, its code to gzk[id].  Returns the slot, or -1
// after max_probe probes or once more than id_limit strata exist.
__device__ __forceinline__ uint64_t key_cas(uint64_t *p, uint64_t e, uint64_t v) {
    return atomicCAS(reinterpret_cast<unsigned long long *>(p), (unsigned long long)e, (unsigned long long)v);
}
__device__ __forceinline__ uint32_t key_cas(uint32_t *p, uint32_t e, uint32_t v) { return atomicCAS(p, e, v); }

template <class K, class Id>
__device__ inline int zinsert(K *keys, Id *ids, uint32_t cap, uint64_t zz, int *counter, int id_limit,
                              uint32_t max_probe, uint64_t *gzk) {
    const K z = (K)zz, empty = (K)kEmptyKey;
    uint32_t h = zhash(zz, cap);
    for (uint32_t p = 0; p < max_probe; ++p) {
        const K k = keys[h];
        if (k == z) return (int)h;
        if (k == empty) {
            const K old = key_cas(&keys[h], empty, z);
            if (old == empty) {
                const int id = atomicAdd(counter, 1);
                if (id >= id_limit) return -1;
                ids[h] = (Id)id;
                if (gzk) gzk[id] = zz;
                return (int)h;
            }
            if (old == z) return (int)h;
        }
        h = (h + 1) & (cap - 1);
    }
    return -1;
}

// As zinsert, without the id: *claimed is set when this call took an empty slot for z (the
// caller hands out the ids of a warp's claims together).  Returns the slot, or -1 after
// max_probe probes.
template <class K>
__device__ __forceinline__ int zclaim(K *keys, uint32_t cap, uint64_t zz, uint32_t max_probe, bool *claimed) {
    const K z = (K)zz, empty = (K)kEmptyKey;
    uint32_t h = zhash(zz, cap);
    for (uint32_t p = 0; p < max_probe; ++p) {
        const K k = keys[h];
        if (k == z) return (int)h;
        if (k == empty) {
            const K old = key_cas(&keys[h], empty, z);
            if (old == empty) {
                *claimed = true;
                return (int)h;
            }
            if (old == z) return (int)h;
        }
        h = (h + 1) & (cap - 1);
    }
    return -1;
}

// Stratum codes of 16 consecutive samples (vector v) from the d Z columns, four column
// loads in flight at a time.  K = uint32_t when every code is below 2^32 (so is every
// prefix of the mixed-radix code).
template <class K>
__device__ __forceinline__ void zcodes16(K (&z)[16], const uint8_t *const *col, const uint32_t *dim, int d,
                                         int64_t v) {
#pragma unroll
    for (int b = 0; b < 16; ++b) z[b] = 0;
    for (int j0 = 0; j0 < d; j0 += 4) {
        uint4 w[4];
#pragma unroll
        for (int t = 0; t < 4; ++t)
            if (j0 + t < d) w[t] = __ldg(reinterpret_cast<const uint4 *>(col[j0 + t]) + v);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            if (j0 + t >= d) break;
            const uint32_t ww[4] = {w[t].x, w[t].y, w[t].z, w[t].w};
            const K dm = dim[j0 + t];
#pragma unroll
            for (int b = 0; b < 16; ++b) z[b] = z[b] * dm + ((ww[b >> 2] >> (8 * (b & 3))) & 0xffu);
        }
    }
}

// Byte offsets of one compact-tier global slot, every region 256-byte aligned.
struct SlotLayout {
    int64_t keys, zk, ids, cnt, cur, sid, wt, ord, tab, rs, total;
};
__host__ __device__ inline int64_t align256(int64_t x) { return (x + 255) & ~(int64_t)255; }
__host__ __device__ inline SlotLayout slot_layout(int64_t S, int64_t cap) {
    SlotLayout L;
    int64_t o = 0;
    L.keys = o; o = align256(o + cap * 8);        // strata hash keys (overflow path)
    L.zk = o;   o = align256(o + (S + 1) * 8);    // stratum code per id (fingerprint only)
    L.ids = o;  o = align256(o + cap * 4);        // id per hash slot (overflow path)
    L.cnt = o;  o = align256(o + (S + 1) * 4);    // samples per stratum -> offsets (overflow path)
    L.cur = o;  o = align256(o + (S + 1) * 4);    // scatter cursors (overflow path)
    L.sid = o;  o = align256(o + (S + 16) * 4);   // slot, then stratum id, per sample
    L.wt = o;   o = align256(o + (int64_t)kWarps * kGlobalWarpTab * 4);  // wide x,y tables, kept zeroed
    L.ord = o;  o = align256(o + (S + 2048) * 2);  // (x << 8) | y codes sorted by stratum (+ partition padding)
    L.tab = o;  o = align256(o + ((int64_t)kDenseMul * S + 64) * 4);  // dense strata x cells counts, kept zeroed
    L.rs = o;   o = align256(o + (S + 2048) * 4);  // partition records: sample index (contributing-sample bitmaps)
    L.total = o;
    return L;
}

// Block-wide exclusive scan of n ints in place (any n), each thread a contiguous chunk.
// s_w: kWarps ints of shared scratch.
__device__ inline void block_exclusive_scan(int *v, int n, int *s_w) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int per = (n + kThreads - 1) / kThreads;
    const int b0 = min(n, tid * per), b1 = min(n, b0 + per);
    int sum = 0;
    for (int i = b0; i < b1; ++i) sum += v[i];
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    __syncthreads();
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    int base = 0;
    for (int w = 0; w < warp; ++w) base += s_w[w];
    int run = base + incl - sum;
    for (int i = b0; i < b1; ++i) {
        const int t = v[i];
        v[i] = run;
        run += t;
    }
    __syncthreads();
}

// Per-thread accumulator of strata terms: FP64 sum for the recheck pass, or FP32
// Neumaier-compensated sum with a running error bound (no FP64 in the common path).
template <bool kFp64>
struct TermAcc {
    double g = 0.0;                          // FP64 pass
    float s = 0.f, c = 0.f, e = 0.f, a = 0.f;  // FP32 pass
    // cell of count O in a stratum of m samples with margins Nx, Ny
    __device__ __forceinline__ void add(int O, int Nx, int Ny, int m) {
        if (kFp64) {
            const double expected = (double)Ny * (double)Nx / (double)m;
            g += 2.0 * O * log(O / expected);
        } else {
            const long long num = (long long)O * m, den = (long long)Nx * Ny;
            if (num == den) return;
            const float q = (float)(num - den) / (float)den;
            const float l = fabsf(q) < 0.5f ? log1pf(q) : logf((float)num / (float)den);
            const float term = 2.0f * (float)O * l;
            const float tt = s + term;
            c += fabsf(s) >= fabsf(term) ? (s - tt) + term : (term - tt) + s;
            s = tt;
            e += 2.0f * (float)O * (2.5e-7f * fminf(1.0f, 2.0f * fabsf(q)) + 2.5e-7f * fabsf(l));
            a += fabsf(term);
        }
    }
    __device__ __forceinline__ void into(Partial &p) const {
        if (kFp64) {
            p.g2 += g;
        } else {
            p.g2 += (double)s + (double)c;
            p.err += (double)e;
            p.abs_g2 += (double)a;
        }
    }
};

// Strata of at most kLaneStratum samples, one thread each, pairwise in registers.
// Larger strata are appended to big[] when collect.
// live (optional): live[k] = 1 when stratum k has two or more values of x and of y.
template <bool kFp64>
__device__ inline Partial score_small_strata(const int *cnt, const uint16_t *gord, int n_obs, int dx, int dy, int *big,
                                             int *n_big, const uint64_t *gzk, bool want_hash, bool collect,
                                             uint8_t *live = nullptr) {
    Partial acc{0, 0.0, 0.0, 0.0, 0ull};
    TermAcc<kFp64> ta;
    for (int k = threadIdx.x; k < n_obs; k += kThreads) {
        const int o0 = cnt[k], m = cnt[k + 1] - o0;
        if (m <= 1 && !want_hash) continue;  // one sample: no G^2 term, no degree of freedom
        if (m > kLaneStratum) {
            if (collect) big[atomicAdd(n_big, 1)] = k;
            continue;
        }
        if (m == 2 && !want_hash) {
            // two samples add one degree of freedom and two cells of 2 ln 2 when they differ in
            // both x and y, and nothing otherwise
            const uint32_t dif = (uint32_t)gord[o0] ^ (uint32_t)gord[o0 + 1];
            const bool both = (dif >> 8) != 0 && (dif & 0xffu) != 0;
            if (both) {
                acc.df += 1;
                ta.add(1, 1, 1, 2);
                ta.add(1, 1, 1, 2);
            }
            if (live) live[k] = both;
            continue;
        }
        // one register per sample: (x << 8) | y; equal cells <=> equal words
        uint32_t pk[kLaneStratum];
#pragma unroll
        for (int i = 0; i < kLaneStratum; ++i) pk[i] = i < m ? (uint32_t)gord[o0 + i] : 0u;
        int ax = 0, ay = 0;
#pragma unroll
        for (int i = 0; i < kLaneStratum; ++i) {
            if (i >= m) break;
            int O = 0, Nx = 0, Ny = 0;
            bool fc = true, fx = true, fy = true;
#pragma unroll
            for (int j = 0; j < kLaneStratum; ++j) {
                if (j >= m) break;
                const uint32_t dif = pk[j] ^ pk[i];
                const bool sc = dif == 0, sx = (dif >> 8) == 0, sy = (dif & 0xffu) == 0;
                O += sc;
                Nx += sx;
                Ny += sy;
                if (j < i) {
                    fc &= !sc;
                    fx &= !sx;
                    fy &= !sy;
                }
            }
            ax += fx;
            ay += fy;
            if (fc) {
                ta.add(O, Nx, Ny, m);
                if (want_hash)
                    acc.hash += cell_mix((gzk[k] * (uint64_t)dx + (pk[i] >> 8)) * (uint64_t)dy + (pk[i] & 0xffu),
                                         (uint32_t)O);
            }
        }
        acc.df += (long long)(max(ax, 1) - 1) * (max(ay, 1) - 1);
        if (live) live[k] = ax >= 2 && ay >= 2;
    }
    ta.into(acc);
    return acc;
}

// Strata listed in big[] (or, when big is null, strata k_first .. k_first + n_big - 1): one
// warp each, dense x,y table read back with atomicExch.
// Strata of up to kRegStratum samples keep their packed (x << 8) | y codes in registers,
// and the next stratum's codes are loaded while the current one is scored.
template <bool kFp64>
__device__ inline Partial score_big_strata(Partial acc, const int *cnt, const uint16_t *gord, const int *big, int n_big,
                                           int dx, int dy, int *wt, const uint64_t *gzk, bool want_hash,
                                           int k_first = 0, uint8_t *live = nullptr) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int dxy = dx * dy;
    int *wni = wt + dxy, *wnj = wni + dx;
    TermAcc<kFp64> ta;
    int b = warp, k = 0, m = 0, o0 = 0, p0 = -1, p1 = -1;
    auto fetch = [&](int bb, int &kk, int &mm, int &oo, int &q0, int &q1) {
        q0 = q1 = -1;
        if (bb >= n_big) return;
        kk = big ? big[bb] : k_first + bb;
        oo = cnt[kk];
        mm = cnt[kk + 1] - oo;
        if (mm <= kRegStratum) {
            if (lane < mm) q0 = gord[oo + lane];
            if (lane + 32 < mm) q1 = gord[oo + 32 + lane];
        }
    };
    fetch(b, k, m, o0, p0, p1);
    for (; b < n_big; b += kWarps) {
        int kn = 0, mn = 0, on = 0, n0 = -1, n1 = -1;
        fetch(b + kWarps, kn, mn, on, n0, n1);
        int ax = 0, ay = 0;
        if (m <= kRegStratum) {
            const int x0 = p0 >> 8, y0 = p0 & 0xff, x1 = p1 >> 8, y1 = p1 & 0xff;
            const int c0 = x0 * dy + y0, c1 = x1 * dy + y1;
            bool nx0 = false, ny0 = false, nx1 = false, ny1 = false;
            if (p0 >= 0) {
                atomicAdd(&wt[c0], 1);
                nx0 = atomicAdd(&wni[x0], 1) == 0;
                ny0 = atomicAdd(&wnj[y0], 1) == 0;
            }
            if (p1 >= 0) {
                atomicAdd(&wt[c1], 1);
                nx1 = atomicAdd(&wni[x1], 1) == 0;
                ny1 = atomicAdd(&wnj[y1], 1) == 0;
            }
            ax = __popc(__ballot_sync(full, nx0)) + __popc(__ballot_sync(full, nx1));
            ay = __popc(__ballot_sync(full, ny0)) + __popc(__ballot_sync(full, ny1));
            __syncwarp();  // the lanes' counts are visible before they are read back
            if (p0 >= 0) {
                const int O = atomicExch(&wt[c0], 0);
                if (O > 0) {
                    ta.add(O, wni[x0], wnj[y0], m);
                    if (want_hash) acc.hash += cell_mix((gzk[k] * (uint64_t)dx + x0) * (uint64_t)dy + y0, (uint32_t)O);
                }
            }
            if (p1 >= 0) {
                const int O = atomicExch(&wt[c1], 0);
                if (O > 0) {
                    ta.add(O, wni[x1], wnj[y1], m);
                    if (want_hash) acc.hash += cell_mix((gzk[k] * (uint64_t)dx + x1) * (uint64_t)dy + y1, (uint32_t)O);
                }
            }
            __syncwarp();
            if (p0 >= 0) {
                wni[x0] = 0;
                wnj[y0] = 0;
            }
            if (p1 >= 0) {
                wni[x1] = 0;
                wnj[y1] = 0;
            }
        } else {
            const int o1 = o0 + m;
            // counts: four codes per lane loaded together, so a stratum in global memory costs
            // one load round trip per 128 samples
            for (int i0 = o0 + lane; i0 < o1; i0 += 128) {
                int q[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) q[u] = i0 + 32 * u < o1 ? (int)gord[i0 + 32 * u] : -1;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (q[u] < 0) break;
                    const int x = q[u] >> 8, y = q[u] & 0xff;
                    atomicAdd(&wt[x * dy + y], 1);
                    ax += atomicAdd(&wni[x], 1) == 0;
                    ay += atomicAdd(&wnj[y], 1) == 0;
                }
            }
            __syncwarp();
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                ax += __shfl_xor_sync(full, ax, o);
                ay += __shfl_xor_sync(full, ay, o);
            }
            for (int i = o0 + lane; i < o1; i += 32) {
                const int p = gord[i];
                const int x = p >> 8, y = p & 0xff;
                const int O = atomicExch(&wt[x * dy + y], 0);
                if (O > 0) {
                    ta.add(O, wni[x], wnj[y], m);
                    if (want_hash) acc.hash += cell_mix((gzk[k] * (uint64_t)dx + x) * (uint64_t)dy + y, (uint32_t)O);
                }
            }
            __syncwarp();
            for (int i = o0 + lane; i < o1; i += 32) {
                const int p = gord[i];
                wni[p >> 8] = 0;
                wnj[p & 0xff] = 0;
            }
        }
        __syncwarp();
        if (lane == 0) {
            acc.df += (long long)(max(ax, 1) - 1) * (max(ay, 1) - 1);
            if (live) live[k] = ax >= 2 && ay >= 2;
        }
        k = kn;
        m = mn;
        o0 = on;
        p0 = n0;
        p1 = n1;
    }
    ta.into(acc);
    return acc;
}

// Dense strata x cells table T[k * dxy + x * dy + y] (k = stratum id), at most 32 cells per
// stratum: lane groups of G = 2^ceil(log2 dxy) lanes, one stratum per group and one cell per
// lane, the margins by shuffles within the group, four strata sets per iteration.
template <bool kFp64>
__device__ inline Partial score_dense_groups(const int *T, int n_obs, int dx, int dy, const uint64_t *gzk,
                                             bool want_hash) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int dxy = dx * dy;
    int lg = 0;
    while ((1 << lg) < dxy) ++lg;
    const int G = 1 << lg, gpw = 32 >> lg, gi = lane >> lg, gl = lane & (G - 1);
    const unsigned gmask = G == 32 ? full : (((1u << G) - 1u) << (gi * G));
    const int x = gl / dy, y = gl - x * dy;
    const bool cell = gl < dxy;
    Partial acc{0, 0.0, 0.0, 0.0, 0ull};
    TermAcc<kFp64> ta;
    // four strata sets per iteration: their loads and shuffle chains are independent
    constexpr int U = 4;
    const int step = kWarps * gpw;
    for (int k0 = warp * gpw; k0 < n_obs; k0 += U * step) {
        int O[U], Nx[U], Ny[U], m[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + u * step + gi;
            O[u] = (cell && k < n_obs) ? __ldcg(T + (int64_t)k * dxy + gl) : 0;
            Nx[u] = 0;
            Ny[u] = 0;
        }
        for (int j = 0; j < dy; ++j) {
#pragma unroll
            for (int u = 0; u < U; ++u) Nx[u] += __shfl_sync(full, O[u], x * dy + j, G);
        }
        for (int i = 0; i < dx; ++i) {
#pragma unroll
            for (int u = 0; u < U; ++u) Ny[u] += __shfl_sync(full, O[u], i * dy + y, G);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) m[u] = O[u];
        for (int o = G >> 1; o > 0; o >>= 1) {
#pragma unroll
            for (int u = 0; u < U; ++u) m[u] += __shfl_xor_sync(full, m[u], o, G);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + u * step + gi;
            const bool valid = cell && k < n_obs;
            const int r = __popc(__ballot_sync(full, valid && y == 0 && Nx[u] > 0) & gmask);
            const int c = __popc(__ballot_sync(full, valid && x == 0 && Ny[u] > 0) & gmask);
            if (valid && gl == 0) acc.df += (long long)(max(r, 1) - 1) * (max(c, 1) - 1);
            if (valid && O[u] > 0) {
                ta.add(O[u], Nx[u], Ny[u], m[u]);
                if (want_hash)
                    acc.hash += cell_mix((gzk[k] * (uint64_t)dx + x) * (uint64_t)dy + y, (uint32_t)O[u]);
            }
        }
    }
    ta.into(acc);
    return acc;
}

// Dense strata x cells table T[k * dxy + x * dy + y] (k = stratum id), at most 32 cells per
// stratum, one thread per stratum: its counts are loaded together (one round trip) into a
// column of shared scratch, the x and y margins summed into two more, then the terms. Each
// thread owns column threadIdx.x of smem (96 ints at stride kThreads: a warp's threads hit
// 32 distinct banks). Every thread of the CTA calls it; returns the thread's share.
template <bool kFp64>
__device__ inline Partial score_dense_rows(const int *T, int n_obs, int dx, int dy, const uint64_t *gzk,
                                           bool want_hash, int *smem) {
    const int dxy = dx * dy;
    int *so = smem + threadIdx.x, *mx = so + 32 * kThreads, *my = mx + 32 * kThreads;
    Partial acc{0, 0.0, 0.0, 0.0, 0ull};
    TermAcc<kFp64> ta;
    for (int k = threadIdx.x; k < n_obs; k += kThreads) {
        const int *row = T + (int64_t)k * dxy;
        int o[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) o[c] = c < dxy ? __ldcg(row + c) : 0;
#pragma unroll
        for (int c = 0; c < 32; ++c)
            if (c < dxy) so[c * kThreads] = o[c];
        for (int i = 0; i < dx; ++i) mx[i * kThreads] = 0;
        for (int j = 0; j < dy; ++j) my[j * kThreads] = 0;
        int m = 0;
        for (int i = 0, c = 0; i < dx; ++i)
            for (int j = 0; j < dy; ++j, ++c) {
                const int v = so[c * kThreads];
                mx[i * kThreads] += v;
                my[j * kThreads] += v;
                m += v;
            }
        int r = 0, q = 0;
        for (int i = 0; i < dx; ++i) r += mx[i * kThreads] > 0;
        for (int j = 0; j < dy; ++j) q += my[j * kThreads] > 0;
        acc.df += (long long)(max(r, 1) - 1) * (max(q, 1) - 1);
        for (int i = 0, c = 0; i < dx; ++i)
            for (int j = 0; j < dy; ++j, ++c) {
                const int O = so[c * kThreads];
                if (O > 0) {
                    ta.add(O, mx[i * kThreads], my[j * kThreads], m);
                    if (want_hash) acc.hash += cell_mix((gzk[k] * (uint64_t)dx + i) * (uint64_t)dy + j, (uint32_t)O);
                }
            }
    }
    ta.into(acc);
    return acc;
}

// Phase timers (ns per phase, summed over tests) when a.dbg is set; off in normal runs.
__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------- tier 2, partitioned strata
// Tests whose strata overflow the shared hash are split into P = 2^lp partitions by the top
// lp bits of the mixed stratum code z * 2^64/phi, so a stratum never spans two partitions.
// One pass writes every sample once as a record (stratum code, (x << 8) | y) to its
// partition's run in the CTA's slot; each partition is then counted and scored in shared
// memory alone:
//   pass 1  the partition's codes are hashed to slots (next bits of the mixed code); a new
//           code appends its slot to occ[] (stratum i = occ[i]) and every slot counts its
//           samples in A[slot];
//   index   strata are ranked by size (1, 2, ..., 8 samples, then larger), so a warp's lanes
//           score strata of one size; A[slot] becomes the rank r and E[1 + r] the count,
//           scanned to the stratum's first sorted position;
//   pass 2  every record is found again and its (x << 8) | y code placed at its stratum's
//           cursor E[1 + r], so afterwards stratum r's samples are ord[E[r] .. E[r + 1]);
//   score   score_small_strata / score_big_strata over the strata.
// No global hash, no per-sample id array and no global scatter of the sorted codes (unless a
// partition holds more samples than the shared sorted array).
// Shared-memory plan (kSmemBytes, PartPlan<K>): keys K[cap] at 0 and A int[cap] after them
// (per-warp x,y tables once pass 2 is done), occ int[lim], E int[lim + 1], sorted codes u16[].
constexpr int kPartProbe = 256;                   // probe bound of the first pass
// Tests of fewer samples keep the compact kernel's global hash: measured on GB300, the
// partitioned path wins at 100,000 samples (1,041 nodes, cards 2-21: 3.85 vs 3.40 M tests/s)
// and loses at 50,000 (100 nodes, cards 2-5: 12.2 vs 13.4 M), where the global hash and the
// dense strata table mostly stay in L2.
constexpr int64_t kPartMinSamples = 65536;
template <class K>
struct PartPlan {
    static constexpr int cap = sizeof(K) == 4 ? 4096 : 2048;  // slots per partition table
    static constexpr int lcap = sizeof(K) == 4 ? 12 : 11;
    static constexpr int lim = cap * 3 / 4;                   // strata per partition at most
    static constexpr int a_off = cap * (int)sizeof(K);
    static constexpr int occ_off = a_off + cap * 4;
    static constexpr int e_off = occ_off + lim * 4;
    static constexpr int ord_off = (e_off + (lim + 1) * 4 + 15) / 16 * 16;
    static constexpr int ord_cap = (kSmemBytes - ord_off) / 2;  // sorted codes kept in shared memory
    static constexpr int wtab = occ_off / 4 / kWarps;            // ints per warp over keys + A
};
static_assert(PartPlan<uint32_t>::ord_cap > 8192 && PartPlan<uint64_t>::ord_cap > 8192, "partition shared plan");
static_assert((1 << PartPlan<uint32_t>::lcap) == PartPlan<uint32_t>::cap, "cap");
static_assert((1 << PartPlan<uint64_t>::lcap) == PartPlan<uint64_t>::cap, "cap");
static_assert(8 * kPartMax <= 2048, "partition padding fits the slot's sorted-code region");
static_assert(PartPlan<uint32_t>::lim <= kPartMinSamples, "stratum-indexed codes fit the zk region");

__device__ __forceinline__ uint64_t zmix(uint64_t z) { return z * 0x9E3779B97F4A7C15ull; }
__device__ __forceinline__ int part_of(uint64_t z, int lp) { return (int)(zmix(z) >> (64 - lp)); }  // lp >= 1
__device__ __forceinline__ uint32_t part_slot(uint64_t z, int lp, int lc) {
    return (uint32_t)((zmix(z) << lp) >> (64 - lc));
}

// Slot of code z, probing from slot h (claimed when absent: the slot is appended to occ[]);
// -1 after max_probe probes or beyond lim strata.
template <class K>
__device__ __forceinline__ int part_insert(K *keys, uint32_t cap, uint32_t h, K z, int max_probe, int *occ,
                                           int *n_occ, int lim) {
    const K empty = (K)kEmptyKey;
    for (int p = 0; p < max_probe; ++p) {
        const K k = keys[h];
        if (k == z) return (int)h;
        if (k == empty) {
            const K old = key_cas(&keys[h], empty, z);
            if (old == empty) {
                const int i = atomicAdd(n_occ, 1);
                if (i >= lim) return -1;
                occ[i] = (int)h;
                return (int)h;
            }
            if (old == z) return (int)h;
        }
        h = (h + 1) & (cap - 1);
    }
    return -1;
}

template <class K>
__device__ __forceinline__ int part_find(const K *keys, uint32_t cap, uint32_t h, K z) {
    for (uint32_t p = 0; p < cap; ++p) {
        if (keys[h] == z) return (int)h;
        h = (h + 1) & (cap - 1);
    }
    return 0;  // unreachable: every code was inserted in pass 1
}

// Eight consecutive records' codes (the run starts on a multiple of 8 records).
template <class K>
__device__ __forceinline__ void load8(K (&z)[8], const K *src) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    if constexpr (sizeof(K) == 4) {
        const uint4 w0 = __ldcg(s4), w1 = __ldcg(s4 + 1);
        z[0] = w0.x; z[1] = w0.y; z[2] = w0.z; z[3] = w0.w;
        z[4] = w1.x; z[5] = w1.y; z[6] = w1.z; z[7] = w1.w;
    } else {
        uint4 w[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) w[i] = __ldcg(s4 + i);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            z[2 * i] = (K)w[i].x | ((K)w[i].y << 32);
            z[2 * i + 1] = (K)w[i].z | ((K)w[i].w << 32);
        }
    }
}

// Partition histogram, offsets (every run padded to a multiple of 8 records) and the
// record pass.  s_poff[P] = records written, padding included.
// Pass 1 computes every stratum code once, stores it to zbuf (coalesced; S codes) and counts
// the partitions.  Pass 2 takes the codes back in chunks of kThreads x 16 samples, sorts a
// chunk's records by partition in shared memory (smem, dead at this point) and copies each
// partition's run out to consecutive records, so the global stores are coalesced.
constexpr int kScatterChunk = kThreads * 16;
// bmr (optional): the parent test's contributing-sample bitmap; samples whose bit is clear get
// no record.  rec_s (optional): each record's sample index, written beside its code.
template <class K, bool kBits>
__device__ __noinline__ void part_scatter_t(const uint8_t *const *col, const uint32_t *dim, int d, int64_t S, int lp,
                                            K *rec_z, uint16_t *rec_xy, int *s_pcnt, int *s_poff, int *s_pcur, K *zbuf,
                                            unsigned char *smem, const uint32_t *bmr, uint32_t *rec_s) {
    if constexpr (!kBits) {
        bmr = nullptr;
        rec_s = nullptr;
    }
    const int tid = threadIdx.x, P = 1 << lp;
    const int64_t nvec = S >> 4;
    const uint8_t *colx = col[d], *coly = col[d + 1];
    K *cz = reinterpret_cast<K *>(smem);
    uint16_t *cxy = reinterpret_cast<uint16_t *>(smem + kScatterChunk * sizeof(K));
    uint8_t *cp = reinterpret_cast<uint8_t *>(smem + kScatterChunk * (sizeof(K) + 2));
    uint32_t *cs = reinterpret_cast<uint32_t *>(smem + kScatterChunk * (sizeof(K) + 3));
    int *lcnt = reinterpret_cast<int *>(smem + kScatterChunk * (sizeof(K) + 7));
    int *lstart = lcnt + kPartMax, *gbase = lstart + kPartMax, *s_ctot = gbase + kPartMax;
    auto live16 = [&](int64_t v) -> uint32_t {
        if constexpr (!kBits) return 0xffffu;
        return bmr ? (__ldcg(bmr + (v >> 1)) >> (16 * (int)(v & 1))) & 0xffffu : 0xffffu;
    };
    auto live1 = [&](int64_t s) -> bool {
        if constexpr (!kBits) return true;
        return !bmr || ((__ldcg(bmr + (s >> 5)) >> (int)(s & 31)) & 1u);
    };
    for (int i = tid; i < P; i += kThreads) s_pcnt[i] = 0;
    __syncthreads();
    for (int64_t v = tid; v < nvec; v += kThreads) {
        K z[16];
        zcodes16(z, col, dim, d, v);
        uint4 *dst = reinterpret_cast<uint4 *>(zbuf + 16 * v);
        if constexpr (sizeof(K) == 4) {
#pragma unroll
            for (int q = 0; q < 4; ++q) dst[q] = make_uint4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q)
                dst[q] = make_uint4((uint32_t)z[2 * q], (uint32_t)(z[2 * q] >> 32), (uint32_t)z[2 * q + 1],
                                    (uint32_t)(z[2 * q + 1] >> 32));
        }
        const uint32_t lv = live16(v);
#pragma unroll
        for (int b = 0; b < 16; ++b) atomicAdd(&s_pcnt[part_of(z[b], lp)], (int)((lv >> b) & 1u));  // no branch
    }
    for (int64_t s = (S & ~(int64_t)15) + tid; s < S; s += kThreads) {
        K z = 0;
        for (int j = 0; j < d; ++j) z = z * (K)dim[j] + col[j][s];
        zbuf[s] = z;
        if (live1(s)) atomicAdd(&s_pcnt[part_of(z, lp)], 1);
    }
    __syncthreads();
    if (tid < 32) {  // padded exclusive scan, eight partitions per lane at most
        const int per = (P + 31) / 32;
        int sum = 0;
        for (int i = 0; i < per; ++i) {
            const int p = tid * per + i;
            if (p < P) sum += (s_pcnt[p] + 7) & ~7;
        }
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (tid >= o) incl += t;
        }
        int run = incl - sum;
        for (int i = 0; i < per; ++i) {
            const int p = tid * per + i;
            if (p < P) {
                s_poff[p] = run;
                s_pcur[p] = run;
                run += (s_pcnt[p] + 7) & ~7;
            }
        }
        if (tid == 31) s_poff[P] = incl;
    }
    __syncthreads();
    const int64_t nchunks = (nvec + kThreads - 1) / kThreads;
    for (int64_t c = 0; c < nchunks; ++c) {
        const int64_t v = c * kThreads + tid;
        const bool have = v < nvec;
        for (int i = tid; i < P; i += kThreads) lcnt[i] = 0;
        __syncthreads();
        K z[16];
        int rk[16];
        uint32_t xx[4] = {0u, 0u, 0u, 0u}, yy[4] = {0u, 0u, 0u, 0u};
        if (have) {
            const uint4 *src = reinterpret_cast<const uint4 *>(zbuf + 16 * v);
            if constexpr (sizeof(K) == 4) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint4 w = __ldcg(src + q);
                    z[4 * q] = w.x;
                    z[4 * q + 1] = w.y;
                    z[4 * q + 2] = w.z;
                    z[4 * q + 3] = w.w;
                }
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const uint4 w = __ldcg(src + q);
                    z[2 * q] = (K)w.x | ((K)w.y << 32);
                    z[2 * q + 1] = (K)w.z | ((K)w.w << 32);
                }
            }
            const uint4 wx = __ldg(reinterpret_cast<const uint4 *>(colx) + v);
            const uint4 wy = __ldg(reinterpret_cast<const uint4 *>(coly) + v);
            xx[0] = wx.x; xx[1] = wx.y; xx[2] = wx.z; xx[3] = wx.w;
            yy[0] = wy.x; yy[1] = wy.y; yy[2] = wy.z; yy[3] = wy.w;
            const uint32_t lv = live16(v);
#pragma unroll
            for (int b = 0; b < 16; ++b) {  // no branch: a left-out sample adds 0 and keeps no rank
                rk[b] = atomicAdd(&lcnt[part_of(z[b], lp)], (int)((lv >> b) & 1u));
                if (!((lv >> b) & 1u)) rk[b] = -1;
            }
        }
        __syncthreads();
        if (tid < 32) {  // chunk offsets per partition, and each run's place in the records
            const int per = (P + 31) / 32;
            int sum = 0;
            for (int i = 0; i < per; ++i) {
                const int p = tid * per + i;
                if (p < P) sum += lcnt[p];
            }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (tid >= o) incl += t;
            }
            int run = incl - sum;
            for (int i = 0; i < per; ++i) {
                const int p = tid * per + i;
                if (p < P) {
                    lstart[p] = run;
                    gbase[p] = lcnt[p] ? atomicAdd(&s_pcur[p], lcnt[p]) : 0;
                    run += lcnt[p];
                }
            }
            if (tid == 31) *s_ctot = incl;  // records of this chunk
        }
        __syncthreads();
        if (have) {
#pragma unroll
            for (int b = 0; b < 16; ++b) {
                if (rk[b] < 0) continue;
                const int p = part_of(z[b], lp), pos = lstart[p] + rk[b], sh = 8 * (b & 3);
                cz[pos] = z[b];
                cxy[pos] = (uint16_t)((((xx[b >> 2] >> sh) & 0xffu) << 8) | ((yy[b >> 2] >> sh) & 0xffu));
                cp[pos] = (uint8_t)p;
                if (rec_s) cs[pos] = (uint32_t)(16 * v + b);
            }
        }
        __syncthreads();
        const int n_in = *s_ctot;
        for (int i = tid; i < n_in; i += kThreads) {
            const int p = cp[i];
            const int g = gbase[p] + (i - lstart[p]);
            rec_z[g] = cz[i];
            rec_xy[g] = cxy[i];
            if (rec_s) rec_s[g] = cs[i];
        }
        __syncthreads();
    }
    for (int64_t s = (S & ~(int64_t)15) + tid; s < S; s += kThreads) {
        if (!live1(s)) continue;
        const K z = zbuf[s];
        const int pos = atomicAdd(&s_pcur[part_of(z, lp)], 1);
        rec_z[pos] = z;
        rec_xy[pos] = (uint16_t)((colx[s] << 8) | coly[s]);
        if (rec_s) rec_s[pos] = (uint32_t)s;
    }
    // padding records carry the empty key (never a stratum code), so a run of partitions
    // can be read as one
    for (int p = tid; p < P; p += kThreads)
        for (int i = s_poff[p] + s_pcnt[p]; i < s_poff[p + 1]; ++i) rec_z[i] = (K)kEmptyKey;
    __syncthreads();
}
static_assert(kScatterChunk * (8 + 7) + 3 * kPartMax * 4 + 4 <= kSmemBytes, "scatter chunk in shared memory");
// without a bitmap to read or write, the plain instance (no per-sample checks)
template <class K>
__device__ inline void part_scatter(const uint8_t *const *col, const uint32_t *dim, int d, int64_t S, int lp, K *rec_z,
                                    uint16_t *rec_xy, int *s_pcnt, int *s_poff, int *s_pcur, K *zbuf, unsigned char *smem,
                                    const uint32_t *bmr, uint32_t *rec_s) {
    if (bmr || rec_s)
        part_scatter_t<K, true>(col, dim, d, S, lp, rec_z, rec_xy, s_pcnt, s_poff, s_pcur, zbuf, smem, bmr, rec_s);
    else
        part_scatter_t<K, false>(col, dim, d, S, lp, rec_z, rec_xy, s_pcnt, s_poff, s_pcur, zbuf, smem, nullptr,
                                 nullptr);
}

// Counts and scores one partition (n records from rec_z/rec_xy + base) in shared memory;
// returns this thread's share of the statistic.  *s_over is set when the partition's codes
// overflow its table (first pass only: the FP64 recheck probes without bound, so it cannot
// fail where the first pass did not).  Thread 0 adds the strata it saw to claims.  Every
// thread of the CTA calls it; it ends on a barrier, so shared memory is free afterwards.
template <bool kFp64, class K>
__device__ __noinline__ Partial part_partition(int lp, const K *rec_z, const uint16_t *rec_xy, int n, int base,
                                               int dx, int dy, unsigned char *smem, uint16_t *gord, int *gwt,
                                               uint64_t *gzk, bool want_hash, int *s_w, int *s_over, int *s_nbig,
                                               int *s_nocc, int *s_bin, int &claims, unsigned long long *dbg) {
    using Plan = PartPlan<K>;
    constexpr uint32_t cap = Plan::cap;
    const int tid = threadIdx.x, warp = tid >> 5;
    K *keys = reinterpret_cast<K *>(smem);
    int *A = reinterpret_cast<int *>(smem + Plan::a_off);
    int *occ = reinterpret_cast<int *>(smem + Plan::occ_off);
    int *E = reinterpret_cast<int *>(smem + Plan::e_off);
    uint16_t *sord = reinterpret_cast<uint16_t *>(smem + Plan::ord_off);
    const int dxy = dx * dy;
    const bool wsmem = dxy + dx + dy <= Plan::wtab;
    int *wt = wsmem ? reinterpret_cast<int *>(smem) + warp * Plan::wtab : gwt + (int64_t)warp * kGlobalWarpTab;
    const int max_probe = kFp64 ? (int)cap : kPartProbe;
    const int lim = Plan::lim;  // the same strata in both passes: the FP64 one cannot exceed it
    Partial acc{0, 0.0, 0.0, 0.0, 0ull};
    // sub-phase timers of thread 0 (FPGM_PHASE_TIMERS): dbg[16..21]
    unsigned long long tp = (dbg && tid == 0) ? gtimer() : 0ull;
    auto lap = [&](int i) {
        if (dbg && tid == 0) {
            const unsigned long long t = gtimer();
            atomicAdd(&dbg[i], t - tp);
            tp = t;
        }
    };
    for (uint32_t i = tid; i < cap; i += kThreads) {
        keys[i] = (K)kEmptyKey;
        A[i] = 0;
    }
    if (tid == 0) *s_nocc = 0;
    if (tid < 10) s_bin[tid] = 0;
    __syncthreads();
    lap(16);
    // pass 1: first probes of eight codes at once; misses take the inserting path
    const int ngroups = (n + 7) >> 3;
    for (int g = tid; g < ngroups; g += kThreads) {
        K z[8];
        load8(z, rec_z + base + 8 * g);
        const int m = n - 8 * g;
        uint32_t h[8];
        K k0[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            h[j] = part_slot(z[j], lp, Plan::lcap);
            k0[j] = j < m ? keys[h[j]] : z[j];
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (j >= m) break;
            int hj = (int)h[j];
            if (k0[j] != z[j]) hj = part_insert(keys, cap, h[j], z[j], max_probe, occ, s_nocc, lim);
            if (hj < 0) {
                *s_over = 1;
                break;
            }
            atomicAdd(&A[hj], 1);
        }
    }
    __syncthreads();
    lap(17);
    if (*s_over == 0) {
        const int n_occ = *s_nocc;
        if (tid == 0) claims += n_occ;
        // strata ranked by size: bins 1..8 samples, 9 for larger ones
        for (int i = tid; i < n_occ; i += kThreads) atomicAdd(&s_bin[min(A[occ[i]], 9)], 1);
        __syncthreads();
        if (tid == 0) {
            int run = 0;
            for (int b = 1; b < 10; ++b) {
                const int c = s_bin[b];
                s_bin[b] = run;
                run += c;
            }
            E[0] = 0;
        }
        __syncthreads();
        for (int i = tid; i < n_occ; i += kThreads) {
            const int sl = occ[i], m = A[sl];
            const int r = atomicAdd(&s_bin[min(m, 9)], 1);
            E[1 + r] = m;
            A[sl] = r;
            if (want_hash) gzk[r] = (uint64_t)keys[sl];
        }
        __syncthreads();
        block_exclusive_scan(E + 1, n_occ, s_w);
        lap(18);
        uint16_t *ord = n <= Plan::ord_cap ? sord : gord + base;
        for (int g = tid; g < ngroups; g += kThreads) {
            K z[8];
            load8(z, rec_z + base + 8 * g);
            const uint4 c = __ldcg(reinterpret_cast<const uint4 *>(rec_xy + base) + g);
            const uint32_t cw[4] = {c.x, c.y, c.z, c.w};
            const int m = n - 8 * g;
            uint32_t h[8];
            K k0[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                h[j] = part_slot(z[j], lp, Plan::lcap);
                k0[j] = j < m ? keys[h[j]] : z[j];
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (j >= m) break;
                const int hj = k0[j] == z[j] ? (int)h[j] : part_find(keys, cap, h[j], z[j]);
                const int pos = atomicAdd(&E[1 + A[hj]], 1);
                ord[pos] = (uint16_t)(cw[j >> 1] >> (16 * (j & 1)));
            }
        }
        __syncthreads();
        lap(19);
        if (wsmem)  // keys and A are dead: per-warp x,y tables
            for (int i = tid; i < Plan::occ_off / 4; i += kThreads) reinterpret_cast<int *>(smem)[i] = 0;
        if (tid == 0) *s_nbig = 0;
        __syncthreads();
        // the larger strata are listed over occ[] (dead since the index step)
        Partial q = score_small_strata<kFp64>(E, ord, n_occ, dx, dy, occ, s_nbig, gzk, want_hash, true);
        __syncthreads();
        lap(20);
        const int n_big = *s_nbig;
        acc = score_big_strata<kFp64>(q, E, ord, occ, n_big, dx, dy, wt, gzk, want_hash);
    }
    __syncthreads();  // before the next partition reuses shared memory
    lap(21);
    return acc;
}

__device__ __forceinline__ void partial_add(Partial &a, const Partial &b) {
    a.df += b.df;
    a.g2 += b.g2;
    a.err += b.err;
    a.abs_g2 += b.abs_g2;
    a.hash += b.hash;
}

// ---------------------------------------------------------------- staged partitions
// A run of consecutive partitions ("super-partition", at most StagePlan<K>::rec records,
// padding included) is copied from the records into shared memory first, so the passes over
// it never wait on global memory:
//   insert  codes hashed to slots as in part_partition; the slot replaces the code in place;
//           samples per slot summed with one atomic per group of equal slots in a warp
//           (match.any), new strata appended to occ[] with one atomic per warp;
//   rank    strata ranked by size (2 .. 8 samples, larger; single-sample strata, which add
//           neither a degree of freedom nor a G^2 term, are left out unless the cell
//           fingerprint is wanted), ranks handed out with one atomic per warp and size;
//   place   (x << 8) | y codes sorted by stratum over the dead hash keys;
//   score   one lane per stratum of at most kLaneStratum samples, one warp per larger one
//           (per-warp x,y tables over the dead records).
// Padding records (a run is padded to 8 records) carry the empty key and are skipped.
template <class K>
struct StagePlan {
    static constexpr int cap = PartPlan<K>::cap, lcap = PartPlan<K>::lcap, lim = PartPlan<K>::lim;
    static constexpr int a_off = cap * (int)sizeof(K);
    static constexpr int occ_off = a_off + cap * 4;
    static constexpr int e_off = occ_off + lim * 4;
    static constexpr int rec_off = (e_off + (lim + 1) * 4 + 15) / 16 * 16;
    static constexpr int rec = (kSmemBytes - rec_off) / ((int)sizeof(K) + 2) / 8 * 8;  // records at most
    static constexpr int xy_off = rec_off + rec * (int)sizeof(K);
    static constexpr int wtab = (rec * ((int)sizeof(K) + 2)) / 4 / kWarps;  // ints per warp over the records
    static constexpr int wtab_z = rec * (int)sizeof(K) / 4 / kWarps;         // ... over the codes alone
};
static_assert(StagePlan<uint32_t>::rec * 2 <= StagePlan<uint32_t>::a_off, "sorted codes over the u32 keys");
static_assert(StagePlan<uint64_t>::rec * 2 <= StagePlan<uint64_t>::a_off, "sorted codes over the u64 keys");
static_assert(StagePlan<uint32_t>::xy_off + StagePlan<uint32_t>::rec * 2 <= kSmemBytes, "u32 stage plan");
static_assert(StagePlan<uint64_t>::xy_off + StagePlan<uint64_t>::rec * 2 <= kSmemBytes, "u64 stage plan");
static_assert(StagePlan<uint32_t>::rec >= 4096 && StagePlan<uint64_t>::rec >= 4096, "stage plan records");

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Eight consecutive staged codes from shared memory (vector loads).
template <class K>
__device__ __forceinline__ void sload8(K (&z)[8], const K *src) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    if constexpr (sizeof(K) == 4) {
        const uint4 w0 = s4[0], w1 = s4[1];
        z[0] = w0.x; z[1] = w0.y; z[2] = w0.z; z[3] = w0.w;
        z[4] = w1.x; z[5] = w1.y; z[6] = w1.z; z[7] = w1.w;
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint4 w = s4[i];
            z[2 * i] = (K)w.x | ((K)w.y << 32);
            z[2 * i + 1] = (K)w.z | ((K)w.w << 32);
        }
    }
}

// The slots of eight consecutive records replace their codes in place (low word of each
// code's place), and are read back the same way.
template <class K>
__device__ __forceinline__ void slot_store8(K *dst, const int (&sl)[8]) {
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    if constexpr (sizeof(K) == 4) {
        d4[0] = make_uint4(sl[0], sl[1], sl[2], sl[3]);
        d4[1] = make_uint4(sl[4], sl[5], sl[6], sl[7]);
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) d4[i] = make_uint4(sl[2 * i], 0u, sl[2 * i + 1], 0u);
    }
}
template <class K>
__device__ __forceinline__ int stage_slot(const K *zr, int i) {
    return reinterpret_cast<const int *>(zr)[i * (int)(sizeof(K) / 4)];
}
template <class K>
__device__ __forceinline__ void slot_load8(int (&sl)[8], const K *src) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    if constexpr (sizeof(K) == 4) {
        const uint4 w0 = s4[0], w1 = s4[1];
        sl[0] = w0.x; sl[1] = w0.y; sl[2] = w0.z; sl[3] = w0.w;
        sl[4] = w1.x; sl[5] = w1.y; sl[6] = w1.z; sl[7] = w1.w;
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint4 w = s4[i];
            sl[2 * i] = (int)w.x;
            sl[2 * i + 1] = (int)w.z;
        }
    }
}

// Counts and scores n records (a multiple of 8, padding included) from base in shared
// memory; n <= StagePlan<K>::rec.  As part_partition: *s_over is set when the strata
// overflow the table (first pass only), claims gets the strata seen, and it ends on a
// barrier.  s_bin: 16 ints of shared scratch.
// bmw / rec_s (optional, first pass only): the test's contributing-sample bitmap, set here for
// the samples of strata with two or more values of x and of y, and the records' sample
// indices (the per-warp x,y tables then live in global memory, so the records' slots survive
// the scoring).
template <bool kFp64, class K>
__device__ __noinline__ Partial part_staged(int lp, const K *rec_z, const uint16_t *rec_xy, int base, int n, int dx,
                                            int dy, unsigned char *smem, int *gwt, uint64_t *gzk, bool want_hash,
                                            int *s_w, int *s_over, int *s_nocc, int *s_bin, int &claims,
                                            unsigned long long *dbg, uint32_t *bmw = nullptr,
                                            const uint32_t *rec_s = nullptr, unsigned long long *lstat = nullptr) {
    using Plan = StagePlan<K>;
    constexpr uint32_t cap = Plan::cap;
    const unsigned full = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    K *keys = reinterpret_cast<K *>(smem);
    int *A = reinterpret_cast<int *>(smem + Plan::a_off);
    int *occ = reinterpret_cast<int *>(smem + Plan::occ_off);
    int *E = reinterpret_cast<int *>(smem + Plan::e_off);
    K *zr = reinterpret_cast<K *>(smem + Plan::rec_off);
    uint16_t *xyr = reinterpret_cast<uint16_t *>(smem + Plan::xy_off);
    uint16_t *sorted = reinterpret_cast<uint16_t *>(smem);  // over the keys once they are dead
    const int dxy = dx * dy;
    const bool bits = !kFp64 && bmw != nullptr;
    // with a bitmap to write, the records' ranks are kept over their x,y codes, so the per-warp
    // tables use the codes' part of the records region only
    const int wtab = bits ? Plan::wtab_z : Plan::wtab;
    const bool wsmem = dxy + dx + dy <= wtab;
    int *wt = wsmem ? reinterpret_cast<int *>(smem + Plan::rec_off) + warp * wtab
                    : gwt + (int64_t)warp * kGlobalWarpTab;
    uint8_t *live = (bits || (!kFp64 && lstat)) ? reinterpret_cast<uint8_t *>(occ) : nullptr;  // per ranked stratum
                                                                                        // (occ is dead then)
    const int max_probe = kFp64 ? (int)cap : kPartProbe;
    const K empty = (K)kEmptyKey;
    Partial acc{0, 0.0, 0.0, 0.0, 0ull};
    // sub-phase timers of thread 0 (FPGM_PHASE_TIMERS): dbg[16..21]
    unsigned long long tp = (dbg && tid == 0) ? gtimer() : 0ull;
    auto lap = [&](int i) {
        if (dbg && tid == 0) {
            const unsigned long long t = gtimer();
            atomicAdd(&dbg[i], t - tp);
            tp = t;
        }
    };
    for (uint32_t i = tid; i < cap; i += kThreads) {
        keys[i] = empty;
        A[i] = 0;
    }
    if (tid == 0) *s_nocc = 0;
    if (tid < 16) s_bin[tid] = 0;
    {  // the records, every load in flight before the first store
        const uint4 *gz = reinterpret_cast<const uint4 *>(rec_z + base);
        const uint4 *gxy = reinterpret_cast<const uint4 *>(rec_xy + base);
        uint4 *sz = reinterpret_cast<uint4 *>(zr), *sxy = reinterpret_cast<uint4 *>(xyr);
        const int nz4 = n * (int)sizeof(K) / 16, nx4 = n / 8;
        for (int i = tid; i < nz4; i += 4 * kThreads) {
            uint4 w[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i + u * kThreads < nz4) w[u] = __ldcg(gz + i + u * kThreads);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i + u * kThreads < nz4) sz[i + u * kThreads] = w[u];
        }
        for (int i = tid; i < nx4; i += kThreads) sxy[i] = __ldcg(gxy + i);
    }
    __syncthreads();
    lap(16);
    // insert: eight records per thread and round; every lane runs every round (warp collectives)
    const int ngroups = n >> 3;
    const int rounds = (ngroups + kThreads - 1) / kThreads;
    for (int rd = 0; rd < rounds; ++rd) {
        const int g = rd * kThreads + tid;
        const bool have = g < ngroups;
        int sl[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) sl[j] = -1;
        unsigned claimed = 0;
        if (have) {
            K z[8];
            sload8(z, zr + 8 * g);
            uint32_t h[8];
            K k0[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                h[j] = part_slot(z[j], lp, Plan::lcap);
                k0[j] = z[j] == empty ? empty : keys[h[j]];
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (z[j] == empty) continue;
                if (k0[j] == z[j]) {
                    sl[j] = (int)h[j];
                    continue;
                }
                uint32_t hh = h[j];
                for (int p = 0; p < max_probe; ++p) {
                    const K k = keys[hh];
                    if (k == z[j]) {
                        sl[j] = (int)hh;
                        break;
                    }
                    if (k == empty) {
                        const K old = key_cas(&keys[hh], empty, z[j]);
                        if (old == empty) {
                            sl[j] = (int)hh;
                            claimed |= 1u << j;
                            break;
                        }
                        if (old == z[j]) {
                            sl[j] = (int)hh;
                            break;
                        }
                    }
                    hh = (hh + 1) & (cap - 1);
                }
                if (sl[j] < 0) *s_over = 1;  // probe bound reached
            }
            slot_store8(zr + 8 * g, sl);
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (sl[j] >= 0) atomicAdd(&A[sl[j]], 1);
        }
        // new strata appended to occ[]: one atomic per warp
        const int c = __popc(claimed);
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(full, incl, o);
            if (lane >= o) incl += t;
        }
        int first = 0;
        if (lane == 31 && incl > 0) first = atomicAdd(s_nocc, incl);
        first = __shfl_sync(full, first, 31) + incl - c;
        while (claimed) {
            const int j = __ffs(claimed) - 1;
            claimed &= claimed - 1;
            if (first < Plan::lim) occ[first] = sl[j];
            ++first;
        }
    }
    __syncthreads();
    const int n_occ = *s_nocc;
    if (n_occ > Plan::lim) *s_over = 1;
    __syncthreads();
    lap(17);
    if (*s_over == 0) {
        if (tid == 0) claims += n_occ;
        // rank by size: bin 0 unscored (single samples), 1 .. 8 samples, 9 larger.  Per warp and
        // round, lane b adds the warp's count of bin b (one atomic instruction for all bins).
        auto bin_of = [&](int m) { return (m <= 1 && !want_hash) ? 0 : (m <= 8 ? m : 9); };
        const int orounds = (n_occ + kThreads - 1) / kThreads;
        for (int rd = 0; rd < orounds; ++rd) {
            const int i = rd * kThreads + tid;
            const int b = i < n_occ ? bin_of(A[occ[i]]) : 0;
            unsigned mine = 0;
#pragma unroll
            for (int bb = 1; bb <= 9; ++bb) {
                const unsigned bal = __ballot_sync(full, b == bb);
                if (lane == bb) mine = bal;
            }
            if (lane >= 1 && lane <= 9 && mine) atomicAdd(&s_bin[lane], __popc(mine));
        }
        __syncthreads();
        if (tid == 0) {
            int run = 0;
            for (int bb = 1; bb <= 9; ++bb) {
                const int cnt = s_bin[bb];
                s_bin[bb] = run;
                if (bb == 9) s_bin[12] = run;  // first stratum of more than kLaneStratum samples
                run += cnt;
            }
            s_bin[15] = run;  // strata scored
            E[0] = 0;
        }
        __syncthreads();
        for (int rd = 0; rd < orounds; ++rd) {
            const int i = rd * kThreads + tid;
            int b = 0, m = 0, s = -1;
            if (i < n_occ) {
                s = occ[i];
                m = A[s];
                b = bin_of(m);
            }
            unsigned mine = 0, bal_b = 0;
#pragma unroll
            for (int bb = 1; bb <= 9; ++bb) {
                const unsigned bal = __ballot_sync(full, b == bb);
                if (lane == bb) mine = bal;
                if (b == bb) bal_b = bal;
            }
            int r0 = 0;
            if (lane >= 1 && lane <= 9 && mine) r0 = atomicAdd(&s_bin[lane], __popc(mine));
            r0 = __shfl_sync(full, r0, b);  // lane b holds this bin's first rank for the warp
            const int r = b > 0 ? r0 + __popc(bal_b & lanemask_lt()) : -1;
            if (s >= 0) {
                if (r >= 0) {
                    E[1 + r] = m;
                    if (want_hash) gzk[r] = (uint64_t)keys[s];
                }
                A[s] = r;  // -1: not scored
            }
        }
        __syncthreads();
        const int n_live = s_bin[15], first_big = s_bin[12];
        block_exclusive_scan(E + 1, n_live, s_w);  // ends with a barrier; the keys are dead
        lap(18);
        // place: (x << 8) | y codes by stratum, one atomic per group of lanes with the same stratum
        for (int rd = 0; rd < rounds; ++rd) {
            const int g = rd * kThreads + tid;
            const bool have = g < ngroups;
            if (have) {
                const uint4 c4 = reinterpret_cast<const uint4 *>(xyr)[g];
                const uint32_t cw[4] = {c4.x, c4.y, c4.z, c4.w};
                int sl[8], r[8];
                slot_load8(sl, zr + 8 * g);
#pragma unroll
                for (int j = 0; j < 8; ++j) r[j] = sl[j] >= 0 ? A[sl[j]] : -1;
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (r[j] >= 0) sorted[atomicAdd(&E[1 + r[j]], 1)] = (uint16_t)(cw[j >> 1] >> (16 * (j & 1)));
                if (bits)  // each record's rank (0xffff: not scored) over its dead x,y code
                    reinterpret_cast<uint4 *>(xyr)[g] =
                        make_uint4(((uint32_t)r[0] & 0xffffu) | ((uint32_t)r[1] << 16),
                                   ((uint32_t)r[2] & 0xffffu) | ((uint32_t)r[3] << 16),
                                   ((uint32_t)r[4] & 0xffffu) | ((uint32_t)r[5] << 16),
                                   ((uint32_t)r[6] & 0xffffu) | ((uint32_t)r[7] << 16));
            }
        }
        __syncthreads();
        if (wsmem)  // the records are dead: per-warp x,y tables
            for (int i = tid; i < kWarps * wtab; i += kThreads)
                reinterpret_cast<int *>(smem + Plan::rec_off)[i] = 0;
        __syncthreads();
        lap(19);
        Partial q = score_small_strata<kFp64>(E, sorted, first_big, dx, dy, nullptr, nullptr, gzk, want_hash, false,
                                              live);
        if (dbg) {
            __syncthreads();
            lap(20);
            if (tid == 0) {  // strata of more than kLaneStratum samples, and their samples
                atomicAdd(&dbg[25], (unsigned long long)(n_live - first_big));
                atomicAdd(&dbg[26], (unsigned long long)(E[n_live] - E[first_big]));
                atomicAdd(&dbg[27], (unsigned long long)n);
            }
        }
        acc = score_big_strata<kFp64>(q, E, sorted, nullptr, n_live - first_big, dx, dy, wt, gzk, want_hash,
                                      first_big, live);
        if (live && lstat) {  // how many of the scored samples lie in contributing strata
            __syncthreads();
            unsigned long long in = 0;
            for (int k = tid; k < n_live; k += kThreads)
                if (live[k]) in += (unsigned long long)(E[k + 1] - E[k]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) in += __shfl_xor_sync(full, in, o);
            if (lane == 0 && in) atomicAdd(&lstat[0], in);
        }
        if (bits) {  // the samples of contributing strata into the test's bitmap
            __syncthreads();
            for (int i = tid; i < n; i += kThreads) {
                const uint32_t r = xyr[i];
                if (r == 0xffffu || !live[r]) continue;
                const uint32_t si = __ldcg(rec_s + base + i);
                atomicOr(&bmw[si >> 5], 1u << (si & 31));
            }
        }
    }
    __syncthreads();  // before the next super-partition reuses shared memory
    lap(21);
    return acc;
}

// Super-partitions: consecutive partitions [sp[i], sp[i + 1]) whose padded records total at
// most rmax (a single partition beyond rmax stands alone).  One thread; returns their count.
__device__ inline int plan_super(const int *pcnt, int P, int rmax, int *sp) {
    int ns = 0, run = 0;
    sp[0] = 0;
    for (int p = 0; p < P; ++p) {
        const int w = (pcnt[p] + 7) & ~7;
        if (run > 0 && run + w > rmax) {
            sp[++ns] = p;
            run = 0;
        }
        run += w;
    }
    sp[++ns] = P;
    return ns;
}

// One super-partition [b0, b1): staged as a whole when its records fit; when its strata
// overflow, its partitions one by one; a partition beyond the staged records goes through
// part_partition (records read from global memory).  *s_over is left set only when a single
// partition overflows.
template <bool kFp64, class K>
__device__ inline Partial part_super(int lp, const K *rec_z, const uint16_t *rec_xy, const int *pcnt, const int *poff,
                                     int b0, int b1, int dx, int dy, unsigned char *smem, uint16_t *gord, int *gwt,
                                     uint64_t *gzk, bool want_hash, int *s_w, int *s_over, int *s_nbig, int *s_nocc,
                                     int *s_bin, int &claims, int rstage, unsigned long long *dbg = nullptr,
                                     uint32_t *bmw = nullptr, const uint32_t *rec_s = nullptr,
                                     int *s_bmbad = nullptr, unsigned long long *lstat = nullptr) {
    const int R = rstage > 0 && rstage < StagePlan<K>::rec ? rstage : StagePlan<K>::rec;
    const int n = poff[b1] - poff[b0];
    if (n == 0) return Partial{0, 0.0, 0.0, 0.0, 0ull};
    if (n <= R) {
        const Partial q = part_staged<kFp64, K>(lp, rec_z, rec_xy, poff[b0], n, dx, dy, smem, gwt, gzk, want_hash, s_w,
                                                s_over, s_nocc, s_bin, claims, dbg, bmw, rec_s, lstat);
        if (*s_over == 0 || b1 - b0 == 1) return q;  // read after part_staged's closing barrier
        __syncthreads();  // every thread has read s_over
        if (threadIdx.x == 0) {
            *s_over = 0;
            if (dbg) atomicAdd(&dbg[24], 1ull);  // super-partitions split again
        }
        __syncthreads();
    }
    Partial acc{0, 0.0, 0.0, 0.0, 0ull};
    for (int b = b0; b < b1; ++b) {
        if (pcnt[b] == 0) continue;
        const int nb = poff[b + 1] - poff[b];
        if (nb > R && bmw && s_bmbad && threadIdx.x == 0) *s_bmbad = 1;  // counted unstaged: no bitmap
        const Partial q =
            nb <= R ? part_staged<kFp64, K>(lp, rec_z, rec_xy, poff[b], nb, dx, dy, smem, gwt, gzk, want_hash, s_w,
                                            s_over, s_nocc, s_bin, claims, dbg, bmw, rec_s, lstat)
                    : part_partition<kFp64, K>(lp, rec_z, rec_xy, pcnt[b], poff[b], dx, dy, smem, gord, gwt, gzk,
                                               want_hash, s_w, s_over, s_nbig, s_nocc, s_bin, claims, dbg);
        if (*s_over) return acc;
        partial_add(acc, q);
    }
    return acc;
}

// Counts and scores every super-partition of a test (sp[0 .. n_sp]: partition boundaries,
// plan_super) in shared memory, one after another; returns this thread's share of the
// statistic (see part_super; stops at the first overflow).  s_pcnt / s_poff: records per
// partition and each partition's first record.
template <bool kFp64, class K>
__device__ __noinline__ Partial part_run(int lp, const K *rec_z, const uint16_t *rec_xy, const int *s_pcnt,
                                         const int *s_poff, const int *sp, int n_sp, int dx, int dy,
                                         unsigned char *smem, uint16_t *gord, int *gwt, uint64_t *gzk, bool want_hash,
                                         int *s_w, int *s_over, int *s_nbig, int *s_nocc, int *s_bin, int &claims,
                                         int rstage, unsigned long long *dbg, uint32_t *bmw = nullptr,
                                         const uint32_t *rec_s = nullptr, int *s_bmbad = nullptr,
                                         unsigned long long *lstat = nullptr) {
    Partial acc{0, 0.0, 0.0, 0.0, 0ull};
    if (dbg && threadIdx.x == 0) atomicAdd(&dbg[22], (unsigned long long)n_sp);
    for (int i = 0; i < n_sp; ++i) {
        const Partial q = part_super<kFp64, K>(lp, rec_z, rec_xy, s_pcnt, s_poff, sp[i], sp[i + 1], dx, dy, smem, gord,
                                               gwt, gzk, want_hash, s_w, s_over, s_nbig, s_nocc, s_bin, claims, rstage,
                                               dbg, bmw, rec_s, s_bmbad, lstat);
        if (*s_over) break;  // read after part_super's closing barrier, same in every thread
        partial_add(acc, q);
    }
    return acc;
}

// FP32 statistic r (block-summed) -> decision: band tables, Wilson-Hilferty beyond them;
// inside the band the FP64 statistic (recheck() returns each thread's share) decides.
// Called by every thread of the CTA; thread 0 records the verdict of a tier-2 test (path 2
// compact strata, 3 partitioned strata).
template <class Recheck>
__device__ inline void decide_record(const WaveArgs &a, int item, const Partial &r, int64_t cells, int path,
                                     int &s_flag, Partial *scratch, Recheck &&recheck) {
    const int tid = threadIdx.x;
    const double err = 2.0 * r.err + 1e-6 * r.abs_g2 + 1e-12;
    int dec = band_decide(r.df, r.g2, err, a.bt);
    if (dec < 0 && r.df > a.bt.dfmax) {
        // beyond the tables: Wilson-Hilferty p of the FP32 statistic, widened by its own
        // error and by the propagated G^2 error (chi-square density <= 0.3/sqrt(df) here)
        if (tid == 0) {
            const double pw = chisq_pvalue_wh(r.g2, (double)r.df);
            const double dist = fabs(pw - a.alpha);
            const double dpb = 2.0 * err * 0.3 / sqrt((double)r.df);
            s_flag = (dist > kBand + kWhMargin && dist > dpb + kWhMargin) ? (pw > a.alpha) : -1;
        }
        __syncthreads();
        dec = s_flag;
    }
    Verdict v{r.df, r.g2, 1.0, 1, 0, 0.0, r.hash};
    if (dec < 0) {
        const Partial r2 = block_sum(recheck(), scratch);
        v.g2 = r2.g2;
        v.rechecked = 1;
        if (tid == 0) {
            v.p = chisq_pvalue(r2.g2, r.df);
            v.indep = v.p > a.alpha;
            v.dp = fabs(v.p - chisq_pvalue(r.g2, r.df));
        }
    } else {
        v.indep = dec;
        if (tid == 0) v.p = (a.detail != nullptr && r.df > 0) ? chisq_pvalue(r.g2, r.df) : (dec ? 1.0 : 0.0);
    }
    if (tid == 0) {
        atomicAdd(&a.stats[ST_LARGE], 1ull);
        record(a, item, v, cells, 0, path);
    }
}

// Tier 2: joint tables too large for shared memory, counted in O(samples):
//  1. the observed Z strata are hashed, each new one taking the next id (shared-memory
//     hash of kZCap32 32-bit or kZCap64 64-bit codes; a global one beyond that);
//  dense path (strata x dx x dy <= kDenseMul n_samples, dx dy <= 32): every sample adds
//     one to T[id][x][y] in the CTA's global slot, and lane groups score the strata from
//     T (score_dense_groups); the table is zeroed again after the decision;
//  otherwise:
//  2. samples are counting-sorted by stratum, stored as packed (x << 8) | y;
//  3. a stratum of at most kLaneStratum samples is scored by one thread with pairwise
//     comparisons; a larger one by one warp that counts its x,y cells in a small dense
//     table and reads each touched cell back with atomicExch(.., 0), so every distinct
//     cell contributes once and the table is left zeroed.  FP32 terms first; the FP64
//     pass runs only when the decision falls inside the recheck band.
template <bool kRetry>
__global__ void __launch_bounds__(kThreads, 2) ci_compact_kernel(WaveArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t *hkeys = reinterpret_cast<uint64_t *>(smem_raw);
    uint16_t *hids = reinterpret_cast<uint16_t *>(smem_raw + kZIdsOff);
    int *scnt = reinterpret_cast<int *>(smem_raw);
    int *scur = reinterpret_cast<int *>(smem_raw + kZCurOff);
    int *swt = reinterpret_cast<int *>(smem_raw + kZTabOff);
    __shared__ const uint8_t *s_col[kMaxCols];
    __shared__ uint32_t s_dim[kMaxCols];
    __shared__ int s_idx, s_over, s_distinct, s_flag, s_seen, s_pick, s_skip;
    __shared__ double s_est;
    __shared__ int s_w[kWarps];
    __shared__ Partial scratch[kWarps];
    const int tid = threadIdx.x;
    const uint32_t gcap = (uint32_t)a.hash_cap_global;
    char *slot = a.slot_mem + (int64_t)blockIdx.x * a.slot_bytes;
    const SlotLayout L = slot_layout(a.slot_S, gcap);
    uint64_t *gkeys = reinterpret_cast<uint64_t *>(slot + L.keys);
    uint64_t *gzk = reinterpret_cast<uint64_t *>(slot + L.zk);
    int *gids = reinterpret_cast<int *>(slot + L.ids);
    int *gcnt = reinterpret_cast<int *>(slot + L.cnt);
    int *gcur = reinterpret_cast<int *>(slot + L.cur);
    int *gsid = reinterpret_cast<int *>(slot + L.sid);
    int *gwt = reinterpret_cast<int *>(slot + L.wt);
    uint16_t *gord = reinterpret_cast<uint16_t *>(slot + L.ord);
    int *gtab = reinterpret_cast<int *>(slot + L.tab);
    const int n2 = a.counters[kRetry ? C_RETRY : C_TIER2];
    const int d = a.d, ncols = d + 2;
    uint64_t *zk = a.want_hash ? gzk : nullptr;
    unsigned long long t_prev = 0;
#define FPGM_PHASE(i)                                                   \
    do {                                                                \
        if (a.dbg && tid == 0) {                                        \
            const unsigned long long t_ = gtimer();                     \
            if ((i) >= 0) atomicAdd(&a.dbg[(i)], t_ - t_prev);          \
            t_prev = t_;                                                \
        }                                                               \
    } while (0)
    for (;;) {
        if (tid == 0) s_idx = atomicAdd(&a.counters[kRetry ? C_WORKR : C_WORK2], 1);
        __syncthreads();
        const int idx = s_idx;
        if (idx >= n2) break;
        FPGM_PHASE(-1);
        const int item = a.lists[(kRetry ? 5 : 2) * a.list_cap + idx];
        const int64_t S = a.var_S[a.item_vars[(int64_t)item * ncols + d]];  // <= the slots' layout size
        int tune_bucket = -1;               // thread 0: the bucket this test's hash-path time goes to
        unsigned long long t_hash = 0;
        const int64_t nvec = S >> 4;
        if (tid < ncols) {
            const int var = a.item_vars[(int64_t)item * ncols + tid];
            s_dim[tid] = a.card[var];
            s_col[tid] = a.cols + a.var_off[var];
        }
        // 1. strata -> ids (shared hash, global if more than kZStrata strata)
        bool global = false;
        // attempt 0: shared hash; 1: global hash sized from where the shared one overflowed
        // (distinct strata grow slower than the samples, so the linear extrapolation bounds
        // them); 2: global hash for every sample (only if 1 overflows)
        int seen = 0;  // vectors hashed when the previous attempt overflowed
        __syncthreads();  // s_dim of this test
        uint64_t dz = 1;
        for (int j = 0; j < d; ++j) dz *= s_dim[j];  // < 2^62 (classified)
        const bool code32 = dz <= 0xFFFFFFFFull;     // codes < dz fit 32 bits, below the empty key
        const int zlimit = code32 ? kZStrata : kZCap64 / 2;
        uint32_t cap = code32 ? (uint32_t)kZCap32 : (uint32_t)kZCap64;
        uint32_t *hkeys32 = reinterpret_cast<uint32_t *>(hkeys);
        bool deferred = false;  // handed to the partitioned kernel
        if (!kRetry && a.wide != nullptr && a.wide_direct && n2 <= a.wide_small_n2) {
            // A wave of few tier-2 tests: every one goes straight to the partition-parallel
            // path, with min(dz, samples) as its strata bound, so no CTA spends the wave on
            // one test's hash or strata scoring alone.
            if (tid == 0) {
                const double est = fmin((double)dz, (double)S);
                const int q = atomicAdd(&a.counters[C_PART], 1);
                a.lists[3 * a.list_cap + q] = item;
                a.lists[4 * a.list_cap + q] = __float_as_int((float)est);
            }
            __syncthreads();
            continue;
        }
        // the autotuner bucket's overflow record may skip the shared-hash attempt
        const int obucket = a.ovf ? tune_index(S, d, (double)dz * s_dim[d] * s_dim[d + 1]) : -1;
        if (!kRetry && tid == 0) {
            double e = 0.0;
            s_skip = ovf_skip(a, obucket, S, &e);
            s_est = e;
            if (s_skip) s_over = 1;  // as after an overflowing attempt 0 (a hand-over keeps it set)
        }
        __syncthreads();
        const bool skip0 = !kRetry && s_skip;
        for (int attempt = kRetry ? 2 : (skip0 ? 1 : 0); attempt < 3; ++attempt) {
            global = attempt >= 1;
            const bool k32 = !global && code32;
            if (attempt == 1) {
                const double est = skip0 ? s_est
                                         : (double)zlimit * (double)(nvec > 1 ? nvec : 1) / (double)(seen > 1 ? seen : 1);
                const bool tail = a.wide != nullptr && n2 <= a.wide_small_n2;
                if (tid == 0) {
                    int b = -1;
                    s_pick = tail || tier2_pick_partitions(a, S, d, (double)dz * s_dim[d] * s_dim[d + 1], &b);
                    tune_bucket = b;
                    t_hash = gtimer();
                }
                __syncthreads();
                if (s_pick) {
                    if (tid == 0) {
                        const int q = atomicAdd(&a.counters[C_PART], 1);
                        a.lists[3 * a.list_cap + q] = item;
                        a.lists[4 * a.list_cap + q] = __float_as_int((float)est);
                    }
                    deferred = true;
                    break;
                }
                cap = 16384u < gcap ? 16384u : gcap;
                while ((double)cap < 2.0 * est && cap < gcap) cap <<= 1;
            } else if (attempt == 2) {
                if (cap == gcap && !kRetry) break;  // attempt 1 had the full size already
                cap = gcap;
            }
            uint64_t *keys = global ? gkeys : hkeys;
            if (k32)
                for (uint32_t i = tid; i < cap; i += kThreads) hkeys32[i] = (uint32_t)kEmptyKey;
            else
                for (uint32_t i = tid; i < cap; i += kThreads) keys[i] = kEmptyKey;
            if (tid == 0) {
                s_over = 0;
                s_distinct = 0;
                s_seen = 0;
            }
            __syncthreads();
            const int limit = global ? (int)(cap / 2) : zlimit;
            const uint32_t max_probe = global ? cap : 64u;
            // every lane runs every round (the ids of a warp's new strata are handed out together)
            const int64_t vrounds = (nvec + kThreads - 1) / kThreads;
            for (int64_t rd = 0; rd < vrounds; ++rd) {
                if (*(volatile int *)&s_over) break;  // one load per warp: the same for its lanes
                const int64_t v = rd * kThreads + tid;
                const bool have = v < nvec;
                int hs[16];
                unsigned claimed = 0;
                bool ok = true;
                if (have) {
                    uint64_t z[16];
                    zcodes16(z, s_col, s_dim, d, v);
                    // first probes of all 16 codes in flight at once; a code found there (the
                    // common case) is done, the others take the inserting path (a stale empty
                    // slot read here is resolved by its compare-and-swap)
#pragma unroll
                    for (int b0 = 0; b0 < 16; b0 += 8) {  // eight at a time (register budget)
                        uint64_t kk[8];
#pragma unroll
                        for (int b = 0; b < 8; ++b) {
                            hs[b0 + b] = (int)zhash(z[b0 + b], cap);
                            kk[b] = k32 ? (uint64_t)hkeys32[hs[b0 + b]] : keys[hs[b0 + b]];
                        }
#pragma unroll
                        for (int b = 0; b < 8; ++b) {
                            if (!ok || kk[b] == z[b0 + b]) continue;
                            bool cl = false;
                            hs[b0 + b] = k32 ? zclaim(hkeys32, cap, z[b0 + b], max_probe, &cl)
                                             : zclaim(keys, cap, z[b0 + b], max_probe, &cl);
                            if (cl) claimed |= 1u << (b0 + b);
                            ok = hs[b0 + b] >= 0;
                        }
                    }
                }
                // ids of the warp's new strata: one atomic per warp
                const int c = __popc(claimed);
                int incl = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if ((tid & 31) >= o) incl += t;
                }
                int first = 0;
                if ((tid & 31) == 31 && incl > 0) first = atomicAdd(&s_distinct, incl);
                first = __shfl_sync(0xffffffffu, first, 31) + incl - c;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    if (!(claimed >> j & 1u)) continue;
                    if (first < limit) {
                        if (global) gids[hs[j]] = first;
                        else hids[hs[j]] = (uint16_t)first;
                        if (zk) zk[first] = k32 ? (uint64_t)hkeys32[hs[j]] : keys[hs[j]];  // the slot holds the code
                    } else {
                        ok = false;
                    }
                    ++first;
                }
                if (!ok) {
                    s_over = 1;
                    s_seen = (int)v + 1;
                } else if (have) {
                    // one 64-byte run per thread, written after the inserts
                    int4 *dst = reinterpret_cast<int4 *>(gsid + v * 16);
                    dst[0] = make_int4(hs[0], hs[1], hs[2], hs[3]);
                    dst[1] = make_int4(hs[4], hs[5], hs[6], hs[7]);
                    dst[2] = make_int4(hs[8], hs[9], hs[10], hs[11]);
                    dst[3] = make_int4(hs[12], hs[13], hs[14], hs[15]);
                }
            }
            for (int64_t s = (S & ~(int64_t)15) + tid; s < S; s += kThreads) {
                if (*(volatile int *)&s_over) break;
                uint64_t z = 0;
                for (int j = 0; j < d; ++j) z = z * s_dim[j] + s_col[j][s];
                const int h = global ? zinsert(keys, gids, cap, z, &s_distinct, limit, max_probe, zk)
                              : k32  ? zinsert(hkeys32, hids, cap, z, &s_distinct, limit, max_probe, zk)
                                     : zinsert(keys, hids, cap, z, &s_distinct, limit, max_probe, zk);
                if (h < 0) {
                    s_over = 1;
                    break;
                }
                gsid[s] = h;
            }
            __syncthreads();
            FPGM_PHASE(attempt > 0 ? 1 : 0);
            seen = s_seen > 0 ? s_seen : (int)nvec;
            if (attempt == 0 && tid == 0 && obucket >= 0) atomicAdd(&a.ovf[8 * obucket + (s_over ? 0 : 1)], 1ull);
            if (!s_over) break;
            __syncthreads();
        }
        if (s_over) {  // deferred, or (cannot happen with cap >= 2 S) flagged instead of guessed
            if (tid == 0 && !deferred) {
                a.flag[item] = 2;
                atomicAdd(&a.stats[ST_UNSUPPORTED], 1ull);
            }
            __syncthreads();
            continue;
        }
        const int n_obs = s_distinct;
        if (tid == 0 && global) ovf_strata(a, obucket, S, n_obs);
        if (a.dbg && tid == 0) {
            atomicAdd(&a.dbg[10], (unsigned long long)n_obs);
            atomicAdd(&a.dbg[11], 1ull);
        }
        const int dy = s_dim[d + 1], dx = s_dim[d];
        const int dxy = dx * dy;
        const uint8_t *colx = s_col[d], *coly = s_col[d + 1];
        // dense strata table when it is small next to the samples and a stratum's cells fit
        // one warp (lane-group scoring); otherwise the counting-sort path
        const bool dense = (int64_t)n_obs * dxy <= (int64_t)kDenseMul * S && dxy <= 32;
        int *cnt = global ? gcnt : scnt;
        int *cur = global ? gcur : scur;
        // stratum ids of larger strata (sorted path): the dead cursors in shared memory, else the free gsid
        int *big = global ? gsid : scur;
        int n_big = 0;
        int *wt = nullptr;           // sorted path: per-warp x,y table
        Partial acc;
        if (dense) {
            if (a.dbg && tid == 0) atomicAdd(&a.dbg[12], 1ull);
            // 2'. strata x cells counted straight into the dense table (kept zeroed between tests)
            for (int64_t v = tid; v < nvec; v += kThreads) {
                const uint4 wx = __ldg(reinterpret_cast<const uint4 *>(colx) + v);
                const uint4 wy = __ldg(reinterpret_cast<const uint4 *>(coly) + v);
                const uint32_t xx[4] = {wx.x, wx.y, wx.z, wx.w}, yy[4] = {wy.x, wy.y, wy.z, wy.w};
                int sid[16];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int4 h = reinterpret_cast<const int4 *>(gsid)[v * 4 + q];
                    sid[4 * q] = h.x;
                    sid[4 * q + 1] = h.y;
                    sid[4 * q + 2] = h.z;
                    sid[4 * q + 3] = h.w;
                }
                // all 16 id lookups before the first increment (the increments could alias them)
#pragma unroll
                for (int b = 0; b < 16; ++b) sid[b] = global ? __ldcg(gids + sid[b]) : (int)hids[sid[b]];
#pragma unroll
                for (int b = 0; b < 16; ++b) {
                    const int q = b >> 2, sh = 8 * (b & 3);
                    const int c = (int)((xx[q] >> sh) & 0xffu) * dy + (int)((yy[q] >> sh) & 0xffu);
                    atomicAdd(&gtab[(int64_t)sid[b] * dxy + c], 1);
                }
            }
            for (int64_t s = (S & ~(int64_t)15) + tid; s < S; s += kThreads) {
                const int sid = global ? gids[gsid[s]] : (int)hids[gsid[s]];
                atomicAdd(&gtab[(int64_t)sid * dxy + colx[s] * dy + coly[s]], 1);
            }
            __syncthreads();
            FPGM_PHASE(7);
            // the hash keys and ids are dead: their 96 KB hold the per-thread scoring columns
            acc = a.dense_rows ? score_dense_rows<false>(gtab, n_obs, dx, dy, zk, a.want_hash != 0,
                                                         reinterpret_cast<int *>(smem_raw))
                               : score_dense_groups<false>(gtab, n_obs, dx, dy, zk, a.want_hash != 0);
            FPGM_PHASE(8);
        } else {
            // 2. counting sort of the samples by stratum
            for (int i = tid; i <= n_obs; i += kThreads) cnt[i] = 0;
            __syncthreads();
            for (int64_t s4 = tid; s4 < (S >> 2); s4 += kThreads) {
                int4 h = reinterpret_cast<int4 *>(gsid)[s4];
                if (global) {
                    h.x = gids[h.x];
                    h.y = gids[h.y];
                    h.z = gids[h.z];
                    h.w = gids[h.w];
                } else {
                    h.x = hids[h.x];
                    h.y = hids[h.y];
                    h.z = hids[h.z];
                    h.w = hids[h.w];
                }
                reinterpret_cast<int4 *>(gsid)[s4] = h;
                atomicAdd(&cnt[h.x], 1);
                atomicAdd(&cnt[h.y], 1);
                atomicAdd(&cnt[h.z], 1);
                atomicAdd(&cnt[h.w], 1);
            }
            for (int64_t s = (S & ~(int64_t)3) + tid; s < S; s += kThreads) {
                const int sid = global ? gids[gsid[s]] : (int)hids[gsid[s]];
                gsid[s] = sid;
                atomicAdd(&cnt[sid], 1);
            }
            __syncthreads();
            FPGM_PHASE(2);
            block_exclusive_scan(cnt, n_obs + 1, s_w);  // cnt -> stratum offsets, cnt[n_obs] = S
            for (int i = tid; i <= n_obs; i += kThreads) cur[i] = cnt[i];
            __syncthreads();
            for (int64_t v = tid; v < nvec; v += kThreads) {
                const uint4 wx = __ldg(reinterpret_cast<const uint4 *>(colx) + v);
                const uint4 wy = __ldg(reinterpret_cast<const uint4 *>(coly) + v);
                const uint32_t xx[4] = {wx.x, wx.y, wx.z, wx.w}, yy[4] = {wy.x, wy.y, wy.z, wy.w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int4 sid = reinterpret_cast<const int4 *>(gsid)[v * 4 + q];
                    const int sv[4] = {sid.x, sid.y, sid.z, sid.w};
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        const int pos = atomicAdd(&cur[sv[b]], 1);
                        gord[pos] = (uint16_t)((((xx[q] >> (8 * b)) & 0xffu) << 8) | ((yy[q] >> (8 * b)) & 0xffu));
                    }
                }
            }
            for (int64_t s = (S & ~(int64_t)15) + tid; s < S; s += kThreads) {
                const int pos = atomicAdd(&cur[gsid[s]], 1);
                gord[pos] = (uint16_t)((colx[s] << 8) | coly[s]);
            }
            __syncthreads();
            FPGM_PHASE(3);
            // 3. score the strata: FP32 terms first, FP64 only inside the recheck band
            const bool wsmem = dxy + dx + dy <= kSparseWarpTab;
            wt = wsmem ? swt + (threadIdx.x >> 5) * kSparseWarpTab : gwt + (int64_t)(threadIdx.x >> 5) * kGlobalWarpTab;
            if (wsmem)  // the table region held ids or cursors until now
                for (int i = tid; i < kWarps * kSparseWarpTab; i += kThreads) swt[i] = 0;
            if (tid == 0) s_over = 0;
            __syncthreads();
            acc = score_small_strata<false>(cnt, gord, n_obs, dx, dy, big, &s_over, zk, a.want_hash != 0, true);
            __syncthreads();
            n_big = s_over;
            FPGM_PHASE(4);
            acc = score_big_strata<false>(acc, cnt, gord, big, n_big, dx, dy, wt, zk, a.want_hash != 0);
            FPGM_PHASE(5);
        }
        const Partial r = block_sum(acc, scratch);
        decide_record(a, item, r, (int64_t)n_obs * dxy, 2, s_flag, scratch, [&]() {
            Partial q;
            if (dense) {
                q = a.dense_rows ? score_dense_rows<true>(gtab, n_obs, dx, dy, nullptr, false,
                                                          reinterpret_cast<int *>(smem_raw))
                                 : score_dense_groups<true>(gtab, n_obs, dx, dy, nullptr, false);
            } else {
                q = score_small_strata<true>(cnt, gord, n_obs, dx, dy, big, nullptr, nullptr, false, false);
                q = score_big_strata<true>(q, cnt, gord, big, n_big, dx, dy, wt, nullptr, false);
            }
            return q;
        });
        if (dense) {  // leave the table zeroed for the next test
            __syncthreads();
            const int64_t ncell = (int64_t)n_obs * dxy;
            for (int64_t i = tid; i < (ncell >> 2); i += kThreads)
                reinterpret_cast<int4 *>(gtab)[i] = make_int4(0, 0, 0, 0);
            for (int64_t i = (ncell & ~(int64_t)3) + tid; i < ncell; i += kThreads) gtab[i] = 0;
        }
        if (tid == 0 && tune_bucket >= 0) {
            atomicAdd(&a.tune_obs[8 * tune_bucket + 2], 1ull);
            atomicAdd(&a.tune_obs[8 * tune_bucket + 3], gtimer() - t_hash);
        }
        FPGM_PHASE(6);
        __syncthreads();
    }
#undef FPGM_PHASE
}

// Tier 2, partitioned: the tests ci_compact_kernel handed over (strata beyond its shared
// hash, at least kPartMinSamples samples), one CTA per test, in the CTA's own slot.  A test
// whose partitions overflow is split again with twice the partitions; past
// 2^part_max_log partitions it goes back to the compact kernel's global hash (retry list,
// ci_compact_kernel<true>).
__global__ void __launch_bounds__(kThreads, 2) ci_part_kernel(WaveArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ const uint8_t *s_col[kMaxCols];
    __shared__ uint32_t s_dim[kMaxCols];
    __shared__ int s_idx, s_over, s_distinct, s_flag, s_nbig, s_nocc;
    __shared__ int s_bin[16];
    __shared__ int s_w[kWarps];
    __shared__ Partial scratch[kWarps];
    __shared__ int s_pcnt[kPartMax], s_poff[kPartMax + 1], s_pcur[kPartMax], s_sp[kPartMax + 1], s_nsp;
    __shared__ const uint32_t *s_bmr;  // parent's contributing-sample bitmap (null: every sample)
    __shared__ uint32_t *s_bmw;        // this test's, being written (null: none)
    __shared__ int s_bmslot, s_bmbad;
    __shared__ unsigned long long *s_lstat;  // this test measures the contributing fraction (null: no)
    const int tid = threadIdx.x;
    char *slot = a.slot_mem + (int64_t)blockIdx.x * a.slot_bytes;
    const SlotLayout L = slot_layout(a.slot_S, (uint32_t)a.hash_cap_global);
    char *rz = slot + L.keys;  // record codes (u32 or u64), S + padding
    uint16_t *rxy = reinterpret_cast<uint16_t *>(slot + L.ids);  // record (x << 8) | y
    uint32_t *rs = reinterpret_cast<uint32_t *>(slot + L.rs);    // record sample index (bitmaps only)
    uint64_t *gzk = reinterpret_cast<uint64_t *>(slot + L.zk);
    int *gwt = reinterpret_cast<int *>(slot + L.wt);
    uint16_t *gord = reinterpret_cast<uint16_t *>(slot + L.ord);
    uint64_t *zk = a.want_hash ? gzk : nullptr;
    const int np = a.counters[C_PART];
    const int d = a.d, ncols = d + 2;
    unsigned long long t_prev = 0;
#define FPGM_PHASE(i)                                                   \
    do {                                                                \
        if (a.dbg && tid == 0) {                                        \
            const unsigned long long t_ = gtimer();                     \
            if ((i) >= 0) atomicAdd(&a.dbg[(i)], t_ - t_prev);          \
            t_prev = t_;                                                \
        }                                                               \
    } while (0)
    for (;;) {
        if (tid == 0) s_idx = atomicAdd(&a.counters[C_WORKP], 1);
        __syncthreads();
        const int idx = s_idx;
        if (idx >= np) break;
        FPGM_PHASE(-1);
        const int item = a.lists[3 * a.list_cap + idx];
        const double est = (double)__int_as_float(a.lists[4 * a.list_cap + idx]);
        const unsigned long long t_part = (tid == 0 && a.tune_obs) ? gtimer() : 0ull;
        const int64_t S = a.var_S[a.item_vars[(int64_t)item * ncols + d]];
        if (tid < ncols) {
            const int var = a.item_vars[(int64_t)item * ncols + tid];
            s_dim[tid] = a.card[var];
            s_col[tid] = a.cols + a.var_off[var];
        }
        if (tid == 0) {  // contributing-sample bitmaps: the parent's (Z minus its last variable), and one to write
            s_bmr = nullptr;
            s_bmw = nullptr;
            s_bmslot = -1;
            s_bmbad = 0;
            if (a.bm_prev_tab && d >= 1) {
                uint16_t v[2 + kMaxCond];
                const int nv = live_key(a.item_vars + (int64_t)item * ncols, d, d - 1, v);
                const int sl = live_find(a.bm_prev_tab, a.bm_prev_tab_cap, v, nv);
                if (sl >= 0) s_bmr = a.bm_prev_pool + (int64_t)sl * a.bm_words;
            }
            if (a.bm_pool) {
                const int sl = atomicAdd(a.bm_count, 1);
                if (sl < a.bm_cap) {
                    s_bmslot = sl;
                    s_bmw = a.bm_pool + (int64_t)sl * a.bm_words;
                }
            }
            // one test in eight (and none of the partition-parallel ones) measures the contributing fraction
            s_lstat = (a.live_stat && (idx & 7) == 0 && !(a.wide != nullptr && idx >= np - (int)gridDim.x))
                          ? a.live_stat
                          : nullptr;
            if (s_lstat) atomicAdd(&s_lstat[1], (unsigned long long)S);  // the test's samples
        }
        __syncthreads();
        if (s_bmw)  // cleared before any bit is set (part_scatter's barriers come first)
            for (int64_t i = tid; i < ((S + 31) >> 5); i += kThreads) s_bmw[i] = 0u;
        uint64_t dz = 1;
        for (int j = 0; j < d; ++j) dz *= s_dim[j];
        const bool code32 = dz <= 0xFFFFFFFFull;
        const int dx = s_dim[d], dy = s_dim[d + 1];
        // Super-partitions of at most rmax records (the staged shared-memory plan), few enough
        // that their strata -- est per sample, which errs high -- fill at most 70% of a table;
        // partitions of about a quarter of that, so that runs of them pack well.
        int rstage = code32 ? StagePlan<uint32_t>::rec : StagePlan<uint64_t>::rec;
        if (a.stage_rec > 0 && a.stage_rec < rstage) rstage = a.stage_rec;
        const int lim = code32 ? StagePlan<uint32_t>::lim : StagePlan<uint64_t>::lim;
        const double ratio = fmax(est / (double)(S > 0 ? S : 1), 1e-6);
        int rmax = (int)fmin((double)rstage, 0.7 * lim / ratio) & ~7;
        if (rmax < 64) rmax = 64;
        int lp = 1;
        const int maxlog = a.part_max_log;
        while ((S >> lp) > rmax / 4 && lp < maxlog) ++lp;
        if (a.wide != nullptr && idx >= np - (int)gridDim.x) {
            // One of the list's last tests (all of them when there are no more tests than
            // CTAs): its records are written here, then its super-partitions are queued for
            // ci_part_wide_kernel, which scores them on whichever CTAs are free.  This CTA
            // takes no further test, so its slot keeps the records.  Super-partitions are cut
            // small enough for about two per CTA over the published tests.
            const int nw = np < (int)gridDim.x ? np : (int)gridDim.x;
            int rw = (int)fmin((double)rmax, (double)S * nw / (2.0 * gridDim.x)) & ~7;
            if (rw < a.wide_part_min) rw = a.wide_part_min < rmax ? a.wide_part_min : rmax;
            int lw = a.wide_min_log < maxlog ? a.wide_min_log : maxlog;
            while ((S >> lw) > rw / 4 && lw < maxlog) ++lw;
            if (code32)
                part_scatter(s_col, s_dim, d, S, lw, reinterpret_cast<uint32_t *>(rz), rxy, s_pcnt, s_poff, s_pcur,
                             reinterpret_cast<uint32_t *>(gzk), smem_raw, s_bmr, s_bmw ? rs : nullptr);
            else
                part_scatter(s_col, s_dim, d, S, lw, reinterpret_cast<uint64_t *>(rz), rxy, s_pcnt, s_poff, s_pcur,
                             reinterpret_cast<uint64_t *>(gzk), smem_raw, s_bmr, s_bmw ? rs : nullptr);
            FPGM_PHASE(14);
            if (tid == 0) s_idx = atomicAdd(&a.counters[C_WIDET], 1);
            __syncthreads();
            WideTest *w = a.wide + s_idx;
            const int P = 1 << lw;
            for (int i = tid; i < P; i += kThreads) {
                w->pcnt[i] = s_pcnt[i];
                w->poff[i] = s_poff[i];
            }
            if (tid == 0) {
                w->poff[P] = s_poff[P];
                int rk = rw;
                if (s_bmr) {  // as in the per-CTA path: fewer records per super-partition with a bitmap
                    int kept = 0;
                    for (int i = 0; i < P; ++i) kept += s_pcnt[i];
                    rk = (int)fmin((double)rw, 0.7 * lim * (double)kept / fmax(est, 1.0)) & ~7;
                    if (rk < 64) rk = 64;
                }
                const int nne = plan_super(s_pcnt, P, rk, w->sp);
                w->item = item;
                w->owner = blockIdx.x;
                w->lp = lw;
                w->code32 = code32;
                w->dx = dx;
                w->dy = dy;
                w->n_items = nne;
                w->done = 0;
                w->over = 0;
                w->n_obs = 0;
                w->df = 0ull;
                w->g2 = 0.0;
                w->err = 0.0;
                w->abs_g2 = 0.0;
                w->hash = 0ull;
                w->bmw = s_bmw;
                w->bm_slot = s_bmslot;
                w->bm_bad = 0;
                const int q0 = atomicAdd(&a.counters[C_WIDEQ], nne);
                for (int i = 0; i < nne; ++i) a.wide_items[q0 + i] = (s_idx << 8) | i;
                if (a.dbg) atomicAdd(&a.dbg[23], 1ull);
            }
            __syncthreads();
            break;
        }
        Partial acc;
        bool over;
        for (;;) {
            if (tid == 0) {
                s_over = 0;
                s_distinct = 0;
            }  // visible after part_scatter's first barrier
            int claims = 0;
            if (code32)
                part_scatter(s_col, s_dim, d, S, lp, reinterpret_cast<uint32_t *>(rz), rxy, s_pcnt, s_poff, s_pcur,
                             reinterpret_cast<uint32_t *>(gzk), smem_raw, s_bmr, s_bmw ? rs : nullptr);
            else
                part_scatter(s_col, s_dim, d, S, lp, reinterpret_cast<uint64_t *>(rz), rxy, s_pcnt, s_poff, s_pcur,
                             reinterpret_cast<uint64_t *>(gzk), smem_raw, s_bmr, s_bmw ? rs : nullptr);
            if (tid == 0) {
                // strata are at most est whichever samples were kept: with a parent's bitmap, as
                // many strata fall on fewer records, so the super-partitions hold fewer records
                int rk = rmax;
                if (s_bmr) {
                    int kept = 0;
                    for (int i = 0; i < (1 << lp); ++i) kept += s_pcnt[i];
                    rk = (int)fmin((double)rmax, 0.7 * lim * (double)kept / fmax(est, 1.0)) & ~7;
                    if (rk < 64) rk = 64;
                }
                s_nsp = plan_super(s_pcnt, 1 << lp, rk, s_sp);
                if (a.dbg) {  // contributing-sample bitmaps: tests with a parent's, samples, records kept
                    atomicAdd(&a.dbg[28], s_bmr ? 1ull : 0ull);
                    atomicAdd(&a.dbg[29], (unsigned long long)S);
                    int kept = 0;
                    for (int i = 0; i < (1 << lp); ++i) kept += s_pcnt[i];
                    atomicAdd(&a.dbg[30], (unsigned long long)kept);
                    atomicAdd(&a.dbg[31], s_bmw ? 1ull : 0ull);
                }
            }
            __syncthreads();
            FPGM_PHASE(14);
            if (code32)
                acc = part_run<false>(lp, reinterpret_cast<const uint32_t *>(rz), rxy, s_pcnt, s_poff, s_sp, s_nsp, dx,
                                      dy, smem_raw, gord, gwt, zk, a.want_hash != 0, s_w, &s_over, &s_nbig, &s_nocc,
                                      s_bin, claims, a.stage_rec, a.dbg, s_bmw, rs, &s_bmbad, s_lstat);
            else
                acc = part_run<false>(lp, reinterpret_cast<const uint64_t *>(rz), rxy, s_pcnt, s_poff, s_sp, s_nsp, dx,
                                      dy, smem_raw, gord, gwt, zk, a.want_hash != 0, s_w, &s_over, &s_nbig, &s_nocc,
                                      s_bin, claims, a.stage_rec, a.dbg, s_bmw, rs, &s_bmbad, s_lstat);
            atomicAdd(&s_distinct, claims);
            __syncthreads();
            over = s_over != 0;
            __syncthreads();  // every thread has read s_over before it is reset
            if (!over || lp >= maxlog) break;
            ++lp;
        }
        if (over) {  // the compact kernel's global hash takes it
            if (tid == 0) {
                const int q = atomicAdd(&a.counters[C_RETRY], 1);
                a.lists[5 * a.list_cap + q] = item;
            }
        } else {
            const int n_obs = s_distinct;
            if (tid == 0) ovf_strata(a, a.ovf ? tune_index(S, d, (double)dz * dx * dy) : -1, S, n_obs);
            if (a.dbg && tid == 0) {
                atomicAdd(&a.dbg[9], (unsigned long long)n_obs);
                atomicAdd(&a.dbg[13], 1ull);
            }
            const Partial r = block_sum(acc, scratch);
            decide_record(a, item, r, (int64_t)n_obs * dx * dy, 3, s_flag, scratch, [&]() {
                int claims = 0;
                return code32 ? part_run<true>(lp, reinterpret_cast<const uint32_t *>(rz), rxy, s_pcnt, s_poff, s_sp,
                                               s_nsp, dx, dy, smem_raw, gord, gwt, nullptr, false, s_w, &s_over,
                                               &s_nbig, &s_nocc, s_bin, claims, a.stage_rec, nullptr)
                              : part_run<true>(lp, reinterpret_cast<const uint64_t *>(rz), rxy, s_pcnt, s_poff, s_sp,
                                               s_nsp, dx, dy, smem_raw, gord, gwt, nullptr, false, s_w, &s_over,
                                               &s_nbig, &s_nocc, s_bin, claims, a.stage_rec, nullptr);
            });
            if (tid == 0 && s_bmw && !s_bmbad) {  // the bitmap is complete: the next level may use it
                uint16_t v[2 + kMaxCond];
                const int nv = live_key(a.item_vars + (int64_t)item * ncols, d, d, v);
                live_insert(a.bm_tab, a.bm_tab_cap, v, nv, s_bmslot);
            }
        }
        if (tid == 0 && a.tune_obs && !a.tune) {  // the partition path's time for the online autotuner
            const int b = tune_index(S, d, (double)dz * dx * dy);
            atomicAdd(&a.tune_obs[8 * b], 1ull);
            atomicAdd(&a.tune_obs[8 * b + 1], gtimer() - t_part);
        }
        FPGM_PHASE(15);
        __syncthreads();
    }
#undef FPGM_PHASE
}

// Partition-parallel scoring of the tests ci_part_kernel published (WideTest): every CTA
// takes (test, partition) items from the queue, counts and scores that partition in shared
// memory from the owner CTA's records, and adds its share to the test's sums.  The CTA that
// finishes a test's last partition decides it -- FP64 recheck over all partitions when the
// statistic falls inside the band -- or, if any partition overflowed its table, hands the
// test to the compact kernel's global hash (retry list, ci_compact_kernel<true>).
__global__ void __launch_bounds__(kThreads, 2) ci_part_wide_kernel(WaveArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_idx, s_over, s_flag, s_nbig, s_nocc, s_last, s_bmbad;
    __shared__ int s_bin[16];
    __shared__ int s_w[kWarps];
    __shared__ Partial scratch[kWarps];
    if (a.wide == nullptr) return;
    const int tid = threadIdx.x;
    char *slot = a.slot_mem + (int64_t)blockIdx.x * a.slot_bytes;
    const SlotLayout L = slot_layout(a.slot_S, (uint32_t)a.hash_cap_global);
    uint64_t *gzk = reinterpret_cast<uint64_t *>(slot + L.zk);
    int *gwt = reinterpret_cast<int *>(slot + L.wt);
    uint16_t *gord = reinterpret_cast<uint16_t *>(slot + L.ord);
    uint64_t *zk = a.want_hash ? gzk : nullptr;
    const int nq = a.counters[C_WIDEQ];
    for (;;) {
        if (tid == 0) s_idx = atomicAdd(&a.counters[C_WIDEW], 1);
        __syncthreads();
        const int idx = s_idx;
        if (idx >= nq) break;
        const int code = a.wide_items[idx];
        WideTest *w = a.wide + (code >> 8);
        const int p = code & 0xff;
        const char *own = a.slot_mem + (int64_t)w->owner * a.slot_bytes;
        const char *rz = own + L.keys;
        const uint16_t *rxy = reinterpret_cast<const uint16_t *>(own + L.ids);
        const uint32_t *rs = reinterpret_cast<const uint32_t *>(own + L.rs);
        const int lp = w->lp, dx = w->dx, dy = w->dy;
        const bool code32 = w->code32 != 0;
        uint32_t *bmw = w->bmw;
        if (tid == 0) {
            s_over = 0;
            s_bmbad = 0;
        }
        __syncthreads();
        int claims = 0;
        const Partial q =
            code32 ? part_super<false, uint32_t>(lp, reinterpret_cast<const uint32_t *>(rz), rxy, w->pcnt, w->poff,
                                                 w->sp[p], w->sp[p + 1], dx, dy, smem_raw, gord, gwt, zk,
                                                 a.want_hash != 0, s_w, &s_over, &s_nbig, &s_nocc, s_bin, claims,
                                                 a.stage_rec, nullptr, bmw, rs, &s_bmbad, nullptr)
                   : part_super<false, uint64_t>(lp, reinterpret_cast<const uint64_t *>(rz), rxy, w->pcnt, w->poff,
                                                 w->sp[p], w->sp[p + 1], dx, dy, smem_raw, gord, gwt, zk,
                                                 a.want_hash != 0, s_w, &s_over, &s_nbig, &s_nocc, s_bin, claims,
                                                 a.stage_rec, nullptr, bmw, rs, &s_bmbad, nullptr);
        const bool over = s_over != 0;  // read after part_super's closing barrier
        const Partial r = block_sum(q, scratch);
        if (tid == 0) {
            if (s_bmbad) atomicExch(&w->bm_bad, 1);
            if (over) {
                atomicExch(&w->over, 1);
            } else {
                atomicAdd(&w->df, r.df);
                atomicAdd(&w->g2, r.g2);
                atomicAdd(&w->err, r.err);
                atomicAdd(&w->abs_g2, r.abs_g2);
                atomicAdd(&w->hash, r.hash);
                atomicAdd(&w->n_obs, claims);
            }
            __threadfence();  // the sums are visible before the partition counts as done
            s_last = atomicAdd(&w->done, 1) == w->n_items - 1;
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            const int item = w->item;
            if (__ldcg(&w->over)) {
                if (tid == 0) {
                    const int qr = atomicAdd(&a.counters[C_RETRY], 1);
                    a.lists[5 * a.list_cap + qr] = item;
                }
            } else {
                Partial R;
                R.df = (long long)__ldcg(&w->df);
                R.g2 = __ldcg(&w->g2);
                R.err = __ldcg(&w->err);
                R.abs_g2 = __ldcg(&w->abs_g2);
                R.hash = __ldcg(&w->hash);
                const int n_obs = __ldcg(&w->n_obs);
                if (a.dbg && tid == 0) {
                    atomicAdd(&a.dbg[9], (unsigned long long)n_obs);
                    atomicAdd(&a.dbg[13], 1ull);
                }
                decide_record(a, item, R, (int64_t)n_obs * dx * dy, 4, s_flag, scratch, [&]() {
                    int cl = 0;
                    return code32 ? part_run<true>(lp, reinterpret_cast<const uint32_t *>(rz), rxy, w->pcnt, w->poff,
                                                   w->sp, w->n_items, dx, dy, smem_raw, gord, gwt, nullptr, false, s_w,
                                                   &s_over, &s_nbig, &s_nocc, s_bin, cl, a.stage_rec, nullptr)
                                  : part_run<true>(lp, reinterpret_cast<const uint64_t *>(rz), rxy, w->pcnt, w->poff,
                                                   w->sp, w->n_items, dx, dy, smem_raw, gord, gwt, nullptr, false, s_w,
                                                   &s_over, &s_nbig, &s_nocc, s_bin, cl, a.stage_rec, nullptr);
                });
                if (tid == 0 && bmw && !__ldcg(&w->bm_bad)) {  // complete: the next level may use it
                    uint16_t v[2 + kMaxCond];
                    const int nv = live_key(a.item_vars + (int64_t)item * (a.d + 2), a.d, a.d, v);
                    live_insert(a.bm_tab, a.bm_tab_cap, v, nv, w->bm_slot);
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- band tables
__global__ void band_table_kernel(double alpha, double *lo, double *hi, int dfmax) {
    const int df = blockIdx.x * blockDim.x + threadIdx.x;
    if (df > dfmax) return;
    if (df == 0) {
        lo[0] = 0.0;
        hi[0] = 0.0;
        return;
    }
    lo[df] = chisq_quantile_upper(alpha + kBand, df);
    hi[df] = chisq_quantile_upper(alpha - kBand, df);
}

// ---------------------------------------------------------------- plain: one test, whole grid, one launch
struct PlainArgs {
    const uint8_t *cols;
    int64_t S;                  // samples of the test's dataset
    const uint8_t *card;
    int32_t ncols;
    int32_t vars[kMaxCols];     // Horner order: z..., x, y
    int64_t col_off[kMaxCols];  // byte offset of each of those columns in cols
    double alpha;
    BandTables bt;
    int32_t want_hash;
    int32_t *gtab;  // zeroed table + marginals
    int32_t *done;  // ticket counter, reset by the last CTA
    fpgm_ci_result *out;
    unsigned long long *stats;
};

__global__ void __launch_bounds__(kThreads) ci_plain_kernel(PlainArgs p) {
    extern __shared__ int smem[];
    __shared__ const uint8_t *s_col[kMaxCols];
    __shared__ uint32_t s_dim[kMaxCols];
    __shared__ Partial scratch[kWarps];
    __shared__ int s_last;
    const int tid = threadIdx.x, lane = tid & 31;
    const int ncols = p.ncols, d = ncols - 2;
    if (tid < ncols) {
        s_dim[tid] = p.card[p.vars[tid]];
        s_col[tid] = p.cols + p.col_off[tid];
    }
    __syncthreads();
    int64_t cells = 1;
    for (int j = 0; j < ncols; ++j) cells *= s_dim[j];
    const int dx = s_dim[d], dy = s_dim[d + 1];
    const int64_t dz = cells / (dx * dy);
    const int64_t marg = dz * (dx + dy + 1);
    const int64_t nvec = p.S >> 4;
    const int64_t per = (nvec + gridDim.x - 1) / gridDim.x;
    const int64_t v0 = min(nvec, per * blockIdx.x), v1 = min(nvec, v0 + per);
    const bool tail = blockIdx.x == 0;
    if (cells + marg <= kCtaInts && cells < 65536) {
        const int stride = (int)cells | 1;
        int R = 1;
        for (int r = 32; r >= 2; r >>= 1)
            if (stride * r <= kCtaInts) { R = r; break; }
        for (int i = tid; i < stride * R; i += kThreads) smem[i] = 0;
        __syncthreads();
        int *mytab = smem + (lane & (R - 1)) * stride;
        for (int64_t v = v0 + tid; v < v1; v += kThreads) {
            uint32_t c2[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (int j = 0; j < ncols; ++j) horner16(c2, __ldg(reinterpret_cast<const uint4 *>(s_col[j]) + v), s_dim[j]);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                atomicAdd(&mytab[c2[q] & 0xffffu], 1);
                atomicAdd(&mytab[c2[q] >> 16], 1);
            }
        }
        if (tail)
            for (int64_t s = (p.S & ~(int64_t)15) + tid; s < p.S; s += kThreads) {
                uint32_t c = 0;
                for (int j = 0; j < ncols; ++j) c = c * s_dim[j] + s_col[j][s];
                atomicAdd(&mytab[c], 1);
            }
        __syncthreads();
        for (int c = tid; c < (int)cells; c += kThreads) {
            int s = 0;
            for (int r = 0; r < R; ++r) s += smem[r * stride + c];
            if (s) atomicAdd(&p.gtab[c], s);
        }
    } else {
        for (int64_t v = v0 * 16 + tid; v < v1 * 16; v += kThreads) {
            uint32_t c = 0;
            for (int j = 0; j < ncols; ++j) c = c * s_dim[j] + s_col[j][v];
            atomicAdd(&p.gtab[c], 1);
        }
        if (tail)
            for (int64_t s = (p.S & ~(int64_t)15) + tid; s < p.S; s += kThreads) {
                uint32_t c = 0;
                for (int j = 0; j < ncols; ++j) c = c * s_dim[j] + s_col[j][s];
                atomicAdd(&p.gtab[c], 1);
            }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(p.done, 1) == (int)gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    int *ct = p.gtab;
    int *ni = ct + cells, *nj = ni + dz * dx, *nk = nj + dz * dy;
    const CtaGroup g{tid};
    const Verdict v = score_dense(g, ct, ni, nj, nk, dx, dy, dz, p.alpha, p.bt, true, p.want_hash != 0, scratch);
    if (tid == 0) {
        fpgm_ci_result r;
        r.table_hash = p.want_hash ? table_hash(ct, cells) : 0;
        r.cell_hash = v.hash;
        r.cells = cells;
        r.df = (int32_t)v.df;
        r.independent = v.indep;
        r.g2 = v.g2;
        r.p_value = v.p;
        r.rechecked = v.rechecked;
        r.path = 1;
        *p.out = r;
        if (v.rechecked) {
            atomicAdd(&p.stats[ST_RECHECK], 1ull);
            if (fabs(v.p - p.alpha) < 1e-12) atomicAdd(&p.stats[ST_NEARTIE], 1ull);
            atomicMax(&p.stats[ST_MAXDP], (unsigned long long)__double_as_longlong(v.dp));
        }
    }
    __syncthreads();
    for (int64_t i = tid; i < cells + marg; i += kThreads) ct[i] = 0;
    if (tid == 0) *p.done = 0;
}

}  // namespace fpgm
