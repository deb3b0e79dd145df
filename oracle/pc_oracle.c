/*
 * oracle/pc_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of FastPGM's PC-stable skeleton phase, used as the
 * checker by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm.
 * Never linked into, or called by, the product library.
 *
 * Followed reference code (paths relative to the FastPGM tree):
 *   data ids       src/fastpgm/Dataset.cpp:459-467 (ids by first appearance),
 *                  :486-488 (cardinality = #distinct observed values)
 *   counting       src/fastpgm/structure_learning/CellTable.cpp:23-72 (dense
 *                  int table n[z][x][y], mixed radix with last Z fastest),
 *                  :226-291 (scan), :242-250 (marginals), :430-455 (2-D case)
 *   df / G^2 / p   src/fastpgm/structure_learning/IndependenceTest.cpp:94-154
 *                  (adjusted df, G^2 in k,i,j order, df==0 -> independent,
 *                  p = 1 - pchisq, independent iff p > alpha) and :295-364
 *   skeleton       src/fastpgm/structure_learning/PCStable.cpp:84-231 (level 0
 *                  over all i<j pairs, then levels d>=1 until FreeDegree <= d),
 *                  :265-388 (adjacency snapshot per level), :399-494 (x side
 *                  then y side per edge), :500-515 (sorted adj minus partner),
 *                  :526-614 (first independent set is the sepset),
 *                  :620-626 (FreeDegree = max |adj| - 1)
 *   combinations   src/fastpgm/ChoiceGenerator.cpp:14-85 (lexicographic)
 *
 * Data are held as int32 columns, like the reference's dataset_columns, and
 * each test allocates and zeroes its dense table, like Counts3D, so the timed
 * CPU baseline does the reference's work per test.  Edges of one level are
 * independent given the level's adjacency snapshot, so they are spread over
 * OpenMP threads; results do not depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "igamma.h"

typedef struct {
    uint64_t table_hash; /* FNV-1a-64 over the int32 joint table in reference cell order (0 when sparse) */
    uint64_t cell_hash;  /* order-free: sum over nonzero cells of mix(cell index, count) */
    int64_t cells;       /* dz * dx * dy */
    int32_t df;
    double g2;
    double p_value;
    int32_t independent;
} oracle_ci_result;

typedef struct {
    int32_t n_levels;
    int64_t tests[64];        /* tests per level, sequential group-size-1 semantics */
    int32_t edges_after[64];  /* edges remaining after each level */
    double seconds[64];
} oracle_pc_stats;

/* ---- data ids (Dataset.cpp:459-467, :486-488) ---- */
void oracle_relabel(const uint8_t *raw, int n_vars, int64_t n_samples, uint8_t *out, uint8_t *card) {
    for (int v = 0; v < n_vars; ++v) {
        int map[256];
        for (int i = 0; i < 256; ++i) map[i] = -1;
        int next = 0;
        const uint8_t *c = raw + (size_t)v * n_samples;
        uint8_t *o = out + (size_t)v * n_samples;
        for (int64_t s = 0; s < n_samples; ++s) {
            int x = c[s];
            if (map[x] < 0) map[x] = next++;
            o[s] = (uint8_t)map[x];
        }
        card[v] = (uint8_t)next;
    }
}

static uint64_t fnv1a_i32(const int32_t *v, int64_t n) {
    uint64_t h = 1469598103934665603ull;
    for (int64_t i = 0; i < n; ++i) {
        uint32_t w = (uint32_t)v[i];
        for (int b = 0; b < 4; ++b) {
            h ^= (w >> (8 * b)) & 0xffu;
            h *= 1099511628211ull;
        }
    }
    return h;
}

static uint64_t cell_mix(uint64_t key, uint32_t count) {
    uint64_t z = key * 0x100000001B3ull + (uint64_t)count + 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

/* Tables beyond this many cells are counted from sorted cell keys instead of a dense array. */
#define ORACLE_DENSE_MAX ((int64_t)1 << 24)

static void finish_result(oracle_ci_result *res, double g2, int64_t df, double alpha) {
    res->df = (int32_t)df;
    res->g2 = g2;
    if (df == 0) {
        res->p_value = 1.0;
        res->independent = 1;
    } else {
        res->p_value = oracle_chisq_pvalue(g2, (int)df);
        res->independent = res->p_value > alpha;
    }
}

/* Same test over the observed cells only: keys (z, x, y) sorted ascending visit the
 * nonzero cells in the reference's k, i, j loop order, so the FP64 sum is the same. */
static int ci_test_sparse(int32_t *const *cols, const uint8_t *card, int64_t S, int x, int y, const int *z, int d,
                          double alpha, oracle_ci_result *res) {
    const uint64_t dx = card[x], dy = card[y], dxy = dx * dy;
    uint64_t radix[64], dz = 1;
    for (int j = d - 1; j >= 0; --j) {
        radix[j] = dz;
        dz *= card[z[j]];
    }
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)S);
    int32_t *ni = (int32_t *)calloc(dx, sizeof(int32_t)), *nj = (int32_t *)calloc(dy, sizeof(int32_t));
    if (!keys || !ni || !nj) {
        free(keys); free(ni); free(nj);
        return -1;
    }
    for (int64_t s = 0; s < S; ++s) {
        uint64_t zc = 0;
        for (int j = 0; j < d; ++j) zc += (uint64_t)cols[z[j]][s] * radix[j];
        keys[s] = (zc * dx + (uint64_t)cols[x][s]) * dy + (uint64_t)cols[y][s];
    }
    qsort(keys, (size_t)S, sizeof(uint64_t), cmp_u64);
    double g2 = 0.0;
    int64_t df = 0;
    uint64_t h = 0;
    int64_t a = 0;
    while (a < S) { /* one stratum: keys with the same key / dxy */
        const uint64_t zk = keys[a] / dxy;
        int64_t b = a;
        while (b < S && keys[b] / dxy == zk) ++b;
        memset(ni, 0, sizeof(int32_t) * dx);
        memset(nj, 0, sizeof(int32_t) * dy);
        for (int64_t t = a; t < b; ++t) {
            const uint64_t c = keys[t] % dxy;
            ni[c / dy]++;
            nj[c % dy]++;
        }
        int alx = 0, aly = 0;
        for (uint64_t i = 0; i < dx; ++i) alx += ni[i] > 0;
        for (uint64_t j = 0; j < dy; ++j) aly += nj[j] > 0;
        alx = alx >= 1 ? alx : 1;
        aly = aly >= 1 ? aly : 1;
        df += (int64_t)(alx - 1) * (aly - 1);
        const long total = (long)(b - a);
        int64_t t = a;
        while (t < b) {
            int64_t u = t;
            while (u < b && keys[u] == keys[t]) ++u;
            const uint64_t c = keys[t] % dxy;
            const long obs = (long)(u - t), row = ni[c / dy], col = nj[c % dy];
            const double expected = (double)col * (double)row / (double)total;
            g2 += 2.0 * obs * log(obs / expected);
            h += cell_mix(keys[t], (uint32_t)obs);
            t = u;
        }
        a = b;
    }
    res->cells = (int64_t)(dz * dxy);
    res->table_hash = 0;
    res->cell_hash = h;
    finish_result(res, g2, df, alpha);
    free(keys); free(ni); free(nj);
    return 0;
}

/* One CI test on int32 columns.  Returns 0, or -1 if the table cannot be allocated. */
static int ci_test_cols(int32_t *const *cols, const uint8_t *card, int64_t S, int x, int y,
                        const int *z, int d, double alpha, int want_hash, oracle_ci_result *res) {
    const int dx = card[x], dy = card[y];
    /* mixed radix over Z, last variable fastest (CellTable.cpp:39-51) */
    int64_t dz = 1;
    int64_t radix[64];
    double dzf = 1.0;
    for (int j = d - 1; j >= 0; --j) {
        radix[j] = dz;
        dz *= card[z[j]];
        dzf *= card[z[j]];
    }
    if (dzf * dx * dy > (double)ORACLE_DENSE_MAX) return ci_test_sparse(cols, card, S, x, y, z, d, alpha, res);
    const int64_t cells = dz * dx * dy;
    int32_t *n = (int32_t *)calloc((size_t)cells, sizeof(int32_t));
    int32_t *ni = (int32_t *)calloc((size_t)(dz * dx), sizeof(int32_t));
    int32_t *nj = (int32_t *)calloc((size_t)(dz * dy), sizeof(int32_t));
    int32_t *nk = (int32_t *)calloc((size_t)dz, sizeof(int32_t));
    if (!n || !ni || !nj || !nk) {
        free(n); free(ni); free(nj); free(nk);
        return -1;
    }
    const int32_t *cx = cols[x], *cy = cols[y];
    if (d == 0) {
        for (int64_t s = 0; s < S; ++s) n[cx[s] * dy + cy[s]]++;
    } else {
        for (int64_t s = 0; s < S; ++s) {
            int64_t zc = 0;
            for (int j = 0; j < d; ++j) zc += (int64_t)cols[z[j]][s] * radix[j];
            n[(zc * dx + cx[s]) * dy + cy[s]]++;
        }
    }
    for (int64_t k = 0; k < dz; ++k)
        for (int i = 0; i < dx; ++i)
            for (int j = 0; j < dy; ++j) {
                int32_t o = n[(k * dx + i) * dy + j];
                ni[k * dx + i] += o;
                nj[k * dy + j] += o;
                nk[k] += o;
            }
    /* IndependenceTest.cpp:94-138 */
    double g2 = 0.0;
    int64_t df = 0;
    for (int64_t k = 0; k < dz; ++k) {
        int alx = 0, aly = 0;
        for (int i = 0; i < dx; ++i) alx += ni[k * dx + i] > 0;
        for (int j = 0; j < dy; ++j) aly += nj[k * dy + j] > 0;
        alx = alx >= 1 ? alx : 1;
        aly = aly >= 1 ? aly : 1;
        df += (int64_t)(alx - 1) * (aly - 1);
        long total = d == 0 ? (long)S : (long)nk[k];
        if (total == 0) continue;
        for (int i = 0; i < dx; ++i) {
            long row = ni[k * dx + i];
            if (row == 0) continue;
            for (int j = 0; j < dy; ++j) {
                long col = nj[k * dy + j];
                long obs = n[(k * dx + i) * dy + j];
                if (col == 0 || obs == 0) continue;
                double expected = (double)col * (double)row / (double)total;
                g2 += 2.0 * obs * log(obs / expected);
            }
        }
    }
    res->cells = cells;
    res->table_hash = want_hash ? fnv1a_i32(n, cells) : 0;
    uint64_t h = 0;
    if (want_hash)
        for (int64_t c = 0; c < cells; ++c)
            if (n[c]) h += cell_mix((uint64_t)c, (uint32_t)n[c]);
    res->cell_hash = h;
    finish_result(res, g2, df, alpha);
    free(n); free(ni); free(nj); free(nk);
    return 0;
}

static int32_t **make_int_columns(const uint8_t *cols, int n, int64_t S) {
    int32_t **c = (int32_t **)malloc(sizeof(int32_t *) * (size_t)n);
    for (int v = 0; v < n; ++v) {
        c[v] = (int32_t *)malloc(sizeof(int32_t) * (size_t)S);
        for (int64_t s = 0; s < S; ++s) c[v][s] = cols[(size_t)v * S + s];
    }
    return c;
}

static void free_int_columns(int32_t **c, int n) {
    for (int v = 0; v < n; ++v) free(c[v]);
    free(c);
}

/* Batch of CI tests: tests[t*(2+d) + {0,1,2..}] = x, y, z1..zd.  Data already relabelled. */
int oracle_ci_tests(const uint8_t *cols, const uint8_t *card, int n_vars, int64_t S, const int32_t *tests,
                    int n_tests, int d, double alpha, int threads, oracle_ci_result *out) {
    int32_t **c = make_int_columns(cols, n_vars, S);
    int err = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
    for (int t = 0; t < n_tests; ++t) {
        const int32_t *tt = tests + (size_t)t * (2 + d);
        int z[64];
        for (int j = 0; j < d; ++j) z[j] = tt[2 + j];
        if (ci_test_cols(c, card, S, tt[0], tt[1], z, d, alpha, 1, &out[t]) != 0) err = -1;
    }
    free_int_columns(c, n_vars);
    return err;
}

/* ---- skeleton ---- */

static int64_t edge_index(int n, int i, int j) { /* Network.cpp:278, i < j */
    return (int64_t)(2 * n - i - 1) * i / 2 + j - i - 1;
}

/* next lexicographic b-combination of [0,a); returns 0 when exhausted (ChoiceGenerator.cpp:55-85) */
static int next_combination(int *c, int a, int b) {
    int i = b - 1;
    while (i >= 0 && c[i] == a - b + i) --i;
    if (i < 0) return 0;
    c[i]++;
    for (int j = i + 1; j < b; ++j) c[j] = c[j - 1] + 1;
    return 1;
}

/*
 * Runs the PC-stable skeleton.  Outputs:
 *   adj[n*n]            final skeleton adjacency (1 = edge kept)
 *   sep_len[E]          for every i<j pair in complete-graph order: -1 if the
 *                       edge survives, else the size of its separating set
 *   sep_vars[E*max_z]   the separating set (sorted ascending, as set<int>)
 *   stats               per-level deterministic test counts and timings
 * depth follows the PCStable ctor (levels d = 1 .. depth-1 after level 0).
 * Returns 0, -1 on bad input, -2 if a sepset exceeds max_z, -3 on allocation failure.
 */
int oracle_pc_skeleton(const uint8_t *cols, const uint8_t *card, int n, int64_t S, double alpha, int depth,
                       int threads, int max_z, uint8_t *adj, int32_t *sep_len, int32_t *sep_vars,
                       oracle_pc_stats *stats) {
    if (n < 2 || S < 1 || max_z < 0 || max_z > 63) return -1;
    if (threads < 1) threads = 1;
    int32_t **c = make_int_columns(cols, n, S);
    const int64_t E = (int64_t)n * (n - 1) / 2;
    for (int64_t e = 0; e < E; ++e) sep_len[e] = -1;
    memset(adj, 0, (size_t)n * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) adj[(size_t)i * n + j] = (uint8_t)(i != j);
    memset(stats, 0, sizeof(*stats));
    int err = 0;

    /* level 0 (PCStable.cpp:133-195) */
    double t0 = omp_get_wtime();
    uint8_t *remove = (uint8_t *)calloc((size_t)E, 1);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int i = 0; i < n - 1; ++i) {
        for (int j = i + 1; j < n; ++j) {
            oracle_ci_result r;
            if (ci_test_cols(c, card, S, i, j, NULL, 0, alpha, 0, &r) != 0) { err = -3; continue; }
            if (r.independent) remove[edge_index(n, i, j)] = 1;
        }
    }
    int64_t remaining = 0;
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            int64_t e = edge_index(n, i, j);
            if (remove[e]) {
                adj[(size_t)i * n + j] = adj[(size_t)j * n + i] = 0;
                sep_len[e] = 0;
            } else {
                ++remaining;
            }
        }
    stats->tests[0] = E;
    stats->edges_after[0] = (int32_t)remaining;
    stats->seconds[0] = omp_get_wtime() - t0;
    stats->n_levels = 1;

    /* level 1 always runs (PCStable.cpp:209-231); later levels only while FreeDegree > d */
    int more = 1, max_deg = 0;

    int32_t *elist = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)(remaining + 1));
    int64_t *etests = (int64_t *)malloc(sizeof(int64_t) * (size_t)(remaining + 1));
    int32_t *esep = (int32_t *)malloc(sizeof(int32_t) * (size_t)(remaining + 1) * (max_z + 1));
    uint8_t *snap = (uint8_t *)malloc((size_t)n * n);

    for (int d = 1; d < depth && more && !err; ++d) {
        if (d > 63) { err = -2; break; }
        t0 = omp_get_wtime();
        memcpy(snap, adj, (size_t)n * n); /* PCStable.cpp:272 */
        int64_t ne = 0;
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j)
                if (adj[(size_t)i * n + j]) { elist[2 * ne] = i; elist[2 * ne + 1] = j; ++ne; }
#pragma omp parallel num_threads(threads)
        {
            int *cand = (int *)malloc(sizeof(int) * (size_t)n);
            int zc[64], z[64];
#pragma omp for schedule(dynamic, 1)
            for (int64_t e = 0; e < ne; ++e) {
                int x = elist[2 * e], y = elist[2 * e + 1];
                int64_t tests = 0;
                int found = 0;
                int32_t *my_sep = esep + (size_t)e * (max_z + 1);
                my_sep[0] = -1;
                for (int side = 0; side < 2 && !found; ++side) {
                    int a = side == 0 ? x : y, b = side == 0 ? y : x;
                    int na = 0;
                    for (int v = 0; v < n; ++v)
                        if (v != b && snap[(size_t)a * n + v]) cand[na++] = v;
                    if (na < d) continue;
                    for (int k = 0; k < d; ++k) zc[k] = k;
                    do {
                        for (int k = 0; k < d; ++k) z[k] = cand[zc[k]];
                        oracle_ci_result r;
                        ++tests;
                        if (ci_test_cols(c, card, S, x, y, z, d, alpha, 0, &r) != 0) { err = -3; break; }
                        if (r.independent) {
                            found = 1;
                            if (d > max_z) { err = -2; break; }
                            my_sep[0] = d;
                            for (int k = 0; k < d; ++k) my_sep[1 + k] = z[k];
                            break;
                        }
                    } while (next_combination(zc, na, d));
                }
                etests[e] = tests;
            }
            free(cand);
        }
        int64_t tot = 0;
        remaining = 0;
        for (int64_t e = 0; e < ne; ++e) {
            tot += etests[e];
            int32_t *my_sep = esep + (size_t)e * (max_z + 1);
            if (my_sep[0] >= 0) {
                int x = elist[2 * e], y = elist[2 * e + 1];
                adj[(size_t)x * n + y] = adj[(size_t)y * n + x] = 0;
                int64_t ei = edge_index(n, x, y);
                sep_len[ei] = my_sep[0];
                for (int k = 0; k < my_sep[0]; ++k) sep_vars[ei * max_z + k] = my_sep[1 + k];
            } else {
                ++remaining;
            }
        }
        max_deg = 0;
        for (int i = 0; i < n; ++i) {
            int dg = 0;
            for (int j = 0; j < n; ++j) dg += adj[(size_t)i * n + j];
            if (dg > max_deg) max_deg = dg;
        }
        more = (max_deg - 1) > d; /* PCStable.cpp:387 */
        if (stats->n_levels < 64) {
            stats->tests[stats->n_levels] = tot;
            stats->edges_after[stats->n_levels] = (int32_t)remaining;
            stats->seconds[stats->n_levels] = omp_get_wtime() - t0;
            stats->n_levels++;
        }
    }
    free(elist); free(etests); free(esep); free(snap); free(remove);
    free_int_columns(c, n);
    return err;
}

/* ---- maximum-likelihood parameters with Laplace smoothing for a known DAG
 * ParameterLearning::LearnParamsKnowStructCompData
 * (src/fastpgm/parameter_learning/ParameterLearning.cpp:22-86): node v's table is over
 * (v, its parents in ascending order) -- PotentialTableBase.cpp:102-130, mixed radix with
 * the last variable fastest, v slowest -- N counts every sample's configuration, N(B) the
 * parent configuration (index mod cum_levels[0]), and
 *   potential[j] = (N[j] + alpha) / (N(B of j) + alpha * card[v]).
 * parent_off[n+1] / parents: each node's parent list (sorted, no repeats: a set in the
 * reference).  out_off[n+1] receives the table offsets; out_pot (when not NULL) the tables.
 * Returns 0, or -1 when a table would exceed 2^31 entries. */
int oracle_mle_cpts(const uint8_t *cols, const uint8_t *card, int n, int64_t S, const int32_t *parent_off,
                    const int32_t *parents, int alpha, int64_t *out_off, double *out_pot) {
    out_off[0] = 0;
    for (int v = 0; v < n; ++v) {
        double size = card[v];
        for (int k = parent_off[v]; k < parent_off[v + 1]; ++k) size *= card[parents[k]];
        if (size > 2147483647.0) return -1;
        out_off[v + 1] = out_off[v] + (int64_t)size;
    }
    if (!out_pot) return 0;
    for (int v = 0; v < n; ++v) {
        const int np = parent_off[v + 1] - parent_off[v];
        const int32_t *par = parents + parent_off[v];
        const int64_t size = out_off[v + 1] - out_off[v];
        const int64_t cum0 = size / card[v]; /* parent configurations */
        int32_t *N = (int32_t *)calloc((size_t)size, sizeof(int32_t));
        int32_t *NB = (int32_t *)calloc((size_t)cum0, sizeof(int32_t));
        if (!N || !NB) { free(N); free(NB); return -1; }
        for (int64_t s = 0; s < S; ++s) {
            int64_t idx = cols[(int64_t)v * S + s];
            for (int k = 0; k < np; ++k) idx = idx * card[par[k]] + cols[(int64_t)par[k] * S + s];
            N[idx]++;
            NB[idx % cum0]++;
        }
        for (int64_t j = 0; j < size; ++j)
            out_pot[out_off[v] + j] = ((double)N[j] + alpha) / ((double)NB[j % cum0] + alpha * card[v]);
        free(N);
        free(NB);
    }
    return 0;
}
