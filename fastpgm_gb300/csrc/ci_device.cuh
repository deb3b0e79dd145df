// Device building blocks of one G^2 conditional-independence test.
//
// A test (x, y | z1..zd) counts the joint table n[z][x][y] over all samples,
// with z the mixed-radix code of (z1..zd), last variable fastest
// (reference: structure_learning/CellTable.cpp:39-51, :254-291), builds the
// marginals N_x+z, N_+yz, N_++z (:242-250), the adjusted degrees of freedom
// and G^2 (IndependenceTest.cpp:94-138), and decides independence as
// df == 0 or p = 1 - P(df/2, G^2/2) > alpha (:140-153).
//
// Precision policy.  Counts are exact int32.  G^2 terms are FP32 with a
// Neumaier-compensated sum and a running error bound.  The decision compares
// G^2 +- bound with two FP64 band-edge tables per df, the G^2 values at which
// p = alpha + 1e-3 and p = alpha - 1e-3 (computed once per alpha with the
// FP64 incomplete gamma below).  A test whose G^2 interval reaches into that
// band -- every test whose p-value may lie within 1e-3 of alpha -- is
// recomputed with FP64 terms and an FP64 p-value.  Outside the band the
// decision equals the FP64 one by monotonicity of p in G^2.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "fastpgm_gb300.h"

namespace fpgm {

constexpr int kMaxCond = FPGM_MAX_COND;
constexpr int kMaxCols = kMaxCond + 2;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kSmemBytes = 96 * 1024;
constexpr int kCtaInts = kSmemBytes / 4;                 // CTA tier: table + marginals
constexpr int kWarpInts = kSmemBytes / 4 / kWarps;      // warp tier: per-warp region
constexpr int kWarpIntsSmall = 2048;                     // ... with 8 KB slices (3 CTAs per SM)
constexpr int kGlobalWarpTab = 255 * 255 + 2 * 255 + 1;  // largest dx*dy + dx + dy
constexpr int kBinomN = 4096;
constexpr int kBinomK = 32;
constexpr double kBand = 1e-3;
constexpr int kBandDfMax = 1 << 15;   // dense tiers have df < cells <= 24,576
constexpr uint64_t kEmptyKey = ~0ull;

// ---------------------------------------------------------------- p-value (FP64)
// Regularised incomplete gamma, written from its series (DLMF 8.7.1) and the
// Legendre continued fraction for Q (DLMF 8.9.2) evaluated by the modified
// Lentz method (Press et al., Numerical Recipes 3rd ed., section 6.2).
__host__ __device__ inline double igamma_p(double a, double x) {
    if (!(x > 0.0)) return 0.0;
    const double eps = 1e-16, tiny = 1e-300;
    const int maxit = 1 << 22;
    double pre = exp(-x + a * log(x) - lgamma(a));
    if (x < a + 1.0) {
        double ap = a, term = 1.0 / a, sum = term;
        for (int n = 1; n < maxit; ++n) {
            ap += 1.0;
            term *= x / ap;
            sum += term;
            if (fabs(term) < fabs(sum) * eps) break;
        }
        return sum * pre;
    }
    double b = x + 1.0 - a, c = 1.0 / tiny, d = 1.0 / b, h = d;
    for (int i = 1; i < maxit; ++i) {
        double an = -i * (i - a);
        b += 2.0;
        d = an * d + b;
        if (fabs(d) < tiny) d = tiny;
        c = b + an / c;
        if (fabs(c) < tiny) c = tiny;
        d = 1.0 / d;
        double del = d * c;
        h *= del;
        if (fabs(del - 1.0) < eps) break;
    }
    return 1.0 - pre * h;
}

// p-value of a chi-square statistic as the reference forms it: 1 - CDF.
__host__ __device__ inline double chisq_pvalue(double g2, long long df) {
    return 1.0 - igamma_p(0.5 * (double)df, 0.5 * g2);
}

// chi-square density, to turn a G^2 error bound into a p-value error bound.
__host__ __device__ inline double chisq_pdf(double x, long long df) {
    if (!(x > 0.0)) return df <= 2 ? 1.0 : 0.0;
    const double k = 0.5 * (double)df;
    return exp((k - 1.0) * log(x) - 0.5 * x - k * 0.69314718055994530942 - lgamma(k));
}

// Wilson-Hilferty approximation of the upper tail P(chi2_k > x).  Only routes tests
// with df beyond the band tables: for k >= 32768 its error is below 3.2e-7 (checked
// against the exact incomplete gamma in the tests) and it is used with a 1e-5 margin,
// inside which the exact FP64 incomplete gamma decides.
__host__ __device__ inline double chisq_pvalue_wh(double x, double k) {
    const double v = 2.0 / (9.0 * k);
    const double z = (cbrt(x / k) - (1.0 - v)) / sqrt(v);
    return 0.5 * erfc(z * 0.70710678118654752440);
}
constexpr double kWhMargin = 1e-5;

// G^2 at which the p-value of df degrees of freedom equals target (bisection;
// p is decreasing in G^2).  Returns 0 for target >= 1 and +inf for target <= 0.
// x with P(chi2_df > x) = target, to 1e-10 relative: Newton's method on the upper tail
// (derivative -pdf) from the Wilson-Hilferty estimate, kept inside a bisection bracket
// (a step leaving the bracket bisects instead).
__host__ __device__ inline double chisq_quantile_upper(double target, long long df) {
    if (target >= 1.0) return 0.0;
    if (target <= 0.0) return 1e300;
    double lo = 0.0, hi = (double)df + 10.0 * sqrt(2.0 * (double)df) + 50.0;
    while (chisq_pvalue(hi, df) > target) hi *= 2.0;
    double x = 0.5 * (lo + hi);
#ifdef __CUDA_ARCH__
    {  // Wilson-Hilferty: chi2_k ~ k (1 - 2/(9k) + z sqrt(2/(9k)))^3, z the normal upper quantile
        const double z = normcdfinv(1.0 - target), c = 2.0 / (9.0 * (double)df);
        const double w = 1.0 - c + z * sqrt(c);
        const double x0 = (double)df * w * w * w;
        if (x0 > lo && x0 < hi) x = x0;
    }
#endif
    for (int it = 0; it < 200; ++it) {
        const double p = chisq_pvalue(x, df);
        if (p > target) lo = x; else hi = x;
        if (hi - lo <= 1e-10 * hi) return 0.5 * (lo + hi);
        const double d = chisq_pdf(x, df);
        double xn = d > 0.0 ? x + (p - target) / d : 0.5 * (lo + hi);
        if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
        if (fabs(xn - x) <= 1e-11 * x) return xn;
        x = xn;
    }
    return x;
}

struct BandTables {
    const double *lo;  // G^2 below lo[df]  =>  p > alpha + band  (independent)
    const double *hi;  // G^2 above hi[df]  =>  p < alpha - band  (dependent)
    int dfmax;
};

// 1 independent, 0 dependent, -1 undecided (FP64 recheck).
__device__ inline int band_decide(long long df, double g, double err, const BandTables &bt) {
    if (df == 0) return 1;
    if (df > bt.dfmax) return -1;
    if (g + err < bt.lo[df]) return 1;
    if (g - err > bt.hi[df]) return 0;
    return -1;
}

// ---------------------------------------------------------------- counting helpers
// 16 samples of one column (one 128-bit load) folded into 8 packed pairs of
// 16-bit Horner codes: pair q holds samples of its low/high halves.  Valid
// while every code stays below 65536 (tables of at most 65536 cells).
__device__ __forceinline__ void horner16(uint32_t (&c2)[8], const uint4 w, const uint32_t dim) {
    const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        c2[2 * q] = c2[2 * q] * dim + __byte_perm(ww[q], 0, 0x4140);      // samples 4q, 4q+1
        c2[2 * q + 1] = c2[2 * q + 1] * dim + __byte_perm(ww[q], 0, 0x4342);  // samples 4q+2, 4q+3
    }
}

// Order-independent fingerprint of a count table: sum over nonzero cells of a
// 64-bit mix of (cell index in reference order, count).
__host__ __device__ inline uint64_t cell_mix(uint64_t key, uint32_t count) {
    uint64_t z = key * 0x100000001B3ull + (uint64_t)count + 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// ---------------------------------------------------------------- thread groups
struct WarpGroup {
    int t;
    __device__ int n() const { return 32; }
    __device__ void sync() const { __syncwarp(); }
};
struct CtaGroup {
    int t;
    __device__ int n() const { return (int)blockDim.x; }
    __device__ void sync() const { __syncthreads(); }
};

struct Partial {
    long long df;
    double g2, err, abs_g2;
    unsigned long long hash;
};

__device__ inline Partial warp_sum(Partial p) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        p.df += __shfl_xor_sync(0xffffffffu, p.df, o);
        p.g2 += __shfl_xor_sync(0xffffffffu, p.g2, o);
        p.err += __shfl_xor_sync(0xffffffffu, p.err, o);
        p.abs_g2 += __shfl_xor_sync(0xffffffffu, p.abs_g2, o);
        p.hash += __shfl_xor_sync(0xffffffffu, p.hash, o);
    }
    return p;
}

// Block-wide sum; the result is valid in every thread.  scratch: kWarps entries.
__device__ inline Partial block_sum(Partial p, Partial *scratch) {
    p = warp_sum(p);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch[warp] = p;
    __syncthreads();
    Partial r{0, 0.0, 0.0, 0.0, 0ull};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        r.df += scratch[w].df;
        r.g2 += scratch[w].g2;
        r.err += scratch[w].err;
        r.abs_g2 += scratch[w].abs_g2;
        r.hash += scratch[w].hash;
    }
    return r;
}

__device__ inline Partial group_sum(const WarpGroup &, Partial p, Partial *) { return warp_sum(p); }
__device__ inline Partial group_sum(const CtaGroup &, Partial p, Partial *scratch) { return block_sum(p, scratch); }

// ---------------------------------------------------------------- scoring
// ct: table [dz][dx][dy]; ni/nj/nk: dz*dx, dz*dy, dz ints of scratch.
// Marginals, then per-thread partial df (strata) -- every thread of g calls it.
template <class G>
__device__ inline long long marginals(const G &g, const int *ct, int *ni, int *nj, int *nk, int dx, int dy,
                                      int64_t dz) {
    const int64_t dxy = (int64_t)dx * dy;
    for (int64_t idx = g.t; idx < dz * dx; idx += g.n()) {
        const int *row = ct + idx * dy;
        int s = 0;
        for (int j = 0; j < dy; ++j) s += row[j];
        ni[idx] = s;
    }
    for (int64_t idx = g.t; idx < dz * dy; idx += g.n()) {
        const int64_t k = idx / dy;
        const int j = (int)(idx - k * dy);
        const int *base = ct + k * dxy + j;
        int s = 0;
        for (int i = 0; i < dx; ++i) s += base[(int64_t)i * dy];
        nj[idx] = s;
    }
    g.sync();
    long long df = 0;
    for (int64_t k = g.t; k < dz; k += g.n()) {
        int alx = 0, aly = 0, tot = 0;
        for (int i = 0; i < dx; ++i) {
            const int v = ni[k * dx + i];
            alx += v > 0;
            tot += v;
        }
        for (int j = 0; j < dy; ++j) aly += nj[k * dy + j] > 0;
        nk[k] = tot;
        alx = alx >= 1 ? alx : 1;
        aly = aly >= 1 ? aly : 1;
        df += (long long)(alx - 1) * (aly - 1);
    }
    g.sync();
    return df;
}

// FP32 G^2 terms 2 O ln(O N_z / (N_x N_y)) over this thread's cells, with exact
// int64 products, Neumaier compensation and a first-order error bound.
// zkeys (optional): stratum code of each table row, for the cell fingerprint.
template <class G>
__device__ inline void g2_fp32(const G &g, const int *ct, const int *ni, const int *nj, const int *nk, int dx, int dy,
                               int64_t cells, const uint64_t *zkeys, bool want_hash, Partial &p) {
    const int64_t dxy = (int64_t)dx * dy;
    float s = 0.f, c = 0.f, e = 0.f, a = 0.f;
    unsigned long long h = 0;
    for (int64_t cell = g.t; cell < cells; cell += g.n()) {
        const int O = ct[cell];
        if (O == 0) continue;
        const int64_t k = cell / dxy;
        const int rem = (int)(cell - k * dxy);
        const int i = rem / dy, j = rem - (rem / dy) * dy;
        if (want_hash) {
            const uint64_t key = zkeys ? (zkeys[k] * (uint64_t)dx + i) * (uint64_t)dy + j : (uint64_t)cell;
            h += cell_mix(key, (uint32_t)O);
        }
        const long long num = (long long)O * nk[k];
        const long long den = (long long)ni[k * dx + i] * nj[k * dy + j];
        if (num == den) continue;
        const float q = (float)(num - den) / (float)den;
        const float l = fabsf(q) < 0.5f ? log1pf(q) : logf((float)num / (float)den);
        const float term = 2.0f * (float)O * l;
        const float tt = s + term;
        c += fabsf(s) >= fabsf(term) ? (s - tt) + term : (term - tt) + s;
        s = tt;
        e += 2.0f * (float)O * (2.5e-7f * fminf(1.0f, 2.0f * fabsf(q)) + 2.5e-7f * fabsf(l));
        a += fabsf(term);
    }
    p.g2 += (double)s + (double)c;
    p.err += (double)e;
    p.abs_g2 += (double)a;
    p.hash += h;
}

// FP64 G^2 terms with the reference's formula: E = N_+yz N_x+z / N_++z, 2 O ln(O / E).
template <class G>
__device__ inline double g2_fp64(const G &g, const int *ct, const int *ni, const int *nj, const int *nk, int dx,
                                 int dy, int64_t cells) {
    const int64_t dxy = (int64_t)dx * dy;
    double s = 0.0;
    for (int64_t cell = g.t; cell < cells; cell += g.n()) {
        const int O = ct[cell];
        if (O == 0) continue;
        const int64_t k = cell / dxy;
        const int rem = (int)(cell - k * dxy);
        const int i = rem / dy, j = rem - (rem / dy) * dy;
        const double expected = (double)nj[k * dy + j] * (double)ni[k * dx + i] / (double)nk[k];
        s += 2.0 * O * log(O / expected);
    }
    return s;
}

struct Verdict {
    long long df;
    double g2, p;
    int indep, rechecked;
    double dp;  // |p(FP32 G^2) - p(FP64 G^2)| when rechecked
    unsigned long long hash;
};

// Full scoring of a dense table held by group g (shared or global memory).
// Every thread of g calls it; the verdict is valid in the group's thread 0.
template <class G>
__device__ inline Verdict score_dense(const G &g, const int *ct, int *ni, int *nj, int *nk, int dx, int dy,
                                      int64_t dz, double alpha, const BandTables &bt, bool want_p, bool want_hash,
                                      Partial *scratch) {
    Partial p{0, 0.0, 0.0, 0.0, 0ull};
    p.df = marginals(g, ct, ni, nj, nk, dx, dy, dz);
    const int64_t cells = dz * dx * dy;
    g2_fp32(g, ct, ni, nj, nk, dx, dy, cells, nullptr, want_hash, p);
    Partial r = group_sum(g, p, scratch);
    Verdict v{r.df, r.g2, 1.0, 1, 0, 0.0, r.hash};
    const double err = 2.0 * r.err + 1e-6 * r.abs_g2 + 1e-12;
    const int dec = band_decide(r.df, r.g2, err, bt);  // uniform across the group
    // p-values are evaluated by the group leader only (FP64 incomplete gamma)
    const bool leader = g.t == 0;
    if (dec < 0) {
        Partial q{0, 0.0, 0.0, 0.0, 0ull};
        q.g2 = g2_fp64(g, ct, ni, nj, nk, dx, dy, cells);
        Partial r2 = group_sum(g, q, scratch);
        v.g2 = r2.g2;
        v.rechecked = 1;
        if (leader) {
            v.p = chisq_pvalue(r2.g2, r.df);
            v.indep = v.p > alpha;
            v.dp = fabs(v.p - chisq_pvalue(r.g2, r.df));
        }
    } else {
        v.indep = dec;
        if (leader) v.p = (want_p && r.df > 0) ? chisq_pvalue(r.g2, r.df) : (r.df == 0 ? 1.0 : (dec ? 1.0 : 0.0));
    }
    return v;  // indep and p are valid in the leader
}

// FNV-1a-64 of the int32 table in cell order (test hook only; one thread).
__device__ inline uint64_t table_hash(const int *ct, int64_t cells) {
    uint64_t h = 1469598103934665603ull;
    for (int64_t i = 0; i < cells; ++i) {
        uint32_t w = (uint32_t)ct[i];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            h ^= (w >> (8 * b)) & 0xffu;
            h *= 1099511628211ull;
        }
    }
    return h;
}

// ---------------------------------------------------------------- combinations
// Binomial table C[n][k], n < kBinomN, k < kBinomK, saturating at UINT64_MAX.
__device__ inline uint64_t binom(const uint64_t *tab, int n, int k) {
    if (k < 0 || n < 0 || k > n) return 0;
    return tab[(int64_t)n * kBinomK + k];
}

// Lexicographic unranking of a d-combination of [0, na) (the order the
// reference's ChoiceGenerator::Next walks, ChoiceGenerator.cpp:55-85):
// rank_lex = C(na,d) - 1 - sum_i C(na-1-c_i, d-i); invert greedily.
__device__ inline void unrank_lex(const uint64_t *btab, int na, int d, uint64_t r, int *c) {
    uint64_t R = binom(btab, na, d) - 1 - r;
    int hi = na - 1;
    for (int i = 0; i < d; ++i) {
        const int k = d - i;
        int lo = k - 1, h = hi;  // largest e in [lo, h] with C(e,k) <= R
        while (lo < h) {
            int mid = (lo + h + 1) >> 1;
            if (binom(btab, mid, k) <= R) lo = mid; else h = mid - 1;
        }
        c[i] = na - 1 - lo;
        R -= binom(btab, lo, k);
        hi = lo - 1;
    }
}

}  // namespace fpgm
