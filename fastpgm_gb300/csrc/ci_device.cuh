// Device building blocks of one G^2 conditional-independence test.
//
// A test (x, y | z1..zd) counts the joint table n[z][x][y] over all samples,
// with z the mixed-radix code of (z1..zd), last variable fastest
// (reference: structure_learning/CellTable.cpp:39-51, :254-291), builds the
// marginals N_x+z, N_+yz, N_++z (:242-250), the adjusted degrees of freedom
// and G^2 (IndependenceTest.cpp:94-138), and p = 1 - P(df/2, G^2/2)
// (:146), independent iff df == 0 or p > alpha (:140-142, :153).
//
// Precision policy: counts are exact int32; G^2 terms are FP32 with a
// Neumaier-compensated sum and a running error bound; the p-value is FP64.
// A test whose p lies within the recheck band of alpha (|p - alpha| < 1e-3,
// widened by the propagated FP32 error) is recomputed with FP64 terms, so
// every decision is an FP64 decision wherever FP32 could flip it.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "fastpgm_gb300.h"

namespace fpgm {

constexpr int kMaxCond = FPGM_MAX_COND;
constexpr int kMaxCols = kMaxCond + 2;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kBinomN = 4096;   // rows of the binomial table
constexpr int kBinomK = 32;     // columns (k <= 31)
constexpr double kBand = 1e-3;  // FP64 recheck band around alpha

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

// chi-square density, used to turn a G^2 error bound into a p error bound.
__host__ __device__ inline double chisq_pdf(double x, long long df) {
    if (!(x > 0.0)) return df <= 2 ? 1.0 : 0.0;
    double k = 0.5 * (double)df;
    return exp((k - 1.0) * log(x) - 0.5 * x - k * 0.69314718055994530942 - lgamma(k));
}

// ---------------------------------------------------------------- test descriptor
struct TestDesc {
    int32_t x, y, d, ncols;
    int32_t dx, dy;
    int32_t R;            // replicas of the shared-memory table
    int32_t path;         // 0 shared memory, 1 global memory, 2 unsupported
    int64_t dz, cells;
    int32_t dims[kMaxCols];             // Z dims, then dx, dy (Horner order)
    const uint8_t *col[kMaxCols];       // matching column pointers
    int32_t z[kMaxCond];
};

// Fills dims/cols/cells from x, y, z and picks the counting path.
// budget_ints: shared-memory ints available for table + marginals.
__device__ inline void desc_finish(TestDesc &t, const uint8_t *cols, int64_t S_pad, const uint8_t *card,
                                   int64_t budget_ints, int64_t large_ints) {
    t.dx = card[t.x];
    t.dy = card[t.y];
    int64_t dz = 1;
    bool over = false;
    for (int k = 0; k < t.d; ++k) {
        int dk = card[t.z[k]];
        t.dims[k] = dk;
        t.col[k] = cols + (int64_t)t.z[k] * S_pad;
        dz *= dk;
        if (dz > ((int64_t)1 << 40)) over = true;
    }
    t.dims[t.d] = t.dx;
    t.col[t.d] = cols + (int64_t)t.x * S_pad;
    t.dims[t.d + 1] = t.dy;
    t.col[t.d + 1] = cols + (int64_t)t.y * S_pad;
    t.ncols = t.d + 2;
    t.dz = dz;
    t.cells = dz * t.dx * t.dy;
    int64_t marg = dz * (t.dx + t.dy + 1);
    t.R = 1;
    if (over) {
        t.path = 2;
        return;
    }
    if (t.cells + marg <= budget_ints) {
        t.path = 0;
        for (int R = 32; R >= 2; R >>= 1)
            if (t.cells * R + t.cells + marg <= budget_ints) { t.R = R; break; }
    } else if (t.cells + marg <= large_ints) {
        t.path = 1;
    } else {
        t.path = 2;
    }
}

// ---------------------------------------------------------------- counting
// Counts samples of vector range [v0, v1) (16 samples per vector) and, if
// tail, the S % 16 leftover samples, into tab (R replicas, skewed layout so
// the lanes of a warp hitting one cell land in different banks).
template <bool kGlobal>
__device__ inline void count_range(const TestDesc &t, int64_t v0, int64_t v1, bool tail, int64_t S, int *tab,
                                   int tid, int nthreads) {
    const int lane = threadIdx.x & 31;
    const int R = t.R, Rm = R - 1;
    const int ncols = t.ncols;
    for (int64_t v = v0 + tid; v < v1; v += nthreads) {
        uint32_t code[16];
#pragma unroll
        for (int b = 0; b < 16; ++b) code[b] = 0;
        for (int j = 0; j < ncols; ++j) {
            const uint4 w = __ldg(reinterpret_cast<const uint4 *>(t.col[j]) + v);
            const uint32_t dim = (uint32_t)t.dims[j];
            const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int b = 0; b < 16; ++b) code[b] = code[b] * dim + ((ww[b >> 2] >> (8 * (b & 3))) & 0xffu);
        }
#pragma unroll
        for (int b = 0; b < 16; ++b) {
            const uint32_t c = code[b];
            if (kGlobal)
                atomicAdd(&tab[c], 1);
            else
                atomicAdd(&tab[(int64_t)c * R + ((lane + (int)c) & Rm)], 1);
        }
    }
    if (tail) {
        for (int64_t s = (S & ~(int64_t)15) + tid; s < S; s += nthreads) {
            uint32_t c = 0;
            for (int j = 0; j < ncols; ++j) c = c * (uint32_t)t.dims[j] + t.col[j][s];
            if (kGlobal)
                atomicAdd(&tab[c], 1);
            else
                atomicAdd(&tab[(int64_t)c * R + ((lane + (int)c) & Rm)], 1);
        }
    }
}

// ---------------------------------------------------------------- reductions
struct Partial {
    long long df;
    double g2, err, abs_g2;
};

__device__ inline Partial block_reduce(Partial p, Partial *scratch /* kWarps */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        p.df += __shfl_down_sync(0xffffffffu, p.df, o);
        p.g2 += __shfl_down_sync(0xffffffffu, p.g2, o);
        p.err += __shfl_down_sync(0xffffffffu, p.err, o);
        p.abs_g2 += __shfl_down_sync(0xffffffffu, p.abs_g2, o);
    }
    if (lane == 0) scratch[warp] = p;
    __syncthreads();
    Partial r{0, 0.0, 0.0, 0.0};
    if (threadIdx.x == 0) {
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            r.df += scratch[w].df;
            r.g2 += scratch[w].g2;
            r.err += scratch[w].err;
            r.abs_g2 += scratch[w].abs_g2;
        }
    }
    __syncthreads();
    return r;  // valid in thread 0
}

struct Verdict {
    long long df;
    double g2, p;
    int indep, rechecked;
    double dp;  // |p32 - p64| when rechecked
};

// ---------------------------------------------------------------- scoring
// ct: compact table [dz][dx][dy]; ni/nj/nk scratch of dz*dx, dz*dy, dz ints.
// Every thread of the block must call this; the verdict is valid in thread 0.
__device__ inline Verdict score_table(const TestDesc &t, const int *ct, int *ni, int *nj, int *nk, double alpha,
                                      Partial *scratch, int tid, int nthreads) {
    const int dx = t.dx, dy = t.dy;
    const int64_t dz = t.dz, dxy = (int64_t)dx * dy;
    for (int64_t idx = tid; idx < dz * dx; idx += nthreads) {
        const int *row = ct + idx * dy;
        int s = 0;
        for (int j = 0; j < dy; ++j) s += row[j];
        ni[idx] = s;
    }
    for (int64_t idx = tid; idx < dz * dy; idx += nthreads) {
        int64_t k = idx / dy;
        int j = (int)(idx - k * dy);
        const int *base = ct + k * dxy + j;
        int s = 0;
        for (int i = 0; i < dx; ++i) s += base[(int64_t)i * dy];
        nj[idx] = s;
    }
    __syncthreads();
    Partial p{0, 0.0, 0.0, 0.0};
    for (int64_t k = tid; k < dz; k += nthreads) {
        int alx = 0, aly = 0, tot = 0;
        for (int i = 0; i < dx; ++i) {
            int v = ni[k * dx + i];
            alx += v > 0;
            tot += v;
        }
        for (int j = 0; j < dy; ++j) aly += nj[k * dy + j] > 0;
        nk[k] = tot;
        alx = alx >= 1 ? alx : 1;
        aly = aly >= 1 ? aly : 1;
        p.df += (long long)(alx - 1) * (aly - 1);
    }
    __syncthreads();
    // FP32 terms 2 O ln(O N_z / (N_x N_y)) with exact int64 products.
    float s = 0.f, c = 0.f, e = 0.f, a = 0.f;
    for (int64_t cell = tid; cell < t.cells; cell += nthreads) {
        const int O = ct[cell];
        if (O == 0) continue;
        const int64_t k = cell / dxy;
        const int rem = (int)(cell - k * dxy);
        const int i = rem / dy, j = rem - (rem / dy) * dy;
        const long long num = (long long)O * nk[k];
        const long long den = (long long)ni[k * dx + i] * nj[k * dy + j];
        if (num == den) continue;
        const float q = (float)(num - den) / (float)den;
        float l;
        if (fabsf(q) < 0.5f)
            l = log1pf(q);
        else
            l = logf((float)num / (float)den);
        const float term = 2.0f * (float)O * l;
        // Neumaier compensated accumulation
        const float tt = s + term;
        if (fabsf(s) >= fabsf(term))
            c += (s - tt) + term;
        else
            c += (term - tt) + s;
        s = tt;
        e += 2.0f * (float)O * (2.5e-7f * fminf(1.0f, 2.0f * fabsf(q)) + 2.5e-7f * fabsf(l));
        a += fabsf(term);
    }
    p.g2 = (double)s + (double)c;
    p.err = (double)e;
    p.abs_g2 = (double)a;
    Partial r = block_reduce(p, scratch);
    __shared__ int s_recheck;
    __shared__ double s_p32;
    Verdict v{0, 0.0, 1.0, 1, 0, 0.0};
    if (tid == 0) {
        v.df = r.df;
        v.g2 = r.g2;
        s_recheck = 0;
        if (r.df == 0) {
            v.p = 1.0;
            v.indep = 1;
        } else {
            const double err = 2.0 * r.err + 1e-6 * r.abs_g2 + 1e-12;
            v.p = chisq_pvalue(r.g2, r.df);
            const double dpb = chisq_pdf(r.g2 > err ? r.g2 - err : 0.0, r.df) * err * 2.0;
            v.indep = v.p > alpha;
            if (fabs(v.p - alpha) < kBand || fabs(v.p - alpha) < dpb) s_recheck = 1;
            s_p32 = v.p;
        }
    }
    __syncthreads();
    if (s_recheck) {
        // FP64 terms, the reference's formula: E = N_+yz * N_x+z / N_++z, 2 O ln(O / E).
        Partial q{0, 0.0, 0.0, 0.0};
        for (int64_t cell = tid; cell < t.cells; cell += nthreads) {
            const int O = ct[cell];
            if (O == 0) continue;
            const int64_t k = cell / dxy;
            const int rem = (int)(cell - k * dxy);
            const int i = rem / dy, j = rem - (rem / dy) * dy;
            const double expected = (double)nj[k * dy + j] * (double)ni[k * dx + i] / (double)nk[k];
            q.g2 += 2.0 * O * log(O / expected);
        }
        Partial r2 = block_reduce(q, scratch);
        if (tid == 0) {
            v.g2 = r2.g2;
            v.p = chisq_pvalue(r2.g2, v.df);
            v.indep = v.p > alpha;
            v.rechecked = 1;
            v.dp = fabs(v.p - s_p32);
        }
    }
    return v;
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
