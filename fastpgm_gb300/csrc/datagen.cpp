// Seeded synthetic Bayesian-network sample generator.
//
// Plays the role of the reference's forward sampler
// (src/fastpgm/SampleSetGenerator.cpp), which seeds from wall-clock time
// (SampleSetGenerator.cpp:36-37) and therefore cannot reproduce a dataset.
// This one is a pure function of its spec:
//   * random DAG over a random topological order with a target edge count and
//     a maximum in-degree;
//   * per-node cardinality drawn from a uniform range plus an optional long
//     tail;
//   * one Dirichlet(alpha) row per parent configuration (Marsaglia-Tsang
//     gamma variates);
//   * forward sampling with one independent random stream per sample, so the
//     output does not depend on the thread count.
// Every floating-point step uses only IEEE basic operations (log/exp are
// evaluated by the series below, not by libm) and the file is compiled with
// -ffp-contract=off, so x86-64 and AArch64 produce identical bytes.
//
// Output: column-major uint8, column v at out + v * n_samples, values are raw
// category indices in [0, card_v).
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

#include "fastpgm_gb300.h"

namespace {

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t &x) {
        uint64_t z = (x += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) s[i] = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {  // xoshiro256**
        uint64_t r = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    double uniform_pos() {  // (0,1)
        double u;
        do { u = uniform(); } while (u <= 0.0);
        return u;
    }
    uint32_t below(uint32_t n) { return (uint32_t)(((next() >> 32) * (uint64_t)n) >> 32); }
};

const double kLn2 = 0.69314718055994530942;

// Natural log from frexp range reduction and the atanh series
// ln m = 2 (t + t^3/3 + t^5/5 + ...), t = (m-1)/(m+1).
double det_log(double x) {
    int e;
    double m = std::frexp(x, &e);  // x = m 2^e, m in [0.5,1)
    if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }
    double t = (m - 1.0) / (m + 1.0), t2 = t * t, term = t, sum = 0.0;
    for (int k = 1; k < 80; k += 2) {
        double add = term / k;
        sum += add;
        if (std::fabs(add) < 1e-18) break;
        term *= t2;
    }
    return 2.0 * sum + e * kLn2;
}

// exp(x) = 2^k e^r with |r| <= ln2/2 and a Taylor series for e^r.
double det_exp(double x) {
    if (x < -745.0) return 0.0;
    double kd = std::floor(x / kLn2 + 0.5);
    double r = x - kd * kLn2;
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 40; ++n) {
        term *= r / n;
        sum += term;
        if (std::fabs(term) < 1e-18) break;
    }
    return std::ldexp(sum, (int)kd);
}

double det_normal(Rng &g) {  // Marsaglia polar method
    for (;;) {
        double u = 2.0 * g.uniform() - 1.0, v = 2.0 * g.uniform() - 1.0;
        double s = u * u + v * v;
        if (s > 0.0 && s < 1.0) return u * std::sqrt(-2.0 * det_log(s) / s);
    }
}

// Gamma(a, 1) variate: Marsaglia & Tsang (2000); a < 1 boosted by U^(1/a).
double det_gamma(Rng &g, double a) {
    if (a < 1.0) {
        double y = det_gamma(g, a + 1.0);
        return y * det_exp(det_log(g.uniform_pos()) / a);
    }
    double d = a - 1.0 / 3.0, c = 1.0 / std::sqrt(9.0 * d);
    for (;;) {
        double x = det_normal(g), v = 1.0 + c * x;
        if (v <= 0.0) continue;
        v = v * v * v;
        double u = g.uniform_pos();
        if (u < 1.0 - 0.0331 * x * x * x * x) return d * v;
        if (det_log(u) < 0.5 * x * x + d * (1.0 - v + det_log(v))) return d * v;
    }
}

}  // namespace

extern "C" int fpgm_generate_network(const fpgm_gen_spec *spec, uint8_t *out_columns,
                                     uint8_t *out_card, int32_t *out_parents) {
    if (!spec || !out_columns || !out_card) return FPGM_ERR_INVALID;
    const int n = spec->n_nodes;
    const int64_t S = spec->n_samples;
    const int maxin = spec->max_indegree;
    if (n < 2 || n > 65535 || S < 1 || maxin < 0 || maxin > 16) return FPGM_ERR_INVALID;
    if (spec->card_min < 2 || spec->card_max < spec->card_min || spec->card_max > 255) return FPGM_ERR_INVALID;
    if (spec->tail_frac > 0.0 && (spec->tail_min < 2 || spec->tail_max < spec->tail_min || spec->tail_max > 255))
        return FPGM_ERR_INVALID;
    if (!(spec->dirichlet_alpha > 0.0)) return FPGM_ERR_INVALID;

    Rng g(spec->seed);
    // random topological order
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    for (int i = n - 1; i > 0; --i) std::swap(order[i], order[g.below((uint32_t)i + 1)]);
    // cardinalities
    std::vector<int> card(n);
    for (int v = 0; v < n; ++v) {
        if (spec->tail_frac > 0.0 && g.uniform() < spec->tail_frac)
            card[v] = spec->tail_min + (int)g.below((uint32_t)(spec->tail_max - spec->tail_min + 1));
        else
            card[v] = spec->card_min + (int)g.below((uint32_t)(spec->card_max - spec->card_min + 1));
    }
    // edges
    int64_t E = spec->n_edges > 0 ? spec->n_edges : (int64_t)std::floor(spec->avg_indegree * n + 0.5);
    std::vector<std::vector<int>> parents(n);
    int64_t added = 0, attempts = 0, max_attempts = 1000 * (E + 1);
    while (added < E && attempts < max_attempts) {
        ++attempts;
        uint32_t p = 1 + g.below((uint32_t)n - 1);
        int child = order[p];
        if ((int)parents[child].size() >= maxin) continue;
        int par = order[g.below(p)];
        if (std::find(parents[child].begin(), parents[child].end(), par) != parents[child].end()) continue;
        parents[child].push_back(par);
        ++added;
    }
    for (int v = 0; v < n; ++v) std::sort(parents[v].begin(), parents[v].end());
    // CPTs as cumulative 2^32-scaled thresholds, row-major [config][value]
    std::vector<std::vector<uint64_t>> cum(n);
    std::vector<std::vector<int64_t>> radix(n);
    for (int v = 0; v < n; ++v) {
        int64_t configs = 1;
        radix[v].assign(parents[v].size(), 1);
        for (int k = (int)parents[v].size() - 1; k >= 0; --k) {
            radix[v][k] = configs;
            configs *= card[parents[v][k]];
        }
        if (configs > (int64_t)1 << 26) return FPGM_ERR_INVALID;
        int c = card[v];
        cum[v].resize((size_t)configs * c);
        std::vector<double> w(c);
        for (int64_t r = 0; r < configs; ++r) {
            double tot = 0.0;
            for (int k = 0; k < c; ++k) { w[k] = det_gamma(g, spec->dirichlet_alpha); tot += w[k]; }
            double acc = 0.0;
            for (int k = 0; k < c; ++k) {
                acc += w[k];
                double f = tot > 0.0 ? acc / tot : (double)(k + 1) / c;
                uint64_t t = (uint64_t)std::floor(f * 4294967296.0);
                if (k == c - 1 || t > 4294967296ull) t = 4294967296ull;
                cum[v][(size_t)r * c + k] = t;
            }
        }
    }
    // forward sampling, one stream per sample
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < S; ++s) {
        Rng gs(spec->seed ^ (0xd1b54a32d192ed03ull * (uint64_t)(s + 1)));
        std::vector<int> val(n);
        for (int p = 0; p < n; ++p) {
            int v = order[p];
            int64_t row = 0;
            for (size_t k = 0; k < parents[v].size(); ++k) row += val[parents[v][k]] * radix[v][k];
            uint64_t u = gs.next() >> 32;
            const uint64_t *cr = &cum[v][(size_t)row * card[v]];
            int x = 0;
            while (x < card[v] - 1 && u >= cr[x]) ++x;
            val[v] = x;
            out_columns[(size_t)v * S + s] = (uint8_t)x;
        }
    }
    for (int v = 0; v < n; ++v) out_card[v] = (uint8_t)card[v];
    if (out_parents) {
        for (int v = 0; v < n; ++v)
            for (int k = 0; k < maxin; ++k)
                out_parents[v * maxin + k] = k < (int)parents[v].size() ? parents[v][k] : -1;
    }
    return FPGM_OK;
}

extern "C" int fpgm_write_csv(const char *path, const uint8_t *columns, int n_vars, int64_t n_samples,
                              const char *name_prefix) {
    if (!path || !columns || n_vars < 1 || n_samples < 1) return FPGM_ERR_INVALID;
    FILE *f = std::fopen(path, "w");
    if (!f) return FPGM_ERR_IO;
    const char *pre = name_prefix ? name_prefix : "V";
    for (int v = 0; v < n_vars; ++v) std::fprintf(f, v ? ",%s%d" : "%s%d", pre, v);
    std::fputc('\n', f);
    std::vector<char> line((size_t)n_vars * 4 + 2);
    for (int64_t s = 0; s < n_samples; ++s) {
        char *p = line.data();
        for (int v = 0; v < n_vars; ++v) {
            unsigned x = columns[(size_t)v * n_samples + s];
            if (v) *p++ = ',';
            if (x >= 100) { *p++ = (char)('0' + x / 100); x %= 100; *p++ = (char)('0' + x / 10); *p++ = (char)('0' + x % 10); }
            else if (x >= 10) { *p++ = (char)('0' + x / 10); *p++ = (char)('0' + x % 10); }
            else *p++ = (char)('0' + x);
        }
        *p++ = '\n';
        std::fwrite(line.data(), 1, (size_t)(p - line.data()), f);
    }
    return std::fclose(f) == 0 ? FPGM_OK : FPGM_ERR_IO;
}
