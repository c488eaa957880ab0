// synth.cpp — seeded synthetic rating matrices with the shapes of the reference's datasets.
//
// The reference trains on Netflix, MovieLens 10M and MovieLens-latest (config/*.ini, prepared
// offline by data/*/prepare_*.py); none of them is available here, so five seeded workloads with
// their shapes stand in:
//   1  1,000 x 500, 20,000 ratings, cells uniform without replacement, values
//      clip(round(3.5 + u.v + N(0, 0.8^2)), 1, 5) from planted rank-8 N(0, 0.3^2) factors;
//      90/10 split; f = 10, lambda = 0.05                                  (toy sets)
//   2  69,878 x 10,677, 10M ratings, row degrees lognormal (median 70, min 20), columns Zipf
//      s = 1.0, half-star values from planted rank-16 factors + N(0, 0.8^2); 90/10; f = 64
//                                                                           (MovieLens 10M)
//   3  480,189 x 17,770, 100M ratings, row degrees heavy-tailed (Lomax, min 1, mean ~209),
//      columns Zipf s = 1.1, integer values 1..5 with marginal {.05,.10,.28,.34,.23} by
//      thresholding planted rank-16 scores + noise; 1.4% test; f = 100, lambda = 0.048 (Netflix)
//   4  config 3 transposed (17,770 x 480,189); f = 128, lambda = 0.05
//   5  283,228 x 58,098, 27M ratings, lognormal rows, Zipf s = 1.0 columns, half-star; 90/10;
//      f = 128, lambda = 0.05                                             (MovieLens latest)
// Every row and column keeps at least one training rating.  Each row draws from its own
// counter-seeded stream, so the bytes depend on (config, seed, scale) only, not on the thread
// count or the machine.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <numeric>
#include <vector>

#include "../../include/als_gb300.h"
#include "internal.h"

namespace {

inline uint64_t splitmix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(splitmix(seed)) {}
    uint64_t next() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    double uniform_pos() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() {  // Box-Muller, one value per call (no cached state)
        double u1 = uniform_pos(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
    uint64_t below(uint64_t n) { return n ? next() % n : 0; }
};

inline uint64_t stream_seed(uint64_t seed, uint64_t tag, uint64_t idx) {
    return splitmix(seed ^ splitmix(tag * 0x100000001B3ull + idx));
}

enum RowModel { ROWS_UNIFORM_CELLS, ROWS_LOGNORMAL, ROWS_LOMAX };
enum ValueModel { VALUES_ROUND_1_5, VALUES_HALF_STAR, VALUES_MARGINAL_1_5 };

struct Spec {
    int64_t m, n, nnz;
    int32_t f;
    float lambda;
    double test_frac;
    RowModel rows;
    double row_a, row_b;  // lognormal: median, sigma; lomax: alpha, mean
    int64_t row_min;
    double col_zipf;      // 0 = uniform
    ValueModel values;
    int rank;
    double factor_sd;
    bool transpose;       // config 4 = config 3 transposed
};

bool spec_of(int config, Spec *s) {
    switch (config) {
    case 1: *s = {1000, 500, 20000, 10, 0.05f, 0.10, ROWS_UNIFORM_CELLS, 0, 0, 1, 0.0,
                  VALUES_ROUND_1_5, 8, 0.3, false}; return true;
    case 2: *s = {69878, 10677, 10000000, 64, 0.05f, 0.10, ROWS_LOGNORMAL, 70.0, 1.19, 20, 1.0,
                  VALUES_HALF_STAR, 16, 0.5, false}; return true;
    case 3: *s = {480189, 17770, 100000000, 100, 0.048f, 0.014, ROWS_LOMAX, 2.2, 209.0, 1, 1.1,
                  VALUES_MARGINAL_1_5, 16, 0.5, false}; return true;
    case 4: *s = {480189, 17770, 100000000, 128, 0.05f, 0.014, ROWS_LOMAX, 2.2, 209.0, 1, 1.1,
                  VALUES_MARGINAL_1_5, 16, 0.5, true}; return true;
    case 5: *s = {283228, 58098, 27000000, 128, 0.05f, 0.10, ROWS_LOGNORMAL, 30.0, 1.52, 1, 1.0,
                  VALUES_HALF_STAR, 16, 0.5, false}; return true;
    }
    return false;
}

struct Result {
    int config = 0;
    uint64_t seed = 0;
    double scale = 0;
    bool valid = false;
    int64_t m = 0, n = 0;
    std::vector<int32_t> ptr, col, trow, tcol;
    std::vector<float> val, tval;
};

std::mutex g_cache_mu;
Result g_cache;

float make_value(ValueModel vm, double score) {
    switch (vm) {
    case VALUES_ROUND_1_5: {
        double v = std::nearbyint(3.5 + score);
        return (float)std::min(5.0, std::max(1.0, v));
    }
    case VALUES_HALF_STAR: {
        double v = std::nearbyint((3.5 + score) * 2.0) / 2.0;
        return (float)std::min(5.0, std::max(0.5, v));
    }
    case VALUES_MARGINAL_1_5: {
        // thresholds at the normal quantiles of the cumulative marginal {.05,.15,.43,.77},
        // scaled by the score's standard deviation (planted rank-16 part 1.0, noise 0.8)
        const double sd = std::sqrt(1.0 + 0.64);
        const double t[4] = {-1.6448536 * sd, -1.0364334 * sd, -0.1763742 * sd, 0.7388468 * sd};
        int v = 1;
        for (int i = 0; i < 4; ++i) v += score > t[i];
        return (float)v;
    }
    }
    return 0.f;
}

// Degrees of all rows summing to exactly `nnz`, each in [dmin, dmax].
std::vector<int64_t> make_degrees(const Spec &sp, int64_t m, int64_t n, int64_t nnz,
                                  double scale, uint64_t seed) {
    std::vector<double> raw((size_t)m);
    const int64_t dmax = std::max<int64_t>(1, n / 2);
    const int64_t dmin = std::max<int64_t>(1, std::min<int64_t>(dmax, (int64_t)std::llround(
                                                                          sp.row_min * (scale < 1 ? scale : 1.0))));
#pragma omp parallel for schedule(static)
    for (int64_t u = 0; u < m; ++u) {
        Rng r(stream_seed(seed, 11, (uint64_t)u));
        if (sp.rows == ROWS_LOGNORMAL) {
            double med = sp.row_a * (scale < 1 ? scale : 1.0);
            raw[u] = med * std::exp(sp.row_b * r.normal());
        } else {  // Lomax: P(D > x) = (1 + x/q)^-alpha, mean q/(alpha-1), shifted to min 1
            double alpha = sp.row_a, q = (sp.row_b - 1.0) * (alpha - 1.0);
            raw[u] = 1.0 + q * (std::pow(1.0 - r.uniform(), -1.0 / alpha) - 1.0);
        }
    }
    std::vector<int64_t> d((size_t)m);
    double factor = 1.0;
    for (int iter = 0; iter < 40; ++iter) {
        int64_t total = 0;
        for (int64_t u = 0; u < m; ++u) {
            int64_t v = (int64_t)std::llround(raw[u] * factor);
            d[u] = std::min(dmax, std::max(dmin, v));
            total += d[u];
        }
        if (total == nnz) break;
        factor *= (double)nnz / (double)total;
    }
    int64_t total = 0;
    for (int64_t u = 0; u < m; ++u) total += d[u];
    // settle the remainder one rating at a time, cycling over rows in order
    for (int64_t u = 0; total != nnz; u = (u + 1) % m) {
        if (total < nnz && d[u] < dmax) { d[u]++; total++; }
        else if (total > nnz && d[u] > dmin) { d[u]--; total--; }
    }
    return d;
}

bool generate(int config, uint64_t seed, double scale, Result *res) {
    Spec sp;
    if (!spec_of(config, &sp)) return false;
    if (!(scale > 0.0) || scale > 1.0) return false;
    const int64_t m = std::max<int64_t>(16, (int64_t)std::llround(sp.m * scale));
    const int64_t n = std::max<int64_t>(16, (int64_t)std::llround(sp.n * scale));
    int64_t nnz = (int64_t)std::llround((double)sp.nnz * scale * scale);
    nnz = std::max<int64_t>(std::max(m, n) * 2, std::min<int64_t>(nnz, m * n / 3));
    const uint64_t gseed = splitmix(seed ^ ((uint64_t)(sp.transpose ? 3 : config) << 56));

    // planted factors
    const int R = sp.rank;
    std::vector<double> P((size_t)(m * R)), Q((size_t)(n * R));
#pragma omp parallel for schedule(static)
    for (int64_t u = 0; u < m; ++u) {
        Rng r(stream_seed(gseed, 21, (uint64_t)u));
        for (int k = 0; k < R; ++k) P[u * R + k] = sp.factor_sd * r.normal();
    }
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < n; ++c) {
        Rng r(stream_seed(gseed, 22, (uint64_t)c));
        for (int k = 0; k < R; ++k) Q[c * R + k] = sp.factor_sd * r.normal();
    }

    std::vector<int64_t> ptr((size_t)m + 1, 0);
    std::vector<int32_t> col;
    if (sp.rows == ROWS_UNIFORM_CELLS) {
        // nnz distinct cells uniformly: partial Fisher-Yates over the m*n cell ids
        Rng r(stream_seed(gseed, 31, 0));
        std::vector<int64_t> cells((size_t)(m * n));
        std::iota(cells.begin(), cells.end(), 0);
        for (int64_t i = 0; i < nnz; ++i) {
            int64_t j = i + (int64_t)r.below((uint64_t)(m * n - i));
            std::swap(cells[i], cells[j]);
        }
        std::sort(cells.begin(), cells.begin() + nnz);
        col.resize((size_t)nnz);
        for (int64_t i = 0; i < nnz; ++i) {
            ptr[cells[i] / n + 1]++;
            col[i] = (int32_t)(cells[i] % n);
        }
        for (int64_t u = 0; u < m; ++u) ptr[u + 1] += ptr[u];
    } else {
        std::vector<int64_t> deg = make_degrees(sp, m, n, nnz, scale, gseed);
        for (int64_t u = 0; u < m; ++u) ptr[u + 1] = ptr[u] + deg[u];
        col.resize((size_t)nnz);
        // column popularity: Zipf over ranks, ranks assigned by a seeded permutation
        std::vector<int64_t> rank_of((size_t)n);
        std::iota(rank_of.begin(), rank_of.end(), 0);
        {
            Rng r(stream_seed(gseed, 41, 0));
            for (int64_t i = n - 1; i > 0; --i)
                std::swap(rank_of[i], rank_of[(int64_t)r.below((uint64_t)(i + 1))]);
        }
        std::vector<double> w((size_t)n), cdf((size_t)n);
        double acc = 0.0;
        for (int64_t c = 0; c < n; ++c) {
            w[c] = std::pow((double)(rank_of[c] + 1), -sp.col_zipf);
            acc += w[c];
            cdf[c] = acc;
        }
        for (int64_t c = 0; c < n; ++c) cdf[c] /= acc;
#pragma omp parallel
        {
            std::vector<int32_t> table;
            std::vector<std::pair<double, int32_t>> keys;
#pragma omp for schedule(dynamic, 64)
            for (int64_t u = 0; u < m; ++u) {
                const int64_t d = ptr[u + 1] - ptr[u];
                int32_t *out = col.data() + ptr[u];
                Rng r(stream_seed(gseed, 51, (uint64_t)u));
                if (d * 16 <= n) {  // rejection with an open-addressing set
                    size_t cap = 16;
                    while (cap < (size_t)(4 * d)) cap <<= 1;
                    table.assign(cap, -1);
                    int64_t got = 0;
                    while (got < d) {
                        double x = r.uniform();
                        int64_t c = std::lower_bound(cdf.begin(), cdf.end(), x) - cdf.begin();
                        if (c >= n) c = n - 1;
                        size_t hsh = (size_t)splitmix((uint64_t)c) & (cap - 1);
                        while (table[hsh] != -1 && table[hsh] != (int32_t)c) hsh = (hsh + 1) & (cap - 1);
                        if (table[hsh] == -1) {
                            table[hsh] = (int32_t)c;
                            out[got++] = (int32_t)c;
                        }
                    }
                } else {  // weighted sampling without replacement by exponential keys
                    keys.resize((size_t)n);
                    for (int64_t c = 0; c < n; ++c)
                        keys[c] = {std::log(r.uniform_pos()) / w[c], (int32_t)c};
                    std::nth_element(keys.begin(), keys.begin() + d, keys.end(),
                                     [](const std::pair<double, int32_t> &a,
                                        const std::pair<double, int32_t> &b) {
                                         return a.first > b.first ||
                                                (a.first == b.first && a.second < b.second);
                                     });
                    for (int64_t i = 0; i < d; ++i) out[i] = keys[i].second;
                }
                std::sort(out, out + d);
            }
        }
    }

    // every column gets a rating: an unsampled column takes over one entry of a column that has
    // more than one, in the first row (scanning from a hashed start) that can give one up
    {
        std::vector<int64_t> cdeg((size_t)n, 0);
        for (int64_t k = 0; k < nnz; ++k) cdeg[col[k]]++;
        for (int64_t c = 0; c < n; ++c) {
            if (cdeg[c] > 0) continue;
            const int64_t start = (int64_t)(splitmix(gseed ^ (uint64_t)c) % (uint64_t)m);
            for (int64_t t = 0; t < m; ++t) {
                const int64_t u = (start + t) % m;
                int32_t *b = col.data() + ptr[u], *e = col.data() + ptr[u + 1];
                if (std::binary_search(b, e, (int32_t)c)) continue;
                int32_t *victim = nullptr;
                for (int32_t *q = b; q < e; ++q)
                    if (cdeg[*q] > 1 && (!victim || cdeg[*q] > cdeg[*victim])) victim = q;
                if (!victim) continue;
                cdeg[*victim]--;
                *victim = (int32_t)c;
                cdeg[c] = 1;
                std::sort(b, e);
                break;
            }
        }
    }

    // values and the train/test split
    std::vector<float> val((size_t)nnz);
    std::vector<uint8_t> is_test((size_t)nnz, 0);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t u = 0; u < m; ++u) {
        Rng r(stream_seed(gseed, 61, (uint64_t)u));
        for (int64_t k = ptr[u]; k < ptr[u + 1]; ++k) {
            const int64_t c = col[k];
            double s = 0.0;
            for (int q = 0; q < R; ++q) s += P[u * R + q] * Q[c * R + q];
            s += 0.8 * r.normal();
            val[k] = make_value(sp.values, s);
            is_test[k] = r.uniform() < sp.test_frac;
        }
    }
    // every row keeps a training rating
    for (int64_t u = 0; u < m; ++u) {
        bool any = false;
        for (int64_t k = ptr[u]; k < ptr[u + 1] && !any; ++k) any = !is_test[k];
        if (!any && ptr[u + 1] > ptr[u]) is_test[ptr[u]] = 0;
    }
    // every column keeps a training rating (its first test rating in row order goes back)
    {
        std::vector<int64_t> ctrain((size_t)n, 0);
        for (int64_t k = 0; k < nnz; ++k)
            if (!is_test[k]) ctrain[col[k]]++;
        for (int64_t k = 0; k < nnz; ++k)
            if (is_test[k] && ctrain[col[k]] == 0) {
                is_test[k] = 0;
                ctrain[col[k]] = 1;
            }
    }

    // emit train CSR + test COO (row-major)
    int64_t ntest = 0;
    for (int64_t k = 0; k < nnz; ++k) ntest += is_test[k];
    res->ptr.assign((size_t)m + 1, 0);
    res->col.resize((size_t)(nnz - ntest));
    res->val.resize((size_t)(nnz - ntest));
    res->trow.resize((size_t)ntest);
    res->tcol.resize((size_t)ntest);
    res->tval.resize((size_t)ntest);
    int64_t a = 0, b = 0;
    for (int64_t u = 0; u < m; ++u) {
        for (int64_t k = ptr[u]; k < ptr[u + 1]; ++k) {
            if (is_test[k]) {
                res->trow[b] = (int32_t)u;
                res->tcol[b] = col[k];
                res->tval[b] = val[k];
                ++b;
            } else {
                res->col[a] = col[k];
                res->val[a] = val[k];
                ++a;
            }
        }
        res->ptr[u + 1] = (int32_t)a;
    }
    res->m = m;
    res->n = n;

    if (sp.transpose) {  // config 4: rows <-> columns, both sets re-sorted row-major
        std::vector<int32_t> tp((size_t)n + 1, 0), ti((size_t)a);
        std::vector<float> tv((size_t)a);
        for (int64_t k = 0; k < a; ++k) tp[res->col[k] + 1]++;
        for (int64_t c = 0; c < n; ++c) tp[c + 1] += tp[c];
        std::vector<int32_t> cur(tp.begin(), tp.end() - 1);
        for (int64_t u = 0; u < m; ++u)
            for (int32_t k = res->ptr[u]; k < res->ptr[u + 1]; ++k) {
                int32_t p = cur[res->col[k]]++;
                ti[p] = (int32_t)u;
                tv[p] = res->val[k];
            }
        std::vector<int64_t> order((size_t)ntest);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) {
            return res->tcol[x] < res->tcol[y];
        });
        std::vector<int32_t> r2((size_t)ntest), c2((size_t)ntest);
        std::vector<float> v2((size_t)ntest);
        for (int64_t i = 0; i < ntest; ++i) {
            r2[i] = res->tcol[order[i]];
            c2[i] = res->trow[order[i]];
            v2[i] = res->tval[order[i]];
        }
        res->ptr.swap(tp);
        res->col.swap(ti);
        res->val.swap(tv);
        res->trow.swap(r2);
        res->tcol.swap(c2);
        res->tval.swap(v2);
        std::swap(res->m, res->n);
    }
    return true;
}

}  // namespace

extern "C" als_status als_synth_shape(int32_t config, int64_t *m, int64_t *n,
                                      int64_t *nnz_total, int32_t *f, float *lambda) {
    Spec sp;
    if (!spec_of(config, &sp))
        return als::set_global_error(ALS_ERR_INVALID_ARG, "config must be 1..5");
    if (m) *m = sp.transpose ? sp.n : sp.m;
    if (n) *n = sp.transpose ? sp.m : sp.n;
    if (nnz_total) *nnz_total = sp.nnz;
    if (f) *f = sp.f;
    if (lambda) *lambda = sp.lambda;
    return ALS_OK;
}

extern "C" als_status als_synth_generate(int32_t config, uint64_t seed, double scale, int64_t *m,
                                         int64_t *n, int64_t *nnz_train, int64_t *nnz_test,
                                         int32_t *row_ptrs, int32_t *col_idxs, float *vals,
                                         int32_t *test_rows, int32_t *test_cols,
                                         float *test_vals) {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    Result &r = g_cache;
    if (!(r.valid && r.config == config && r.seed == seed && r.scale == scale)) {
        r = Result();
        if (!generate(config, seed, scale, &r))
            return als::set_global_error(ALS_ERR_INVALID_ARG,
                                         "config must be 1..5 and scale in (0, 1]");
        r.config = config;
        r.seed = seed;
        r.scale = scale;
        r.valid = true;
    }
    if (m) *m = r.m;
    if (n) *n = r.n;
    if (nnz_train) *nnz_train = (int64_t)r.col.size();
    if (nnz_test) *nnz_test = (int64_t)r.trow.size();
    bool want = row_ptrs || col_idxs || vals || test_rows || test_cols || test_vals;
    if (!want) return ALS_OK;
    if (row_ptrs) std::memcpy(row_ptrs, r.ptr.data(), sizeof(int32_t) * r.ptr.size());
    if (col_idxs) std::memcpy(col_idxs, r.col.data(), sizeof(int32_t) * r.col.size());
    if (vals) std::memcpy(vals, r.val.data(), sizeof(float) * r.val.size());
    if (test_rows) std::memcpy(test_rows, r.trow.data(), sizeof(int32_t) * r.trow.size());
    if (test_cols) std::memcpy(test_cols, r.tcol.data(), sizeof(int32_t) * r.tcol.size());
    if (test_vals) std::memcpy(test_vals, r.tval.data(), sizeof(float) * r.tval.size());
    if (row_ptrs && col_idxs && vals && test_rows && test_cols && test_vals) r = Result();
    return ALS_OK;
}
