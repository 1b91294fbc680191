// Planted box-QP generator for the synthetic workloads.
//
// Every draw comes from one splitmix64 stream per instance, in a fixed order:
// graph edges -> diagonal -> per-variable bounds -> planted pattern and x* -> duals z.
// Q is PSD and diagonally dominant by construction (weighted Laplacian + positive
// diagonal, or grid Laplacian + shift), the planted duals are strictly complementary
// (|z_j| >= dual_lo at every active bound), and c = -Q x* + z, so x* is the unique
// optimum.  Host arithmetic is compiled with -ffp-contract=off and the objective is
// accumulated in double-double, so every host produces the same bits.
//
// Family 2 restates the reference's own published-number harness
// (02-software/solver/src/scale_benchmark.cpp:13-18): tridiagonal Q (2.02 / -1), bounds
// [0, 3], x*_j = 0.5 + (s mod 10001)/10000 from the 32-bit LCG s <- 1664525 s + 1013904223
// started at 26119, c = -Q x*, known objective -sum_j x*_j (Q x*)_j / 2.
#include "boxqp.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

struct bqp_planted {
    int64_t n = 0;
    std::vector<int32_t> rowptr, col;
    std::vector<double> val, c, lower, upper, xstar, z;
    double fstar = 0;
};

extern "C" uint64_t bqp_splitmix64(uint64_t* state) {
    uint64_t z = (*state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

namespace {
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() { return bqp_splitmix64(&s); }
    // U[0,1) with 53 random bits.
    double u01() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }
    double uniform(double a, double b) { return a + (b - a) * u01(); }
    // Uniform integer in [0, n) by multiply-shift.
    int64_t index(int64_t n) {
        unsigned __int128 p = static_cast<unsigned __int128>(next()) * static_cast<uint64_t>(n);
        return static_cast<int64_t>(p >> 64);
    }
};

// Double-double accumulation (Knuth TwoSum, Dekker TwoProduct via Veltkamp split);
// written without FMA so that it rounds the same on every host.
struct DD {
    double hi = 0, lo = 0;
    static void two_sum(double a, double b, double& s, double& e) {
        s = a + b;
        double bb = s - a;
        e = (a - (s - bb)) + (b - bb);
    }
    static void split(double a, double& h, double& l) {
        const double f = 134217729.0;  // 2^27 + 1
        double t = f * a;
        h = t - (t - a);
        l = a - h;
    }
    static void two_prod(double a, double b, double& p, double& e) {
        p = a * b;
        double ah, al, bh, bl;
        split(a, ah, al);
        split(b, bh, bl);
        e = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
    }
    void add(double a) {
        double s, e;
        two_sum(hi, a, s, e);
        e += lo;
        two_sum(s, e, hi, lo);
    }
    void add_prod(double a, double b) {
        double p, e;
        two_prod(a, b, p, e);
        add(p);
        add(e);
    }
    double value() const { return hi + lo; }
};

struct Edge {
    uint64_t key;  // a * n + b with a < b
    uint32_t seq;
    double w;
};

void plant(const bqp_planted_spec& s, Rng& rng, bqp_planted& p) {
    const int64_t n = p.n;
    p.lower.resize(n);
    p.upper.resize(n);
    p.xstar.resize(n);
    p.z.resize(n);
    if (s.bounds_mode == 1) {
        for (int64_t i = 0; i < n; ++i) {
            p.lower[i] = rng.uniform(-1.0, -0.5);
            p.upper[i] = rng.uniform(0.5, 1.0);
        }
    } else {
        std::fill(p.lower.begin(), p.lower.end(), s.lower);
        std::fill(p.upper.begin(), p.upper.end(), s.upper);
    }
    std::vector<int8_t> pattern(n);
    for (int64_t i = 0; i < n; ++i) {
        double r = rng.u01();
        if (r < s.frac_lower) {
            pattern[i] = -1;
            p.xstar[i] = p.lower[i];
        } else if (r < s.frac_lower + s.frac_upper) {
            pattern[i] = 1;
            p.xstar[i] = p.upper[i];
        } else {
            pattern[i] = 0;
            p.xstar[i] = p.lower[i] + (p.upper[i] - p.lower[i]) * rng.uniform(s.interior_lo, s.interior_hi);
        }
    }
    for (int64_t i = 0; i < n; ++i) {
        if (pattern[i] < 0) p.z[i] = rng.uniform(s.dual_lo, s.dual_hi);
        else if (pattern[i] > 0) p.z[i] = -rng.uniform(s.dual_lo, s.dual_hi);
        else p.z[i] = 0.0;
    }
    // c = -Q x* + z, Q x* summed in CSR order; f* = sum_i x*_i (Qx*)_i / 2 + c_i x*_i.
    p.c.resize(n);
    DD f;
    for (int64_t i = 0; i < n; ++i) {
        double q = 0;
        for (int32_t k = p.rowptr[i]; k < p.rowptr[i + 1]; ++k) q += p.val[k] * p.xstar[p.col[k]];
        p.c[i] = -q + p.z[i];
        f.add_prod(0.5 * p.xstar[i], q);
        f.add_prod(p.c[i], p.xstar[i]);
    }
    p.fstar = f.value();
}

bool build_graph(const bqp_planted_spec& s, Rng& rng, bqp_planted& p) {
    const int64_t n = p.n;
    const int64_t m = static_cast<int64_t>(s.edges_per_vertex) * n;
    std::vector<Edge> edges;
    edges.reserve(static_cast<size_t>(m));
    for (int64_t e = 0; e < m; ++e) {
        int64_t a = rng.index(n), b = rng.index(n);
        double w = rng.uniform(s.weight_lo, s.weight_hi);
        if (a == b) continue;
        if (a > b) std::swap(a, b);
        edges.push_back({static_cast<uint64_t>(a) * static_cast<uint64_t>(n) + static_cast<uint64_t>(b),
                         static_cast<uint32_t>(e), w});
    }
    std::sort(edges.begin(), edges.end(), [](const Edge& x, const Edge& y) {
        return x.key != y.key ? x.key < y.key : x.seq < y.seq;
    });
    // Merge duplicate edges by summing weights in draw order.
    size_t out = 0;
    for (size_t k = 0; k < edges.size();) {
        Edge e = edges[k++];
        while (k < edges.size() && edges[k].key == e.key) e.w += edges[k++].w;
        edges[out++] = e;
    }
    edges.resize(out);
    std::vector<double> diag(n);
    for (int64_t i = 0; i < n; ++i) diag[i] = rng.uniform(s.diag_lo, s.diag_hi);
    std::vector<int32_t> count(n + 1, 0), low(n, 0);
    std::vector<double> degree(n, 0.0);
    for (const Edge& e : edges) {
        int64_t a = static_cast<int64_t>(e.key / static_cast<uint64_t>(n));
        int64_t b = static_cast<int64_t>(e.key % static_cast<uint64_t>(n));
        count[a + 1]++;
        count[b + 1]++;
        low[b]++;
        degree[a] += e.w;
        degree[b] += e.w;
    }
    p.rowptr.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        int64_t next = static_cast<int64_t>(p.rowptr[i]) + count[i + 1] + 1;
        if (next > 2000000000LL) return false;
        p.rowptr[i + 1] = static_cast<int32_t>(next);
    }
    const int64_t nnz = p.rowptr[n];
    p.col.resize(nnz);
    p.val.resize(nnz);
    std::vector<int32_t> lowpos(n), highpos(n);
    for (int64_t i = 0; i < n; ++i) {
        int32_t d = p.rowptr[i] + low[i];
        p.col[d] = static_cast<int32_t>(i);
        p.val[d] = degree[i] + diag[i];
        lowpos[i] = p.rowptr[i];
        highpos[i] = d + 1;
    }
    // Edges are sorted by (a, b): row b receives its lower entries in ascending a, row a
    // its upper entries in ascending b, so every row comes out sorted by column.
    for (const Edge& e : edges) {
        int64_t a = static_cast<int64_t>(e.key / static_cast<uint64_t>(n));
        int64_t b = static_cast<int64_t>(e.key % static_cast<uint64_t>(n));
        p.col[lowpos[b]] = static_cast<int32_t>(a);
        p.val[lowpos[b]++] = -e.w;
        p.col[highpos[a]] = static_cast<int32_t>(b);
        p.val[highpos[a]++] = -e.w;
    }
    return true;
}

void build_grid(const bqp_planted_spec& s, bqp_planted& p) {
    const int64_t side = s.grid_side, n = side * side;
    p.rowptr.assign(n + 1, 0);
    p.col.clear();
    p.val.clear();
    p.col.reserve(5 * n);
    p.val.reserve(5 * n);
    for (int64_t r = 0; r < side; ++r) {
        for (int64_t q = 0; q < side; ++q) {
            int64_t i = r * side + q;
            if (r > 0) { p.col.push_back(static_cast<int32_t>(i - side)); p.val.push_back(-1.0); }
            if (q > 0) { p.col.push_back(static_cast<int32_t>(i - 1)); p.val.push_back(-1.0); }
            p.col.push_back(static_cast<int32_t>(i));
            p.val.push_back(4.0 + s.shift);
            if (q + 1 < side) { p.col.push_back(static_cast<int32_t>(i + 1)); p.val.push_back(-1.0); }
            if (r + 1 < side) { p.col.push_back(static_cast<int32_t>(i + side)); p.val.push_back(-1.0); }
            p.rowptr[i + 1] = static_cast<int32_t>(p.col.size());
        }
    }
}

void build_tridiagonal(const bqp_planted_spec& s, bqp_planted& p) {
    const int64_t n = p.n;
    p.rowptr.assign(n + 1, 0);
    p.col.clear();
    p.val.clear();
    for (int64_t i = 0; i < n; ++i) {
        if (i > 0) { p.col.push_back(static_cast<int32_t>(i - 1)); p.val.push_back(-1.0); }
        p.col.push_back(static_cast<int32_t>(i));
        p.val.push_back(2.02);
        if (i + 1 < n) { p.col.push_back(static_cast<int32_t>(i + 1)); p.val.push_back(-1.0); }
        p.rowptr[i + 1] = static_cast<int32_t>(p.col.size());
    }
    p.lower.assign(n, 0.0);
    p.upper.assign(n, 3.0);
    p.xstar.resize(n);
    p.z.assign(n, 0.0);
    p.c.resize(n);
    uint32_t state = static_cast<uint32_t>(s.seed);
    for (int64_t j = 0; j < n; ++j) {
        state = 1664525u * state + 1013904223u;
        p.xstar[j] = .5 + double(state % 10001) / 10000;
    }
    DD f;
    for (int64_t j = 0; j < n; ++j) {
        double hx = 2.02 * p.xstar[j] - (j ? p.xstar[j - 1] : 0) - (j + 1 < n ? p.xstar[j + 1] : 0);
        p.c[j] = -hx;
        f.add_prod(-0.5 * p.xstar[j], hx);
    }
    p.fstar = f.value();
}
}  // namespace

extern "C" {

int bqp_planted_preset(int32_t preset, uint64_t seed, int64_t index, int64_t n_override, bqp_planted_spec* spec) {
    if (!spec) return BQP_ERR_INVALID;
    bqp_planted_spec s;
    std::memset(&s, 0, sizeof(s));
    s.seed = seed;
    s.diag_lo = 0.5;
    s.diag_hi = 2.0;
    s.weight_lo = 0.1;
    s.weight_hi = 1.0;
    s.dual_lo = 0.1;
    s.dual_hi = 1.0;
    switch (preset) {
    case 0:  // n = 10,000 random graph, 5 edges/vertex, [0, 1], 30/30/40, interior U(0.1, 0.9)
        s.family = 0; s.n = 10000; s.edges_per_vertex = 5; s.lower = 0; s.upper = 1;
        s.frac_lower = 0.3; s.frac_upper = 0.3; s.interior_lo = 0.1; s.interior_hi = 0.9;
        break;
    case 1:  // n = 1,000,000 random graph, 7 edges/vertex, [-1, 1], 25/25/50, interior U(-0.9, 0.9)
        s.family = 0; s.n = 1000000; s.edges_per_vertex = 7; s.lower = -1; s.upper = 1;
        s.frac_lower = 0.25; s.frac_upper = 0.25; s.interior_lo = 0.05; s.interior_hi = 0.95;
        break;
    case 2:  // 1024 x 1024 grid Laplacian + 1e-3 I, l ~ U[-1,-.5], u ~ U[.5,1], 20/20/60
        s.family = 1; s.grid_side = 1024; s.n = 1024 * 1024; s.shift = 1e-3; s.bounds_mode = 1;
        s.frac_lower = 0.2; s.frac_upper = 0.2; s.interior_lo = 0.05; s.interior_hi = 0.95;
        break;
    case 3: {  // instance `index` of the uneven batch: n log-uniform [64, 16384], 2..6 edges/vertex
        uint64_t st = seed ^ (0xD1B54A32D192ED03ULL * static_cast<uint64_t>(index + 1));
        uint64_t inst_seed = bqp_splitmix64(&st);
        Rng r(inst_seed);
        double ln = r.uniform(std::log(64.0), std::log(16384.0));
        s.family = 0;
        s.n = static_cast<int64_t>(std::floor(std::exp(ln)));
        s.edges_per_vertex = 2 + static_cast<int32_t>(r.index(5));
        s.lower = 0;
        s.upper = r.uniform(0.5, 2.0);
        s.seed = r.next();
        s.frac_lower = 0.3; s.frac_upper = 0.3; s.interior_lo = 0.1; s.interior_hi = 0.9;
        break;
    }
    case 4: {  // request `index` of the serving stream: n log-uniform [1000, 200000], 5 edges/vertex
        uint64_t st = seed ^ (0x9FB21C651E98DF25ULL * static_cast<uint64_t>(index + 1));
        uint64_t req_seed = bqp_splitmix64(&st);
        Rng r(req_seed);
        double ln = r.uniform(std::log(1000.0), std::log(200000.0));
        s.family = 0;
        s.n = static_cast<int64_t>(std::floor(std::exp(ln)));
        s.edges_per_vertex = 5; s.lower = 0; s.upper = 1;
        s.seed = r.next();
        s.frac_lower = 0.3; s.frac_upper = 0.3; s.interior_lo = 0.1; s.interior_hi = 0.9;
        break;
    }
    case 5:  // the reference's tridiagonal scale family
        s.family = 2; s.n = 10000; s.seed = 26119; s.lower = 0; s.upper = 3;
        break;
    default:
        return BQP_ERR_INVALID;
    }
    if (n_override > 0) {
        if (s.family == 1) {
            int64_t side = static_cast<int64_t>(std::llround(std::sqrt(static_cast<double>(n_override))));
            if (side * side != n_override) return BQP_ERR_INVALID;
            s.grid_side = static_cast<int32_t>(side);
            s.n = n_override;
        } else {
            s.n = n_override;
        }
    }
    *spec = s;
    return BQP_OK;
}

bqp_planted* bqp_planted_create(const bqp_planted_spec* spec) {
    if (!spec) return nullptr;
    const bqp_planted_spec& s = *spec;
    bqp_planted* p = new (std::nothrow) bqp_planted;
    if (!p) return nullptr;
    try {
        if (s.family == 0) {
            if (s.n < 2 || s.n > 200000000LL || s.edges_per_vertex < 0) { delete p; return nullptr; }
            p->n = s.n;
            Rng rng(s.seed);
            if (!build_graph(s, rng, *p)) { delete p; return nullptr; }
            plant(s, rng, *p);
        } else if (s.family == 1) {
            if (s.grid_side < 2 || static_cast<int64_t>(s.grid_side) * s.grid_side > 200000000LL) { delete p; return nullptr; }
            p->n = static_cast<int64_t>(s.grid_side) * s.grid_side;
            Rng rng(s.seed);
            build_grid(s, *p);
            plant(s, rng, *p);
        } else if (s.family == 2) {
            if (s.n < 2 || s.n > 200000000LL) { delete p; return nullptr; }
            p->n = s.n;
            build_tridiagonal(s, *p);
        } else {
            delete p;
            return nullptr;
        }
    } catch (...) {
        delete p;
        return nullptr;
    }
    return p;
}

int bqp_planted_info(const bqp_planted* p, int64_t* n, int64_t* nnz, int64_t* nnz_lower, double* fstar) {
    if (!p) return BQP_ERR_INVALID;
    if (n) *n = p->n;
    if (nnz) *nnz = p->rowptr.empty() ? 0 : p->rowptr[p->n];
    if (nnz_lower) {
        int64_t diag = 0;
        for (int64_t i = 0; i < p->n; ++i)
            for (int32_t k = p->rowptr[i]; k < p->rowptr[i + 1]; ++k) if (p->col[k] == i) ++diag;
        *nnz_lower = (static_cast<int64_t>(p->rowptr[p->n]) + diag) / 2;
    }
    if (fstar) *fstar = p->fstar;
    return BQP_OK;
}

int bqp_planted_copy(const bqp_planted* p, int32_t* rowptr, int32_t* col, double* val, double* c,
                     double* lower, double* upper, double* xstar, double* z) {
    if (!p) return BQP_ERR_INVALID;
    const size_t n = static_cast<size_t>(p->n), nnz = static_cast<size_t>(p->rowptr[p->n]);
    if (rowptr) std::memcpy(rowptr, p->rowptr.data(), (n + 1) * sizeof(int32_t));
    if (col) std::memcpy(col, p->col.data(), nnz * sizeof(int32_t));
    if (val) std::memcpy(val, p->val.data(), nnz * sizeof(double));
    if (c) std::memcpy(c, p->c.data(), n * sizeof(double));
    if (lower) std::memcpy(lower, p->lower.data(), n * sizeof(double));
    if (upper) std::memcpy(upper, p->upper.data(), n * sizeof(double));
    if (xstar) std::memcpy(xstar, p->xstar.data(), n * sizeof(double));
    if (z) std::memcpy(z, p->z.data(), n * sizeof(double));
    return BQP_OK;
}

int bqp_planted_copy_lower(const bqp_planted* p, int64_t* hrow, int64_t* hcol, double* hval) {
    if (!p || !hrow || !hcol || !hval) return BQP_ERR_INVALID;
    int64_t t = 0;
    for (int64_t i = 0; i < p->n; ++i) {
        for (int32_t k = p->rowptr[i]; k < p->rowptr[i + 1]; ++k) {
            if (p->col[k] > i) break;
            hrow[t] = i;
            hcol[t] = p->col[k];
            hval[t] = p->val[k];
            ++t;
        }
    }
    return BQP_OK;
}

void bqp_planted_free(bqp_planted* p) { delete p; }

}  // extern "C"
