// Host-side problem assembly for the box-QP engine: full symmetric CSR from the
// reference's lower-triangle triplets, the convexity gate and the Gershgorin bound.
//
//  - CSR: same result as mirroring into per-row lists (02-software/solver/src/accelerated_qp.cpp:20-24)
//    and merging each row with a std::map (include/sparse_matrix.hpp:10-17), but built by a
//    parallel stable bucket sort in O(nnz) instead of O(nnz log deg) map inserts.  Rows are
//    filled in triplet order and then stable-sorted by column, so duplicates are summed in input
//    order.
//  - check_convex_hessian (src/qp_admm.cpp:30-62): diagonal dominance with a non-negative
//    diagonal proves PSD in O(nnz); otherwise the same congruence-scaled sparse LDL^T with
//    complete fill and a 4M fill budget decides.
#include "boxqp.h"
#include "workers.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <numeric>
#include <thread>
#include <utility>
#include <vector>

extern "C" {

int bqp_csr_from_lower(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
                       double sign, int32_t* rowptr, int32_t* col, double* val, int64_t* nnz_out) {
    if (n <= 0 || nh < 0 || !rowptr || (nh && (!hrow || !hcol || !hval || !col || !val))) return BQP_ERR_INVALID;
    if (n > 2000000000LL) return BQP_ERR_INVALID;
    try {
        // Parallel stable bucket sort.  Triplets are cut into T consecutive chunks and rows into
        // row blocks; every (chunk, block) pair gets its own slot range, placed in chunk order
        // within each block, so a row's entries keep triplet order (duplicates are summed in
        // input order, as the per-row map merge does).  Each block then sorts its rows by column
        // (stable) and merges duplicates; a prefix over the blocks places the output.
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const int T = static_cast<int>(std::min<int64_t>(std::min<int64_t>(hw, 32), std::max<int64_t>(1, nh / 200000)));
        const int64_t rows_per_block = 256;
        const int64_t B = (n + rows_per_block - 1) / rows_per_block;
        std::vector<int64_t> cnt(static_cast<size_t>(T) * static_cast<size_t>(B), 0);
        std::vector<int> bad(static_cast<size_t>(T), 0);
        auto chunk = [&](int t, int64_t* k0, int64_t* k1) {
            *k0 = nh * t / T;
            *k1 = nh * (t + 1) / T;
        };
        auto parallel = [&](auto&& fn) {
            bqp::WorkerPool::get().run(T, [&](int64_t t) { fn(static_cast<int>(t)); });
        };
        parallel([&](int t) {
            int64_t k0, k1;
            chunk(t, &k0, &k1);
            int64_t* c = cnt.data() + static_cast<size_t>(t) * static_cast<size_t>(B);
            for (int64_t k = k0; k < k1; ++k) {
                const int64_t i = hrow[k], j = hcol[k];
                if (i < 0 || i >= n || j < 0 || j >= n) {
                    bad[t] = 1;
                    return;
                }
                c[i / rows_per_block]++;
                if (i != j) c[j / rows_per_block]++;
            }
        });
        for (int t = 0; t < T; ++t) if (bad[t]) return BQP_ERR_INVALID;
        // slot ranges: block-major, chunk order inside a block
        std::vector<int64_t> block_start(static_cast<size_t>(B) + 1, 0);
        int64_t run = 0;
        for (int64_t bl = 0; bl < B; ++bl) {
            block_start[bl] = run;
            for (int t = 0; t < T; ++t) {
                int64_t& c = cnt[static_cast<size_t>(t) * static_cast<size_t>(B) + bl];
                const int64_t here = c;
                c = run;
                run += here;
            }
        }
        block_start[B] = run;
        struct Entry {
            int32_t row, col;
            double val;
        };
        std::unique_ptr<Entry[]> e(new Entry[static_cast<size_t>(std::max<int64_t>(run, 1))]);
        parallel([&](int t) {
            int64_t k0, k1;
            chunk(t, &k0, &k1);
            int64_t* pos = cnt.data() + static_cast<size_t>(t) * static_cast<size_t>(B);
            for (int64_t k = k0; k < k1; ++k) {
                const int32_t i = static_cast<int32_t>(hrow[k]), j = static_cast<int32_t>(hcol[k]);
                const double v = sign * hval[k];
                e[pos[i / rows_per_block]++] = Entry{i, j, v};
                if (i != j) e[pos[j / rows_per_block]++] = Entry{j, i, v};
            }
        });
        // per block: stable counting sort by row, stable sort by column, merge duplicates, drop
        // zeros; the merged entries are written back at the start of the block's range
        std::vector<int64_t> block_nnz(static_cast<size_t>(B), 0);
        std::vector<int32_t> row_nnz(static_cast<size_t>(n), 0);
        const int64_t blocks_per_task = (B + T - 1) / T;
        parallel([&](int t) {
            std::vector<Entry> tmp;
            std::vector<int64_t> rstart(static_cast<size_t>(rows_per_block) + 1);
            for (int64_t bl = t * blocks_per_task; bl < std::min<int64_t>(B, (t + 1) * blocks_per_task); ++bl) {
                const int64_t s0 = block_start[bl], s1 = block_start[bl + 1];
                const int64_t r0 = bl * rows_per_block, r1 = std::min<int64_t>(n, r0 + rows_per_block);
                std::fill(rstart.begin(), rstart.end(), 0);
                for (int64_t k = s0; k < s1; ++k) rstart[e[k].row - r0 + 1]++;
                for (int64_t r = 0; r < r1 - r0; ++r) rstart[r + 1] += rstart[r];
                tmp.resize(static_cast<size_t>(s1 - s0));
                std::vector<int64_t> fill(rstart.begin(), rstart.end() - 1);
                for (int64_t k = s0; k < s1; ++k) tmp[fill[e[k].row - r0]++] = e[k];
                int64_t out = s0;
                for (int64_t r = 0; r < r1 - r0; ++r) {
                    Entry* b = tmp.data() + rstart[r];
                    Entry* end = tmp.data() + rstart[r + 1];
                    if (end - b > 64) {
                        std::stable_sort(b, end, [](const Entry& x, const Entry& y) { return x.col < y.col; });
                    } else {
                        for (Entry* k = b + 1; k < end; ++k) {
                            const Entry item = *k;
                            Entry* m = k;
                            while (m != b && (m - 1)->col > item.col) {
                                *m = *(m - 1);
                                --m;
                            }
                            *m = item;
                        }
                    }
                    const int64_t row_out0 = out;
                    for (Entry* k = b; k != end;) {
                        const int32_t c = k->col;
                        double sum = 0.0;
                        while (k != end && k->col == c) {
                            sum += k->val;
                            ++k;
                        }
                        if (sum != 0) e[out++] = Entry{static_cast<int32_t>(r0 + r), c, sum};
                    }
                    row_nnz[r0 + r] = static_cast<int32_t>(out - row_out0);
                }
                block_nnz[bl] = out - s0;
            }
        });
        std::vector<int64_t> block_out(static_cast<size_t>(B) + 1, 0);
        for (int64_t bl = 0; bl < B; ++bl) block_out[bl + 1] = block_out[bl] + block_nnz[bl];
        const int64_t nnz = block_out[B];
        if (nnz > 2000000000LL) return BQP_ERR_INVALID;
        parallel([&](int t) {
            for (int64_t bl = t * blocks_per_task; bl < std::min<int64_t>(B, (t + 1) * blocks_per_task); ++bl) {
                const int64_t r0 = bl * rows_per_block, r1 = std::min<int64_t>(n, r0 + rows_per_block);
                int64_t o = block_out[bl];
                for (int64_t r = r0; r < r1; ++r) {
                    rowptr[r] = static_cast<int32_t>(o);
                    o += row_nnz[r];
                }
                const Entry* src = e.get() + block_start[bl];
                for (int64_t k = 0; k < block_nnz[bl]; ++k) {
                    col[block_out[bl] + k] = src[k].col;
                    val[block_out[bl] + k] = src[k].val;
                }
            }
        });
        rowptr[n] = static_cast<int32_t>(nnz);
        if (nnz_out) *nnz_out = nnz;
        return BQP_OK;
    } catch (...) {
        return BQP_ERR_NO_MEMORY;
    }
}

int bqp_check_convex(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
                     int32_t maximize) {
    if (n <= 0 || nh < 0) return -1;
    const double sign = maximize ? -1.0 : 1.0;
    try {
        std::vector<double> diagonal(static_cast<size_t>(n), 0.0), radius(static_cast<size_t>(n), 0.0);
        for (int64_t k = 0; k < nh; ++k) {
            if (hrow[k] < 0 || hrow[k] >= n || hcol[k] < 0 || hcol[k] >= n || !std::isfinite(hval[k])) return -1;
            if (hrow[k] == hcol[k]) diagonal[hrow[k]] += sign * hval[k];
            else {
                radius[hrow[k]] += std::abs(hval[k]);
                radius[hcol[k]] += std::abs(hval[k]);
            }
        }
        bool dominant = true;
        for (int64_t j = 0; j < n; ++j) {
            if (diagonal[j] < 0 || (diagonal[j] == 0 && radius[j] > 0)) return 0;
            if (diagonal[j] < radius[j]) dominant = false;
        }
        if (dominant) return 1;
        // column k holds entries (i, k), i >= k, scaled by 1/sqrt(d_i d_k)
        std::vector<std::map<int64_t, double>> column(static_cast<size_t>(n));
        for (int64_t k = 0; k < nh; ++k) {
            int64_t i = std::max(hrow[k], hcol[k]), j = std::min(hrow[k], hcol[k]);
            if (diagonal[i] > 0 && diagonal[j] > 0) column[j][i] += sign * hval[k] / std::sqrt(diagonal[i] * diagonal[j]);
        }
        int64_t fill = nh;
        std::vector<std::pair<int64_t, double>> below;
        for (int64_t k = 0; k < n; ++k) {
            auto found = column[k].find(k);
            double d = found != column[k].end() ? found->second : 0.0;
            if (d < -1e-12) return 0;
            below.clear();
            for (const auto& a : column[k]) if (a.first > k) below.push_back(a);
            if (d <= 1e-12) {
                for (const auto& a : below) if (std::abs(a.second) > 1e-10) return 0;
                continue;
            }
            for (size_t u = 0; u < below.size(); ++u) {
                for (size_t v = u; v < below.size(); ++v) {
                    int64_t i = below[u].first, j = below[v].first;
                    auto& target = column[i];
                    auto at = target.find(j);
                    if (at == target.end()) {
                        if (++fill > 4000000) return 0;
                        at = target.emplace(j, 0.0).first;
                    }
                    at->second -= below[u].second * below[v].second / d;
                }
            }
            column[k].clear();
        }
        return 1;
    } catch (...) {
        return -1;
    }
}

double bqp_gershgorin(int64_t n, const int32_t* rowptr, const double* val) {
    double lipschitz = 0;
    for (int64_t i = 0; i < n; ++i) {
        double sum = 0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) sum += std::abs(val[k]);
        lipschitz = std::max(lipschitz, sum);
    }
    return lipschitz;
}

double bqp_dot_ld(int64_t n, const double* a, const double* b) {
    long double s = 0;
    for (int64_t j = 0; j < n; ++j) s += static_cast<long double>(a[j]) * b[j];
    return static_cast<double>(s);
}

}  // extern "C"
