// Host-side problem assembly for the box-QP engine: full symmetric CSR from the
// reference's lower-triangle triplets, the convexity gate and the Gershgorin bound.
//
//  - CSR: same result as mirroring into per-row lists (02-software/solver/src/accelerated_qp.cpp:20-24)
//    and merging each row with a std::map (include/sparse_matrix.hpp:10-17), but built by
//    counting sort in O(nnz) instead of O(nnz log deg) map inserts.  Rows are filled in triplet
//    order and then stable-sorted by column, so duplicates are summed in input order.
//  - check_convex_hessian (src/qp_admm.cpp:30-62): diagonal dominance with a non-negative
//    diagonal proves PSD in O(nnz); otherwise the same congruence-scaled sparse LDL^T with
//    complete fill and a 4M fill budget decides.
#include "boxqp.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <utility>
#include <vector>

extern "C" {

int bqp_csr_from_lower(int64_t n, int64_t nh, const int64_t* hrow, const int64_t* hcol, const double* hval,
                       double sign, int32_t* rowptr, int32_t* col, double* val, int64_t* nnz_out) {
    if (n <= 0 || nh < 0 || !rowptr || (nh && (!hrow || !hcol || !hval || !col || !val))) return BQP_ERR_INVALID;
    try {
        std::vector<int64_t> count(static_cast<size_t>(n) + 1, 0);
        for (int64_t k = 0; k < nh; ++k) {
            if (hrow[k] < 0 || hrow[k] >= n || hcol[k] < 0 || hcol[k] >= n) return BQP_ERR_INVALID;
            count[hrow[k] + 1]++;
            if (hrow[k] != hcol[k]) count[hcol[k] + 1]++;
        }
        for (int64_t i = 0; i < n; ++i) count[i + 1] += count[i];
        const int64_t total = count[n];
        std::vector<std::pair<int64_t, double>> e(static_cast<size_t>(total));
        std::vector<int64_t> fill(count.begin(), count.end() - 1);
        for (int64_t k = 0; k < nh; ++k) {
            double v = sign * hval[k];
            e[fill[hrow[k]]++] = {hcol[k], v};
            if (hrow[k] != hcol[k]) e[fill[hcol[k]]++] = {hrow[k], v};
        }
        int64_t nnz = 0;
        rowptr[0] = 0;
        for (int64_t i = 0; i < n; ++i) {
            auto b = e.begin() + count[i], t = e.begin() + count[i + 1];
            if (t - b > 1)
                std::stable_sort(b, t, [](const std::pair<int64_t, double>& x, const std::pair<int64_t, double>& y) {
                    return x.first < y.first;
                });
            for (auto k = b; k != t;) {
                int64_t c = k->first;
                double s = 0.0;
                while (k != t && k->first == c) { s += k->second; ++k; }
                if (s != 0) {
                    col[nnz] = static_cast<int32_t>(c);
                    val[nnz] = s;
                    ++nnz;
                }
            }
            if (nnz > 2000000000LL) return BQP_ERR_INVALID;
            rowptr[i + 1] = static_cast<int32_t>(nnz);
        }
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

}  // extern "C"
