// Secondary lookup keys (the reference's useSecondaryLookup: two active planes for the implicit
// arrangement, src/implicit_arrangement.cpp:276-283; three materials for the material interface,
// src/material_interface.cpp:320-327).
//
// The canonical record of a tet depends only on the combinatorial type of its arrangement, which is
// fixed by the oriented matroid of the rows involved (tet faces e_0..e_3 and the function rows):
//   two planes P, Q:       signs of P and Q at the four corners and of the six 2x2 minors
//                          P_i Q_j - P_j Q_i (the 4x4 determinants {e_a, e_b, P, Q});
//   three materials m0..2: signs of m_b - m_a at the four corners (three pairs) and of the six 3x3
//                          minors det[[m0_c, m0_d, 1], [m1_c, m1_d, 1], [m2_c, m2_d, 1]].
// Each sign is exact (filtered, with an exact fallback).  The key is the base-3 number of the signs
// (14 or 18 digits, below 2^29).  Only tets whose rows are pairwise distinct groups use a key: the
// record then carries the labels 4, 5 (and 6) and nothing specific to the tet.
#pragma once
#include "exact.cuh"

namespace ria {

// exact sign of a*d - b*c, or 2 if the exact evaluation overflowed (inputs within key_range: a
// product is zero only when a factor is, so two zero products decide the sign without the exact path)
RIA_HD int sign_det2(double a, double b, double c, double d) {
    const double x = a * d, y = b * c;
    if (x == 0.0 && y == 0.0) return 0;
    const double v = x - y;
    const double bound = 4.0 * kU * (fabs(x) + fabs(y));
    if (v > bound) return 1;
    if (v < -bound) return -1;
    double M[4] = {a, b, c, d};
    return det_sign_exact(M, 2);
}

RIA_HD int sign_det3(const double* M) {
    double perm = 0.0;
    const double v = det_fp(M, 3, perm);
    const double bound = det_err_coeff(3) * perm;
    if (v > bound) return 1;
    if (v < -bound) return -1;
    double W[9];
    for (int i = 0; i < 9; ++i) W[i] = M[i];
    return det_sign_exact(W, 3);
}

RIA_HD int sign_of(double x) { return (x > 0.0) - (x < 0.0); }

// Keys are only formed for values in [1e-70, 1e70] (or zero): no product of up to three of them
// leaves the normal FP64 range, so the filters' relative bounds and the exact fallback hold.
RIA_HD bool key_range(const double* v, int n) {
    for (int i = 0; i < n; ++i) {
        const double a = fabs(v[i]);
        if (a != 0.0 && (a < 1e-70 || a > 1e70)) return false;
    }
    return true;
}

// two planes P = rows[0..3], Q = rows[4..7]
RIA_HD bool ia_key2(const double* rows, uint32_t& key) {
    if (!key_range(rows, 8)) return false;
    const double* P = rows;
    const double* Q = rows + 4;
    uint32_t k = 0;
    for (int c = 0; c < 4; ++c) k = 3 * k + (uint32_t)(sign_of(P[c]) + 1);
    for (int c = 0; c < 4; ++c) k = 3 * k + (uint32_t)(sign_of(Q[c]) + 1);
    for (int i = 0; i < 4; ++i)
        for (int j = i + 1; j < 4; ++j) {
            const int s = sign_det2(P[i], P[j], Q[i], Q[j]);
            if (s == 2) return false;
            k = 3 * k + (uint32_t)(s + 1);
        }
    key = k;
    return true;
}

// three planes P, Q, R = rows[0..3], rows[4..7], rows[8..11]: their signs at the corners, the 2x2
// minors of each pair on each corner pair, and the 3x3 minors of (P, Q, R) on each corner triple
// (the 4x4 determinants {e_a, P, Q, R}); 34 base-3 digits
RIA_HD bool ia_key3(const double* rows, uint64_t& key) {
    if (!key_range(rows, 12)) return false;
    uint64_t k = 0;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) k = 3 * k + (uint64_t)(sign_of(rows[4 * r + c]) + 1);
    const int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
    for (int p = 0; p < 3; ++p)
        for (int i = 0; i < 4; ++i)
            for (int j = i + 1; j < 4; ++j) {
                const double* X = rows + 4 * pa[p];
                const double* Y = rows + 4 * pb[p];
                const int s = sign_det2(X[i], X[j], Y[i], Y[j]);
                if (s == 2) return false;
                k = 3 * k + (uint64_t)(s + 1);
            }
    for (int skip = 0; skip < 4; ++skip) {
        double M[9];
        for (int r = 0; r < 3; ++r) {
            int cc = 0;
            for (int c = 0; c < 4; ++c)
                if (c != skip) M[3 * r + cc++] = rows[4 * r + c];
        }
        const int s = sign_det3(M);
        if (s == 2) return false;
        k = 3 * k + (uint64_t)(s + 1);
    }
    key = k;
    return true;
}

// three materials, rows m[0..3], m[4..7], m[8..11]
RIA_HD bool mi_key3(const double* m, uint32_t& key) {
    if (!key_range(m, 12)) return false;
    uint32_t k = 0;
    const int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
    for (int p = 0; p < 3; ++p)
        for (int c = 0; c < 4; ++c) {
            const double x = m[4 * pb[p] + c], y = m[4 * pa[p] + c];
            k = 3 * k + (uint32_t)((x > y) - (x < y) + 1);
        }
    for (int c = 0; c < 4; ++c)
        for (int d = c + 1; d < 4; ++d) {
            double M[9];
            for (int r = 0; r < 3; ++r) {
                M[3 * r] = m[4 * r + c];
                M[3 * r + 1] = m[4 * r + d];
                M[3 * r + 2] = 1.0;
            }
            const int s = sign_det3(M);
            if (s == 2) return false;
            k = 3 * k + (uint32_t)(s + 1);
        }
    key = k;
    return true;
}

// three materials pairwise different (no grouping of identical materials)
RIA_HD bool mi_distinct3(const double* m) {
    for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 3; ++b) {
            bool same = true;
            for (int c = 0; c < 4; ++c) same = same && m[4 * a + c] == m[4 * b + c];
            if (same) return false;
        }
    return true;
}

}  // namespace ria
