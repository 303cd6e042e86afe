// CPU oracle (test infrastructure only): exact sign predicates for the per-tet cut.
//
// The reference delegates its per-tet cut to the third-party library
// qnzhou/simplicial_arrangement (GIT_TAG main, unpinned; cmake/simplicial_arrangement.cmake:6-10),
// which is not vendored.  Its robustness rests on exact orientation predicates over FP64
// plane/material values.  This header restates that idea from the published method:
//   * a semi-static FP64 filter (value and a rigorous forward error bound), and
//   * an exact fallback with floating-point expansion arithmetic (J. R. Shewchuk,
//     "Adaptive Precision Floating-Point Arithmetic and Fast Robust Geometric Predicates",
//     Discrete & Computational Geometry 18, 1997: Two-Sum, Two-Product, Grow-Expansion).
// Only tests/, the smoke check and bench.py's CPU baseline use this code.
#pragma once
#include <cmath>
#include <cstdlib>
#include <cstdint>
#include <vector>

namespace oracle {

using Exp = std::vector<double>;  // nonoverlapping, increasing magnitude, zero-free

inline void two_sum(double a, double b, double& x, double& y) {
    x = a + b;
    double bv = x - a;
    double av = x - bv;
    double br = b - bv;
    double ar = a - av;
    y = ar + br;
}

inline void two_prod(double a, double b, double& x, double& y) {
    x = a * b;
    y = std::fma(a, b, -x);
}

// h = e + b (Grow-Expansion with zero elimination).
inline Exp grow(const Exp& e, double b) {
    Exp h;
    h.reserve(e.size() + 1);
    double q = b;
    for (double ei : e) {
        double qn, hh;
        two_sum(q, ei, qn, hh);
        q = qn;
        if (hh != 0.0) h.push_back(hh);
    }
    if (q != 0.0) h.push_back(q);
    return h;
}

inline Exp add(const Exp& e, const Exp& f) {
    Exp h = e;
    for (double fj : f) h = grow(h, fj);
    return h;
}

// e * b, summed component by component through Grow-Expansion (exact).
inline Exp scale(const Exp& e, double b) {
    Exp h;
    if (b == 0.0) return h;
    for (double ei : e) {
        double x, y;
        two_prod(ei, b, x, y);
        if (y != 0.0) h = grow(h, y);
        if (x != 0.0) h = grow(h, x);
    }
    return h;
}

inline int exp_sign(const Exp& e) {
    if (e.empty()) return 0;
    return e.back() > 0 ? 1 : -1;
}

// Exact determinant of an n x n row-major matrix (n <= 5) by Laplace expansion on row `row`
// over the columns in `cols`.
inline Exp det_exact_rec(const double* M, int n, int row, unsigned cols) {
    int rem = n - row;
    if (rem == 1) {
        for (int c = 0; c < n; ++c)
            if (cols & (1u << c)) {
                double v = M[row * n + c];
                return v == 0.0 ? Exp{} : Exp{v};
            }
        return Exp{};
    }
    if (rem == 2) {
        int c0 = -1, c1 = -1;
        for (int c = 0; c < n; ++c)
            if (cols & (1u << c)) {
                if (c0 < 0) c0 = c; else c1 = c;
            }
        double a = M[row * n + c0], b = M[row * n + c1];
        double c = M[(row + 1) * n + c0], d = M[(row + 1) * n + c1];
        double x1, y1, x2, y2;
        two_prod(a, d, x1, y1);
        two_prod(b, c, x2, y2);
        Exp r;
        if (y1 != 0.0) r = grow(r, y1);
        if (x1 != 0.0) r = grow(r, x1);
        if (y2 != 0.0) r = grow(r, -y2);
        if (x2 != 0.0) r = grow(r, -x2);
        return r;
    }
    Exp acc;
    int idx = 0;
    for (int c = 0; c < n; ++c) {
        if (!(cols & (1u << c))) continue;
        double v = M[row * n + c];
        if (v != 0.0) {
            Exp sub = det_exact_rec(M, n, row + 1, cols & ~(1u << c));
            Exp t = scale(sub, (idx & 1) ? -v : v);
            acc = add(acc, t);
        }
        ++idx;
    }
    return acc;
}

inline int det_sign_exact(const double* M, int n) {
    if (n == 0) return 1;
    return exp_sign(det_exact_rec(M, n, 0, (1u << n) - 1));
}

// FP64 determinant with the permanent of |M| (same Laplace order).  The forward error of the
// computed value is below (c_n + 1) * u * perm with c_1 = 0, c_2 = 2, c_n = c_{n-1} + n.
inline double det_fp_rec(const double* M, int n, int row, unsigned cols, double& perm) {
    int rem = n - row;
    if (rem == 1) {
        for (int c = 0; c < n; ++c)
            if (cols & (1u << c)) {
                perm = std::fabs(M[row * n + c]);
                return M[row * n + c];
            }
        perm = 0;
        return 0;
    }
    double acc = 0, pacc = 0;
    int idx = 0;
    for (int c = 0; c < n; ++c) {
        if (!(cols & (1u << c))) continue;
        double v = M[row * n + c];
        double p;
        double sub = det_fp_rec(M, n, row + 1, cols & ~(1u << c), p);
        double t = v * sub;
        acc = (idx & 1) ? acc - t : acc + t;
        pacc = pacc + std::fabs(v) * p;
        ++idx;
    }
    perm = pacc;
    return acc;
}

constexpr double kU = 1.1102230246251565e-16;  // 2^-53

inline double det_err_coeff(int n) {
    static const double c[6] = {0, 0, 2, 5, 9, 14};
    return 2.0 * (c[n] + 1.0) * kU;  // factor 2: slack for second-order terms and perm rounding
}

// Predicate cache of one arrangement vertex.
//
// A vertex P lies on the face of the tet spanned by the free corners S (|S| = s); its
// homogeneous barycentric coordinates on S are the cofactors N of an m x (m+1) system A:
//   implicit arrangement : rows = m = s-1 implicit planes restricted to S  (cols = S)
//   material interface   : rows = m = s   materials restricted to S, with a trailing 1
//                          column (cols = S + level)
// For a query row r (length m+1): det([A; r]) = sum_i r_i N_i; the sign of the query at P is
// sign(det([A; r])) * sigma, where sigma = sign(det([A; z])) and z is the normalisation row
// (all ones on S, 0 on the level column).
struct VCache {
    int m = 0;          // number of defining rows
    int s = 0;          // free corners
    int S[4] = {0, 0, 0, 0};
    double A[4 * 5];    // defining rows, (m) x (m+1)
    double N[5];        // sigma-normalised FP64 cofactors
    double E[5];        // error bounds of N
    int sigma = 1;
    bool mi = false;
};

// Build the cache from explicit rows over free corners.  `rows` holds m rows of 4 corner values;
// for MI the trailing 1 column is appended here.
inline void vcache_build(VCache& c, bool mi, int s, const int* S, int m, const double* const* rows) {
    if (s < 1 || s > 4 || m < 0 || m > 4) std::abort();  // a vertex of a tet: at most 4 corners and rows
    c.mi = mi;
    c.s = s;
    c.m = m;
    for (int i = 0; i < s; ++i) c.S[i] = S[i];
    int nc = m + 1;
    for (int r = 0; r < m; ++r) {
        for (int i = 0; i < s; ++i) c.A[r * nc + i] = rows[r][S[i]];
        if (mi) c.A[r * nc + s] = 1.0;
    }
    // cofactors: N_i = (-1)^(m+i) det(A without column i)
    double minor[16];
    for (int i = 0; i < nc; ++i) {
        for (int r = 0; r < m; ++r) {
            int cc = 0;
            for (int j = 0; j < nc; ++j)
                if (j != i) minor[r * m + cc++] = c.A[r * nc + j];
        }
        double perm = 0;
        double v = (m == 0) ? 1.0 : det_fp_rec(minor, m, 0, (1u << m) - 1, perm);
        double sg = ((m + i) & 1) ? -1.0 : 1.0;
        c.N[i] = sg * v;
        c.E[i] = (m <= 1) ? 0.0 : det_err_coeff(m) * perm;  // 0x0 / 1x1 minors are exact
    }
    // sigma: all exact cofactors on S share one sign (P lies in the closed tet)
    int sig = 0;
    for (int i = 0; i < s; ++i)
        if (std::fabs(c.N[i]) > c.E[i]) {
            sig = c.N[i] > 0 ? 1 : -1;
            break;
        }
    if (sig == 0) {
        double M[25];
        for (int r = 0; r < m; ++r)
            for (int j = 0; j < nc; ++j) M[r * nc + j] = c.A[r * nc + j];
        for (int j = 0; j < nc; ++j) M[m * nc + j] = (j < s) ? 1.0 : 0.0;
        sig = det_sign_exact(M, nc);
    }
    c.sigma = sig;  // 0 only for a singular (dependent) defining set
    for (int i = 0; i < nc; ++i) c.N[i] *= (double)sig;
}

// Sign at P of a query row given by 4 corner values q (and, for MI, the level term 1).
// `exact_calls` counts filter failures (statistics only).
inline int vcache_query(const VCache& c, const double* q, long* exact_calls = nullptr) {
    int nc = c.m + 1;
    double r[5];
    for (int i = 0; i < c.s; ++i) r[i] = q[c.S[i]];
    if (c.mi) r[c.s] = 1.0;
    double v = 0, mag = 0, err = 0;
    for (int i = 0; i < nc; ++i) {
        double t = r[i] * c.N[i];
        v += t;
        mag += std::fabs(t);
        err += std::fabs(r[i]) * c.E[i];
    }
    double bound = 1.01 * ((double)(nc + 1) * kU * mag + err);
    if (v > bound) return 1;
    if (v < -bound) return -1;
    if (bound == 0.0) return 0;
    if (exact_calls) ++*exact_calls;
    double M[25];
    for (int rr = 0; rr < c.m; ++rr)
        for (int j = 0; j < nc; ++j) M[rr * nc + j] = c.A[rr * nc + j];
    for (int j = 0; j < nc; ++j) M[c.m * nc + j] = r[j];
    return det_sign_exact(M, nc) * c.sigma;
}

// Exact a*b == c*d.
inline bool prod_eq(double a, double b, double c, double d) {
    double x1, y1, x2, y2;
    two_prod(a, b, x1, y1);
    two_prod(c, d, x2, y2);
    return x1 == x2 && y1 == y2;
}

// Exact rank test: are the given rows (length n <= 5) linearly independent?
inline bool rows_independent(const double* const* rows, int r, int n) {
    if (r == 0) return true;
    if (r > n) return false;
    // try every r-subset of columns
    for (unsigned cols = 0; cols < (1u << n); ++cols) {
        if (__builtin_popcount(cols) != r) continue;
        double M[25];
        for (int i = 0; i < r; ++i) {
            int cc = 0;
            for (int j = 0; j < n; ++j)
                if (cols & (1u << j)) M[i * r + cc++] = rows[i][j];
        }
        if (det_sign_exact(M, r) != 0) return true;
    }
    return false;
}

}  // namespace oracle
