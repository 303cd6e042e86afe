// Exact sign predicates for the per-tet cut (device code; also compiled for the host in a
// test-only harness).
//
// The reference's per-tet cut lives in the third-party library qnzhou/simplicial_arrangement
// (not vendored; called at src/implicit_arrangement.cpp:279,283 and
// src/material_interface.cpp:323,327), whose robustness rests on exact orientation predicates over
// FP64 inputs.  Here every predicate is the sign of a small determinant of input doubles:
//   * a semi-static FP64 filter: the value and a rigorous forward error bound, and
//   * an exact fallback with floating-point expansion arithmetic (J. R. Shewchuk, "Adaptive
//     Precision Floating-Point Arithmetic and Fast Robust Geometric Predicates", DCG 18, 1997:
//     Two-Sum, Fast-Two-Sum, Two-Product (through fma), Grow-Expansion and Compress).
// Expansions have a fixed capacity; an input whose exact value does not fit reports failure
// (the caller turns it into RIA_EDEGENERATE) instead of guessing.
#pragma once
#include <cstdint>
#include <cmath>
#include <cstring>

#if defined(__CUDACC__)
#define RIA_HD __host__ __device__ __forceinline__
#define RIA_HDI __host__ __device__
#else
#define RIA_HD inline
#define RIA_HDI inline
#endif

namespace ria {

constexpr double kU = 1.1102230246251565e-16;  // 2^-53

RIA_HD void two_sum(double a, double b, double& x, double& y) {
    x = a + b;
    double bv = x - a;
    double av = x - bv;
    double br = b - bv;
    double ar = a - av;
    y = ar + br;
}

RIA_HD void fast_two_sum(double a, double b, double& x, double& y) {  // |a| >= |b|
    x = a + b;
    double bv = x - a;
    y = b - bv;
}

RIA_HD void two_prod(double a, double b, double& x, double& y) {
    x = a * b;
    y = fma(a, b, -x);
}

template <int CAP>
struct Expn {
    int n;
    double c[CAP];  // nonoverlapping, increasing magnitude, zero-free
};

// h += b in place (Grow-Expansion with zero elimination).
template <int CAP>
RIA_HD bool exp_grow(Expn<CAP>& h, double b) {
    double q = b;
    int j = 0;
    for (int i = 0; i < h.n; ++i) {
        double qn, hh;
        two_sum(q, h.c[i], qn, hh);
        q = qn;
        if (hh != 0.0) h.c[j++] = hh;
    }
    if (q != 0.0) {
        if (j >= CAP) return false;
        h.c[j++] = q;
    }
    h.n = j;
    return true;
}

// Compress in place (the result is nonoverlapping and as short as the method makes it).
template <int CAP>
RIA_HD void exp_compress(Expn<CAP>& e) {
    const int m = e.n;
    if (m <= 1) return;
    double Q = e.c[m - 1];
    int bottom = m - 1;
    for (int i = m - 2; i >= 0; --i) {
        double s, q;
        fast_two_sum(Q, e.c[i], s, q);
        if (q != 0.0) {
            e.c[bottom--] = s;
            Q = q;
        } else {
            Q = s;
        }
    }
    e.c[bottom] = Q;
    int top = 0;
    for (int i = bottom + 1; i < m; ++i) {
        double s, q;
        fast_two_sum(e.c[i], Q, s, q);
        if (q != 0.0) e.c[top++] = q;
        Q = s;
    }
    e.c[top++] = Q;
    e.n = top;
}

template <int CAP>
RIA_HD int exp_sign(const Expn<CAP>& e) {
    if (e.n == 0) return 0;
    return e.c[e.n - 1] > 0.0 ? 1 : -1;
}

// acc += sub * v (exact); compresses as it goes.
template <int CAP, int CAP2>
RIA_HD bool exp_add_scaled(Expn<CAP>& acc, const Expn<CAP2>& sub, double v) {
    for (int i = 0; i < sub.n; ++i) {
        double x, y;
        two_prod(sub.c[i], v, x, y);
        if (acc.n + 2 > CAP) {
            exp_compress(acc);
            if (acc.n + 2 > CAP) return false;
        }
        if (y != 0.0 && !exp_grow(acc, y)) return false;
        if (x != 0.0 && !exp_grow(acc, x)) return false;
    }
    exp_compress(acc);
    return true;
}

// Exact determinant of rows row..n-1 of an n x n row-major matrix over the columns in `cols`,
// by Laplace expansion.  R = n - row (compile-time depth).
template <int R, int CAP>
RIA_HDI bool det_rec(const double* M, int n, int row, unsigned cols, Expn<CAP>& out) {
    if constexpr (R == 1) {
        out.n = 0;
        for (int c = 0; c < n; ++c)
            if (cols & (1u << c)) {
                double v = M[row * n + c];
                if (v != 0.0) {
                    out.c[0] = v;
                    out.n = 1;
                }
                return true;
            }
        return true;
    } else if constexpr (R == 2) {
        int c0 = -1, c1 = -1;
        for (int c = 0; c < n; ++c)
            if (cols & (1u << c)) {
                if (c0 < 0) c0 = c;
                else c1 = c;
            }
        double a = M[row * n + c0], b = M[row * n + c1];
        double cc = M[(row + 1) * n + c0], d = M[(row + 1) * n + c1];
        double x1, y1, x2, y2;
        two_prod(a, d, x1, y1);
        two_prod(b, cc, x2, y2);
        out.n = 0;
        exp_grow(out, y1);
        exp_grow(out, x1);
        exp_grow(out, -y2);
        exp_grow(out, -x2);
        exp_compress(out);
        return true;
    } else {
        out.n = 0;
        int idx = 0;
        for (int c = 0; c < n; ++c) {
            if (!(cols & (1u << c))) continue;
            double v = M[row * n + c];
            if (v != 0.0) {
                Expn<CAP> sub;
                if (!det_rec<R - 1, CAP>(M, n, row + 1, cols & ~(1u << c), sub)) return false;
                if (!exp_add_scaled(out, sub, (idx & 1) ? -v : v)) return false;
            }
            ++idx;
        }
        return true;
    }
}

// Sign of an exact n x n determinant (n <= 5).  Returns 2 on capacity overflow.
template <int CAP = 48>
RIA_HDI int det_sign_exact(const double* M, int n) {
    Expn<CAP> e;
    bool ok = true;
    switch (n) {
        case 0:
            return 1;
        case 1:
            return M[0] > 0 ? 1 : (M[0] < 0 ? -1 : 0);
        case 2:
            ok = det_rec<2, CAP>(M, 2, 0, 3u, e);
            break;
        case 3:
            ok = det_rec<3, CAP>(M, 3, 0, 7u, e);
            break;
        case 4:
            ok = det_rec<4, CAP>(M, 4, 0, 15u, e);
            break;
        case 5:
            ok = det_rec<5, CAP>(M, 5, 0, 31u, e);
            break;
        default:
            return 2;
    }
    if (!ok) return 2;
    return exp_sign(e);
}

// FP64 determinant (same Laplace order) and the permanent of |M|; the forward error of the value
// is below (c_n + 1) u perm with c_1 = 0, c_2 = 2, c_n = c_{n-1} + n.
template <int R>
RIA_HD double det_fp_rec(const double* M, int n, int row, unsigned cols, double& perm) {
    if constexpr (R == 1) {
        for (int c = 0; c < n; ++c)
            if (cols & (1u << c)) {
                perm = fabs(M[row * n + c]);
                return M[row * n + c];
            }
        perm = 0.0;
        return 0.0;
    } else {
        double acc = 0.0, pacc = 0.0;
        int idx = 0;
        for (int c = 0; c < n; ++c) {
            if (!(cols & (1u << c))) continue;
            double v = M[row * n + c];
            double p;
            double sub = det_fp_rec<R - 1>(M, n, row + 1, cols & ~(1u << c), p);
            double t = v * sub;
            acc = (idx & 1) ? acc - t : acc + t;
            pacc = pacc + fabs(v) * p;
            ++idx;
        }
        perm = pacc;
        return acc;
    }
}

RIA_HD double det_fp(const double* M, int n, double& perm) {
    switch (n) {
        case 1:
            return det_fp_rec<1>(M, 1, 0, 1u, perm);
        case 2:
            return det_fp_rec<2>(M, 2, 0, 3u, perm);
        case 3:
            return det_fp_rec<3>(M, 3, 0, 7u, perm);
        case 4:
            return det_fp_rec<4>(M, 4, 0, 15u, perm);
        default:
            perm = 0.0;
            return 1.0;
    }
}

RIA_HD double det_err_coeff(int n) {
    // 2 (c_n + 1) u; the factor 2 covers second-order terms and the rounding of perm itself
    return n <= 1 ? 0.0 : (n == 2 ? 6.0 * kU : (n == 3 ? 12.0 * kU : (n == 4 ? 20.0 * kU : 30.0 * kU)));
}

// ---------------------------------------------------------------------------------------------
// Per-vertex predicate cache.
//
// A vertex P lies on the face of the tet spanned by the free corners S (|S| = s).  Its
// homogeneous barycentric coordinates on S are the cofactors N of an m x (m+1) system A:
//   implicit arrangement: m = s-1 implicit planes restricted to S (columns S);
//   material interface:   m = s materials restricted to S plus a trailing 1 (columns S, level).
// For a query row r: det([A; r]) = sum_i r_i N_i and the sign of the query at P is
// sign(det([A; r])) * sigma with sigma = sign(det([A; z])), z = (1 on S, 0 on the level column).
struct VCache {
    float N[5];  // sigma * cofactors from the FP32 filter (valid when f32)
    float E[5];  // their error bounds against the exact cofactors of the FP64 inputs
    int8_t s, m;
    int8_t mi;
    int8_t sigma;
    uint8_t S[4];
    uint8_t f32;
};

// ---- FP32 filter
//
// GB300 issues FP32 at many times its FP64 rate, so the predicates are tried in FP32 first.  Inputs
// are truncated to FP32 bit-exactly with integer operations (relative error below 2^-23); a
// nonzero input outside [2^-24, 2^24) leaves the FP32 filter out for that vertex or query.  With
// every input in that range no product of up to five inputs leaves the normal FP32 range; products
// of inputs with cancelled (possibly subnormal) minors are covered by an absolute term 2^-60 that
// exceeds the worst accumulated underflow error (fewer than 2^7 products, each off by at most
// 2^-150 and scaled by at most 2^72 through the remaining levels).

constexpr float kU32 = 5.9604644775390625e-8f;       // 2^-24
constexpr float kAbs32 = 8.673617379884035e-19f;      // 2^-60

RIA_HD bool to_f32(double x, float& f) {
#if defined(__CUDA_ARCH__)
    const uint64_t b = (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, 8);
#endif
    const uint64_t mag = b & 0x7FFFFFFFFFFFFFFFull;
    if (mag == 0) {
        f = 0.0f;
        return true;
    }
    const int e = (int)(mag >> 52) - 1023;
    if (e < -24 || e > 23) return false;
    const uint32_t fb = ((uint32_t)(b >> 32) & 0x80000000u) | ((uint32_t)(e + 127) << 23) |
                        ((uint32_t)(mag >> 29) & 0x7FFFFFu);
#if defined(__CUDA_ARCH__)
    f = __int_as_float((int)fb);
#else
    std::memcpy(&f, &fb, 4);
#endif
    return true;
}

RIA_HD int popc32(unsigned x) {
#if defined(__CUDA_ARCH__)
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}

// All M+1 maximal minors of an M x (M+1) matrix (signed as cofactors of an appended row) and their
// permanents, from shared minors of the bottom rows: the minor of rows M-j..M-1 on a column set is
// the Laplace expansion along row M-j, so each value is the same expansion as a full recursive
// Laplace evaluation, with its error bound (c_1 = 0, c_j = c_{j-1} + j).
template <int M>
RIA_HD void cofactors_f32(const float* A, float* N, float* P) {
    constexpr int NC = M + 1;
    float D[1 << NC], Q[1 << NC];
#pragma unroll
    for (int mask = 1; mask < (1 << NC); ++mask) {
        const int j = popc32((unsigned)mask);
        if (j > M) continue;
        const int row = M - j;
        float acc = 0.0f, pacc = 0.0f;
        int t = 0;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            if (!(mask & (1 << c))) continue;
            const float a = A[row * NC + c];
            const int sub = mask & ~(1 << c);
            if (j == 1) {
                acc = a;
                pacc = fabsf(a);
            } else {
                const float term = a * D[sub];
                acc = (t & 1) ? acc - term : acc + term;
                pacc = pacc + fabsf(a) * Q[sub];
            }
            ++t;
        }
        D[mask] = acc;
        Q[mask] = pacc;
    }
#pragma unroll
    for (int i = 0; i < NC; ++i) {
        const int mask = ((1 << NC) - 1) & ~(1 << i);
        const float v = (M == 0) ? 1.0f : D[mask];
        N[i] = ((M + i) & 1) ? -v : v;
        P[i] = (M == 0) ? 0.0f : Q[mask];
    }
}

// (2M + c_M) u with 2% headroom: 2M u for the truncated inputs, c_M u for the evaluation
RIA_HD float err_coeff_f32(int m) {
    const float k = m <= 0 ? 0.0f : (m == 1 ? 2.0f : (m == 2 ? 6.0f : (m == 3 ? 11.0f : 17.0f)));
    return 1.02f * k * kU32;
}

// ---- FP64 filter (the fallback when the FP32 filter cannot decide)

RIA_HD void cofactors_f64(const double* A, int m, double* N, double* E) {
    const int nc = m + 1;
    for (int i = 0; i < nc; ++i) {
        double minor[16];
        for (int r = 0; r < m; ++r) {
            int cc = 0;
            for (int j = 0; j < nc; ++j)
                if (j != i) minor[r * m + cc++] = A[r * nc + j];
        }
        double perm = 0.0;
        double v = (m == 0) ? 1.0 : det_fp(minor, m, perm);
        N[i] = ((m + i) & 1) ? -v : v;
        E[i] = det_err_coeff(m) * perm;
    }
}

RIA_HD void vcache_matrix(const VCache& c, const double* const* rows, double* A) {
    const int nc = c.m + 1;
    for (int r = 0; r < c.m; ++r) {
        for (int i = 0; i < c.s; ++i) A[r * nc + i] = rows[r][c.S[i]];
        if (c.mi) A[r * nc + c.s] = 1.0;
    }
}

// rows[r] points at the 4 corner values of defining row r.  Returns false when sigma cannot be
// decided by the filters and `exact` is false (or the exact evaluation overflowed).
RIA_HD bool vcache_build(VCache& c, bool mi, int s, const uint8_t* S, int m, const double* const* rows, bool exact) {
    c.mi = mi;
    c.s = (int8_t)s;
    c.m = (int8_t)m;
    for (int i = 0; i < 4; ++i) c.S[i] = i < s ? S[i] : 0;
    const int nc = m + 1;
    double A[4 * 5];
    vcache_matrix(c, rows, A);
    float A32[4 * 5];
    bool ok = true;
    for (int k = 0; k < m * nc; ++k) ok = to_f32(A[k], A32[k]) && ok;
    c.f32 = ok ? 1 : 0;
    int sig = 0;
    if (ok) {
        float P[5];
        switch (m) {
            case 0: cofactors_f32<0>(A32, c.N, P); break;
            case 1: cofactors_f32<1>(A32, c.N, P); break;
            case 2: cofactors_f32<2>(A32, c.N, P); break;
            case 3: cofactors_f32<3>(A32, c.N, P); break;
            default: cofactors_f32<4>(A32, c.N, P); break;
        }
        const float k = err_coeff_f32(m);
        for (int i = 0; i < nc; ++i) c.E[i] = P[i] == 0.0f ? 0.0f : k * P[i] + kAbs32;
        for (int i = 0; i < s; ++i)
            if (fabsf(c.N[i]) > c.E[i]) {
                sig = c.N[i] > 0.0f ? 1 : -1;
                break;
            }
    }
    if (sig == 0) {
        double N[5], E[5];
        cofactors_f64(A, m, N, E);
        for (int i = 0; i < s; ++i)
            if (fabs(N[i]) > E[i]) {
                sig = N[i] > 0 ? 1 : -1;
                break;
            }
    }
    if (sig == 0) {
        if (!exact) return false;
        double M[25];
        for (int r = 0; r < m; ++r)
            for (int j = 0; j < nc; ++j) M[r * nc + j] = A[r * nc + j];
        for (int j = 0; j < nc; ++j) M[m * nc + j] = (j < s) ? 1.0 : 0.0;
        sig = det_sign_exact(M, nc);
        if (sig == 0 || sig == 2) return false;
    }
    c.sigma = (int8_t)sig;
    if (ok)
        for (int i = 0; i < nc; ++i) c.N[i] = sig > 0 ? c.N[i] : -c.N[i];
    return true;
}

// Sign of the query row q (4 corner values) at the vertex: -1, 0, 1; or 2 when the filters cannot
// decide and `exact` is false (or the exact evaluation overflowed).  `rows` are the defining rows.
RIA_HD int vcache_query(const VCache& c, const double* q, const double* const* rows, bool exact) {
    const int nc = c.m + 1;
    double r[5];
    for (int i = 0; i < c.s; ++i) r[i] = q[c.S[i]];
    if (c.mi) r[c.s] = 1.0;
    if (c.f32) {
        float r32[5];
        bool ok = true;
        for (int i = 0; i < nc; ++i) ok = to_f32(r[i], r32[i]) && ok;
        if (ok) {
            // |v32 - v| <= 1.02 ((nc + 2) u mag + sum |r_i| E_i) + 2^-60: nc u for the evaluation, 2u for
            // the truncated query, the cofactor bounds E for the rest
            float v = 0.0f, mag = 0.0f, err = 0.0f;
            bool zero = true;
            for (int i = 0; i < nc; ++i) {
                const float t = r32[i] * c.N[i];
                v = v + t;
                mag = mag + fabsf(t);
                err = err + fabsf(r32[i]) * c.E[i];
                zero = zero && (r32[i] == 0.0f || (c.N[i] == 0.0f && c.E[i] == 0.0f));
            }
            if (zero) return 0;  // every term is exactly zero
            const float bound = 1.02f * ((float)(nc + 2) * kU32 * mag + err) + kAbs32;
            if (v > bound) return 1;
            if (v < -bound) return -1;
        }
    }
    double A[4 * 5];
    vcache_matrix(c, rows, A);
    double N[5], E[5];
    cofactors_f64(A, c.m, N, E);
    double v = 0.0, mag = 0.0, err = 0.0;
    for (int i = 0; i < nc; ++i) {
        double t = r[i] * (N[i] * (double)c.sigma);
        v += t;
        mag += fabs(t);
        err += fabs(r[i]) * E[i];
    }
    double bound = 1.01 * ((double)(nc + 1) * kU * mag + err);
    if (v > bound) return 1;
    if (v < -bound) return -1;
    if (bound == 0.0) return 0;
    if (!exact) return 2;
    double M[25];
    for (int rr = 0; rr < c.m; ++rr)
        for (int j = 0; j < nc; ++j) M[rr * nc + j] = A[rr * nc + j];
    for (int j = 0; j < nc; ++j) M[c.m * nc + j] = r[j];
    int sg = det_sign_exact(M, nc);
    if (sg == 2) return 2;
    return sg * c.sigma;
}

// Exact a*b == c*d.
RIA_HD bool prod_eq(double a, double b, double c, double d) {
    double x1, y1, x2, y2;
    two_prod(a, b, x1, y1);
    two_prod(c, d, x2, y2);
    return x1 == x2 && y1 == y2;
}

// Exact rank test: are the r rows (n columns, n <= 5) linearly independent?  Returns 2 on
// overflow of the exact evaluation.
RIA_HD int rows_independent(const double* rows, int r, int n) {
    if (r == 0) return 1;
    if (r > n) return 0;
    for (unsigned cols = 0; cols < (1u << n); ++cols) {
        int pc = 0;
        for (int j = 0; j < n; ++j) pc += (cols >> j) & 1;
        if (pc != r) continue;
        double M[25];
        for (int i = 0; i < r; ++i) {
            int cc = 0;
            for (int j = 0; j < n; ++j)
                if (cols & (1u << j)) M[i * r + cc++] = rows[i * n + j];
        }
        int sg = det_sign_exact(M, r);
        if (sg == 2) return 2;
        if (sg != 0) return 1;
    }
    return 0;
}

}  // namespace ria
