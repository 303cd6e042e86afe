// Stages (a) and (b): sampling the implicit functions at the grid vertices, per-vertex sign /
// argmax masks, and the ordered compaction of the active tets.
//
//   sampling     the external implicit_functions library (app/implicit_arrangement.cpp:59);
//                formulas in include/ria.h.  One thread per vertex loops over the functions
//                (no divergence across a warp), combining per-axis terms tabulated once per grid;
//                the block's rows of the row-major V x F matrix go through shared memory so the
//                stores stay coalesced; the per-vertex masks come out of the same loop.
//   IA signs     src/implicit_arrangement.cpp:53-77   (pos/neg bit masks, F <= 64)
//   IA filter    src/implicit_arrangement.cpp:82-116  (active = not all corners strictly + and not
//                all strictly -:  ~(p0&p1&p2&p3 | n0&n1&n2&n3))
//   MI argmax    src/material_interface.cpp:53-92     (mask of the materials equal to the maximum)
//   MI filter    src/material_interface.cpp:94-152
// The compaction keeps tet order (per-block counts, an exclusive scan, warp-ballot ranks) so the
// active-function CRS and the first-occurrence numbering of the extraction follow the reference.
#include <math_constants.h>

#include "device_common.cuh"
#include "launch.hpp"
#include "sqrt_rn.cuh"

namespace ria {

namespace {

constexpr int kTileV = 32;
constexpr int kBlock = 256;

// the sign of a value from its bits, off the FP64 pipe: 1 positive, -1 negative, 0 for zeros and
// NaN (the outcomes of v > 0 and v < 0)
__device__ __forceinline__ int value_sign(double v) {
    const long long b = __double_as_longlong(v);
    const unsigned long long mag = (unsigned long long)b & 0x7FFFFFFFFFFFFFFFull;
    if (mag == 0 || mag > 0x7FF0000000000000ull) return 0;
    return b < 0 ? -1 : 1;
}

// masks of one vertex row held in shared memory
template <bool MI>
__device__ __forceinline__ ulonglong2 row_masks(const double* row, int F, int& nzero) {
    ulonglong2 m;
    if (!MI) {
        uint64_t pos = 0, neg = 0;
        for (int f = 0; f < F; ++f) {
            const int sg = value_sign(row[f]);
            if (sg > 0) pos |= bit64(f);
            else if (sg < 0) neg |= bit64(f);
        }
        nzero = F - __popcll(pos) - __popcll(neg);
        m.x = pos;
        m.y = neg;
    } else {
        double mx = row[0];
        for (int f = 1; f < F; ++f)
            if (row[f] > mx) mx = row[f];
        uint64_t tie = 0;
        for (int f = 0; f < F; ++f)
            if (row[f] == mx) tie |= bit64(f);
        nzero = __popcll(tie) > 1 ? 1 : 0;
        m.x = tie;
        m.y = 0;
    }
    return m;
}

__device__ __forceinline__ void block_add(unsigned long long* dst, int v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, (unsigned long long)v);
}

// Separable evaluation.  Every function of include/ria.h starts with terms that depend on a single
// coordinate (n_a (x_a - p_a), d_a^2, v_a = x_a - p_a and v_a u_a); on a grid they are tabulated per
// axis once, and each vertex only performs the operations that mix the axes, in the same order as
// the full formula, so the result is bit-identical to evaluating the formula at the vertex.
__device__ __forceinline__ void axis_parts(const ria_function& f, int a, double x, double& w0, double& w1) {
    switch (f.type) {
        case RIA_FUNC_PLANE:
            w0 = f.p[3 + a] * (x - f.p[a]);
            w1 = 0.0;
            break;
        case RIA_FUNC_SPHERE:
        case RIA_FUNC_SPHERE_SQUARED: {
            double d = x - f.p[a];
            w0 = d * d;
            w1 = 0.0;
            break;
        }
        case RIA_FUNC_CYLINDER:
        case RIA_FUNC_TORUS: {
            double d = x - f.p[a];
            w0 = d;
            w1 = d * f.p[3 + a];
            break;
        }
        default:
            w0 = w1 = 0.0;
    }
}

// Every formula starts with the sum of its x and y terms: w0 (plane, spheres) or w1 (cylinder,
// torus).  On a grid it is tabulated per (x, y) column; `s` is that first sum.  Square roots go
// through sqrt_rn (correctly rounded like sqrt, on the integer and FP32 pipes).
__device__ __forceinline__ bool first_sum_of_w1(int type) { return type == RIA_FUNC_CYLINDER || type == RIA_FUNC_TORUS; }

__device__ __forceinline__ double combine_from_sum(const ria_function& f, double s, const double w0[3],
                                                   const double w1[3]) {
    double v;
    switch (f.type) {
        case RIA_FUNC_PLANE:
            v = s + w0[2];
            break;
        case RIA_FUNC_SPHERE:
            v = f.p[3] - sqrt_rn(s + w0[2]);
            break;
        case RIA_FUNC_SPHERE_SQUARED:
            v = f.p[3] * f.p[3] - (s + w0[2]);
            break;
        case RIA_FUNC_CYLINDER: {
            double t = s + w1[2];
            double wx = w0[0] - t * f.p[3], wy = w0[1] - t * f.p[4], wz = w0[2] - t * f.p[5];
            v = f.p[6] - sqrt_rn((wx * wx + wy * wy) + wz * wz);
            break;
        }
        case RIA_FUNC_TORUS: {
            double h = s + w1[2];
            double wx = w0[0] - h * f.p[3], wy = w0[1] - h * f.p[4], wz = w0[2] - h * f.p[5];
            double rho = sqrt_rn((wx * wx + wy * wy) + wz * wz);
            double a = rho - f.p[6];
            v = f.p[7] - sqrt_rn(a * a + h * h);
            break;
        }
        default:
            v = 0.0;
    }
    // negation flips the sign bit (IEEE 754 negate, exact for every value, NaN included); done on the
    // integer pipe, since the FP64 pipe bounds this kernel.  The XOR is written in PTX: written in C++,
    // the compiler recognises a conditional floating-point negation and issues it as an FP64
    // addition (one per function and vertex, whether or not the function is flipped)
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned long long flip = f.flipped ? 0x8000000000000000ull : 0ull;
    asm("xor.b64 %0, %0, %1;" : "+l"(b) : "l"(flip));
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ double combine_parts(const ria_function& f, const double w0[3], const double w1[3]) {
    const double s = first_sum_of_w1(f.type) ? w1[0] + w1[1] : w0[0] + w0[1];
    return combine_from_sum(f, s, w0, w1);
}

// grid coordinates per axis (src/io.cpp:104-106): coords[a * N + n]
__global__ void k_grid_coords(GridDesc g, int N, double* __restrict__ coords) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * N) return;
    const int a = idx / N, n = idx - a * N;
    coords[idx] = ((double)n / (double)(N - 1)) * (g.bmax[a] - g.bmin[a]) + g.bmin[a];
}

// per-axis terms: tab[((f * 3 + a) * 2 + w) * N + n]
__global__ void k_axis_tables(const ria_function* __restrict__ funcs, int F, const double* __restrict__ coords, int N,
                              double* __restrict__ tab) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= F * 3 * N) return;
    const int n = idx % N, fa = idx / N, a = fa % 3, f = fa / 3;
    double w0, w1;
    axis_parts(funcs[f], a, coords[a * N + n], w0, w1);
    tab[(fa * 2 + 0) * N + n] = w0;
    tab[(fa * 2 + 1) * N + n] = w1;
}

// first sums per (x, y) column: xy[(f * N + i) * N + j] (one FP64 addition per column and function
// instead of one per vertex; the same operands, so the same bits)
__global__ void k_xy_tables(const ria_function* __restrict__ funcs, int F, const double* __restrict__ tab, int N,
                            double* __restrict__ xy) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)F * N * N) return;
    const int j = (int)(idx % N), i = (int)((idx / N) % N), f = (int)(idx / ((int64_t)N * N));
    const double* t = tab + (size_t)f * 6 * N;
    const int w = first_sum_of_w1(funcs[f].type) ? 1 : 0;
    xy[idx] = t[w * N + i] + t[(2 + w) * N + j];
}

constexpr int kSampleBlock = 128;

// One thread per vertex, a loop over the functions (uniform across the warp); the block's rows are
// staged in shared memory and stored row by row, so the V x F stores stay coalesced.
template <bool MI, bool GRID>
__global__ void __launch_bounds__(kSampleBlock) k_sample(const ria_function* __restrict__ funcs, int F,
                                                         const double* __restrict__ tab,
                                                         const double* __restrict__ xy, int N,
                                                         const double* __restrict__ pts, int64_t V,
                                                         double* __restrict__ fv, ulonglong2* __restrict__ vmask,
                                                         unsigned long long* __restrict__ n_zero) {
    extern __shared__ double tile[];
    const int stride = F + 1;
    const int64_t v0 = (int64_t)blockIdx.x * kSampleBlock;
    const int64_t v = v0 + threadIdx.x;
    const bool valid = v < V;
    int ix[3] = {0, 0, 0};
    double x[3] = {0.0, 0.0, 0.0};
    if (valid) {
        if (GRID) {
            const int vi = (int)v;
            ix[0] = vi / (N * N);
            ix[1] = (vi / N) % N;
            ix[2] = vi % N;
        } else {
            x[0] = pts[3 * v];
            x[1] = pts[3 * v + 1];
            x[2] = pts[3 * v + 2];
        }
    }
    uint64_t m0 = 0, m1 = 0;
    double mx = 0.0;
    for (int f = 0; f < F; ++f) {
        const ria_function& fn = funcs[f];
        double w0[3], w1[3];
        double val;
        if (GRID) {
            const double* t = tab + (size_t)f * 6 * N;
            for (int a = 0; a < 3; ++a) {
                w0[a] = t[(2 * a) * N + ix[a]];
                w1[a] = t[(2 * a + 1) * N + ix[a]];
            }
            val = combine_from_sum(fn, xy[((size_t)f * N + ix[0]) * N + ix[1]], w0, w1);
        } else {
            for (int a = 0; a < 3; ++a) axis_parts(fn, a, x[a], w0[a], w1[a]);
            val = combine_parts(fn, w0, w1);
        }
        tile[threadIdx.x * stride + f] = val;
        if (!MI) {
            const int sg = value_sign(val);
            if (sg > 0) m0 |= bit64(f);
            else if (sg < 0) m1 |= bit64(f);
        } else {
            if (f == 0 || val > mx) {
                mx = val;
                m0 = bit64(f);
            } else if (val == mx) {
                m0 |= bit64(f);
            }
        }
    }
    int nz = 0;
    if (valid && vmask) {
        vmask[v] = make_ulonglong2(m0, m1);
        nz = MI ? (__popcll(m0) > 1) : (F - __popcll(m0) - __popcll(m1));
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r < kSampleBlock; r += kSampleBlock / 32) {
        if (v0 + r >= V) break;
        double* dst = fv + (v0 + r) * F;
        for (int c = lane; c < F; c += 32) dst[c] = tile[r * stride + c];
    }
    if (n_zero) block_add(n_zero, nz);
}

template <bool MI>
__global__ void __launch_bounds__(kBlock) k_vertex_masks(const double* __restrict__ fv, int64_t V, int F,
                                                         ulonglong2* __restrict__ vmask,
                                                         unsigned long long* __restrict__ n_zero) {
    extern __shared__ double tile[];
    const int stride = F + 1;
    const int64_t v0 = (int64_t)blockIdx.x * kTileV;
    const int nel = kTileV * F;
    for (int e = threadIdx.x; e < nel; e += blockDim.x) {
        int lv = e / F, f = e - lv * F;
        int64_t v = v0 + lv;
        if (v < V) tile[lv * stride + f] = fv[v * F + f];
    }
    __syncthreads();
    int nz = 0;
    if (threadIdx.x < kTileV) {
        int64_t v = v0 + threadIdx.x;
        if (v < V) vmask[v] = row_masks<MI>(tile + threadIdx.x * stride, F, nz);
    }
    if (threadIdx.x < 32) block_add(n_zero, nz);
}

// Active functions of tet t.  IA: from the sign masks.  MI: candidates are the argmax sets of the
// corners; with at least two of them, add every material above the corner-wise minimum of the
// candidates at more than one corner (src/material_interface.cpp:104-145).
template <bool MI>
__device__ __forceinline__ uint64_t tet_active(const ulonglong2* __restrict__ vmask, const double* __restrict__ fv,
                                               int F, const int64_t v[4]) {
    const uint64_t full = (F == 64) ? ~0ull : (bit64(F) - 1);
    if (!MI) {
        ulonglong2 m0 = vmask[v[0]], m1 = vmask[v[1]], m2 = vmask[v[2]], m3 = vmask[v[3]];
        uint64_t ap = m0.x & m1.x & m2.x & m3.x;
        uint64_t an = m0.y & m1.y & m2.y & m3.y;
        return ~(ap | an) & full;
    } else {
        uint64_t cand = vmask[v[0]].x | vmask[v[1]].x | vmask[v[2]].x | vmask[v[3]].x;
        if (__popcll(cand) < 2) return 0;
        double min_h[4];
        for (int c = 0; c < 4; ++c) {
            min_h[c] = 1.7976931348623157e308;
            uint64_t cm = cand;
            while (cm) {
                int m = __ffsll((long long)cm) - 1;
                cm &= cm - 1;
                double x = fv[v[c] * F + m];
                if (x < min_h[c]) min_h[c] = x;
            }
        }
        uint64_t act = cand;
        for (int j = 0; j < F; ++j) {
            int g = 0;
            for (int c = 0; c < 4; ++c) g += fv[v[c] * F + j] > min_h[c];
            if (g > 1) act |= bit64(j);
        }
        return act & full;
    }
}

// sign pattern index of a lookup-table tet: sum over corners of (s_c + 1) 3^c
template <bool MI>
__device__ __forceinline__ int tet_pattern(const ulonglong2* __restrict__ vmask, const double* __restrict__ fv, int F,
                                           const int64_t v[4], uint64_t act) {
    int p = 0, w = 1;
    if (!MI) {
        int j = __ffsll((long long)act) - 1;
        for (int c = 0; c < 4; ++c) {
            ulonglong2 m = vmask[v[c]];
            int s = ((m.x >> j) & 1) ? 1 : (((m.y >> j) & 1) ? -1 : 0);
            p += (s + 1) * w;
            w *= 3;
        }
    } else {
        int a = __ffsll((long long)act) - 1;
        int b = __ffsll((long long)(act & (act - 1))) - 1;
        for (int c = 0; c < 4; ++c) {
            double fa = fv[v[c] * F + a], fb = fv[v[c] * F + b];
            int s = fb > fa ? 1 : (fb < fa ? -1 : 0);
            p += (s + 1) * w;
            w *= 3;
        }
    }
    return p;
}

// bin of a general-case tet: the heaviest (most active functions) first, so that a warp cuts tets of
// one size and the longest cuts start first
template <bool MI>
__device__ __forceinline__ int gen_bin(int k) {
    const int kk = k - (MI ? 1 : 0);
    return kGenBins - (kk < kGenBins ? kk : kGenBins);
}

// per block: the active count, then the general-case count of each bin; layout [1 + kGenBins][nb]
template <bool MI>
__global__ void __launch_bounds__(kBlock) k_filter_count(const ulonglong2* __restrict__ vmask,
                                                         const double* __restrict__ fv, int F, TetSrc ts, int64_t T,
                                                         bool use_table, uint32_t* __restrict__ blk,
                                                         unsigned long long* __restrict__ khist) {
    __shared__ uint32_t bins[kGenBins];
    if (threadIdx.x < kGenBins) bins[threadIdx.x] = 0;
    const int64_t t = (int64_t)blockIdx.x * kBlock + threadIdx.x;
    int k = 0;
    if (t < T) {
        int64_t v[4];
        ts.get(t, v);
        k = __popcll(tet_active<MI>(vmask, fv, F, v));
    }
    const int ka = MI ? 2 : 1;
    int act = k > 0;
    int gen = act && !(use_table && k == ka);
    int na = __syncthreads_count(act);  // also orders the zeroing of bins before the adds
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const unsigned same = __match_any_sync(full, gen ? gen_bin<MI>(k) : -1);
    if (gen && lane == __ffs(same) - 1) atomicAdd(&bins[gen_bin<MI>(k)], (uint32_t)__popc(same));
    int h0 = __syncthreads_count(k == ka);
    int h1 = __syncthreads_count(k == ka + 1);
    int h2 = __syncthreads_count(k > ka + 1);
    if (threadIdx.x == 0) {
        blk[blockIdx.x] = (uint32_t)na;
        if (h0) atomicAdd(&khist[0], (unsigned long long)h0);
        if (h1) atomicAdd(&khist[1], (unsigned long long)h1);
        if (h2) atomicAdd(&khist[2], (unsigned long long)h2);
    }
    if (threadIdx.x < kGenBins) blk[(1 + threadIdx.x) * (int64_t)gridDim.x + blockIdx.x] = bins[threadIdx.x];
}

template <bool MI>
__global__ void __launch_bounds__(kBlock) k_filter_scatter(const ulonglong2* __restrict__ vmask,
                                                           const double* __restrict__ fv, int F, TetSrc ts,
                                                           int64_t T, bool use_table,
                                                           const uint32_t* __restrict__ blk_off,
                                                           const IASum4* __restrict__ table_sum, FilterOut out) {
    __shared__ int wa[kBlock / 32];
    __shared__ int wg[kGenBins][kBlock / 32];
    for (int i = threadIdx.x; i < kGenBins * (kBlock / 32); i += kBlock) (&wg[0][0])[i] = 0;
    const int64_t t = (int64_t)blockIdx.x * kBlock + threadIdx.x;
    uint64_t act = 0;
    int64_t v[4] = {0, 0, 0, 0};
    if (t < T) {
        ts.get(t, v);
        act = tet_active<MI>(vmask, fv, F, v);
    }
    const int k = __popcll(act);
    const int ka = MI ? 2 : 1;
    const bool isact = k > 0;
    const bool isgen = isact && !(use_table && k == ka);
    const int bin = isgen ? gen_bin<MI>(k) : -1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1;
    const unsigned ba = __ballot_sync(0xFFFFFFFFu, isact);
    const unsigned same = __match_any_sync(0xFFFFFFFFu, bin);
    __syncthreads();  // wg zeroed
    if (lane == 0) wa[warp] = __popc(ba);
    if (isgen && lane == __ffs(same) - 1) wg[bin][warp] = __popc(same);
    __syncthreads();
    int pa = 0, pg = 0;
    for (int w = 0; w < warp; ++w) {
        pa += wa[w];
        if (isgen) pg += wg[bin][w];
    }
    if (isact) {
        uint32_t a = blk_off[blockIdx.x] + pa + __popc(ba & lt);
        out.act_tet[a] = (uint32_t)t;
        out.act_mask[a] = act;
        if (isgen) {
            const uint32_t base_g = blk_off[(1 + bin) * (int64_t)gridDim.x + blockIdx.x] - blk_off[gridDim.x];
            out.gen[base_g + pg + __popc(same & lt)] = a;
            out.act_desc[a] = 0;
        } else {
            int p = tet_pattern<MI>(vmask, fv, F, v, act);
            out.act_desc[a] = kTableBit | (uint64_t)p;
            out.act_sum[a] = table_sum[p];
        }
    }
}

__global__ void k_check_tets(const int64_t* __restrict__ tets, int64_t n, int64_t V, uint32_t* status) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t v = tets[i];
        if (v < 0 || v >= V) {
            raise_status(status, ST_BADINPUT);
            return;
        }
    }
}

// ---- batched grids

__device__ __forceinline__ int upper_index(const int64_t* base, int n, int64_t x) {
    // largest p in [0, n) with base[p] <= x (base ascending, base[0] = 0)
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int upper_index32(const uint32_t* base, int n, uint32_t x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One block holds vertices of one problem.  Coordinates follow src/io.cpp:104-106 and every value
// is the full formula at the vertex (the same operations, in the same order, as the separable grid
// sampler), so each problem's values equal those of its own grid call.
template <bool MI>
__global__ void __launch_bounds__(kBatchSampleBlock)
    k_batch_sample(const BatchProblem* __restrict__ probs, int n, const uint32_t* __restrict__ blk_off,
                   const ria_function* __restrict__ funcs, int Fmax, double* __restrict__ pts,
                   double* __restrict__ fv, ulonglong2* __restrict__ vmask, unsigned long long* __restrict__ n_zero,
                   unsigned long long* __restrict__ n_zero_p) {
    extern __shared__ double tile[];
    const int stride = Fmax + 1;
    const int p = upper_index32(blk_off, n, blockIdx.x);
    const BatchProblem pr = probs[p];
    const int N = pr.res + 1;
    const int64_t Vp = (int64_t)N * N * N;
    const int64_t l0 = (int64_t)(blockIdx.x - blk_off[p]) * kBatchSampleBlock;
    const int64_t lv = l0 + threadIdx.x;
    const bool valid = lv < Vp;
    double x[3] = {0.0, 0.0, 0.0};
    if (valid) {
        const int vi = (int)lv;
        const int ix[3] = {vi / (N * N), (vi / N) % N, vi % N};
        for (int a = 0; a < 3; ++a)
            x[a] = ((double)ix[a] / (double)(N - 1)) * (pr.bmax[a] - pr.bmin[a]) + pr.bmin[a];
        double* dst = pts + 3 * (pr.vbase + lv);
        dst[0] = x[0];
        dst[1] = x[1];
        dst[2] = x[2];
    }
    uint64_t m0 = 0, m1 = 0;
    double mx = 0.0;
    for (int f = 0; f < Fmax; ++f) {
        double val;
        if (f < pr.F) {
            const ria_function& fn = funcs[pr.foff + f];
            double w0[3], w1[3];
            for (int a = 0; a < 3; ++a) axis_parts(fn, a, x[a], w0[a], w1[a]);
            val = combine_parts(fn, w0, w1);
        } else {
            val = MI ? -CUDART_INF : 1.0;
        }
        tile[threadIdx.x * stride + f] = val;
        if (!MI) {
            const int sg = value_sign(val);
            if (sg > 0) m0 |= bit64(f);
            else if (sg < 0) m1 |= bit64(f);
        } else {
            if (f == 0 || val > mx) {
                mx = val;
                m0 = bit64(f);
            } else if (val == mx) {
                m0 |= bit64(f);
            }
        }
    }
    int nz = 0;
    if (valid) {
        vmask[pr.vbase + lv] = make_ulonglong2(m0, m1);
        nz = MI ? (__popcll(m0) > 1) : (Fmax - __popcll(m0) - __popcll(m1));
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    for (int r = warp; r < kBatchSampleBlock; r += kBatchSampleBlock / 32) {
        if (l0 + r >= Vp) break;
        double* dst = fv + (pr.vbase + l0 + r) * Fmax;
        for (int c = lane; c < Fmax; c += 32) dst[c] = tile[r * stride + c];
    }
    block_add(n_zero, nz);
    block_add(n_zero_p + p, nz);
}

__global__ void k_batch_tets(const BatchProblem* __restrict__ probs, const int64_t* __restrict__ tet_base, int n,
                             int64_t T, int64_t* __restrict__ tets) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < T; t += (int64_t)gridDim.x * blockDim.x) {
        const int p = upper_index(tet_base, n, t);
        int64_t v[4];
        grid_tet(t - tet_base[p], probs[p].res, v);
        const int64_t vb = probs[p].vbase;
        longlong2* dst = reinterpret_cast<longlong2*>(tets + 4 * t);
        dst[0] = make_longlong2(v[0] + vb, v[1] + vb);
        dst[1] = make_longlong2(v[2] + vb, v[3] + vb);
    }
}

// first index i in [0, m) with key(i) >= x (key non-decreasing), or m
template <class Key>
__device__ __forceinline__ int64_t lower_index(int64_t m, int64_t x, Key key) {
    int64_t lo = 0, hi = m;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (key(mid) < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__global__ void k_batch_ranges(const int64_t* __restrict__ tet_base, int n, const int64_t* __restrict__ verts,
                               int64_t n_verts, const int64_t* __restrict__ fto, const int64_t* __restrict__ ftets,
                               int64_t n_faces, int64_t* __restrict__ vert_first, int64_t* __restrict__ face_first) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > n) return;
    if (p == n) {
        vert_first[n] = n_verts;
        face_first[n] = n_faces;
        return;
    }
    const int64_t tb = tet_base[p];
    vert_first[p] = lower_index(n_verts, tb, [&](int64_t i) { return verts[11 * i]; });
    face_first[p] = lower_index(n_faces, tb, [&](int64_t f) { return ftets[2 * fto[f]]; });
}

// stats4[4 p + 0..3]: active tets, k == a, k == a + 1, k > a + 1 (a = 1 IA, 2 MI)
template <bool MI>
__global__ void k_batch_active_stats(const int64_t* __restrict__ tet_base, int n, const uint32_t* __restrict__ act_tet,
                                     const uint64_t* __restrict__ act_mask, int64_t A,
                                     unsigned long long* __restrict__ stats4) {
    const int ka = MI ? 2 : 1;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A; i += (int64_t)gridDim.x * blockDim.x) {
        const int p = upper_index(tet_base, n, (int64_t)act_tet[i]);
        const int k = __popcll(act_mask[i]);
        unsigned long long* st = stats4 + 4 * p;
        atomicAdd(st, 1ull);
        atomicAdd(st + (k == ka ? 1 : (k == ka + 1 ? 2 : 3)), 1ull);
    }
}

template <bool MI, bool GRID>
void set_sample_smem(size_t smem) {
    if (smem > 48 * 1024) {  // once per process (thread-safe static initialisation)
        static const bool done =
            cudaFuncSetAttribute(k_sample<MI, GRID>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024) ==
            cudaSuccess;
        (void)done;
    }
}

}  // namespace

void launch_grid_coords(const GridDesc& g, double* coords, cudaStream_t s) {
    const int N = (int)g.res + 1;
    k_grid_coords<<<(3 * N + 127) / 128, 128, 0, s>>>(g, N, coords);
    note_launch();
}

void launch_sample_grid(bool mi, const ria_function* d_funcs, int F, const GridDesc& g, const double* coords,
                        double* tab, double* xy, double* fv, ulonglong2* vmask, unsigned long long* n_zero,
                        cudaStream_t s) {
    const int N = (int)g.res + 1;
    const int64_t V = (int64_t)N * N * N;
    k_axis_tables<<<(F * 3 * N + 127) / 128, 128, 0, s>>>(d_funcs, F, coords, N, tab);
    note_launch();
    const int64_t nxy = (int64_t)F * N * N;
    k_xy_tables<<<(unsigned)((nxy + 127) / 128), 128, 0, s>>>(d_funcs, F, tab, N, xy);
    note_launch();
    const unsigned blocks = (unsigned)((V + kSampleBlock - 1) / kSampleBlock);
    const size_t smem = sizeof(double) * kSampleBlock * (F + 1);
    if (mi) {
        set_sample_smem<true, true>(smem);
        k_sample<true, true><<<blocks, kSampleBlock, smem, s>>>(d_funcs, F, tab, xy, N, nullptr, V, fv, vmask, n_zero);
    } else {
        set_sample_smem<false, true>(smem);
        k_sample<false, true><<<blocks, kSampleBlock, smem, s>>>(d_funcs, F, tab, xy, N, nullptr, V, fv, vmask, n_zero);
    }
    note_launch();
}

void launch_sample_points(const ria_function* d_funcs, int F, const double* pts, int64_t V, double* fv,
                          ulonglong2* vmask, unsigned long long* n_zero, cudaStream_t s) {
    if (V == 0) return;
    const unsigned blocks = (unsigned)((V + kSampleBlock - 1) / kSampleBlock);
    const size_t smem = sizeof(double) * kSampleBlock * (F + 1);
    set_sample_smem<false, false>(smem);
    k_sample<false, false><<<blocks, kSampleBlock, smem, s>>>(d_funcs, F, nullptr, nullptr, 0, pts, V, fv, vmask, n_zero);
    note_launch();
}

void launch_vertex_masks(bool mi, const double* fv, int64_t V, int F, ulonglong2* vmask, unsigned long long* n_zero,
                         cudaStream_t s) {
    const int64_t blocks = (V + kTileV - 1) / kTileV;
    if (blocks == 0) return;
    const size_t smem = sizeof(double) * kTileV * (F + 1);
    if (mi)
        {
            k_vertex_masks<true><<<(unsigned)blocks, kBlock, smem, s>>>(fv, V, F, vmask, n_zero);
            note_launch();
        }
    else
        {
            k_vertex_masks<false><<<(unsigned)blocks, kBlock, smem, s>>>(fv, V, F, vmask, n_zero);
            note_launch();
        }
}

void launch_batch_sample(bool mi, const BatchProblem* probs, int n, const uint32_t* blk_off, uint32_t n_blocks,
                         const ria_function* funcs, int Fmax, double* pts, double* fv, ulonglong2* vmask,
                         unsigned long long* n_zero, unsigned long long* n_zero_p, cudaStream_t s) {
    if (n_blocks == 0) return;
    const size_t smem = sizeof(double) * kBatchSampleBlock * (Fmax + 1);
    if (smem > 48 * 1024) {  // once per process and mode (thread-safe static initialisation)
        if (mi) {
            static const bool done =
                cudaFuncSetAttribute(k_batch_sample<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024) ==
                cudaSuccess;
            (void)done;
        } else {
            static const bool done =
                cudaFuncSetAttribute(k_batch_sample<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024) ==
                cudaSuccess;
            (void)done;
        }
    }
    if (mi)
        k_batch_sample<true><<<n_blocks, kBatchSampleBlock, smem, s>>>(probs, n, blk_off, funcs, Fmax, pts, fv, vmask,
                                                                       n_zero, n_zero_p);
    else
        k_batch_sample<false><<<n_blocks, kBatchSampleBlock, smem, s>>>(probs, n, blk_off, funcs, Fmax, pts, fv, vmask,
                                                                        n_zero, n_zero_p);
    note_launch();
}

void launch_batch_tets(const BatchProblem* probs, const int64_t* tet_base, int n, int64_t T, int64_t* tets,
                       cudaStream_t s) {
    if (T == 0) return;
    int64_t blocks = (T + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_batch_tets<<<(unsigned)blocks, 256, 0, s>>>(probs, tet_base, n, T, tets);
    note_launch();
}

void launch_batch_ranges(const int64_t* tet_base, int n, const int64_t* verts, int64_t n_verts,
                         const int64_t* face_tet_offsets, const int64_t* face_tets, int64_t n_faces,
                         int64_t* vert_first, int64_t* face_first, cudaStream_t s) {
    k_batch_ranges<<<(unsigned)((n + 1 + 127) / 128), 128, 0, s>>>(tet_base, n, verts, n_verts, face_tet_offsets,
                                                                    face_tets, n_faces, vert_first, face_first);
    note_launch();
}

void launch_batch_active_stats(bool mi, const int64_t* tet_base, int n, const uint32_t* act_tet,
                               const uint64_t* act_mask, int64_t A, unsigned long long* stats4, cudaStream_t s) {
    if (A == 0) return;
    int64_t blocks = (A + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (mi) k_batch_active_stats<true><<<(unsigned)blocks, 256, 0, s>>>(tet_base, n, act_tet, act_mask, A, stats4);
    else k_batch_active_stats<false><<<(unsigned)blocks, 256, 0, s>>>(tet_base, n, act_tet, act_mask, A, stats4);
    note_launch();
}

void launch_check_tets(const int64_t* d_tets, int64_t T, int64_t V, uint32_t* status, cudaStream_t s) {
    if (T == 0) return;
    const int64_t n = 4 * T;
    int64_t blocks = (n + kBlock - 1) / kBlock;
    if (blocks > 152 * 32) blocks = 152 * 32;
    {
        k_check_tets<<<(unsigned)blocks, kBlock, 0, s>>>(d_tets, n, V, status);
        note_launch();
    }
}

int64_t filter_num_blocks(int64_t T) { return (T + kBlock - 1) / kBlock; }

void launch_filter_count(bool mi, const ulonglong2* vmask, const double* fv, int F, const int64_t* d_tets,
                         const GridDesc& g, int64_t T, bool use_table, uint32_t* blk, unsigned long long* khist,
                         cudaStream_t s) {
    const int64_t nb = filter_num_blocks(T);
    if (nb == 0) return;
    TetSrc ts{d_tets, g.res};
    if (mi)
        {
            k_filter_count<true><<<(unsigned)nb, kBlock, 0, s>>>(vmask, fv, F, ts, T, use_table, blk, khist);
            note_launch();
        }
    else
        {
            k_filter_count<false><<<(unsigned)nb, kBlock, 0, s>>>(vmask, fv, F, ts, T, use_table, blk, khist);
            note_launch();
        }
}

void launch_filter_scatter(bool mi, const ulonglong2* vmask, const double* fv, int F, const int64_t* d_tets,
                           const GridDesc& g, int64_t T, bool use_table, const uint32_t* blk_off,
                           const IASum4* table_sum, FilterOut out, cudaStream_t s) {
    const int64_t nb = filter_num_blocks(T);
    if (nb == 0) return;
    TetSrc ts{d_tets, g.res};
    if (mi)
        {
            k_filter_scatter<true><<<(unsigned)nb, kBlock, 0, s>>>(vmask, fv, F, ts, T, use_table, blk_off, table_sum, out);
            note_launch();
        }
    else
        {
            k_filter_scatter<false><<<(unsigned)nb, kBlock, 0, s>>>(vmask, fv, F, ts, T, use_table, blk_off, table_sum, out);
            note_launch();
        }
}

}  // namespace ria
