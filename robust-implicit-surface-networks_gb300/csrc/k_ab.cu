// Stages (a) and (b): sampling the implicit functions at the grid vertices, per-vertex sign /
// argmax masks, and the ordered compaction of the active tets.
//
//   sampling     the external implicit_functions library (app/implicit_arrangement.cpp:59);
//                formulas in include/ria.h.  One thread per (vertex, function) element of the
//                row-major V x F matrix, so stores are coalesced; a block stages a 32-vertex tile in
//                shared memory and derives the per-vertex masks from it.
//   IA signs     src/implicit_arrangement.cpp:53-77   (pos/neg bit masks, F <= 64)
//   IA filter    src/implicit_arrangement.cpp:82-116  (active = not all corners strictly + and not
//                all strictly -:  ~(p0&p1&p2&p3 | n0&n1&n2&n3))
//   MI argmax    src/material_interface.cpp:53-92     (mask of the materials equal to the maximum)
//   MI filter    src/material_interface.cpp:94-152
// The compaction keeps tet order (per-block counts, an exclusive scan, warp-ballot ranks) so the
// active-function CRS and the first-occurrence numbering of the extraction follow the reference.
#include "device_common.cuh"
#include "launch.hpp"

namespace ria {

namespace {

constexpr int kTileV = 32;
constexpr int kBlock = 256;

__device__ __forceinline__ double eval_function(const ria_function& f, double x, double y, double z) {
    double v = 0.0;
    switch (f.type) {
        case RIA_FUNC_PLANE:
            v = (f.p[3] * (x - f.p[0]) + f.p[4] * (y - f.p[1])) + f.p[5] * (z - f.p[2]);
            break;
        case RIA_FUNC_SPHERE:
        case RIA_FUNC_SPHERE_SQUARED: {
            double dx = x - f.p[0], dy = y - f.p[1], dz = z - f.p[2];
            double d2 = (dx * dx + dy * dy) + dz * dz;
            v = (f.type == RIA_FUNC_SPHERE) ? f.p[3] - sqrt(d2) : f.p[3] * f.p[3] - d2;
            break;
        }
        case RIA_FUNC_CYLINDER: {
            double vx = x - f.p[0], vy = y - f.p[1], vz = z - f.p[2];
            double t = (vx * f.p[3] + vy * f.p[4]) + vz * f.p[5];
            double wx = vx - t * f.p[3], wy = vy - t * f.p[4], wz = vz - t * f.p[5];
            v = f.p[6] - sqrt((wx * wx + wy * wy) + wz * wz);
            break;
        }
        case RIA_FUNC_TORUS: {
            double vx = x - f.p[0], vy = y - f.p[1], vz = z - f.p[2];
            double h = (vx * f.p[3] + vy * f.p[4]) + vz * f.p[5];
            double wx = vx - h * f.p[3], wy = vy - h * f.p[4], wz = vz - h * f.p[5];
            double rho = sqrt((wx * wx + wy * wy) + wz * wz);
            double a = rho - f.p[6];
            v = f.p[7] - sqrt(a * a + h * h);
            break;
        }
        default:
            v = 0.0;
    }
    return f.flipped ? -v : v;
}

// masks of one vertex row held in shared memory
template <bool MI>
__device__ __forceinline__ ulonglong2 row_masks(const double* row, int F, int& nzero) {
    ulonglong2 m;
    if (!MI) {
        uint64_t pos = 0, neg = 0;
        for (int f = 0; f < F; ++f) {
            double x = row[f];
            if (x > 0.0) pos |= bit64(f);
            else if (x < 0.0) neg |= bit64(f);
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

template <bool MI>
__global__ void __launch_bounds__(kBlock) k_sample_grid(const ria_function* __restrict__ funcs, int F, PtSrc ps,
                                                        int64_t V, double* __restrict__ fv,
                                                        ulonglong2* __restrict__ vmask,
                                                        unsigned long long* __restrict__ n_zero) {
    extern __shared__ double tile[];
    const int stride = F + 1;
    const int64_t v0 = (int64_t)blockIdx.x * kTileV;
    const int nel = kTileV * F;
    for (int e = threadIdx.x; e < nel; e += blockDim.x) {
        int lv = e / F, f = e - lv * F;
        int64_t v = v0 + lv;
        if (v < V) {
            double p[3];
            ps.get(v, p);
            double val = eval_function(funcs[f], p[0], p[1], p[2]);
            fv[v * F + f] = val;
            tile[lv * stride + f] = val;
        }
    }
    __syncthreads();
    int nz = 0;
    if (threadIdx.x < kTileV) {
        int64_t v = v0 + threadIdx.x;
        if (v < V) vmask[v] = row_masks<MI>(tile + threadIdx.x * stride, F, nz);
    }
    if (threadIdx.x < 32) block_add(n_zero, nz);
}

__global__ void __launch_bounds__(kBlock) k_sample_points(const ria_function* __restrict__ funcs, int F,
                                                          const double* __restrict__ pts, int64_t V,
                                                          double* __restrict__ fv) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= V * F) return;
    int64_t v = e / F;
    int f = (int)(e - v * F);
    fv[e] = eval_function(funcs[f], pts[3 * v], pts[3 * v + 1], pts[3 * v + 2]);
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

template <bool MI>
__global__ void __launch_bounds__(kBlock) k_filter_count(const ulonglong2* __restrict__ vmask,
                                                         const double* __restrict__ fv, int F, TetSrc ts, int64_t T,
                                                         bool use_table, uint32_t* __restrict__ blk,
                                                         unsigned long long* __restrict__ khist) {
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
    int na = __syncthreads_count(act);
    int ng = __syncthreads_count(gen);
    int h0 = __syncthreads_count(k == ka);
    int h1 = __syncthreads_count(k == ka + 1);
    int h2 = __syncthreads_count(k > ka + 1);
    if (threadIdx.x == 0) {
        blk[blockIdx.x] = (uint32_t)na;
        blk[gridDim.x + blockIdx.x] = (uint32_t)ng;
        if (h0) atomicAdd(&khist[0], (unsigned long long)h0);
        if (h1) atomicAdd(&khist[1], (unsigned long long)h1);
        if (h2) atomicAdd(&khist[2], (unsigned long long)h2);
    }
}

template <bool MI>
__global__ void __launch_bounds__(kBlock) k_filter_scatter(const ulonglong2* __restrict__ vmask,
                                                           const double* __restrict__ fv, int F, TetSrc ts,
                                                           int64_t T, bool use_table,
                                                           const uint32_t* __restrict__ blk_off,
                                                           const IASum4* __restrict__ table_sum, FilterOut out) {
    __shared__ int wa[kBlock / 32], wg[kBlock / 32];
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
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1;
    unsigned ba = __ballot_sync(0xFFFFFFFFu, isact), bg = __ballot_sync(0xFFFFFFFFu, isgen);
    if (lane == 0) {
        wa[warp] = __popc(ba);
        wg[warp] = __popc(bg);
    }
    __syncthreads();
    int pa = 0, pg = 0;
    for (int w = 0; w < warp; ++w) {
        pa += wa[w];
        pg += wg[w];
    }
    const uint32_t base_a = blk_off[blockIdx.x];
    const uint32_t base_g = blk_off[gridDim.x + blockIdx.x] - blk_off[gridDim.x];
    if (isact) {
        uint32_t a = base_a + pa + __popc(ba & lt);
        out.act_tet[a] = (uint32_t)t;
        out.act_mask[a] = act;
        if (isgen) {
            out.gen[base_g + pg + __popc(bg & lt)] = a;
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

PtSrc grid_pts(const GridDesc& g) {
    PtSrc p;
    p.pts = nullptr;
    p.res = g.res;
    for (int a = 0; a < 3; ++a) {
        p.bmin[a] = g.bmin[a];
        p.bmax[a] = g.bmax[a];
    }
    return p;
}

}  // namespace

void launch_sample_grid(bool mi, const ria_function* d_funcs, int F, const GridDesc& g, double* fv,
                        ulonglong2* vmask, unsigned long long* n_zero, cudaStream_t s) {
    const int64_t N = g.res + 1;
    const int64_t V = N * N * N;
    const int64_t blocks = (V + kTileV - 1) / kTileV;
    const size_t smem = sizeof(double) * kTileV * (F + 1);
    if (mi)
        {
            k_sample_grid<true><<<(unsigned)blocks, kBlock, smem, s>>>(d_funcs, F, grid_pts(g), V, fv, vmask, n_zero);
            note_launch();
        }
    else
        {
            k_sample_grid<false><<<(unsigned)blocks, kBlock, smem, s>>>(d_funcs, F, grid_pts(g), V, fv, vmask, n_zero);
            note_launch();
        }
}

void launch_sample_points(const ria_function* d_funcs, int F, const double* pts, int64_t V, double* fv, cudaStream_t s) {
    const int64_t n = V * F;
    if (n == 0) return;
    {
        k_sample_points<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(d_funcs, F, pts, V, fv);
        note_launch();
    }
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
