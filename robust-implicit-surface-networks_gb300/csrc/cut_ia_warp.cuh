// Per-tet implicit arrangement, one warp per tet (the same algorithm and canonical record as
// cut_ia.cuh, which runs one thread per tet).
//
// A heavy tet (four or more planes) is a long chain of plane insertions over tens of vertices and
// faces.  Run by one thread, its state (several KB) lives in local memory, and a warp of such
// threads holds far more state than L1 keeps; run by a warp, the state sits in shared memory and
// each insertion's per-vertex, per-face and per-cell steps run across the lanes:
//   A  the sign of every vertex against the plane (exact predicates)
//   B  the cells the plane crosses (OR-reductions of per-face side masks)
//   C  one new vertex per crossing edge (edges deduplicated in a shared hash, numbered by slot)
//   D  every face rebuilt with its new vertices and split in two when crossed (scans give each
//      face's loop offset and the id of its negative part, in face order as the serial cut does)
//   E  every crossed cell split, its cap face chained from the cap edges of its faces
//   F  cell references of the faces on the negative side
// Vertex ids of step C differ from the serial cut's; the canonical form depends only on labels,
// sign vectors and geometry, so the record is the same byte for byte.
//
// `Lanes` is the cooperating group: a full warp on the device; a single lane on the host, where
// every lane-parallel loop becomes the serial loop (the host build checks the algorithm against
// the oracle without a GPU).
#pragma once
#include "cut_ia.cuh"

namespace ria {

// A group of G lanes of one warp (G = 32: the whole warp; G = 16: either half), lanes numbered
// from 0 within the group.  Ballots return group-relative masks.
template <int G>
struct LanesG {
#if defined(__CUDA_ARCH__)
    static constexpr int W = G;
    int lane;       // within the group
    int base;       // first warp lane of the group
    unsigned mask;  // the group's lanes in the warp
    __device__ __forceinline__ static LanesG of_thread(int warp_lane) {
        LanesG g;
        g.lane = warp_lane & (G - 1);
        g.base = warp_lane & ~(G - 1);
        g.mask = G == 32 ? 0xFFFFFFFFu : (((1u << G) - 1u) << g.base);
        return g;
    }
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
    __device__ __forceinline__ unsigned ballot(bool p) const {
        const unsigned b = __ballot_sync(mask, p);
        return G == 32 ? b : ((b >> base) & ((1u << G) - 1u));
    }
    __device__ __forceinline__ unsigned or_all(unsigned x) const { return __reduce_or_sync(mask, x); }
    __device__ __forceinline__ int add_all(int x) const { return (int)__reduce_add_sync(mask, (unsigned)x); }
    __device__ __forceinline__ int below(unsigned m) const { return __popc(m & ((1u << lane) - 1u)); }
    __device__ __forceinline__ int count(unsigned m) const { return __popc(m); }
    template <class T>
    __device__ __forceinline__ T bcast(T x) const { return __shfl_sync(mask, x, 0, G); }
#else
    static constexpr int W = 1;
    int lane = 0;
    static LanesG of_thread(int) { return LanesG{}; }
    void sync() const {}
    unsigned ballot(bool p) const { return p ? 1u : 0u; }
    unsigned or_all(unsigned x) const { return x; }
    int add_all(int x) const { return x; }
    int below(unsigned) const { return 0; }
    int count(unsigned m) const { return m ? 1 : 0; }
    template <class T>
    T bcast(T x) const { return x; }
#endif
    // exclusive prefix of `x` over the lanes of one round, plus the round's total
    RIA_HD int scan(int x, int& total) const {
#if defined(__CUDA_ARCH__)
        int v = x;
        for (int d = 1; d < G; d <<= 1) {
            int y = __shfl_up_sync(mask, v, d, G);
            if (lane >= d) v += y;
        }
        total = __shfl_sync(mask, v, G - 1, G);
        return v - x;
#else
        total = x;
        return 0;
#endif
    }
};
using Lanes = LanesG<32>;

constexpr int kWarpMaxK = 16;      // active planes of a tet the warp cut takes
constexpr int kEdgeSlots = 128;    // shared hash of the crossing edges of one insertion
constexpr int kCapEdges = 16;      // edges of one cap face

template <int MV, int MF, int ML>
struct IAWarpCut {
    static_assert(MV <= 255 && MF <= 65535, "ids");
    static constexpr int MC = 32;  // cells: one 32-bit mask
    double pl[4 * kWarpMaxK];
    uint8_t rep[kWarpMaxK];
    int k, nv, nf, nc, cur, lused;
    int fail;  // a step that cannot complete: CUT_DEFER (capacity) or CUT_FAIL
    uint8_t lab[MV][3];
    uint64_t mask[MV];
    VCache vc[MV];
    int8_t sg[MV];
    uint8_t fsupp[MF], fpos[MF], fneg[MF];
    uint16_t foff[MF], flen[MF];
    uint8_t loops[2][ML];
    uint64_t csign[MC];
    // per insertion
    int8_t fside[MF];
    uint8_t cwa[MF], cwb[MF];  // cap edge of the face: the two zero vertices bounding its negative run
    int8_t chas[MF];
    uint8_t cneg_of[MC];
    uint16_t capoff[MC];  // loop offset of the cap face of a crossed cell
    // scratch of one step at a time: crossing edges (cd), cap faces (e), canonical
    // form (can)
    union {
        struct {
            uint32_t eslot[kEdgeSlots];  // crossing edge key + 1 (u | w << 8, u < w); 0 = empty
            uint8_t evert[kEdgeSlots];
        } cd;
        struct {
            uint32_t capn[MC];             // cap edges gathered per crossed cell
            uint8_t capet[MC][kCapEdges];  // edge tail and head, oriented outward for the cell
            uint8_t capeh[MC][kCapEdges];
        } e;
        struct {
            uint8_t vnew[MV], vorder[MV], live[MV];
            uint8_t cnew[MC], corder[MC];
            uint16_t forder[MF], floff[MF];
            uint32_t fkey[MF];
        } can;
    } sc;
    int nv_live, loop_total;

    RIA_HD void set_fail(int code) { fail = code; }

    RIA_HD bool build_cache(int v) {
        bool bound[4] = {false, false, false, false};
        const double* rows[3];
        int m = 0;
        for (int t = 0; t < 3; ++t) {
            const int l = lab[v][t];
            if (l < 4)
                bound[l] = true;
            else
                rows[m++] = pl + 4 * (l - 4);
        }
        uint8_t S[4];
        int s = 0;
        for (int c = 0; c < 4; ++c)
            if (!bound[c]) S[s++] = (uint8_t)c;
        return vcache_build(vc[v], false, s, S, m, rows, true);
    }

    RIA_HD int query(int v, const double* q) const {
        const double* rows[3];
        int m = 0;
        for (int t = 0; t < 3; ++t)
            if (lab[v][t] >= 4) rows[m++] = pl + 4 * (lab[v][t] - 4);
        return vcache_query(vc[v], q, rows, true);
    }

    RIA_HD int edge_vertex(int u, int w) const {
        const uint32_t key = (uint32_t)(u < w ? (u | (w << 8)) : (w | (u << 8))) + 1u;
        uint32_t h = (key * 2654435761u) >> 25;
        for (int p = 0; p < kEdgeSlots; ++p) {
            const uint32_t s = sc.cd.eslot[(h + p) & (kEdgeSlots - 1)];
            if (s == key) return sc.cd.evert[(h + p) & (kEdgeSlots - 1)];
            if (s == 0) return -1;
        }
        return -1;
    }

    // the face loop with the new vertices of its crossing edges inserted (n entries)
    RIA_HD int full_loop(int f, uint8_t* full, int cap) const {
        const int L = flen[f];
        int n = 0;
        for (int j = 0; j < L; ++j) {
            const int u = loops[cur][foff[f] + j], w = loops[cur][foff[f] + (j + 1 == L ? 0 : j + 1)];
            if (n >= cap) return -1;
            full[n++] = (uint8_t)u;
            if (sg[u] * sg[w] < 0) {
                if (n >= cap) return -1;
                const int e = edge_vertex(u, w);
                if (e < 0) return -1;
                full[n++] = (uint8_t)e;
            }
        }
        return n;
    }

    // Planes are in pl[0 .. 4k).  Returns CUT_OK, CUT_DEFER (capacity) or CUT_FAIL.
    template <class LT>
    RIA_HDI int run(const LT& L, int kk) {
        const int lane = L.lane;
        if (lane == 0) {
            k = kk;
            fail = CUT_OK;
        }
        L.sync();
        // groups: rep[i] is the smallest plane exactly proportional to plane i (an equivalence on
        // the planes with two or more nonzero values), as ia_group_planes finds it serially
        for (int i = lane; i < kk; i += L.W) {
            const double* a = pl + 4 * i;
            int nz = 0, last = -1;
            for (int c = 0; c < 4; ++c)
                if (a[c] != 0.0) {
                    ++nz;
                    last = c;
                }
            uint8_t r = (uint8_t)(4 + i);
            if (nz == 0) {
                r = 0xFF;
            } else if (nz == 1) {
                r = (uint8_t)last;
            } else {
                for (int j = 0; j < i; ++j) {
                    const double* b = pl + 4 * j;
                    int nzb = 0;
                    for (int c = 0; c < 4; ++c) nzb += b[c] != 0.0;
                    if (nzb < 2) continue;
                    bool prop = true;
                    for (int x = 0; x < 4 && prop; ++x)
                        for (int y = x + 1; y < 4 && prop; ++y)
                            if (!prod_eq(a[x], b[y], a[y], b[x])) prop = false;
                    if (prop) {
                        r = (uint8_t)(4 + j);
                        break;
                    }
                }
            }
            rep[i] = r;
        }
        // the tet
        for (int c = lane; c < 4; c += L.W) {
            int t = 0;
            for (int b = 0; b < 4; ++b)
                if (b != c) lab[c][t++] = (uint8_t)b;
            mask[c] = 0xFull & ~bit64(c);
            sg[c] = 0;
            if (!build_cache(c)) set_fail(CUT_FAIL);
            fsupp[c] = (uint8_t)c;
            fpos[c] = 0;
            fneg[c] = kNoCell;
            foff[c] = (uint16_t)(3 * c);
            flen[c] = 3;
            for (int j = 0; j < 3; ++j) loops[0][3 * c + j] = (uint8_t)tet_face_inward(c, j);
        }
        if (lane == 0) {
            nv = 4;
            nf = 4;
            nc = 1;
            cur = 0;
            lused = 12;
            csign[0] = 0;
        }
        L.sync();
        if (fail != CUT_OK) return fail;

        for (int i = 0; i < kk; ++i) {
            if (rep[i] != 4 + i) continue;
            const int q = 4 + i;
            const double* qv = pl + 4 * i;
            const int nv0 = nv, nf0 = nf, nc0 = nc, nb = cur ^ 1;
            // A: vertex signs
            for (int v = lane; v < nv0; v += L.W) {
                const int s = query(v, qv);
                if (s == 2) set_fail(CUT_FAIL);
                sg[v] = (int8_t)(s == 2 ? 0 : s);
                if (s == 0) mask[v] |= bit64(q);
            }
            for (int t = lane; t < kEdgeSlots; t += L.W) sc.cd.eslot[t] = 0;
            L.sync();
            if (fail != CUT_OK) return fail;
            // B and C in one pass over the faces: the cells the plane crosses (OR-reductions of the
            // faces' side masks) and the crossing edges, into the shared hash (a crossing edge only
            // exists when some face has both signs, so a plane that crosses no cell inserts none)
            unsigned cp = 0, cn = 0;
            for (int f = lane; f < nf0; f += L.W) {
                bool hp = false, hn = false;
                const int Lf = flen[f];
                for (int j = 0; j < Lf; ++j) {
                    const int u = loops[cur][foff[f] + j], w = loops[cur][foff[f] + (j + 1 == Lf ? 0 : j + 1)];
                    const int su = sg[u];
                    hp = hp || su > 0;
                    hn = hn || su < 0;
                    if (su * sg[w] >= 0) continue;
                    const uint32_t key = (uint32_t)(u < w ? (u | (w << 8)) : (w | (u << 8))) + 1u;
                    uint32_t h = (key * 2654435761u) >> 25;
                    bool placed = false;
                    for (int p = 0; p < kEdgeSlots && !placed; ++p) {
                        uint32_t* slot = &sc.cd.eslot[(h + p) & (kEdgeSlots - 1)];
#if defined(__CUDA_ARCH__)
                        const uint32_t old = atomicCAS(slot, 0u, key);
#else
                        const uint32_t old = *slot;
                        if (old == 0) *slot = key;
#endif
                        placed = old == 0 || old == key;
                    }
                    if (!placed) set_fail(CUT_DEFER);
                }
                const unsigned cells = (1u << fpos[f]) | (fneg[f] != kNoCell ? (1u << fneg[f]) : 0u);
                if (hp) cp |= cells;
                if (hn) cn |= cells;
            }
            cp = L.or_all(cp);
            cn = L.or_all(cn);
            const unsigned strad = cp & cn;
            for (int c = lane; c < nc0; c += L.W)
                if (!((strad >> c) & 1) && ((cp >> c) & 1)) csign[c] |= bit64(q);
            L.sync();
            if (!strad) continue;
            if (fail != CUT_OK) return fail;
            // new vertices, numbered by slot
            int added = 0;
            for (int base = 0; base < kEdgeSlots; base += L.W) {
                const int t = base + lane;
                const uint32_t key = sc.cd.eslot[t];
                const unsigned m = L.ballot(key != 0);
                if (key) {
                    const int id = nv0 + added + L.below(m);
                    if (id >= MV) {
                        set_fail(CUT_DEFER);
                    } else {
                        sc.cd.evert[t] = (uint8_t)id;
                        const int u = (int)((key - 1u) & 0xFF), w = (int)((key - 1u) >> 8);
                        const uint64_t em = mask[u] & mask[w];
                        if (popc64u(em) < 2) {  // an edge lies on two planes; guards the labels below
                            set_fail(CUT_FAIL);
                        }
                        const int p1 = popc64u(em) < 2 ? 0 : ctz64(em);
                        const int p2 = popc64u(em) < 2 ? 1 : ctz64(em & ~bit64(p1));
                        lab[id][0] = (uint8_t)p1;
                        lab[id][1] = (uint8_t)p2;
                        lab[id][2] = (uint8_t)q;
                        mask[id] = em | bit64(q);
                        sg[id] = 0;
                        if (!build_cache(id)) set_fail(CUT_FAIL);
                    }
                }
                added += L.count(m);
            }
            L.sync();
            if (fail != CUT_OK) return fail;
            // D: every face rebuilt in one pass: its loop with the new vertices, its split, its cap
            // edge, then (after the round's scans give offsets and ids) its loop(s) written
            int nsplit = 0, nused = 0;
            for (int base = 0; base < nf0; base += L.W) {
                const int f = base + lane;
                int out = 0, n = -1, j0 = -1, lp = 0, ln = 0;
                bool split = false;
                uint8_t full[MV + 8];
                if (f < nf0) {
                    n = full_loop(f, full, MV + 8);
                    if (n < 0) {
                        set_fail(CUT_DEFER);
                    } else {
                        bool hp = false, hn = false;
                        for (int j = 0; j < n; ++j) {
                            hp = hp || sg[full[j]] > 0;
                            hn = hn || sg[full[j]] < 0;
                            lp += sg[full[j]] >= 0;
                            ln += sg[full[j]] <= 0;
                        }
                        chas[f] = 0;
                        for (int j = 0; j < n; ++j) {
                            const int prev = full[j == 0 ? n - 1 : j - 1];
                            if (sg[full[j]] < 0 && sg[prev] >= 0) {
                                j0 = j;
                                break;
                            }
                        }
                        if (j0 >= 0) {
                            int j1 = j0;
                            while (sg[full[(j1 + 1) % n]] < 0) j1 = (j1 + 1) % n;
                            const int wa = full[(j0 - 1 + n) % n], wb = full[(j1 + 1) % n];
                            if (wa != wb) {
                                chas[f] = 1;
                                cwa[f] = (uint8_t)wa;
                                cwb[f] = (uint8_t)wb;
                            }
                        }
                        if (hp && hn) {
                            split = true;
                            fside[f] = 2;
                            out = lp + ln;
                        } else {
                            fside[f] = hp ? 1 : -1;
                            out = n;
                        }
                    }
                }
                int tot_out = 0;
                const int off = L.scan(out, tot_out);
                const unsigned sm = L.ballot(split);
                const bool fits = nused + tot_out <= ML && nf0 + nsplit + L.count(sm) <= MF;
                if (!fits) set_fail(CUT_DEFER);
                if (fits && f < nf0 && n >= 0) {
                    int w = nused + off;
                    if (split) {
                        // positive part keeps id f, negative part becomes face nf0 + rank; it starts at wa
                        const int g = nf0 + nsplit + L.below(sm);
                        fsupp[g] = fsupp[f];
                        fpos[g] = fpos[f];
                        fneg[g] = fneg[f];
                        foff[f] = (uint16_t)w;
                        flen[f] = (uint16_t)lp;
                        for (int j = 0; j < n; ++j)
                            if (sg[full[j]] >= 0) loops[nb][w++] = full[j];
                        foff[g] = (uint16_t)w;
                        flen[g] = (uint16_t)ln;
                        const int jstart = (j0 - 1 + n) % n;
                        for (int t = 0; t < n; ++t) {
                            const int v = full[(jstart + t) % n];
                            if (sg[v] <= 0) loops[nb][w++] = (uint8_t)v;
                        }
                    } else {
                        foff[f] = (uint16_t)w;
                        flen[f] = (uint16_t)n;
                        for (int j = 0; j < n; ++j) loops[nb][w++] = full[j];
                    }
                }
                nused += tot_out;
                nsplit += L.count(sm);
            }
            L.sync();
            if (fail != CUT_OK) return fail;
            const int nf1 = nf0 + nsplit;
            L.sync();
            // E0: the cap edges of the crossed cells, gathered per cell (lanes over faces)
            for (int c = lane; c < nc0; c += L.W) sc.e.capn[c] = 0;
            L.sync();
            for (int f = lane; f < nf0; f += L.W) {
                if (!chas[f]) continue;
                for (int side = 0; side < 2; ++side) {
                    const int c = side ? fneg[f] : fpos[f];
                    if (c == kNoCell || !((strad >> c) & 1)) continue;
#if defined(__CUDA_ARCH__)
                    const uint32_t slot = atomicAdd(&sc.e.capn[c], 1u);
#else
                    const uint32_t slot = sc.e.capn[c]++;
#endif
                    if (slot >= (uint32_t)kCapEdges) continue;
                    // the face loop runs outward for its negative cell
                    sc.e.capet[c][slot] = side ? cwa[f] : cwb[f];
                    sc.e.capeh[c][slot] = side ? cwb[f] : cwa[f];
                }
            }
            L.sync();
            // E1: new cells, cap-face sizes
            int ncells = 0, ncap_used = 0;
            for (int base = 0; base < nc0; base += L.W) {
                const int c = base + lane;
                const bool st = c < nc0 && ((strad >> c) & 1);
                const unsigned m = L.ballot(st);
                int nedge = 0;
                if (st) {
                    const int id = nc0 + ncells + L.below(m);
                    if (id >= MC) set_fail(CUT_DEFER);
                    cneg_of[c] = (uint8_t)(id < MC ? id : 0);
                    nedge = (int)sc.e.capn[c];
                    if (nedge > kCapEdges) set_fail(CUT_DEFER);
                    if (nedge < 3) set_fail(CUT_FAIL);  // an open cap cannot happen with exact signs
                } else if (c < nc0) {
                    cneg_of[c] = kNoCell;
                }
                int tot = 0;
                const int off = L.scan(nedge, tot);
                if (st) capoff[c] = (uint16_t)(nused + ncap_used + off);
                ncells += L.count(m);
                ncap_used += tot;
            }
            if (nf1 + ncells > MF || nused + ncap_used > ML) set_fail(CUT_DEFER);
            L.sync();
            if (fail != CUT_OK) return fail;
            // E2: split cells, chain the cap faces (face id nf1 + rank among the crossed cells)
            for (int c = lane; c < nc0; c += L.W) {
                if (!((strad >> c) & 1)) continue;
                const int id = cneg_of[c];
                const int g = nf1 + (id - nc0);
                csign[id] = csign[c];
                csign[c] |= bit64(q);
                const int nedge = (int)sc.e.capn[c];
                const uint8_t* et = sc.e.capet[c];
                const uint8_t* eh = sc.e.capeh[c];
                int w = capoff[c];
                fsupp[g] = (uint8_t)q;
                fpos[g] = (uint8_t)c;
                fneg[g] = (uint8_t)id;
                foff[g] = (uint16_t)w;
                flen[g] = (uint16_t)nedge;
                int curv = et[0];
                for (int t = 0; t < nedge; ++t) {
                    loops[nb][w++] = (uint8_t)curv;
                    int nxt = -1;
                    for (int e = 0; e < nedge; ++e)
                        if (et[e] == curv) {
                            nxt = eh[e];
                            break;
                        }
                    if (nxt < 0) {
                        set_fail(CUT_FAIL);
                        break;
                    }
                    curv = nxt;
                }
                if (curv != et[0]) set_fail(CUT_FAIL);
            }
            L.sync();
            if (fail != CUT_OK) return fail;
            // F: cell references of faces on the negative side (negative parts and whole faces)
            for (int f = lane; f < nf1; f += L.W) {
                if (f < nf0 && fside[f] != -1) continue;
                if (fpos[f] != kNoCell && cneg_of[fpos[f]] != kNoCell) fpos[f] = cneg_of[fpos[f]];
                if (fneg[f] != kNoCell && cneg_of[fneg[f]] != kNoCell) fneg[f] = cneg_of[fneg[f]];
            }
            L.sync();
            if (lane == 0) {
                nv = nv0 + added;
                nf = nf1 + ncells;
                nc = nc0 + ncells;
                cur = nb;
                lused = nused + ncap_used;
            }
            L.sync();
        }
        return CUT_OK;
    }

    RIA_HD uint32_t vkey(int v) const { return ((uint32_t)lab[v][0] << 16) | ((uint32_t)lab[v][1] << 8) | lab[v][2]; }

    RIA_HD uint32_t face_key(int f) const {
        uint32_t s0 = 0xFF, s1 = 0xFF, s2 = 0xFF;
        for (int j = 0; j < flen[f]; ++j) {
            const uint32_t v = sc.can.vnew[loops[cur][foff[f] + j]];
            if (v < s0) {
                s2 = s1;
                s1 = s0;
                s0 = v;
            } else if (v < s1) {
                s2 = s1;
                s1 = v;
            } else if (v < s2) {
                s2 = v;
            }
        }
        return ((uint32_t)fsupp[f] << 24) | (s0 << 16) | (s1 << 8) | s2;
    }

    RIA_HD bool plane_is_iso(int p) const {
        if (p > 3) return true;
        for (int j = 0; j < k; ++j)
            if (rep[j] == p) return true;
        return false;
    }

    // ranks instead of sorts, ties broken by id as the serial cut's stable insertion sorts do (face
    // ids are the serial cut's: positive parts keep their id, negative parts and cap faces follow in
    // face and cell order)
    template <class LT>
    RIA_HDI void canonicalize(const LT& L) {
        const int lane = L.lane;
        for (int v = lane; v < nv; v += L.W) sc.can.live[v] = 0;
        L.sync();
        for (int f = lane; f < nf; f += L.W)
            for (int j = 0; j < flen[f]; ++j) sc.can.live[loops[cur][foff[f] + j]] = 1;
        L.sync();
        int nl = 0;
        for (int v = lane; v < nv; v += L.W) nl += sc.can.live[v];
        nl = L.add_all(nl);
        for (int v = lane; v < nv; v += L.W) sc.can.fkey[v] = sc.can.live[v] ? vkey(v) : 0xFFFFFFFFu;  // vertex keys first
        L.sync();
        for (int v = lane; v < nv; v += L.W) {
            if (!sc.can.live[v]) continue;
            const uint32_t kv = sc.can.fkey[v];
            int r = 0;
            for (int u = 0; u < nv; ++u) r += sc.can.fkey[u] < kv || (sc.can.fkey[u] == kv && u < v);
            sc.can.vnew[v] = (uint8_t)r;
            sc.can.vorder[r] = (uint8_t)v;
        }
        for (int c = lane; c < nc; c += L.W) {
            int r = 0;
            for (int d = 0; d < nc; ++d) r += csign[d] < csign[c] || (csign[d] == csign[c] && d < c);
            sc.can.cnew[c] = (uint8_t)r;
            sc.can.corder[r] = (uint8_t)c;
        }
        L.sync();
        int lt = 0;
        for (int f = lane; f < nf; f += L.W) {
            sc.can.fkey[f] = face_key(f);
            lt += flen[f];
        }
        lt = L.add_all(lt);
        L.sync();
        for (int f = lane; f < nf; f += L.W) {
            int r = 0;
            for (int g = 0; g < nf; ++g) r += sc.can.fkey[g] < sc.can.fkey[f] || (sc.can.fkey[g] == sc.can.fkey[f] && g < f);  // stable
            sc.can.forder[r] = (uint16_t)f;
        }
        L.sync();
        // loop offsets in sorted order
        int acc = 0;
        for (int base = 0; base < nf; base += L.W) {
            const int i = base + lane;
            const int len = i < nf ? flen[sc.can.forder[i]] : 0;
            int tot = 0;
            const int off = L.scan(len, tot);
            if (i < nf) sc.can.floff[i] = (uint16_t)(acc + off);
            acc += tot;
        }
        if (lane == 0) {
            nv_live = nl;
            loop_total = lt;
        }
        L.sync();
    }

    RIA_HD int record_size() const { return 10 + k + 3 * nv_live + 8 * nf + 2 * loop_total + 8 * nc; }

    // the canonical record (record_size() bytes) and the extraction summary, written by the lanes
    template <class LT>
    RIA_HDI void emit(const LT& L, uint8_t* dst, IASummary& sum) {
        const int lane = L.lane;
        auto w16 = [&](int o, int v) {
            dst[o] = (uint8_t)(v & 0xFF);
            dst[o + 1] = (uint8_t)((v >> 8) & 0xFF);
        };
        if (lane == 0) {
            dst[0] = 1;
            dst[1] = (uint8_t)k;
            w16(2, nv_live);
            w16(4, nf);
            w16(6, nc);
            w16(8, loop_total);
        }
        for (int i = lane; i < k; i += L.W) dst[10 + i] = rep[i];
        const int ov = 10 + k, ofc = ov + 3 * nv_live, olp = ofc + 8 * nf, oc = olp + 2 * loop_total;
        for (int i = lane; i < nv_live; i += L.W)
            for (int t = 0; t < 3; ++t) dst[ov + 3 * i + t] = lab[sc.can.vorder[i]][t];
        for (int v = lane; v < nv; v += L.W) sc.can.live[v] = 0;  // reused: vertex on an iso face
        L.sync();
        int niso = 0, nloop = 0, nbnd = 0;
        for (int i = lane; i < nf; i += L.W) {
            const int f = sc.can.forder[i];
            const int o = ofc + 8 * i;
            dst[o] = fsupp[f];
            dst[o + 1] = (uint8_t)(fneg[f] == kNoCell ? 1 : 0);
            w16(o + 2, sc.can.cnew[fpos[f]]);
            w16(o + 4, fneg[f] == kNoCell ? 0xFFFF : sc.can.cnew[fneg[f]]);
            w16(o + 6, flen[f]);
            const int Lf = flen[f];
            const bool iso = plane_is_iso(fsupp[f]);
            if (iso) {
                ++niso;
                nloop += Lf;
                if (fneg[f] == kNoCell) ++nbnd;
            }
            int jm = 0;
            for (int j = 1; j < Lf; ++j)
                if (sc.can.vnew[loops[cur][foff[f] + j]] < sc.can.vnew[loops[cur][foff[f] + jm]]) jm = j;
            for (int t = 0; t < Lf; ++t) {
                const int v = loops[cur][foff[f] + (jm + t) % Lf];
                w16(olp + 2 * (sc.can.floff[i] + t), sc.can.vnew[v]);
                if (iso) sc.can.live[v] = 1;
            }
        }
        for (int i = lane; i < nc; i += L.W) {
            const uint64_t s = csign[sc.can.corder[i]];
            for (int b = 0; b < 8; ++b) dst[oc + 8 * i + b] = (uint8_t)((s >> (8 * b)) & 0xFF);
        }
        niso = L.add_all(niso);
        nloop = L.add_all(nloop);
        nbnd = L.add_all(nbnd);
        L.sync();
        int nisov = 0;
        for (int v = lane; v < nv; v += L.W) nisov += sc.can.live[v];
        nisov = L.add_all(nisov);
        sum.n_iso_v = (uint16_t)nisov;
        sum.n_iso_f = (uint16_t)niso;
        sum.n_iso_loop = (uint16_t)nloop;
        sum.n_bnd_f = (uint16_t)nbnd;
    }
};

}  // namespace ria
